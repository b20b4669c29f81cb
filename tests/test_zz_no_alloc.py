"""nqes_apply_S_static: S·v for callers that cannot call cudaMalloc (code
running inside a CUDA graph capture, hosts whose device memory belongs to
their own pool allocator, loops that cannot take cudaMalloc's implicit
synchronisation). The entry point works on device buffers the caller already
owns and keeps its intermediates in the library's fixed 16 MiB device array.

The test allocates the caller's buffers itself (as such a caller would have
done up front), calls the entry point through the C ABI twice in a row, and
checks each result against the CPU oracle's S·v (the matrix-free operator of
code/rbm.cc:660-683 over the oracle's own samples, which are the GPU's bit for
bit) and against the context-based nqes_apply_S, to the 1e-11 relative
tolerance of the other S·v parity tests. It also checks that sizes beyond the
array are refused with a message, including sizes whose sum would overflow.
This file is collected last so that a failure here comes after every other
test ran."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
import helpers

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


@pytest.mark.parametrize("real", [True, False])
def test_static_scratch_sv_matches_apply_S(pkg, real):
    torch = pytest.importorskip("torch")
    N, M, K = 8, 16, 2
    J = helpers.synthetic_j(N)
    weights = helpers.random_weights(N, M, K, 0.1, 5, real=real)
    ctx = pkg.Context(N, M, K, J, 0.595)
    ctx.set_weights(*weights)
    orc = helpers.Oracle(N, M, K, J, 0.595)
    orc.set_weights(*weights)
    chains, m = 16, 25
    ctx.sr_step(777, chains, m, 8, 0.1, 2.0, 1e-9, 500)
    orc.sr_step(777, chains, m, 8, 0.1, 2.0, 1e-9, 500, store_o=True)
    assert np.array_equal(ctx.get_samples()[0], orc.samples(chains * m)[0])
    ns, P = chains * m, ctx.P
    O = ctx.get_O(0, ns)
    o, skk, _ = ctx.get_moments()
    dt = np.float64 if real else np.complex128
    conv = (lambda z: np.ascontiguousarray(z.real)) if real else (lambda z: np.ascontiguousarray(z))
    dev = lambda z: torch.from_numpy(conv(z).view(np.float64).copy()).cuda()
    O_d, o_d, skk_d = dev(O), dev(o), dev(skk)
    out_d = torch.empty_like(o_d)
    lib = pkg.load_library()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(3)
    for call in range(2):
        v = rng.normal(size=P) + (0 if real else 1j) * rng.normal(size=P)
        v_d = dev(v)
        st = lib.nqes_apply_S_static(ctypes.c_void_p(O_d.data_ptr()), ctypes.c_void_p(o_d.data_ptr()),
                                     ctypes.c_void_p(skk_d.data_ptr()), ctypes.c_void_p(v_d.data_ptr()),
                                     ctypes.c_void_p(out_d.data_ptr()), ns, P, 0 if real else 1, stream)
        assert st == pkg.OK, lib.nqes_last_error(None)
        torch.cuda.synchronize()
        got = out_d.cpu().numpy().view(np.float64 if real else np.complex128)
        for want in (orc.apply_S(v), ctx.apply_S(v)):
            if real:
                want = want.real
            assert rel_err(got, want) < 1e-11, (call, rel_err(got, want))
    # Sizes beyond the static array are refused, with a description.
    st = lib.nqes_apply_S_static(ctypes.c_void_p(O_d.data_ptr()), ctypes.c_void_p(o_d.data_ptr()),
                                 ctypes.c_void_p(skk_d.data_ptr()), ctypes.c_void_p(v_d.data_ptr()),
                                 ctypes.c_void_p(out_d.data_ptr()), 1 << 40, P, 0, stream)
    assert st == pkg.ERR_INVALID
    assert b"static scratch" in lib.nqes_last_error(None)
    # n_samples + n_params would wrap around in 64 bits: refused all the same
    big = (1 << 63) - 1
    for ns_, p_ in ((big, big), (big, P), (ns, big)):
        st = lib.nqes_apply_S_static(ctypes.c_void_p(O_d.data_ptr()), ctypes.c_void_p(o_d.data_ptr()),
                                     ctypes.c_void_p(skk_d.data_ptr()), ctypes.c_void_p(v_d.data_ptr()),
                                     ctypes.c_void_p(out_d.data_ptr()), ns_, p_, 0, stream)
        assert st == pkg.ERR_INVALID, (ns_, p_)
        assert b"static scratch" in lib.nqes_last_error(None)
    ctx.close()
