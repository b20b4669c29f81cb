"""In-tree build of libnqes.so (CUDA, sm_103a) and the drop-in executables.

    python nqes-trapped-ion_gb300/build.py [--verbose]

Translation units are compiled in parallel with one -gencode for sm_103a and
linked into nqes-trapped-ion_gb300/lib/libnqes.so. No cmake, no torch
extension machinery: the library is a plain C-ABI shared object.
"""
import concurrent.futures as cf
import os
import shutil
import struct
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["kernels_sample.cu", "kernels_sample_mixed.cu", "kernels_sample_warp.cu", "kernels_sample_warp_k34.cu",
           "kernels_solve.cu", "kernels_sv_fused.cu", "kernels_factored.cu", "kernels_factored_tc.cu", "nqes_api.cu",
           "sv_static.cu", "nqes_server.cc"]
HEADERS = ["nqes_math.cuh", "pcg64.cuh", "nqes_internal.h", "tma_stage.cuh", "sample_warp.cuh", "tc_util.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnqes")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "nqes.h")]
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc(), "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE,
           "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build_library(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    lib = os.path.join(LIBDIR, "libnqes.so")
    if _stale(lib, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", lib, *objs, "-lcudart", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libnqes.so failed:\n{r.stderr}")
    return lib




# ---- drop-in executables ----
CLI = os.path.join(PKG, "cli")
BINDIR = os.path.join(PKG, "bin")
CLI_SOURCES = ["cmdline.cc", "matv5.cc"]
CLI_HEADERS = ["cmdline.h", "matv5.h", "small_eig.h"]
JMATDIR = os.path.join(CLI, "jmat")
# The reference's build list (code/build.sh:28), the K=4 precision shape and
# N50 M150 K2, the shape of the reference's published trapped-ion runs
# (data/energy/ion_N50_M150_K2_*).
DEFAULT_SHAPES = [(8, 16, 2), (8, 32, 2), (16, 32, 2), (16, 64, 2), (32, 64, 2), (32, 128, 2), (64, 128, 2),
                  (64, 256, 2), (128, 256, 2), (64, 128, 4), (50, 150, 2)]


def jmat_header(n):
    """Jmat{n}.h in the build folder: the reference's compiled-in couplings
    (code/build.sh:34 writes them with code/load_jmat.py) as
    `RealScalar Jmat[n][n]`, each value an exact hexadecimal floating literal,
    from cli/jmat/Ising2d_N{n}_alpha1.0.f64 (raw little-endian float64,
    row-major; written by cli/jmat/make_jmat.py). None when there is no file for n."""
    src = os.path.join(JMATDIR, f"Ising2d_N{n}_alpha1.0.f64")
    if not os.path.exists(src):
        return None
    os.makedirs(OBJDIR, exist_ok=True)
    hdr = os.path.join(OBJDIR, f"Jmat{n}.h")
    if _stale(hdr, [src]):
        with open(src, "rb") as f:
            raw = f.read()
        if len(raw) != 8 * n * n:
            raise RuntimeError(f"{src}: {len(raw)} bytes, expected {8 * n * n}")
        vals = struct.unpack(f"<{n * n}d", raw)
        rows = ["{" + ",".join(float.hex(v) for v in vals[i * n:(i + 1) * n]) + "}" for i in range(n)]
        tmp = hdr + ".tmp"
        with open(tmp, "w") as f:
            f.write(f"RealScalar Jmat[{n}][{n}] = {{\n" + ",\n".join(rows) + "};\n")
        os.replace(tmp, hdr)
    return hdr


def _gxx():
    return shutil.which("g++") or "g++"


def _cli_object(src):
    obj = os.path.join(OBJDIR, "cli_" + os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CLI, src)] + [os.path.join(CLI, h) for h in CLI_HEADERS]
    if _stale(obj, deps):
        r = subprocess.run([_gxx(), "-std=c++20", "-O2", "-fPIC", "-c", os.path.join(CLI, src), "-o", obj],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {src}:\n{r.stderr}")
    return obj


def _cli_binary(shape, objs, lib):
    n, m, k = shape
    name = f"rbm-matfree-N{n}-M{m}-K{k}-opt"
    out = os.path.join(BINDIR, name)
    jh = jmat_header(n)
    deps = [os.path.join(CLI, "rbm_main.cc"), lib, os.path.join(INCLUDE, "nqes.h")] + objs + \
        [os.path.join(CLI, h) for h in CLI_HEADERS] + ([jh] if jh else [])
    if _stale(out, deps):
        jdef = [f'-DJMAT_INC="{os.path.basename(jh)}"', "-I", OBJDIR] if jh else []
        cmd = [_gxx(), "-std=c++20", "-O2", f"-DNUM_SPINS={n}", f"-DNUM_HIDDEN_UNITS={m}", f"-DNUM_EIGENSTATES={k}",
               *jdef, "-I", INCLUDE, "-I", CLI, os.path.join(CLI, "rbm_main.cc"), *objs, "-L", LIBDIR, "-lnqes",
               "-Wl,-rpath,$ORIGIN/../lib", "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {name}:\n{r.stderr}")
    if n <= 16:  # the reference names its N <= 16 builds without "matfree"
        alias = os.path.join(BINDIR, f"rbm-N{n}-M{m}-K{k}-opt")
        if not os.path.exists(alias):
            os.symlink(name, alias)
    return out


def build_cli(shapes=None):
    """Builds rbm-matfree-N{N}-M{M}-K{K}-opt for each (N, M, K)."""
    lib = build_library()
    os.makedirs(BINDIR, exist_ok=True)
    objs = [_cli_object(s) for s in CLI_SOURCES]
    for n in sorted({sh[0] for sh in (shapes or DEFAULT_SHAPES)}):
        jmat_header(n)  # before the parallel links: shapes that share N share the header
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        return list(ex.map(lambda sh: _cli_binary(sh, objs, lib), shapes or DEFAULT_SHAPES))


def main():
    print(build_library(verbose="--verbose" in sys.argv))
    for b in build_cli():
        print(b)


if __name__ == "__main__":
    main()
