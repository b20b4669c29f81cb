// Drop-in executable rbm-matfree-N{N}-M{M}-K{K}-opt.
//
// The shape is fixed at compile time (NUM_SPINS, NUM_HIDDEN_UNITS,
// NUM_EIGENSTATES), as in the reference's build (code/build.sh:28-42); every
// SR step, the correlation stage and all device work run in libnqes through
// its C ABI. This file is the host orchestration of code/rbm.cc:1121-1327
// (run, main): seed handling and the "Random seed is" line, weight loading /
// initialisation / gauge, the lrate and lambda schedules, per-step sorted
// per-site energies in Eigen's row-vector format, the convergence test, the
// correlation functions written with --correlation-data, --dump-rbm, and the
// exit codes (1 for -c 0, 127 for a floating-point error with
// --throw-fperror, 255 for command-line errors).

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "cmdline.h"
#include "matv5.h"
#include "nqes.h"
#include "small_eig.h"

#ifndef NUM_SPINS
#error "NUM_SPINS, NUM_HIDDEN_UNITS and NUM_EIGENSTATES must be defined"
#endif

using nqes_cli::cplx;
using nqes_cli::MatArray;
using nqes_cli::Model;

namespace {

constexpr int N = NUM_SPINS, M = NUM_HIDDEN_UNITS, K = NUM_EIGENSTATES;

// Errors reported like the reference's uncaught exceptions (code/except.h).
class CliError : public std::exception {
    std::string msg_;

public:
    explicit CliError(std::string m) : msg_(std::move(m)) {}
    const char *what() const noexcept override { return msg_.c_str(); }
};
class MatioCreateFileError : public CliError {
public:
    explicit MatioCreateFileError(const std::string &f) : CliError("libmatio: failed to open/create file " + f + ".") {}
};
class MatioReadVarError : public CliError {
public:
    explicit MatioReadVarError(const std::string &v) : CliError("libmatio: failed to read variable " + v + ".") {}
};
class MatioInvalidVarError : public CliError {
public:
    MatioInvalidVarError(const std::string &v, const std::string &why)
        : CliError("libmatio: variable " + v + " is invalid (" + why + ")") {}
};

struct Weights {
    std::vector<cplx> a, b, w;  // K×N, K×M, K×N×M (library layout)
    explicit Weights(int k = K) : a(size_t(k) * N), b(size_t(k) * M), w(size_t(k) * N * M) {}
};

// load_rbm (code/rbm.cc:272-385): complex double a (K×N), b (K×M), w (K×N×M),
// stored column-major.
Weights load_rbm(const std::string &fname, int kk) {
    std::map<std::string, MatArray> vars;
    std::string err;
    if (!nqes_cli::mat_read(fname, vars, err)) throw MatioCreateFileError(fname);
    auto get = [&](const char *name, bool check_type_first, int rank, std::vector<size_t> dims) -> const MatArray & {
        auto it = vars.find(name);
        if (it == vars.end()) throw MatioReadVarError(name);
        const MatArray &v = it->second;
        if (check_type_first) {
            if (!v.is_double) throw MatioInvalidVarError(name, "floating point type mismatch");
            if (!v.is_complex) throw MatioInvalidVarError(name, "not a complex matrix");
        } else {
            if (!v.is_complex) throw MatioInvalidVarError(name, "not a complex matrix");
            if (!v.is_double) throw MatioInvalidVarError(name, "floating point type mismatch");
        }
        if (int(v.dims.size()) != rank)
            throw MatioInvalidVarError(name, rank == 2 ? "not a rank 2 matrix" : "not a rank 3 matrix");
        for (int d = 0; d < rank; d++)
            if (v.dims[d] != dims[d]) {
                if (rank == 2) throw MatioInvalidVarError(name, d == 0 ? "invalid row dimension" : "invalid column dimension");
                throw MatioInvalidVarError(name, "invalid dimension " + std::to_string(d));
            }
        return v;
    };
    const MatArray &a = get("a", true, 2, {size_t(kk), size_t(N)});
    const MatArray &b = get("b", false, 2, {size_t(kk), size_t(M)});
    const MatArray &w = get("w", true, 3, {size_t(kk), size_t(N), size_t(M)});
    Weights r(kk);
    for (int k = 0; k < kk; k++) {
        for (int i = 0; i < N; i++) r.a[k * N + i] = cplx(a.re[i * kk + k], a.im[i * kk + k]);
        for (int j = 0; j < M; j++) r.b[k * M + j] = cplx(b.re[j * kk + k], b.im[j * kk + k]);
        for (int i = 0; i < N; i++)
            for (int j = 0; j < M; j++) {
                const size_t src = size_t(j) * kk * N + size_t(i) * kk + k;
                r.w[(size_t(k) * N + i) * M + j] = cplx(w.re[src], w.im[src]);
            }
    }
    return r;
}

// dump_rbm (code/rbm.cc:405-471): <prefix>N{N}M{M}K{K}.mat, uncompressed.
void dump_rbm(const Weights &r, const std::string &prefix) {
    std::ostringstream ss;
    ss << prefix << "N" << N << "M" << M << "K" << K << ".mat";
    MatArray a, b, w;
    a.dims = {size_t(K), size_t(N)};
    b.dims = {size_t(K), size_t(M)};
    w.dims = {size_t(K), size_t(N), size_t(M)};
    a.is_complex = b.is_complex = w.is_complex = true;
    a.re.resize(K * N); a.im.resize(K * N);
    b.re.resize(K * M); b.im.resize(K * M);
    w.re.resize(size_t(K) * N * M); w.im.resize(size_t(K) * N * M);
    for (int k = 0; k < K; k++) {
        for (int i = 0; i < N; i++) {
            a.re[i * K + k] = r.a[k * N + i].real();
            a.im[i * K + k] = r.a[k * N + i].imag();
        }
        for (int j = 0; j < M; j++) {
            b.re[j * K + k] = r.b[k * M + j].real();
            b.im[j * K + k] = r.b[k * M + j].imag();
        }
        for (int i = 0; i < N; i++)
            for (int j = 0; j < M; j++) {
                const size_t dst = size_t(j) * K * N + size_t(i) * K + k;
                w.re[dst] = r.w[(size_t(k) * N + i) * M + j].real();
                w.im[dst] = r.w[(size_t(k) * N + i) * M + j].imag();
            }
    }
    std::string err;
    if (!nqes_cli::mat_write(ss.str(), {{"a", a}, {"b", b}, {"w", w}}, err)) throw MatioCreateFileError(ss.str());
}

// dump_corrs (code/rbm.cc:828-889): real x, z (N×K) and xx, zz (N×N×K).
void dump_corrs(const std::vector<double> &x, const std::vector<double> &z, const std::vector<double> &xx,
                const std::vector<double> &zz, const std::string &fname) {
    MatArray X, Z, XX, ZZ;
    X.dims = Z.dims = {size_t(N), size_t(K)};
    XX.dims = ZZ.dims = {size_t(N), size_t(N), size_t(K)};
    X.re.resize(N * K); Z.re.resize(N * K);
    XX.re.resize(size_t(N) * N * K); ZZ.re.resize(size_t(N) * N * K);
    for (int k = 0; k < K; k++) {
        for (int i = 0; i < N; i++) {
            X.re[k * N + i] = x[i * K + k];
            Z.re[k * N + i] = z[i * K + k];
        }
        for (int j = 0; j < N; j++)
            for (int i = 0; i < N; i++) {
                XX.re[size_t(k) * N * N + j * N + i] = xx[(size_t(i) * N + j) * K + k];
                ZZ.re[size_t(k) * N * N + j * N + i] = zz[(size_t(i) * N + j) * K + k];
            }
    }
    std::string err;
    if (!nqes_cli::mat_write(fname, {{"x", X}, {"z", Z}, {"xx", XX}, {"zz", ZZ}}, err)) throw MatioCreateFileError(fname);
}

// The coupling of each model in the lower triangle of J: the ising-like
// models as 2 sum_{i>j} J_ij s_i s_j (code/rbm.cc:963-1031), the
// Heisenberg-like ones as sum_{i>j} J_ij (sx sx + sy sy + delta sz sz)
// (code/rbm.cc:1064-1089).
std::vector<double> build_J(const nqes_cli::CmdArgs &args) {
    std::vector<double> J(size_t(N) * N, 0.0);
    switch (args.model) {
    case Model::HS:  // J_ij = 1 / d_ij^2, d_ij = (N / pi) sin(pi (i - j) / N)
        for (int i = 1; i < N; i++)
            for (int j = 0; j < i; j++) {
                const double d = std::sin(M_PI * (i - j) / N) * N / M_PI;
                J[i * N + j] = 1.0 / (d * d);
            }
        break;
    case Model::XXZ:  // -1 on the bonds of the periodic chain
        for (int i = 1; i < N; i++) J[i * N + i - 1] = -1.0;
        if (N > 2) J[(N - 1) * N + 0] = -1.0;
        break;
    case Model::Ising:  // -sum_i s_i s_{i-1}
        for (int i = 1; i < N; i++) J[i * N + i - 1] = -0.5;
        break;
    case Model::PeriodicIsing:  // -sum_i s_i s_{i-1 mod N}
        for (int i = 1; i < N; i++) J[i * N + i - 1] = -0.5;
        if (N > 1) J[(N - 1) * N + 0] += -0.5;
        break;
    case Model::LongRange:  // 2 sum_{i>j} (i-j)^-0.2 s_i s_j
        for (int i = 1; i < N; i++)
            for (int j = 0; j < i; j++) J[i * N + j] = std::pow(double(i - j), -0.2);
        break;
    case Model::TrappedIon:
    default:
        if (args.jmat == "synthetic") {
            // the power-law chain J_ij = |i-j|^-1.2 (max |J| = 1) of the benchmark inputs
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++) J[i * N + j] = i == j ? 0.0 : std::pow(double(std::abs(i - j)), -1.2);
        } else if (!args.jmat.empty()) {
            std::map<std::string, MatArray> vars;
            std::string err;
            if (!nqes_cli::mat_read(args.jmat, vars, err)) throw MatioCreateFileError(args.jmat);
            auto it = vars.find("J");
            if (it == vars.end()) throw MatioReadVarError("J");
            if (it->second.dims.size() != 2 || it->second.dims[0] != size_t(N) || it->second.dims[1] != size_t(N))
                throw MatioInvalidVarError("J", "not an N x N matrix");
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++) J[i * N + j] = it->second.re[size_t(j) * N + i];
        } else {
#ifdef JMAT_INC
            // The reference's compiled-in couplings (code/build.sh:34-41, code/rbm.cc:1015):
            // Jmat/Ising2d_N{N}_alpha1.0.mat, generated into Jmat{N}.h by build.py.
            using RealScalar = double;
#include JMAT_INC
            static_assert(sizeof(Jmat) == sizeof(double) * N * N, "Jmat must be N x N");
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++) J[i * N + j] = Jmat[i][j];
#else
            // The reference has no Jmat file for this N and would not compile.
            throw CliError("no compiled-in trapped-ion couplings for N = " + std::to_string(N) +
                           "; pass --jmat <file.mat> or --jmat synthetic");
#endif
        }
        break;
    }
    return J;
}

// Eigen's default row-vector output: each value at the stream precision,
// right-aligned to the widest, separated by one space.
void print_row(const std::vector<double> &v) {
    std::vector<std::string> s;
    size_t width = 0;
    for (double x : v) {
        std::ostringstream o;
        o << x;
        s.push_back(o.str());
        width = std::max(width, s.back().size());
    }
    for (size_t t = 0; t < v.size(); t++) {
        if (t) std::cout << " ";
        std::cout << std::setw(int(width)) << s[t];
    }
    std::cout << std::endl;
}

void check(nqes_ctx *ctx, int st) {
    if (st != NQES_OK) {
        std::cerr << "nqes: " << nqes_last_error(ctx) << std::endl;
        std::exit(1);
    }
}

// --throw-fperror: the reference traps FP exceptions and exits 127
// (code/rbm.cc:1248-1292). Here the library reports non-finite values as
// NQES_ERR_NONFINITE, and the host checks its own results, instead of a
// hardware trap (which would also fire inside the CUDA runtime).
void fp_error_exit() {
    std::cerr << "Floating point error occured. Exiting." << std::endl;
    std::exit(127);
}

// --dump-states / --dump-ham / --dump-deriv (code/rbm.cc:473-524, 1150-1172):
// Phi, E = Phi^+ H Phi or the log-derivatives O at every multi-spin
// configuration (row k = bits k N .. k N + N - 1 of the enumeration index),
// evaluated on the device in chunks, written as the complex variable "s" of
// <prefix>N{N}M{M}K{K}.mat, dimensions [2^(K N), rows, cols] without the
// singleton ones, column-major. Only built for K N < 32, as the reference.
enum class DumpWhat { Phi, E, O };
void dump_states(nqes_ctx *ctx, const std::string &prefix, DumpWhat what) {
    if (N * K >= 32) return;
    constexpr int L = N + M + N * M, P = K * L;
    const uint64_t n = 1ULL << (K * N), mask = (1ULL << N) - 1;
    const int rows = what == DumpWhat::O ? P : K, cols = what == DumpWhat::O ? 1 : K;
    MatArray s;
    s.is_complex = true;
    s.dims = {size_t(n)};
    if (rows > 1) s.dims.push_back(size_t(rows));
    if (cols > 1) s.dims.push_back(size_t(cols));
    s.re.assign(size_t(n) * rows * cols, 0.0);
    s.im.assign(size_t(n) * rows * cols, 0.0);
    const uint64_t chunk = 1ULL << 14;
    std::vector<uint64_t> cfg(chunk * K);
    std::vector<cplx> out(chunk * size_t(rows) * cols);
    for (uint64_t base = 0; base < n; base += chunk) {
        const int cnt = int(std::min<uint64_t>(chunk, n - base));
        for (int c = 0; c < cnt; c++)
            for (int k = 0; k < K; k++) cfg[size_t(c) * K + k] = ((base + c) >> (k * N)) & mask;
        double *o = reinterpret_cast<double *>(out.data());
        check(ctx, nqes_evaluate(ctx, cfg.data(), cnt, what == DumpWhat::Phi ? o : nullptr, nullptr,
                                 what == DumpWhat::E ? o : nullptr, what == DumpWhat::O ? o : nullptr));
        for (int c = 0; c < cnt; c++)
            for (int i = 0; i < rows; i++)
                for (int j = 0; j < cols; j++) {
                    const cplx v = out[size_t(c) * rows * cols + size_t(i) * cols + j];
                    const size_t at = (size_t(j) * rows + i) * n + base + c;
                    s.re[at] = v.real();
                    s.im[at] = v.imag();
                }
    }
    std::ostringstream fname;
    fname << prefix << "N" << N << "M" << M << "K" << K << ".mat";
    std::string err;
    if (!nqes_cli::mat_write(fname.str(), {{"s", s}}, err)) throw MatioCreateFileError(fname.str());
}

void run(const nqes_cli::CmdArgs &args) {
    std::random_device rd;
    const uint64_t seed = args.seed.value_or(rd());
    std::cout << "Random seed is " << seed << std::endl;
    const std::vector<double> J = build_J(args);
    if (!args.dump_jmat.empty()) {
        MatArray A;
        A.dims = {size_t(N), size_t(N)};
        A.re.resize(size_t(N) * N);
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) A.re[size_t(j) * N + i] = J[size_t(i) * N + j];  // column-major
        std::string err;
        if (!nqes_cli::mat_write(args.dump_jmat, {{"J", A}}, err)) throw MatioCreateFileError(args.dump_jmat);
        return;
    }
    nqes_ctx *ctx = nullptr;
    if (nqes_create(N, M, K, J.data(), args.h, args.device, &ctx) != NQES_OK) {
        std::cerr << "nqes: " << nqes_last_error(nullptr) << std::endl;
        std::exit(1);
    }
    if (args.model == Model::HS || args.model == Model::XXZ)  // delta 1 (hs), -1 (xxz): code/rbm.cc:1314-1325
        check(ctx, nqes_set_hamiltonian(ctx, NQES_HAM_HEISENBERG_LIKE, args.model == Model::HS ? 1.0 : -1.0));
    Weights rbm;
    if (!args.load_rbm.empty()) {
        rbm = load_rbm(args.load_rbm, K);
        if (args.apply_gauge)
            for (int k = 0; k < K; k++)
                for (int i = 1; i < N; i += 2) rbm.a[k * N + i] += cplx(0, args.inverse_gauge ? M_PI_2 : -M_PI_2);
        check(ctx, nqes_set_weights(ctx, reinterpret_cast<double *>(rbm.a.data()),
                                    reinterpret_cast<double *>(rbm.b.data()), reinterpret_cast<double *>(rbm.w.data())));
    } else if (!args.load_single_rbm.empty()) {
        Weights one = load_rbm(args.load_single_rbm, 1);
        for (int k = 0; k < K; k++) {
            const double sgn = k == 0 ? 1.0 : -1.0;
            for (int i = 0; i < N; i++) rbm.a[k * N + i] = sgn * one.a[i];
            for (int j = 0; j < M; j++) rbm.b[k * M + j] = one.b[j];
            for (int t = 0; t < N * M; t++) rbm.w[size_t(k) * N * M + t] = sgn * one.w[t];
        }
        check(ctx, nqes_set_weights(ctx, reinterpret_cast<double *>(rbm.a.data()),
                                    reinterpret_cast<double *>(rbm.b.data()), reinterpret_cast<double *>(rbm.w.data())));
    } else {
        check(ctx, nqes_init_weights(ctx, seed));
    }
    if (!args.dump_states.empty()) dump_states(ctx, args.dump_states, DumpWhat::Phi);
    if (!args.dump_ham.empty()) dump_states(ctx, args.dump_ham, DumpWhat::E);
    if (!args.dump_deriv.empty()) dump_states(ctx, args.dump_deriv, DumpWhat::O);

    double reglam = args.reglam0, lrate = args.lrate0;
    std::vector<double> best(K, 0.0);
    std::vector<cplx> e_mat(K * K);
    for (int iter = 0; iter < args.niters; iter++) {
        nqes_step_info info;
        const int st = nqes_sr_step(ctx, seed + uint64_t(iter) * args.ncpus, args.ncpus, args.mc_steps_percpu,
                                    args.burn_in_steps, std::max(lrate, args.lrate_cutoff),
                                    std::max(reglam, args.reglam_cutoff), args.minres_rtol, args.minres_maxit,
                                    reinterpret_cast<double *>(e_mat.data()), &info);
        if (st == NQES_ERR_NONFINITE) {
            if (args.throw_fperror) fp_error_exit();
        } else {
            check(ctx, st);
        }
        for (auto &z : e_mat) {
            z /= double(N);
            if (args.throw_fperror && !(std::isfinite(z.real()) && std::isfinite(z.imag()))) fp_error_exit();
        }
        reglam *= args.reglam_decay;
        lrate *= args.lratef;
        std::vector<cplx> ev(K), vec(K * K);
        nqes_cli::small_eig(e_mat.data(), K, ev.data(), vec.data());
        std::vector<double> evals(K);
        for (int k = 0; k < K; k++) evals[k] = ev[k].real();
        std::sort(evals.begin(), evals.end());
        print_row(evals);
        double d2 = 0, s_new = 0, s_best = 0;
        for (int k = 0; k < K; k++) {
            d2 += (evals[k] - best[k]) * (evals[k] - best[k]);
            s_new += evals[k];
            s_best += best[k];
        }
        if (iter && std::sqrt(d2) < args.tol) {
            std::cout << "Converged after " << iter + 1 << " steps." << std::endl;
            break;
        }
        if (!iter || s_new < s_best) best = evals;
    }

    // Correlation functions with the eigenvectors of the last e_mat, columns
    // ordered by eigenvalue (code/rbm.cc:1198-1232).
    std::vector<cplx> ev(K), evecs(K * K);
    nqes_cli::small_eig(e_mat.data(), K, ev.data(), evecs.data());
    std::vector<int> idx(K);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int p, int q) { return ev[p].real() < ev[q].real(); });
    std::vector<double> x(N * K), z(N * K), xx(size_t(N) * N * K), zz(size_t(N) * N * K);
    const int st = nqes_correlations(ctx, seed + uint64_t(args.niters) * args.ncpus, args.ncpus, args.mc_steps_percpu,
                                     args.burn_in_steps, reinterpret_cast<const double *>(evecs.data()), x.data(),
                                     z.data(), xx.data(), zz.data());
    if (st == NQES_ERR_NONFINITE && args.throw_fperror) fp_error_exit();
    if (st != NQES_ERR_NONFINITE) check(ctx, st);
    std::vector<double> sx(N * K), sz(N * K), sxx(size_t(N) * N * K), szz(size_t(N) * N * K);
    for (int k = 0; k < K; k++) {
        for (int i = 0; i < N; i++) {
            sx[i * K + k] = x[i * K + idx[k]];
            sz[i * K + k] = z[i * K + idx[k]];
        }
        for (int t = 0; t < N * N; t++) {
            sxx[size_t(t) * K + k] = xx[size_t(t) * K + idx[k]];
            szz[size_t(t) * K + k] = zz[size_t(t) * K + idx[k]];
        }
    }
    dump_corrs(sx, sz, sxx, szz, args.correlation_data);

    if (!args.dump_rbm.empty()) {
        check(ctx, nqes_get_weights(ctx, reinterpret_cast<double *>(rbm.a.data()), reinterpret_cast<double *>(rbm.b.data()),
                                    reinterpret_cast<double *>(rbm.w.data())));
        if (args.apply_gauge)
            for (int k = 0; k < K; k++)
                for (int i = 1; i < N; i += 2) rbm.a[k * N + i] -= cplx(0, M_PI_2);
        dump_rbm(rbm, args.dump_rbm);
    }
    nqes_destroy(ctx);
}

}  // namespace

int main(int argc, char *argv[]) {
    std::ostringstream welcome;
    welcome << "This program computes the lowest " << K << " energy eigenstates of the transverse field Ising model "
            << "with " << N << " spins using RBMs with " << M << " hidden units." << std::endl;
    const nqes_cli::CmdArgs args = nqes_cli::parse_args(argc, argv, welcome.str(), N * K < 32);
    if (!args.ncpus) {
        std::cerr << "Number of CPU cores cannot be zero." << std::endl;
        return 1;
    }
    run(args);
    return 0;
}
