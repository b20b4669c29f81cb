// CPU oracle — test infrastructure only.
//
// A C++ restatement of the reference's variational Monte Carlo / stochastic
// reconfiguration step for K multi-RBM states (code/rbm.cc), with the shape
// (N spins, M hidden units, K states) as runtime values instead of template
// parameters. It is used by tests/ as the parity checker for the CUDA library,
// and by bench.py as the timed CPU baseline ("port" of the reference's
// rbm-matfree build: OpenMP over chains, matrix-free S·v that recomputes every
// log-derivative on every MINRES-QLP iteration, code/rbm.cc:660-683).
// The product never links or calls this file.
//
// The reference itself cannot be compiled here (it needs Eigen3 and libmatio),
// so this restatement is pinned (a) for the RNG and the solver against the
// reference's own header-only pcg_random.h and minresqlp.h (oracle/ref_harness.cc,
// golden vectors in tests/golden/), and (b) for the physics against direct
// evaluation of the definitions and exact diagonalisation (tests/).
//
// Conventions shared with the C ABI in include/nqes.h:
//   * complex arrays are interleaved (re, im) doubles;
//   * a is K×N, b is K×M, w is K×N×M (index (k*N+i)*M+j), all row-major;
//   * a spin configuration is ceil(N/64) uint64 words, bit i set = spin i down
//     (sigma_i = -1), the std::bitset convention of code/rbm.cc:77-83;
//   * Phi is K×K row-major, Phi[k][kk] = psi_kk(s_k) (code/rbm.cc:146-171);
//   * tanh(theta) is M×K² row-major, column k*K+kk (code/rbm.cc:163-166);
//   * O (log-derivatives) is K·L per sample, [k][a_i | b_j | w_{i*M+j}]
//     (code/rbm.cc:199-239).
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "minres_qlp.h"
#include "pcg64.h"

namespace nqes_oracle {
namespace {

inline bool spin_bit(const uint64_t *s, int i) { return (s[i >> 6] >> (i & 63)) & 1ULL; }
inline void spin_flip(uint64_t *s, int i) { s[i >> 6] ^= (1ULL << (i & 63)); }

// Determinant of a small K×K row-major complex matrix. K <= 3 use the direct
// cofactor formulas of Eigen's fixed-size determinant (code/rbm.cc:216 etc.);
// larger K use LU with partial pivoting.
cplx small_det(const cplx *m, int K) {
    if (K == 1) return m[0];
    if (K == 2) return m[0] * m[3] - m[2] * m[1];
    if (K == 3) {
        // Cofactor expansion along the first column.
        auto e = [&](int r, int c) { return m[r * 3 + c]; };
        auto h3 = [&](int a, int b, int c) { return e(a, 0) * (e(b, 1) * e(c, 2) - e(b, 2) * e(c, 1)); };
        return h3(0, 1, 2) - h3(1, 0, 2) + h3(2, 0, 1);
    }
    std::vector<cplx> a(m, m + K * K);
    cplx d = 1;
    for (int c = 0; c < K; c++) {
        int p = c;
        for (int r = c + 1; r < K; r++)
            if (std::abs(a[r * K + c]) > std::abs(a[p * K + c])) p = r;
        if (a[p * K + c] == cplx(0)) return cplx(0);
        if (p != c) {
            for (int j = 0; j < K; j++) std::swap(a[p * K + j], a[c * K + j]);
            d = -d;
        }
        d *= a[c * K + c];
        for (int r = c + 1; r < K; r++) {
            cplx f = a[r * K + c] / a[c * K + c];
            for (int j = c; j < K; j++) a[r * K + j] -= f * a[c * K + j];
        }
    }
    return d;
}

// Inverse by Gauss-Jordan with partial pivoting. Returns false when singular.
// For an invertible Phi this equals the complete-orthogonal-decomposition
// pseudo-inverse the reference takes (code/rbm.cc:547,608).
bool small_inv(const cplx *m, cplx *inv, int K) {
    std::vector<cplx> a(m, m + K * K);
    for (int i = 0; i < K * K; i++) inv[i] = 0;
    for (int i = 0; i < K; i++) inv[i * K + i] = 1;
    for (int c = 0; c < K; c++) {
        int p = c;
        for (int r = c + 1; r < K; r++)
            if (std::abs(a[r * K + c]) > std::abs(a[p * K + c])) p = r;
        if (a[p * K + c] == cplx(0)) return false;
        if (p != c)
            for (int j = 0; j < K; j++) {
                std::swap(a[p * K + j], a[c * K + j]);
                std::swap(inv[p * K + j], inv[c * K + j]);
            }
        cplx piv = cplx(1) / a[c * K + c];
        for (int j = 0; j < K; j++) {
            a[c * K + j] *= piv;
            inv[c * K + j] *= piv;
        }
        for (int r = 0; r < K; r++) {
            if (r == c) continue;
            cplx f = a[r * K + c];
            if (f == cplx(0)) continue;
            for (int j = 0; j < K; j++) {
                a[r * K + j] -= f * a[c * K + j];
                inv[r * K + j] -= f * inv[c * K + j];
            }
        }
    }
    return true;
}

void small_mul(const cplx *A, const cplx *B, cplx *C, int K) {
    for (int r = 0; r < K; r++)
        for (int c = 0; c < K; c++) {
            cplx s = 0;
            for (int t = 0; t < K; t++) s += A[r * K + t] * B[t * K + c];
            C[r * K + c] = s;
        }
}

struct Oracle {
    int N, M, K, L, P, NW;
    std::vector<double> J;  // N×N row-major; the lower triangle J[i][j], i > j, is used
    double h;
    int ham = 0;            // 0: ising-like (J, h); 1: Heisenberg-like (J, delta)
    double delta = 0;
    std::vector<cplx> a, b, w;

    // Per-sample storage of the last sr_step, for the matrix-free S·v
    // (code/rbm.cc:581-589, 628-632).
    int Ns = 0;
    std::vector<uint64_t> st_spin;
    std::vector<cplx> st_phi, st_phiinv, st_tanh;
    std::vector<cplx> st_o, st_skk;  // normalised o and lambda-scaled skk_diag
    std::vector<cplx> st_f;
    std::vector<cplx> st_eloc;       // per-sample local energies (trace of E)
    std::vector<cplx> st_emat;       // per-sample K×K E matrices
    std::vector<uint64_t> st_accept; // accepted proposals per chain
    QlpInfo last_info;

    Oracle(int n, int m, int k, const double *Jm, double hh)
        : N(n), M(m), K(k), L(n + m + n * m), P(k * (n + m + n * m)), NW((n + 63) / 64),
          J(Jm, Jm + size_t(n) * n), h(hh), a(size_t(k) * n), b(size_t(k) * m), w(size_t(k) * n * m) {}

    const cplx &A(int kk, int i) const { return a[size_t(kk) * N + i]; }
    const cplx &B(int kk, int j) const { return b[size_t(kk) * M + j]; }
    const cplx &W(int kk, int i, int j) const { return w[(size_t(kk) * N + i) * M + j]; }

    // theta_j for RBM kk at configuration s (code/rbm.cc:134-143).
    cplx theta(int j, const uint64_t *s, int kk) const {
        cplx r = B(kk, j);
        for (int i = 0; i < N; i++) r += spin_bit(s, i) ? -W(kk, i, j) : W(kk, i, j);
        return r;
    }

    // Grand wave function Phi and tanh(theta) (code/rbm.cc:146-171).
    void state_fcn(const uint64_t *spin, cplx *phi, cplx *tanh_theta) const {
        const int KK = K * K;
        for (int k = 0; k < K; k++) {
            const uint64_t *s = spin + size_t(k) * NW;
            for (int kk = 0; kk < K; kk++) {
                cplx p = 0;
                for (int i = 0; i < N; i++) p += spin_bit(s, i) ? -A(kk, i) : A(kk, i);
                p = std::exp(p);
                for (int j = 0; j < M; j++) {
                    cplx th = theta(j, s, kk);
                    p *= std::cosh(th);
                    if (tanh_theta) tanh_theta[size_t(j) * KK + k * K + kk] = std::tanh(th);
                }
                phi[k * K + kk] = p;
            }
        }
    }

    // Single flip of spin i in configuration k (code/rbm.cc:176-190).
    void flip_state_fcn(int k, int i, const uint64_t *spin, cplx *phi, cplx *tanh_theta) const {
        const int KK = K * K;
        const bool down = spin_bit(spin + size_t(k) * NW, i);
        for (int kk = 0; kk < K; kk++) {
            phi[k * K + kk] *= std::exp(down ? 2.0 * A(kk, i) : -2.0 * A(kk, i));
            for (int j = 0; j < M; j++) {
                cplx ws = down ? -2.0 * W(kk, i, j) : 2.0 * W(kk, i, j);
                cplx &t = tanh_theta[size_t(j) * KK + k * K + kk];
                cplx th = t;
                cplx denom = std::cosh(ws) - th * std::sinh(ws);
                t = (th * std::cosh(ws) - std::sinh(ws)) / denom;
                phi[k * K + kk] *= denom;
            }
        }
    }

    // Log-derivatives O, as the determinants the reference takes
    // (code/rbm.cc:199-239).
    void deriv(const uint64_t *spin, const cplx *phi, const cplx *phi_inv, const cplx *tanh_theta,
               cplx *out) const {
        const int KK = K * K;
        std::vector<cplx> d(KK), prod(KK);
        auto det_of = [&](const std::vector<cplx> &dphi) {
            small_mul(phi_inv, dphi.data(), prod.data(), K);
            return small_det(prod.data(), K);
        };
        for (int k = 0; k < K; k++) {
            cplx *o = out + size_t(k) * L;
            for (int i = 0; i < N; i++) {
                d.assign(phi, phi + KK);
                for (int kk = 0; kk < K; kk++)
                    if (spin_bit(spin + size_t(kk) * NW, i)) d[kk * K + k] = -d[kk * K + k];
                o[i] = det_of(d);
            }
            for (int j = 0; j < M; j++) {
                d.assign(phi, phi + KK);
                for (int kk = 0; kk < K; kk++) d[kk * K + k] *= tanh_theta[size_t(j) * KK + kk * K + k];
                o[N + j] = det_of(d);
            }
            for (int i = 0; i < N; i++)
                for (int j = 0; j < M; j++) {
                    d.assign(phi, phi + KK);
                    for (int kk = 0; kk < K; kk++) {
                        d[kk * K + k] *= tanh_theta[size_t(j) * KK + kk * K + k];
                        if (spin_bit(spin + size_t(kk) * NW, i)) d[kk * K + k] = -d[kk * K + k];
                    }
                    o[N + M + i * M + j] = det_of(d);
                }
        }
    }

    // 2 * sum_{i>j} J_ij sigma_i sigma_j (code/rbm.cc:1011-1031).
    double jterm(const uint64_t *s) const {
        double r = 0;
        for (int i = 1; i < N; i++)
            for (int j = 0; j < i; j++) {
                double p = J[size_t(i) * N + j];
                if (spin_bit(s, i) ^ spin_bit(s, j)) p = -p;
                r += p;
            }
        return r * 2.0;
    }

    // Heisenberg-like: H = sum_{i>j} J_ij (sx_i sx_j + sy_i sy_j + delta sz_i sz_j)
    // (code/rbm.cc:1091-1119): for every pair and row k, two sequential single
    // flips when the spins differ (res += J (2 Phi' - delta Phi)), else
    // res += J delta Phi; E = Phi^-1 res.
    void local_energy_hs(const uint64_t *spin, const cplx *phi, const cplx *phi_inv,
                         const cplx *tanh_theta, cplx *E) const {
        const int KK = K * K;
        std::vector<cplx> res(KK, cplx(0)), phip(KK), tp(size_t(M) * KK);
        std::vector<uint64_t> sp(size_t(K) * NW);
        for (int i = 1; i < N; i++)
            for (int j = 0; j < i; j++) {
                const double p = J[size_t(i) * N + j];
                sp.assign(spin, spin + size_t(K) * NW);
                phip.assign(phi, phi + KK);
                tp.assign(tanh_theta, tanh_theta + size_t(M) * KK);
                for (int k = 0; k < K; k++) {
                    const uint64_t *sk = spin + size_t(k) * NW;
                    if (spin_bit(sk, i) != spin_bit(sk, j)) {
                        flip_state_fcn(k, i, sp.data(), phip.data(), tp.data());
                        sp[size_t(k) * NW + (i >> 6)] ^= 1ULL << (i & 63);
                        flip_state_fcn(k, j, sp.data(), phip.data(), tp.data());
                        for (int kk = 0; kk < K; kk++)
                            res[k * K + kk] += p * (2.0 * phip[k * K + kk] - delta * phi[k * K + kk]);
                    } else {
                        for (int kk = 0; kk < K; kk++) res[k * K + kk] += p * delta * phi[k * K + kk];
                    }
                }
            }
        small_mul(phi_inv, res.data(), E, K);
    }

    // E = Phi^-1 (diag(J(s_k)) Phi - h sum_i Phi(flip i in every row))
    // (code/rbm.cc:1042-1062).
    void local_energy(const uint64_t *spin, const cplx *phi, const cplx *phi_inv,
                      const cplx *tanh_theta, cplx *E) const {
        if (ham == 1) return local_energy_hs(spin, phi, phi_inv, tanh_theta, E);
        const int KK = K * K;
        std::vector<cplx> res(phi, phi + KK), sx(KK, cplx(0)), phip(KK), tp(size_t(M) * KK);
        for (int k = 0; k < K; k++) {
            double jk = jterm(spin + size_t(k) * NW);
            for (int kk = 0; kk < K; kk++) res[k * K + kk] *= jk;
        }
        for (int i = 0; i < N; i++) {
            phip.assign(phi, phi + KK);
            tp.assign(tanh_theta, tanh_theta + size_t(M) * KK);
            for (int k = 0; k < K; k++) flip_state_fcn(k, i, spin, phip.data(), tp.data());
            for (int t = 0; t < KK; t++) sx[t] += phip[t];
        }
        for (int t = 0; t < KK; t++) res[t] -= h * sx[t];
        small_mul(phi_inv, res.data(), E, K);
    }

    void invert_or_flag(const cplx *phi, cplx *phi_inv, bool &singular) const {
        singular = !small_inv(phi, phi_inv, K);
        if (singular)
            for (int t = 0; t < K * K; t++) phi_inv[t] = 0;
    }

    // One sweep (code/rbm.cc:530-552): proposals k outer, i inner, one uniform
    // draw each, accept iff u <= min(1, |det Phi'|^2 / |det Phi|^2).
    uint64_t mc_step(uint64_t *spin, Pcg64 &rg, cplx *phi, cplx *phi_inv, cplx *tanh_theta,
                     bool &singular, uint64_t *proposal_log = nullptr) const {
        const int KK = K * K;
        cplx det_phi = small_det(phi, K);
        std::uniform_real_distribution<double> unif(0, 1);
        std::vector<cplx> phip(KK), tp(size_t(M) * KK);
        uint64_t acc = 0;
        for (int k = 0; k < K; k++)
            for (int i = 0; i < N; i++) {
                phip.assign(phi, phi + KK);
                tp.assign(tanh_theta, tanh_theta + size_t(M) * KK);
                flip_state_fcn(k, i, spin, phip.data(), tp.data());
                cplx det_p = small_det(phip.data(), K);
                double prob = det_phi == cplx(0) ? 1.0 : std::norm(det_p) / std::norm(det_phi);
                double u = unif(rg);
                bool accept = u <= std::min(1.0, prob);
                if (proposal_log) *proposal_log++ = accept;
                if (accept) {
                    spin_flip(spin + size_t(k) * NW, i);
                    det_phi = det_p;
                    std::copy(phip.begin(), phip.end(), phi);
                    invert_or_flag(phi, phi_inv, singular);
                    std::copy(tp.begin(), tp.end(), tanh_theta);
                    acc++;
                }
            }
        return acc;
    }

    // Start configuration: K·N Bernoulli(1/2) draws, k-major (code/rbm.cc:98-119).
    void init_spin(Pcg64 &rg, uint64_t *spin) const {
        std::bernoulli_distribution d(0.5);
        std::fill(spin, spin + size_t(K) * NW, 0);
        for (int k = 0; k < K; k++)
            for (int i = 0; i < N; i++)
                if (d(rg)) spin_flip(spin + size_t(k) * NW, i);
    }

    // Reference weight initialisation from pcg64(seed-1) (code/rbm.cc:241-270, 1127).
    void init_weights(uint64_t seed) {
        Pcg64 rg(seed - 1);
        std::normal_distribution<double> nd;
        for (int k = 0; k < K; k++) {
            for (int i = 0; i < N; i++) {
                double re = nd(rg), im = nd(rg);
                a[size_t(k) * N + i] = cplx{re, im} / cplx{std::sqrt(double(N))};
            }
            for (int j = 0; j < M; j++) {
                double re = nd(rg), im = nd(rg);
                b[size_t(k) * M + j] = cplx{re, im} / cplx{std::sqrt(double(M))};
            }
            for (int i = 0; i < N; i++)
                for (int j = 0; j < M; j++) {
                    double re = nd(rg), im = nd(rg);
                    w[(size_t(k) * N + i) * M + j] = cplx{re, im} / cplx{std::sqrt(double(N * M))};
                }
        }
    }

    // One SR step (code/rbm.cc:561-719). Returns e_mat / Ns in emat_out.
    int sr_step(uint64_t seed, int C, int m, int burn, double lr, double reglam, double rtol,
                uint64_t maxit, bool store_o, cplx *emat_out, int nthreads) {
        const int KK = K * K;
        Ns = C * m;
        st_spin.assign(size_t(Ns) * K * NW, 0);
        st_phi.assign(size_t(Ns) * KK, 0);
        st_phiinv.assign(size_t(Ns) * KK, 0);
        st_tanh.assign(size_t(Ns) * M * KK, 0);
        st_eloc.assign(Ns, 0);
        st_emat.assign(size_t(Ns) * KK, 0);
        st_accept.assign(C, 0);
        std::vector<cplx> Ost;
        if (store_o) Ost.assign(size_t(Ns) * P, 0);

        // Per-chain partial sums, combined in chain order afterwards.
        std::vector<cplx> po(size_t(C) * P), pf(size_t(C) * P), ps(size_t(C) * P);
        std::vector<cplx> pe(size_t(C) * KK), pl(C);
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : bad)
        for (int c = 0; c < C; c++) {
            Pcg64 rg(seed + uint64_t(c));
            std::vector<uint64_t> spin(size_t(K) * NW);
            std::vector<cplx> phi(KK), phi_inv(KK), tnh(size_t(M) * KK), E(KK), der(P);
            bool singular = false;
            init_spin(rg, spin.data());
            state_fcn(spin.data(), phi.data(), tnh.data());
            invert_or_flag(phi.data(), phi_inv.data(), singular);
            uint64_t acc = 0;
            for (int t = 0; t < burn; t++)
                acc += mc_step(spin.data(), rg, phi.data(), phi_inv.data(), tnh.data(), singular);
            cplx *o = &po[size_t(c) * P], *f = &pf[size_t(c) * P], *s2 = &ps[size_t(c) * P];
            for (int t = 0; t < m; t++) {
                acc += mc_step(spin.data(), rg, phi.data(), phi_inv.data(), tnh.data(), singular);
                if (singular) bad++;
                local_energy(spin.data(), phi.data(), phi_inv.data(), tnh.data(), E.data());
                cplx en = 0;
                for (int k = 0; k < K; k++) en += E[k * K + k];
                for (int q = 0; q < KK; q++) pe[size_t(c) * KK + q] += E[q];
                pl[c] += en;
                deriv(spin.data(), phi.data(), phi_inv.data(), tnh.data(), der.data());
                for (int p = 0; p < P; p++) {
                    o[p] += der[p];
                    s2[p] += der[p] * std::conj(der[p]);
                    f[p] += en * std::conj(der[p]);
                }
                size_t idx = size_t(c) * m + t;
                std::copy(spin.begin(), spin.end(), st_spin.begin() + idx * K * NW);
                std::copy(phi.begin(), phi.end(), st_phi.begin() + idx * KK);
                std::copy(phi_inv.begin(), phi_inv.end(), st_phiinv.begin() + idx * KK);
                std::copy(tnh.begin(), tnh.end(), st_tanh.begin() + idx * M * KK);
                std::copy(E.begin(), E.end(), st_emat.begin() + idx * KK);
                st_eloc[idx] = en;
                if (store_o) std::copy(der.begin(), der.end(), Ost.begin() + idx * P);
            }
            st_accept[c] = acc;
        }

        std::vector<cplx> o(P, 0), skk(P, 0), f(P, 0), e_mat(KK, 0);
        cplx eloc = 0;
        for (int c = 0; c < C; c++) {
            for (int p = 0; p < P; p++) {
                o[p] += po[size_t(c) * P + p];
                skk[p] += ps[size_t(c) * P + p];
                f[p] += pf[size_t(c) * P + p];
            }
            for (int q = 0; q < KK; q++) e_mat[q] += pe[size_t(c) * KK + q];
            eloc += pl[c];
        }
        // Normalisation (code/rbm.cc:640-650).
        eloc /= double(Ns);
        for (int p = 0; p < P; p++) {
            o[p] /= double(Ns);
            skk[p] /= double(Ns);
            skk[p] -= std::norm(o[p]);
            skk[p] *= reglam;
            f[p] /= double(Ns);
            f[p] -= eloc * std::conj(o[p]);
        }
        st_o = o;
        st_skk = skk;
        st_f = f;

        // Matrix-free S·v (code/rbm.cc:660-683).
        auto Sv = [&](const CVec &v, CVec &res) { apply_S(v, res, store_o ? &Ost : nullptr, nthreads); };
        CVec x;
        last_info = minres_qlp(Sv, f, x, rtol, maxit);

        // Update (code/rbm.cc:699-717).
        for (int k = 0; k < K; k++) {
            for (int i = 0; i < N; i++) a[size_t(k) * N + i] -= lr * x[size_t(k) * L + i];
            for (int j = 0; j < M; j++) b[size_t(k) * M + j] -= lr * x[size_t(k) * L + N + j];
            for (int i = 0; i < N; i++)
                for (int j = 0; j < M; j++)
                    w[(size_t(k) * N + i) * M + j] -= lr * x[size_t(k) * L + N + M + size_t(i) * M + j];
        }
        for (int q = 0; q < KK; q++) emat_out[q] = e_mat[q] / double(Ns);
        return bad;
    }

    // (S v)_l = (1/Ns) sum_s conj(O_sl) (O_s · v) + skk_l v_l - (o · v) conj(o_l).
    void apply_S(const CVec &v, CVec &res, const std::vector<cplx> *Ost, int nthreads) const {
        const int KK = K * K;
        const int nchunk = std::max(1, std::min(Ns, 256));
        std::vector<cplx> part(size_t(nchunk) * P, 0);
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int ch = 0; ch < nchunk; ch++) {
            std::vector<cplx> der(P);
            cplx *acc = &part[size_t(ch) * P];
            int s0 = int(int64_t(Ns) * ch / nchunk), s1 = int(int64_t(Ns) * (ch + 1) / nchunk);
            for (int s = s0; s < s1; s++) {
                const cplx *d;
                if (Ost) {
                    d = &(*Ost)[size_t(s) * P];
                } else {
                    deriv(&st_spin[size_t(s) * K * NW], &st_phi[size_t(s) * KK], &st_phiinv[size_t(s) * KK],
                          &st_tanh[size_t(s) * M * KK], der.data());
                    d = der.data();
                }
                cplx dv = 0;
                for (int p = 0; p < P; p++) dv += d[p] * v[p];
                for (int p = 0; p < P; p++) acc[p] += dv * std::conj(d[p]);
            }
        }
        res.assign(P, 0);
        for (int ch = 0; ch < nchunk; ch++)
            for (int p = 0; p < P; p++) res[p] += part[size_t(ch) * P + p];
        cplx ov = 0;
        for (int p = 0; p < P; p++) ov += st_o[p] * v[p];
        for (int p = 0; p < P; p++) {
            res[p] /= double(Ns);
            res[p] += st_skk[p] * v[p] - ov * std::conj(st_o[p]);
        }
    }

    // Correlation functions x, z, xx, zz (code/rbm.cc:730-826). The four
    // reference passes share one seed and therefore one set of chains; this
    // restatement walks those chains once and evaluates the four observables
    // on every sample. Output is the reference's correlation_fcn result,
    // res(i, k) = Re diag(V^-1 <Phi^-1 F_i> V)_k, before the eigenvalue sort.
    void correlations(uint64_t seed, int C, int m, int burn, const cplx *evecs, double *xo, double *zo,
                      double *xxo, double *zzo, int nthreads) const {
        const int KK = K * K;
        const size_t R1 = size_t(N) * KK, R2 = size_t(N) * N * KK;
        std::vector<cplx> cx(size_t(C) * R1), cz(size_t(C) * R1), cxx(size_t(C) * R2), czz(size_t(C) * R2);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
        for (int c = 0; c < C; c++) {
            Pcg64 rg(seed + uint64_t(c));
            std::vector<uint64_t> spin(size_t(K) * NW), sp(size_t(K) * NW);
            std::vector<cplx> phi(KK), phi_inv(KK), tnh(size_t(M) * KK), F(KK), mat(KK);
            bool singular = false;
            init_spin(rg, spin.data());
            state_fcn(spin.data(), phi.data(), tnh.data());
            invert_or_flag(phi.data(), phi_inv.data(), singular);
            for (int t = 0; t < burn; t++) mc_step(spin.data(), rg, phi.data(), phi_inv.data(), tnh.data(), singular);
            for (int t = 0; t < m; t++) {
                mc_step(spin.data(), rg, phi.data(), phi_inv.data(), tnh.data(), singular);
                for (int i = 0; i < N; i++) {
                    // sigma^x_i: state_fcn with spin i flipped in every row (code/rbm.cc:773-781).
                    sp = spin;
                    for (int k = 0; k < K; k++) spin_flip(&sp[size_t(k) * NW], i);
                    state_fcn(sp.data(), F.data(), nullptr);
                    small_mul(phi_inv.data(), F.data(), mat.data(), K);
                    for (int q = 0; q < KK; q++) cx[size_t(c) * R1 + size_t(i) * KK + q] += mat[q];
                    // sigma^z_i: rows with spin i down change sign (code/rbm.cc:799-810).
                    F = phi;
                    for (int k = 0; k < K; k++)
                        if (spin_bit(&spin[size_t(k) * NW], i))
                            for (int kk = 0; kk < K; kk++) F[k * K + kk] = -F[k * K + kk];
                    small_mul(phi_inv.data(), F.data(), mat.data(), K);
                    for (int q = 0; q < KK; q++) cz[size_t(c) * R1 + size_t(i) * KK + q] += mat[q];
                }
                for (int i = 0; i < N; i++)
                    for (int j = 0; j < N; j++) {
                        const size_t row = size_t(i) * N + j;
                        // sigma^x_i sigma^x_j (code/rbm.cc:784-796).
                        sp = spin;
                        for (int k = 0; k < K; k++) {
                            spin_flip(&sp[size_t(k) * NW], i);
                            spin_flip(&sp[size_t(k) * NW], j);
                        }
                        state_fcn(sp.data(), F.data(), nullptr);
                        small_mul(phi_inv.data(), F.data(), mat.data(), K);
                        for (int q = 0; q < KK; q++) cxx[size_t(c) * R2 + row * KK + q] += mat[q];
                        // sigma^z_i sigma^z_j (code/rbm.cc:813-826).
                        F = phi;
                        for (int k = 0; k < K; k++)
                            if (spin_bit(&spin[size_t(k) * NW], i) ^ spin_bit(&spin[size_t(k) * NW], j))
                                for (int kk = 0; kk < K; kk++) F[k * K + kk] = -F[k * K + kk];
                        small_mul(phi_inv.data(), F.data(), mat.data(), K);
                        for (int q = 0; q < KK; q++) czz[size_t(c) * R2 + row * KK + q] += mat[q];
                    }
            }
        }
        std::vector<cplx> vinv(KK), tmp(KK), tmp2(KK), mat(KK);
        small_inv(evecs, vinv.data(), K);
        const double ns = double(C) * m;
        auto finish = [&](const std::vector<cplx> &acc, size_t rows, double *out) {
            for (size_t r = 0; r < rows; r++) {
                for (int q = 0; q < KK; q++) {
                    cplx s = 0;
                    for (int c = 0; c < C; c++) s += acc[size_t(c) * rows * KK + r * KK + q];
                    mat[q] = s / ns;
                }
                small_mul(vinv.data(), mat.data(), tmp.data(), K);
                small_mul(tmp.data(), evecs, tmp2.data(), K);
                for (int k = 0; k < K; k++) out[r * K + k] = tmp2[k * K + k].real();
            }
        };
        finish(cx, N, xo);
        finish(cz, N, zo);
        finish(cxx, size_t(N) * N, xxo);
        finish(czz, size_t(N) * N, zzo);
    }

    // One chain's trajectory for chain-level parity: the spin configuration
    // after every sweep (burn-in included) and each proposal's accept bit.
    void chain_trajectory(uint64_t seed, int sweeps, uint64_t *spins_out, uint64_t *accept_out) const {
        const int KK = K * K;
        Pcg64 rg(seed);
        std::vector<uint64_t> spin(size_t(K) * NW);
        std::vector<cplx> phi(KK), phi_inv(KK), tnh(size_t(M) * KK);
        bool singular = false;
        init_spin(rg, spin.data());
        state_fcn(spin.data(), phi.data(), tnh.data());
        invert_or_flag(phi.data(), phi_inv.data(), singular);
        for (int t = 0; t < sweeps; t++) {
            mc_step(spin.data(), rg, phi.data(), phi_inv.data(), tnh.data(), singular,
                    accept_out ? accept_out + size_t(t) * K * N : nullptr);
            std::copy(spin.begin(), spin.end(), spins_out + size_t(t) * K * NW);
        }
    }
};

inline const cplx *C(const double *p) { return reinterpret_cast<const cplx *>(p); }
inline cplx *C(double *p) { return reinterpret_cast<cplx *>(p); }

}  // namespace
}  // namespace nqes_oracle

using nqes_oracle::cplx;
using nqes_oracle::Oracle;
using nqes_oracle::C;

extern "C" {

void *orc_create(int N, int M, int K, const double *J, double h) { return new Oracle(N, M, K, J, h); }
void orc_set_hamiltonian(void *op, int form, double delta) {
    Oracle *o = static_cast<Oracle *>(op);
    o->ham = form;
    o->delta = delta;
}
void orc_destroy(void *o) { delete static_cast<Oracle *>(o); }

void orc_set_weights(void *op, const double *a, const double *b, const double *w) {
    auto *o = static_cast<Oracle *>(op);
    std::copy(C(a), C(a) + o->a.size(), o->a.begin());
    std::copy(C(b), C(b) + o->b.size(), o->b.begin());
    std::copy(C(w), C(w) + o->w.size(), o->w.begin());
}
void orc_get_weights(void *op, double *a, double *b, double *w) {
    auto *o = static_cast<Oracle *>(op);
    std::copy(o->a.begin(), o->a.end(), C(a));
    std::copy(o->b.begin(), o->b.end(), C(b));
    std::copy(o->w.begin(), o->w.end(), C(w));
}
void orc_init_weights(void *op, uint64_t seed) { static_cast<Oracle *>(op)->init_weights(seed); }

void orc_state(void *op, const uint64_t *spin, double *phi, double *tanh_theta) {
    static_cast<Oracle *>(op)->state_fcn(spin, C(phi), tanh_theta ? C(tanh_theta) : nullptr);
}

// E (K×K) and O (P) at a configuration, from a fresh state_fcn.
int orc_local(void *op, const uint64_t *spin, double *E, double *O) {
    auto *o = static_cast<Oracle *>(op);
    const int KK = o->K * o->K;
    std::vector<cplx> phi(KK), inv(KK), tnh(size_t(o->M) * KK);
    o->state_fcn(spin, phi.data(), tnh.data());
    bool sing = false;
    o->invert_or_flag(phi.data(), inv.data(), sing);
    if (sing) return 1;
    if (E) o->local_energy(spin, phi.data(), inv.data(), tnh.data(), C(E));
    if (O) o->deriv(spin, phi.data(), inv.data(), tnh.data(), C(O));
    return 0;
}

// Full SR step. info: [flag, iters, qlp_iters, relres, anorm, acond, xnorm, accept_total, singular_samples]
int orc_sr_step(void *op, uint64_t seed, int C_, int m, int burn, double lr, double reglam, double rtol,
                uint64_t maxit, int store_o, double *emat, double *info, int nthreads) {
    auto *o = static_cast<Oracle *>(op);
    int bad = o->sr_step(seed, C_, m, burn, lr, reglam, rtol, maxit, store_o != 0, C(emat), nthreads);
    if (info) {
        info[0] = o->last_info.flag;
        info[1] = double(o->last_info.iters);
        info[2] = double(o->last_info.qlp_iters);
        info[3] = o->last_info.relres;
        info[4] = o->last_info.anorm;
        info[5] = o->last_info.acond;
        info[6] = o->last_info.xnorm;
        uint64_t acc = 0;
        for (auto x : o->st_accept) acc += x;
        info[7] = double(acc);
        info[8] = bad;
    }
    return 0;
}

// Per-sample records of the last sr_step.
void orc_samples(void *op, uint64_t *spins, double *eloc, double *emat) {
    auto *o = static_cast<Oracle *>(op);
    if (spins) std::copy(o->st_spin.begin(), o->st_spin.end(), spins);
    if (eloc) std::copy(o->st_eloc.begin(), o->st_eloc.end(), C(eloc));
    if (emat) std::copy(o->st_emat.begin(), o->st_emat.end(), C(emat));
}
// o (mean O), skk (lambda-scaled diagonal), f (force) of the last sr_step.
void orc_moments(void *op, double *o_, double *skk, double *f) {
    auto *o = static_cast<Oracle *>(op);
    if (o_) std::copy(o->st_o.begin(), o->st_o.end(), C(o_));
    if (skk) std::copy(o->st_skk.begin(), o->st_skk.end(), C(skk));
    if (f) std::copy(o->st_f.begin(), o->st_f.end(), C(f));
}
// O row of stored sample s of the last sr_step.
void orc_sample_deriv(void *op, int s, double *out) {
    auto *o = static_cast<Oracle *>(op);
    const int KK = o->K * o->K;
    o->deriv(&o->st_spin[size_t(s) * o->K * o->NW], &o->st_phi[size_t(s) * KK], &o->st_phiinv[size_t(s) * KK],
             &o->st_tanh[size_t(s) * o->M * KK], C(out));
}
// Matrix-free S·v with the moments and samples of the last sr_step.
void orc_apply_S(void *op, const double *v, double *out, int nthreads) {
    auto *o = static_cast<Oracle *>(op);
    nqes_oracle::CVec vv(C(v), C(v) + o->P), res;
    o->apply_S(vv, res, nullptr, nthreads);
    std::copy(res.begin(), res.end(), C(out));
}

void orc_correlations(void *op, uint64_t seed, int C_, int m, int burn, const double *evecs, double *x, double *z,
                      double *xx, double *zz, int nthreads) {
    static_cast<Oracle *>(op)->correlations(seed, C_, m, burn, C(evecs), x, z, xx, zz, nthreads);
}

void orc_chain(void *op, uint64_t seed, int sweeps, uint64_t *spins_out, uint64_t *accept_out) {
    static_cast<Oracle *>(op)->chain_trajectory(seed, sweeps, spins_out, accept_out);
}

// Raw pcg64 outputs and the two libstdc++ distributions the reference draws.
void orc_pcg64(uint64_t seed, int n, uint64_t *out) {
    nqes_oracle::Pcg64 rg(seed);
    for (int i = 0; i < n; i++) out[i] = rg();
}
void orc_uniform(uint64_t seed, int n, double *out) {
    nqes_oracle::Pcg64 rg(seed);
    std::uniform_real_distribution<double> u(0, 1);
    for (int i = 0; i < n; i++) out[i] = u(rg);
}
void orc_bernoulli(uint64_t seed, int n, uint8_t *out) {
    nqes_oracle::Pcg64 rg(seed);
    std::bernoulli_distribution d(0.5);
    for (int i = 0; i < n; i++) out[i] = d(rg);
}

// MINRES-QLP on a dense Hermitian P×P matrix (row-major complex).
int orc_minresqlp_dense(int n, const double *A, const double *b, double rtol, uint64_t maxit, double *x,
                        double *info) {
    const cplx *Am = C(A);
    auto op = [&](const nqes_oracle::CVec &v, nqes_oracle::CVec &out) {
        out.assign(n, 0);
        for (int r = 0; r < n; r++) {
            cplx s = 0;
            for (int c = 0; c < n; c++) s += Am[size_t(r) * n + c] * v[c];
            out[r] = s;
        }
    };
    nqes_oracle::CVec bb(C(b), C(b) + n), xx;
    auto in = nqes_oracle::minres_qlp(op, bb, xx, rtol, maxit);
    std::copy(xx.begin(), xx.end(), C(x));
    if (info) {
        info[0] = in.flag;
        info[1] = double(in.iters);
        info[2] = double(in.qlp_iters);
        info[3] = in.relres;
    }
    return in.flag;
}

}  // extern "C"
