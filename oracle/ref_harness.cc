// CPU oracle — test infrastructure only.
//
// Runs the reference's own header-only components, compiled from where they
// lie in the reference tree (code/pcg_random.h, code/pcg_extras.h,
// code/minresqlp.h; see oracle/Makefile), to produce golden vectors that pin
// the oracle restatement (oracle/pcg64.h, oracle/minres_qlp.h, the weight
// initialisation in oracle/nqes_oracle.cc). The rest of code/rbm.cc cannot be
// compiled here (Eigen3 and libmatio are absent).
//
// Output: JSON on stdout, consumed by tests/golden/make_golden.py.
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "minresqlp.h"
#include "pcg_random.h"

using cplx = std::complex<double>;

// The minimal vector interface code/minresqlp.h needs (code/minresqlp.h:73-79):
// RealScalar, size, norm, dot (conjugating the left operand), Zero, and
// element-wise arithmetic with real scalars.
struct RVec {
    using RealScalar = double;
    std::vector<cplx> d;
    RVec() = default;
    explicit RVec(size_t n) : d(n) {}
    size_t size() const { return d.size(); }
    static RVec Zero(size_t n) { return RVec(n); }
    double norm() const {
        double s = 0;
        for (auto &z : d) s += std::norm(z);
        return std::sqrt(s);
    }
    cplx dot(const RVec &o) const {
        cplx s = 0;
        for (size_t i = 0; i < d.size(); i++) s += std::conj(d[i]) * o.d[i];
        return s;
    }
    RVec &operator+=(const RVec &o) { for (size_t i = 0; i < d.size(); i++) d[i] += o.d[i]; return *this; }
    RVec &operator-=(const RVec &o) { for (size_t i = 0; i < d.size(); i++) d[i] -= o.d[i]; return *this; }
};
inline RVec operator+(RVec a, const RVec &b) { return a += b; }
inline RVec operator-(RVec a, const RVec &b) { return a -= b; }
inline RVec operator-(RVec a) { for (auto &z : a.d) z = -z; return a; }
inline RVec operator*(RVec a, double s) { for (auto &z : a.d) z *= s; return a; }
inline RVec operator*(double s, RVec a) { for (auto &z : a.d) z *= s; return a; }
inline RVec operator/(RVec a, double s) { for (auto &z : a.d) z /= s; return a; }

static void print_u64s(const char *key, const std::vector<uint64_t> &v, bool last = false) {
    printf("\"%s\": [", key);
    for (size_t i = 0; i < v.size(); i++) printf("%s\"%llu\"", i ? "," : "", (unsigned long long)v[i]);
    printf("]%s\n", last ? "" : ",");
}
static void print_dbls(const char *key, const std::vector<double> &v, bool last = false) {
    printf("\"%s\": [", key);
    for (size_t i = 0; i < v.size(); i++) printf("%s%.17g", i ? "," : "", v[i]);
    printf("]%s\n", last ? "" : ",");
}

int main() {
    printf("{\n");
    // 1. Raw pcg64 streams, uniform doubles and Bernoulli bits for several
    //    seeds, through libstdc++'s distributions exactly as code/rbm.cc:103,535.
    const uint64_t seeds[] = {0ULL, 1ULL, 42ULL, 2201341417ULL, 18446744073709551615ULL, 123456789012345ULL};
    printf("\"rng\": [\n");
    for (size_t si = 0; si < sizeof(seeds) / sizeof(seeds[0]); si++) {
        const int n = 512;
        std::vector<uint64_t> raw(n);
        std::vector<double> uni(n), bern(n);
        {
            pcg64 rg(seeds[si]);
            for (int i = 0; i < n; i++) raw[i] = rg();
        }
        {
            pcg64 rg(seeds[si]);
            std::uniform_real_distribution<double> u(0, 1);
            for (int i = 0; i < n; i++) uni[i] = u(rg);
        }
        {
            pcg64 rg(seeds[si]);
            std::bernoulli_distribution b(0.5);
            for (int i = 0; i < n; i++) bern[i] = b(rg);
        }
        // Long-stream checksums: wrapping sum and xor of the first 10^6 raw
        // outputs, and the exact sum of the first 10^6 uniforms in draw order.
        uint64_t sum = 0, x = 0;
        double usum = 0;
        {
            pcg64 rg(seeds[si]);
            for (int i = 0; i < 1000000; i++) { uint64_t r = rg(); sum += r; x ^= r; }
            pcg64 rg2(seeds[si]);
            std::uniform_real_distribution<double> u(0, 1);
            for (int i = 0; i < 1000000; i++) usum += u(rg2);
        }
        printf("{\"seed\": \"%llu\", \"sum1e6\": \"%llu\", \"xor1e6\": \"%llu\", \"usum1e6\": %.17g,\n",
               (unsigned long long)seeds[si], (unsigned long long)sum, (unsigned long long)x, usum);
        print_u64s("raw", raw);
        print_dbls("uniform", uni);
        print_dbls("bernoulli", bern, true);
        printf("}%s\n", si + 1 < sizeof(seeds) / sizeof(seeds[0]) ? "," : "");
    }
    printf("],\n");

    // 2. Reference weight initialisation order (code/rbm.cc:241-270) with
    //    pcg64(seed - 1) (code/rbm.cc:1127): N=3, M=6, K=2, seed=7.
    {
        const int N = 3, M = 6, K = 2;
        pcg64 rg(7 - 1);
        std::normal_distribution<double> nd;
        std::vector<double> out;
        for (int k = 0; k < K; k++) {
            for (int i = 0; i < N; i++) {
                cplx v = cplx{nd(rg), nd(rg)} / cplx{std::sqrt(N)};
                out.push_back(v.real()); out.push_back(v.imag());
            }
            for (int i = 0; i < M; i++) {
                cplx v = cplx{nd(rg), nd(rg)} / cplx{std::sqrt(M)};
                out.push_back(v.real()); out.push_back(v.imag());
            }
            for (int i = 0; i < N; i++)
                for (int j = 0; j < M; j++) {
                    cplx v = cplx{nd(rg), nd(rg)} / cplx{std::sqrt(N * M)};
                    out.push_back(v.real()); out.push_back(v.imag());
                }
        }
        printf("\"init\": {\"N\": %d, \"M\": %d, \"K\": %d, \"seed\": 7,\n", N, M, K);
        print_dbls("weights", out, true);
        printf("},\n");
    }

    // 3. MINRES-QLP on Hermitian systems built from a seeded pcg64 stream:
    //    A = G^H G / n + mu I (mu > 0: positive definite; mu < 0: indefinite),
    //    right-hand side b from the same stream.
    printf("\"minresqlp\": [\n");
    struct Case { int n; double mu; double rtol; unsigned long long maxit; uint64_t seed; };
    const Case cases[] = {{12, 0.5, 1e-10, ~0ULL, 11}, {40, 0.05, 1e-9, ~0ULL, 12}, {40, -0.3, 1e-9, ~0ULL, 13},
                          {64, 1e-3, 1e-12, ~0ULL, 14}, {64, 0.01, 1e-9, 7ULL, 15}, {30, 0.0, 1e-10, ~0ULL, 16}};
    for (size_t ci = 0; ci < sizeof(cases) / sizeof(cases[0]); ci++) {
        const Case &cs = cases[ci];
        const int n = cs.n;
        pcg64 rg(cs.seed);
        std::uniform_real_distribution<double> u(-1, 1);
        std::vector<cplx> G(size_t(n) * n), A(size_t(n) * n);
        for (auto &z : G) z = cplx(u(rg), u(rg));
        // Case 6 has a rank-deficient G (last 5 rows zero) and mu = 0: singular A.
        if (cs.mu == 0.0)
            for (int r = n - 5; r < n; r++)
                for (int c = 0; c < n; c++) G[size_t(r) * n + c] = 0;
        for (int r = 0; r < n; r++)
            for (int c = 0; c < n; c++) {
                cplx s = 0;
                for (int t = 0; t < n; t++) s += std::conj(G[size_t(t) * n + r]) * G[size_t(t) * n + c];
                A[size_t(r) * n + c] = s / double(n) + (r == c ? cs.mu : 0.0);
            }
        RVec b(n);
        for (auto &z : b.d) z = cplx(u(rg), u(rg));
        RVec x(n);
        auto op = [&](const RVec &v) {
            RVec o(n);
            for (int r = 0; r < n; r++) {
                cplx s = 0;
                for (int c = 0; c < n; c++) s += A[size_t(r) * n + c] * v.d[c];
                o.d[r] = s;
            }
            return o;
        };
        auto res = minresqlp(op, b, x, cs.rtol, cs.maxit);
        std::vector<double> Ad, bd, xd;
        for (auto &z : A) { Ad.push_back(z.real()); Ad.push_back(z.imag()); }
        for (auto &z : b.d) { bd.push_back(z.real()); bd.push_back(z.imag()); }
        for (auto &z : x.d) { xd.push_back(z.real()); xd.push_back(z.imag()); }
        printf("{\"n\": %d, \"rtol\": %.17g, \"maxit\": \"%llu\", \"flag\": %d,\n", n, cs.rtol, cs.maxit, int(res.flag));
        print_dbls("A", Ad);
        print_dbls("b", bd);
        print_dbls("x", xd, true);
        printf("}%s\n", ci + 1 < sizeof(cases) / sizeof(cases[0]) ? "," : "");
    }
    printf("]\n}\n");
    return 0;
}
