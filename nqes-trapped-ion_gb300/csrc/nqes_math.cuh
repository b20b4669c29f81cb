// Scalar arithmetic shared by every kernel of the library.
//
// Kernels are written once over a scalar type S that is either `double`
// (real arithmetic: all weights, J and h real, so every amplitude, ratio,
// local energy and log-derivative is real) or `cplx` (complex arithmetic, the
// general case of code/rbm.cc:25-26). With real inputs the complex algebra of
// the reference stays exactly real, so the real instantiation computes the
// same quantities with a quarter of the FP64 work.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace nqes {

struct __align__(16) cplx {
    double re, im;
};

__host__ __device__ __forceinline__ cplx mk(double r, double i) { return cplx{r, i}; }
__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return {-a.re, -a.im}; }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
    return {fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re)};
}
__host__ __device__ __forceinline__ cplx operator*(cplx a, double s) { return {a.re * s, a.im * s}; }
__host__ __device__ __forceinline__ cplx operator*(double s, cplx a) { return {a.re * s, a.im * s}; }
__host__ __device__ __forceinline__ cplx operator/(cplx a, double s) { return {a.re / s, a.im / s}; }
__host__ __device__ __forceinline__ cplx &operator+=(cplx &a, cplx b) { a = a + b; return a; }
__host__ __device__ __forceinline__ cplx &operator-=(cplx &a, cplx b) { a = a - b; return a; }
__host__ __device__ __forceinline__ cplx &operator*=(cplx &a, cplx b) { a = a * b; return a; }
__host__ __device__ __forceinline__ bool operator==(cplx a, cplx b) { return a.re == b.re && a.im == b.im; }

// Scalar-type traits: one name per operation for both real and complex S.
__host__ __device__ __forceinline__ double re(double x) { return x; }
__host__ __device__ __forceinline__ double re(cplx x) { return x.re; }
__host__ __device__ __forceinline__ double im(double) { return 0.0; }
__host__ __device__ __forceinline__ double im(cplx x) { return x.im; }
__host__ __device__ __forceinline__ double conj(double x) { return x; }
__host__ __device__ __forceinline__ cplx conj(cplx x) { return {x.re, -x.im}; }
__host__ __device__ __forceinline__ double norm2(double x) { return x * x; }
__host__ __device__ __forceinline__ double norm2(cplx x) { return fma(x.re, x.re, x.im * x.im); }
template <class S> __host__ __device__ __forceinline__ S one();
template <> __host__ __device__ __forceinline__ double one<double>() { return 1.0; }
template <> __host__ __device__ __forceinline__ cplx one<cplx>() { return {1.0, 0.0}; }
template <class S> __host__ __device__ __forceinline__ S zero();
template <> __host__ __device__ __forceinline__ double zero<double>() { return 0.0; }
template <> __host__ __device__ __forceinline__ cplx zero<cplx>() { return {0.0, 0.0}; }
template <class S> __host__ __device__ __forceinline__ S from_c(cplx z);
template <> __host__ __device__ __forceinline__ double from_c<double>(cplx z) { return z.re; }
template <> __host__ __device__ __forceinline__ cplx from_c<cplx>(cplx z) { return z; }
__host__ __device__ __forceinline__ cplx to_c(double x) { return {x, 0.0}; }
__host__ __device__ __forceinline__ cplx to_c(cplx x) { return x; }
// a*b + c
__host__ __device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }
__host__ __device__ __forceinline__ cplx mad(cplx a, cplx b, cplx c) {
    return {fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im))};
}
// conj(a)*b + c
__host__ __device__ __forceinline__ double cmad(double a, double b, double c) { return fma(a, b, c); }
__host__ __device__ __forceinline__ cplx cmad(cplx a, cplx b, cplx c) {
    return {fma(a.re, b.re, fma(a.im, b.im, c.re)), fma(a.re, b.im, fma(-a.im, b.re, c.im))};
}
__host__ __device__ __forceinline__ double inv(double x) { return 1.0 / x; }
__host__ __device__ __forceinline__ cplx inv(cplx x) {
    double d = 1.0 / fma(x.re, x.re, x.im * x.im);
    return {x.re * d, -x.im * d};
}
__host__ __device__ __forceinline__ bool finite(double x) { return isfinite(x); }
__host__ __device__ __forceinline__ bool finite(cplx x) { return isfinite(x.re) && isfinite(x.im); }
__host__ __device__ __forceinline__ bool is_zero(double x) { return x == 0.0; }
__host__ __device__ __forceinline__ bool is_zero(cplx x) { return x.re == 0.0 && x.im == 0.0; }

// Elementary functions.
__device__ __forceinline__ double cexp_(double x) { return exp(x); }
__device__ __forceinline__ cplx cexp_(cplx z) {
    double e = exp(z.re), s, c;
    sincos(z.im, &s, &c);
    return {e * c, e * s};
}
__device__ __forceinline__ double ccosh_(double x) { return cosh(x); }
__device__ __forceinline__ cplx ccosh_(cplx z) {
    double s, c;
    sincos(z.im, &s, &c);
    return {cosh(z.re) * c, sinh(z.re) * s};
}
__device__ __forceinline__ double csinh_(double x) { return sinh(x); }
__device__ __forceinline__ cplx csinh_(cplx z) {
    double s, c;
    sincos(z.im, &s, &c);
    return {sinh(z.re) * c, cosh(z.re) * s};
}
__device__ __forceinline__ double ctanh_(double x) { return tanh(x); }
// tanh(x+iy) = (sinh 2x + i sin 2y) / (cosh 2x + cos 2y), with the large-|x|
// limit taken explicitly so that no inf/inf arises.
__device__ __forceinline__ cplx ctanh_(cplx z) {
    if (fabs(z.re) > 20.0) {
        double s, c;
        sincos(2.0 * z.im, &s, &c);
        double e = exp(-2.0 * fabs(z.re));
        return {copysign(1.0, z.re), 2.0 * s * e};
    }
    double s, c;
    sincos(2.0 * z.im, &s, &c);
    double d = cosh(2.0 * z.re) + c;
    return {sinh(2.0 * z.re) / d, s / d};
}

// Exact power-of-two scaling (used to keep rows of Phi in range without
// changing any ratio): x * 2^e for real and complex.
__device__ __forceinline__ double scale2(double x, int e) { return ldexp(x, e); }
__device__ __forceinline__ cplx scale2(cplx x, int e) { return {ldexp(x.re, e), ldexp(x.im, e)}; }
// Binary exponent of the larger component (0 for zero), from the bit pattern.
__device__ __forceinline__ int expo(double x) {
    int hi = __double2hiint(x);
    int e = (hi >> 20) & 0x7ff;
    return e == 0 ? -1023 : e - 1023;
}
__device__ __forceinline__ int expo(cplx x) { return max(expo(x.re), expo(x.im)); }

// Warp-level reductions.
__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ cplx shfl_xor(cplx v, int m) {
    return {__shfl_xor_sync(0xffffffffu, v.re, m), __shfl_xor_sync(0xffffffffu, v.im, m)};
}
template <class S> __device__ __forceinline__ S warp_sum(S v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v = v + shfl_xor(v, m);
    return v;
}
template <class S> __device__ __forceinline__ S warp_prod(S v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v = v * shfl_xor(v, m);
    return v;
}

// Small K×K (K <= 4) row-major matrix helpers, run by one thread.
template <class S> __host__ __device__ inline S small_det(const S *m, int K) {
    if (K == 1) return m[0];
    if (K == 2) return m[0] * m[3] - m[2] * m[1];
    if (K == 3) {
        auto h3 = [&](int a, int b, int c) {
            return m[a * 3] * (m[b * 3 + 1] * m[c * 3 + 2] - m[b * 3 + 2] * m[c * 3 + 1]);
        };
        return h3(0, 1, 2) - h3(1, 0, 2) + h3(2, 0, 1);
    }
    // K == 4: Laplace expansion along the first column.
    S d = zero<S>();
    for (int r = 0; r < 4; r++) {
        int rr[3], t = 0;
        for (int q = 0; q < 4; q++)
            if (q != r) rr[t++] = q;
        auto e = [&](int a, int c) { return m[rr[a] * 4 + c]; };
        S minor = e(0, 1) * (e(1, 2) * e(2, 3) - e(1, 3) * e(2, 2)) - e(1, 1) * (e(0, 2) * e(2, 3) - e(0, 3) * e(2, 2)) +
                  e(2, 1) * (e(0, 2) * e(1, 3) - e(0, 3) * e(1, 2));
        S term = m[r * 4] * minor;
        d = (r & 1) ? d - term : d + term;
    }
    return d;
}

// Inverse by Gauss-Jordan with partial pivoting; false when singular.
template <class S> __host__ __device__ inline bool small_inv(const S *m, S *out, int K) {
    S a[16];
    for (int t = 0; t < K * K; t++) {
        a[t] = m[t];
        out[t] = zero<S>();
    }
    for (int t = 0; t < K; t++) out[t * K + t] = one<S>();
    for (int c = 0; c < K; c++) {
        int p = c;
        double best = norm2(a[c * K + c]);
        for (int r = c + 1; r < K; r++) {
            double v = norm2(a[r * K + c]);
            if (v > best) {
                best = v;
                p = r;
            }
        }
        if (best == 0.0) return false;
        if (p != c)
            for (int j = 0; j < K; j++) {
                S t1 = a[p * K + j];
                a[p * K + j] = a[c * K + j];
                a[c * K + j] = t1;
                S t2 = out[p * K + j];
                out[p * K + j] = out[c * K + j];
                out[c * K + j] = t2;
            }
        S piv = inv(a[c * K + c]);
        for (int j = 0; j < K; j++) {
            a[c * K + j] = a[c * K + j] * piv;
            out[c * K + j] = out[c * K + j] * piv;
        }
        for (int r = 0; r < K; r++) {
            if (r == c) continue;
            S f = a[r * K + c];
            for (int j = 0; j < K; j++) {
                a[r * K + j] = a[r * K + j] - f * a[c * K + j];
                out[r * K + j] = out[r * K + j] - f * out[c * K + j];
            }
        }
    }
    return true;
}

// Moore-Penrose pseudo-inverse of a K×K matrix (K <= 4), the role of Eigen's
// completeOrthogonalDecomposition().pseudoInverse() (code/rbm.cc:547, 608),
// by full-rank factorisation: the columns that Gram-Schmidt finds
// independent (residual norm above 1e-14 of the largest column norm, a
// relative rank threshold as the decomposition's) form C (K×r), A = C F with
// F = (C^H C)^-1 C^H A, and A+ = F^H (F F^H)^-1 (C^H C)^-1 C^H. Returns the
// rank r; a zero matrix gives zero.
template <class S> __host__ __device__ inline int small_pinv(const S *a, S *out, int K) {
    S q[16], c[16], f[16], g[16], gi[16], h[16], hi[16], t1[16];
    int sel[4], r = 0;
    double maxn = 0.0;
    for (int j = 0; j < K; j++) {
        double n = 0.0;
        for (int i = 0; i < K; i++) n += norm2(a[i * K + j]);
        maxn = n > maxn ? n : maxn;
    }
    for (int t = 0; t < K * K; t++) out[t] = zero<S>();
    for (int j = 0; j < K && maxn > 0.0; j++) {
        S v[4];
        for (int i = 0; i < K; i++) v[i] = a[i * K + j];
        for (int t = 0; t < r; t++) {
            S d = zero<S>();
            for (int i = 0; i < K; i++) d = d + conj(q[i * 4 + t]) * v[i];
            for (int i = 0; i < K; i++) v[i] = v[i] - q[i * 4 + t] * d;
        }
        double n2 = 0.0;
        for (int i = 0; i < K; i++) n2 += norm2(v[i]);
        if (n2 > 1e-28 * maxn) {
            const double s = 1.0 / sqrt(n2);
            for (int i = 0; i < K; i++) q[i * 4 + r] = v[i] * s;
            sel[r++] = j;
        }
    }
    if (r == 0) return 0;
    for (int i = 0; i < K; i++)  // C = the selected columns (K×r)
        for (int t = 0; t < r; t++) c[i * r + t] = a[i * K + sel[t]];
    for (int s1 = 0; s1 < r; s1++)  // G = C^H C (r×r)
        for (int s2 = 0; s2 < r; s2++) {
            S acc = zero<S>();
            for (int i = 0; i < K; i++) acc = acc + conj(c[i * r + s1]) * c[i * r + s2];
            g[s1 * r + s2] = acc;
        }
    if (!small_inv(g, gi, r)) return r;
    for (int s1 = 0; s1 < r; s1++)  // t1 = G^-1 C^H (r×K)
        for (int i = 0; i < K; i++) {
            S acc = zero<S>();
            for (int s2 = 0; s2 < r; s2++) acc = acc + gi[s1 * r + s2] * conj(c[i * r + s2]);
            t1[s1 * K + i] = acc;
        }
    for (int s1 = 0; s1 < r; s1++)  // F = G^-1 C^H A (r×K)
        for (int j = 0; j < K; j++) {
            S acc = zero<S>();
            for (int i = 0; i < K; i++) acc = acc + t1[s1 * K + i] * a[i * K + j];
            f[s1 * K + j] = acc;
        }
    for (int s1 = 0; s1 < r; s1++)  // H = F F^H (r×r)
        for (int s2 = 0; s2 < r; s2++) {
            S acc = zero<S>();
            for (int j = 0; j < K; j++) acc = acc + f[s1 * K + j] * conj(f[s2 * K + j]);
            h[s1 * r + s2] = acc;
        }
    if (!small_inv(h, hi, r)) return r;
    for (int j = 0; j < K; j++)  // A+ = F^H H^-1 (G^-1 C^H)
        for (int i = 0; i < K; i++) {
            S acc = zero<S>();
            for (int s1 = 0; s1 < r; s1++) {
                S u = zero<S>();
                for (int s2 = 0; s2 < r; s2++) u = u + hi[s1 * r + s2] * t1[s2 * K + i];
                acc = acc + conj(f[s1 * K + j]) * u;
            }
            out[j * K + i] = acc;
        }
    return r;
}

// ---- e^{-x}, x >= 0, from a table (the Phi row rebuilds of the decision-warp sampler) ----
// x = n/64 + r with n = rint(64 x) and |r| <= 1/128, so e^{-x} = T[n] e^{-r}
// with T[n] = e^{-n/64} (a table of kExpTabN entries built with exp() when a
// context is created) and e^{-r} from its Taylor polynomial of degree 6
// (truncation below (1/128)^7 / 7! < 2^-58). r = x - n/64 is exact (n = 0, or
// n/64 within 1/128 of x >= 1/128). About 1.5 ulp, ten FP64 operations
// against the ~25 of exp(). Beyond the table (x > 40) e^{-x} < 2^-57, under
// half an ulp of the 1 it is added to, and 0 is returned; NaN stays NaN.
constexpr int kExpTabN = 2561;
__device__ __forceinline__ double exp_neg_tab(double x, const double *__restrict__ tab) {
    const double t = x * 64.0;
    if (!(t < 2560.0)) return t >= 2560.0 ? 0.0 : x;  // x is NaN in the second case
    // rint(t) by the 1.5 * 2^52 shift (t in [0, 2560)): the integer in the low word
    const double sh = t + 6755399441055744.0;
    const int n = __double2loint(sh);
    const double r = fma(sh - 6755399441055744.0, -0.015625, x);
    const double q = -r;
    double p = 1.0 / 720.0;
    p = fma(p, q, 1.0 / 120.0);
    p = fma(p, q, 1.0 / 24.0);
    p = fma(p, q, 1.0 / 6.0);
    p = fma(p, q, 0.5);
    p = fma(p, q, 1.0);
    p = fma(p, q, 1.0);
    return __ldg(tab + n) * p;
}

// ---- double-float (hi + lo FP32 pairs) on the FP32 pipe ----

// d as hi + lo: hi = d cut to 24 significant bits, lo = the remaining 29
// bits rounded to 24, by integer operations (no FP64 instruction), so that
// |d - hi - lo| <= 2^-48 |d|; |d| < 2^-126 gives 0. Returns false when
// |d| >= 2^127 or d is not finite.
__device__ __forceinline__ bool df_split(double d, float &hi, float &lo) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
    const unsigned hw = unsigned(b >> 32), lw = unsigned(b);
    const unsigned ax = hw & 0x7fffffffu, sgn = hw & 0x80000000u;
    // biased exponent e = ax >> 20; hi is representable as a normal float for
    // 897 <= e <= 1150: exponent e - 896, mantissa the top 23 of d's 52 bits
    const bool nrm = ax >= 0x38100000u;
    const unsigned hb = __funnelshift_l(lw, ax - 0x38000000u, 3);
    hi = __uint_as_float(nrm ? (hb | sgn) : sgn);
    // lo = sign * r * 2^(e - 1075) with r the low 29 mantissa bits; the scale
    // is a normal float for e >= 949 (below, |lo| < 2^-149 |...|: dropped)
    const unsigned e = ax >> 20;
    const float sc = __uint_as_float((e - 948u) << 23);
    const float l = __uint2float_rn(lw & 0x1fffffffu) * sc;
    lo = e >= 949u ? __uint_as_float(__float_as_uint(l) | sgn) : 0.f;
    return ax < 0x47f00000u;
}

// (sh, sl) += (ah + al) (bh + bl): the product to 2^-48 relative (its FMA
// error term and the two cross terms), added with TwoSum into sh and the
// rounding error and low terms into sl.
__device__ __forceinline__ void df_fma(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// (ah, al) *= (bh, bl): the product to a few 2^-48, renormalised
__device__ __forceinline__ void df_mul(float &ah, float &al, float bh, float bl) {
    const float p = ah * bh;
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    ah = __fadd_rn(p, e);
    al = __fsub_rn(e, __fsub_rn(ah, p));
}

// (ah, al) += (bh, bl)
__device__ __forceinline__ void df_acc(float &ah, float &al, float bh, float bl) {
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    ah = s;
    al = __fadd_rn(al, __fadd_rn(err, bl));
}


// Two double-float lanes at once with the packed FP32 instructions of sm_100
// and later (add/sub/mul/fma .f32x2 on 64-bit register pairs): one
// instruction does a lane's operation for both, with per-lane round to
// nearest, so results equal two scalar evaluations bit for bit.
__device__ __forceinline__ uint64_t f2_pack(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t r, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// df_fma on two lanes: (sh, sl) += (ah + al)(bh + bl), with bn = -bh given
// (the products' negations are exact, so no negation instruction is needed):
// -p = ah bn, the product's error fma(ah, bh, -p), the cross terms, TwoSum of
// sh + p from the negated product.
__device__ __forceinline__ void df_fma2(uint64_t &sh, uint64_t &sl, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                        uint64_t bn) {
    const uint64_t pn = f2_mul(ah, bn);
    uint64_t e = f2_fma(ah, bh, pn);
    e = f2_fma(ah, bl, e);
    e = f2_fma(al, bh, e);
    const uint64_t s = f2_sub(sh, pn);
    const uint64_t bb = f2_sub(s, sh);
    const uint64_t err = f2_sub(f2_sub(sh, f2_sub(s, bb)), f2_add(pn, bb));
    sh = s;
    sl = f2_add(sl, f2_add(err, e));
}

}  // namespace nqes
