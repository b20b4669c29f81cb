// Eigenvalues and eigenvectors of a small general complex matrix (K <= 4),
// replacing Eigen's eigenvalues() and ComplexEigenSolver in the reference's
// driver (code/rbm.cc:1186, 1198-1205): Householder reduction to Hessenberg
// form, shifted QR iterations with complex Givens rotations (Wilkinson shifts,
// exceptional shifts on stagnation) to the Schur form A = Q T Q^H, then
// eigenvectors by back-substitution in T, mapped through Q, unit-normalised.
#pragma once
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

namespace nqes_cli {

using cplx = std::complex<double>;

// A: n×n row-major. evals[q] = q-th diagonal of T; evecs: n×n row-major with
// column q the eigenvector of evals[q].
inline void small_eig(const cplx *A, int n, cplx *evals, cplx *evecs) {
    const double eps = std::numeric_limits<double>::epsilon();
    std::vector<cplx> T(A, A + n * n), Q(n * n, 0.0);
    for (int t = 0; t < n; t++) Q[t * n + t] = 1.0;
    auto at = [&](std::vector<cplx> &m, int r, int c) -> cplx & { return m[r * n + c]; };
    // Hessenberg reduction
    for (int k = 0; k + 2 < n; k++) {
        double nx = 0;
        for (int r = k + 1; r < n; r++) nx += std::norm(at(T, r, k));
        nx = std::sqrt(nx);
        if (nx == 0) continue;
        std::vector<cplx> v(n, 0.0);
        const cplx x0 = at(T, k + 1, k);
        const cplx ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cplx(1.0);
        for (int r = k + 1; r < n; r++) v[r] = at(T, r, k);
        v[k + 1] += ph * nx;
        double nv = 0;
        for (auto &z : v) nv += std::norm(z);
        nv = std::sqrt(nv);
        for (auto &z : v) z /= nv;
        // T <- (I - 2 v v^H) T (I - 2 v v^H), Q <- Q (I - 2 v v^H)
        for (int c = 0; c < n; c++) {
            cplx s = 0;
            for (int r = 0; r < n; r++) s += std::conj(v[r]) * at(T, r, c);
            for (int r = 0; r < n; r++) at(T, r, c) -= 2.0 * v[r] * s;
        }
        for (int r = 0; r < n; r++) {
            cplx s = 0, sq = 0;
            for (int c = 0; c < n; c++) {
                s += at(T, r, c) * v[c];
                sq += at(Q, r, c) * v[c];
            }
            for (int c = 0; c < n; c++) {
                at(T, r, c) -= 2.0 * s * std::conj(v[c]);
                at(Q, r, c) -= 2.0 * sq * std::conj(v[c]);
            }
        }
    }
    // shifted QR on the Hessenberg matrix
    int hi = n - 1, iter = 0, total = 0;
    while (hi > 0 && total < 10000) {
        int l = hi;
        while (l > 0 && std::abs(at(T, l, l - 1)) > eps * (std::abs(at(T, l, l)) + std::abs(at(T, l - 1, l - 1)))) l--;
        if (l > 0) at(T, l, l - 1) = 0.0;
        if (l == hi) {
            hi--;
            iter = 0;
            continue;
        }
        const cplx a = at(T, hi - 1, hi - 1), b = at(T, hi - 1, hi), c = at(T, hi, hi - 1), d = at(T, hi, hi);
        cplx mu;
        if (iter > 0 && iter % 10 == 0) {
            mu = d + std::abs(c) * cplx(0.75, 0.43);  // exceptional shift
        } else {
            const cplx tr = a + d, det = a * d - b * c;
            const cplx disc = std::sqrt(tr * tr / 4.0 - det);
            const cplx m1 = tr / 2.0 + disc, m2 = tr / 2.0 - disc;
            mu = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
        }
        for (int k = l; k <= hi; k++) at(T, k, k) -= mu;
        std::vector<double> cs(n);
        std::vector<cplx> sn(n);
        for (int k = l; k < hi; k++) {
            const cplx x = at(T, k, k), y = at(T, k + 1, k);
            const double r = std::hypot(std::abs(x), std::abs(y));
            double cc;
            cplx s;
            if (r == 0) {
                cc = 1;
                s = 0;
            } else if (std::abs(x) == 0) {
                cc = 0;
                s = std::conj(y) / std::abs(y);
            } else {
                cc = std::abs(x) / r;
                s = (x / std::abs(x)) * std::conj(y) / r;
            }
            cs[k] = cc;
            sn[k] = s;
            for (int j = k; j < n; j++) {
                const cplx t1 = at(T, k, j), t2 = at(T, k + 1, j);
                at(T, k, j) = cc * t1 + s * t2;
                at(T, k + 1, j) = -std::conj(s) * t1 + cc * t2;
            }
        }
        for (int k = l; k < hi; k++) {
            const double cc = cs[k];
            const cplx s = sn[k];
            for (int r = 0; r <= std::min(k + 2, hi); r++) {
                const cplx t1 = at(T, r, k), t2 = at(T, r, k + 1);
                at(T, r, k) = cc * t1 + std::conj(s) * t2;
                at(T, r, k + 1) = -s * t1 + cc * t2;
            }
            for (int r = 0; r < n; r++) {
                const cplx q1 = at(Q, r, k), q2 = at(Q, r, k + 1);
                at(Q, r, k) = cc * q1 + std::conj(s) * q2;
                at(Q, r, k + 1) = -s * q1 + cc * q2;
            }
        }
        for (int k = l; k <= hi; k++) at(T, k, k) += mu;
        iter++;
        total++;
    }
    double tnorm = 0;
    for (auto &z : T) tnorm = std::max(tnorm, std::abs(z));
    for (int k = 0; k < n; k++) {
        evals[k] = at(T, k, k);
        std::vector<cplx> y(n, 0.0);
        y[k] = 1.0;
        for (int j = k - 1; j >= 0; j--) {
            cplx s = 0;
            for (int l2 = j + 1; l2 <= k; l2++) s += at(T, j, l2) * y[l2];
            cplx den = at(T, j, j) - at(T, k, k);
            if (std::abs(den) < eps * tnorm) den = eps * tnorm;
            y[j] = -s / den;
        }
        double nrm = 0;
        std::vector<cplx> v(n, 0.0);
        for (int r = 0; r < n; r++) {
            for (int c = 0; c < n; c++) v[r] += at(Q, r, c) * y[c];
            nrm += std::norm(v[r]);
        }
        nrm = std::sqrt(nrm);
        for (int r = 0; r < n; r++) evecs[r * n + k] = v[r] / nrm;
    }
}

}  // namespace nqes_cli
