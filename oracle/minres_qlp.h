// CPU oracle — test infrastructure only. Nothing in the product links this file.
//
// Restatement of the reference's MINRES-QLP solver (code/minresqlp.h:112-456),
// which is the published MINRES-QLP method of Choi, Paige & Saunders (SIAM J.
// Sci. Comput. 33(4), 2011) for Hermitian A x = b. The reference is called with
// shift = 0, maxxnorm = 1e7, Acondlim = 1e15, TranCond = 1e7
// (code/rbm.cc:661-683). The steps follow the reference in order, including
// two properties a user of its results depends on:
//   * alfa = Re(r3^H v) (code/minresqlp.h:171);
//   * the plain-MINRES branch is taken only when a stop flag has already been
//     raised in the same iteration (code/minresqlp.h:253), so ordinary
//     iterations run the QLP update (code/minresqlp.h:262-299).
// Vector norms and dots are plain sums in index order (the reference uses
// Eigen's, code/minresqlp.h:125,173,178), so results agree to rounding.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <limits>
#include <vector>

namespace nqes_oracle {

using cplx = std::complex<double>;
using CVec = std::vector<cplx>;

struct QlpInfo {
    int flag = -2;
    uint64_t iters = 0;
    uint64_t qlp_iters = 0;
    double relres = 0, anorm = 0, acond = 0, xnorm = 0;
};

namespace qlp_detail {

inline double sgn(double a) { return std::copysign(1.0, a); }

// Stable Givens rotation [c s; s -c] [a; b] = [r; 0]  (code/minresqlp.h:85-110).
inline void givens(double a, double b, double &c, double &s, double &r) {
    if (b == 0) {
        c = (a == 0) ? 1.0 : sgn(a);
        s = 0;
        r = std::fabs(a);
    } else if (a == 0) {
        c = 0;
        s = sgn(b);
        r = std::fabs(b);
    } else if (std::fabs(b) > std::fabs(a)) {
        double t = a / b;
        s = sgn(b) / std::sqrt(1 + t * t);
        c = s * t;
        r = b / s;
    } else {
        double t = b / a;
        c = sgn(a) / std::sqrt(1 + t * t);
        s = c * t;
        r = a / c;
    }
}

inline double vnorm(const CVec &v) {
    double s = 0;
    for (const auto &z : v) s += std::norm(z);
    return std::sqrt(s);
}

// Re(sum conj(a_i) b_i)
inline double re_dot(const CVec &a, const CVec &b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i].real() * b[i].real() + a[i].imag() * b[i].imag();
    return s;
}

}  // namespace qlp_detail

// Solves A x = b for Hermitian A given as a callable out = A(v).
inline QlpInfo minres_qlp(const std::function<void(const CVec &, CVec &)> &A, const CVec &b,
                          CVec &x, double rtol, uint64_t maxit, double maxxnorm = 1e7,
                          double acondlim = 1e15, double trancond = 1e7) {
    using namespace qlp_detail;
    const size_t n = b.size();
    const double kTiny = std::numeric_limits<double>::min();
    const double kEps = std::numeric_limits<double>::epsilon();
    enum { kInternal = -2, kEigvec = -1, kZero = 0, kConv = 1, kConvLS = 2, kEps1 = 3,
           kEpsLS = 4, kEigConv = 5, kXNorm = 6, kACond = 7, kMaxIt = 8, kSingular = 9 };

    CVec r1(b), r2(b), r3(b), v(n), Av(n);
    CVec w(n), wl(n), wl2(n), xl2(n);
    x.assign(n, cplx(0));
    const double beta1 = vnorm(b);

    int flag = kInternal;
    uint64_t iters = 0, qlp = 0;
    double beta = 0, tau = 0, taul = 0, phi = beta1, betan = beta1, gmin = 0, gminl = 0;
    double cs = -1, sn = 0, cr1 = -1, sr1 = 0, cr2 = -1, sr2 = 0, dltan = 0, eplnn = 0;
    double gama = 0, gamal = 0, gamal2 = 0, eta = 0, etal = 0, etal2 = 0;
    double vepln = 0, veplnl = 0, veplnl2 = 0, ul3 = 0, ul2 = 0, ul = 0, u = 0;
    double gama_qlp = 0, gamal_qlp = 0, vepln_qlp = 0, u_qlp = 0, ul_qlp = 0;
    double rnorm = betan, xnorm = 0, xl2norm = 0, axnorm = 0, anorm = 0, acond = 1;
    double relres = rnorm / (beta1 + 1e-50);

    if (beta1 == 0) flag = kZero;

    while (flag == kInternal && iters < maxit) {
        // Lanczos step.
        iters++;
        const double betal = beta;
        beta = betan;
        for (size_t i = 0; i < n; i++) v[i] = r3[i] / beta;
        A(v, Av);
        r3 = Av;
        if (iters > 1) {
            const double q = beta / betal;
            for (size_t i = 0; i < n; i++) r3[i] -= r1[i] * q;
        }
        const double alfa = re_dot(r3, v);
        {
            const double q = alfa / beta;
            for (size_t i = 0; i < n; i++) r3[i] -= r2[i] * q;
        }
        r1 = r2;
        r2 = r3;
        betan = vnorm(r3);
        if (iters == 1 && betan == 0) {
            if (alfa == 0) {
                flag = kZero;
            } else {
                flag = kEigvec;
                for (size_t i = 0; i < n; i++) x[i] = b[i] / alfa;
            }
            break;
        }
        const double pnorm = std::sqrt(betal * betal + alfa * alfa + betan * betan);

        // Previous left rotation Q_{k-1}.
        const double dbar = dltan;
        double dlta = cs * dbar + sn * alfa;
        const double epln = eplnn;
        const double gbar = sn * dbar - cs * alfa;
        eplnn = sn * betan;
        dltan = -cs * betan;
        const double dlta_qlp = dlta;
        // Current left rotation Q_k.
        const double gamal3 = gamal2;
        gamal2 = gamal;
        gamal = gama;
        givens(gbar, betan, cs, sn, gama);
        const double gama_tmp = gama;
        const double taul2 = taul;
        taul = tau;
        tau = cs * phi;
        axnorm = std::sqrt(axnorm * axnorm + tau * tau);
        phi = sn * phi;
        // Previous right rotation P_{k-2,k}.
        if (iters > 2) {
            veplnl2 = veplnl;
            etal2 = etal;
            etal = eta;
            const double dlta_tmp = sr2 * vepln - cr2 * dlta;
            veplnl = cr2 * vepln + sr2 * dlta;
            dlta = dlta_tmp;
            eta = sr2 * gama;
            gama = -cr2 * gama;
        }
        // Current right rotation P_{k-1,k}.
        if (iters > 1) {
            givens(gamal, dlta, cr1, sr1, gamal);
            vepln = sr1 * gama;
            gama = -cr1 * gama;
        }

        // Solution-norm recurrences.
        const double ul4 = ul3;
        ul3 = ul2;
        if (iters > 2) ul2 = (taul2 - etal2 * ul4 - veplnl2 * ul3) / gamal2;
        if (iters > 1) ul = (taul - etal * ul3 - veplnl * ul2) / gamal;
        const double xnorm_tmp = std::sqrt(xl2norm * xl2norm + ul2 * ul2 + ul * ul);
        if (std::fabs(gama) > kTiny && xnorm_tmp < maxxnorm) {
            u = (tau - eta * ul2 - vepln * ul) / gama;
            if (std::sqrt(xnorm_tmp * xnorm_tmp + u * u) > maxxnorm) {
                u = 0;
                flag = kXNorm;
            }
        } else {
            u = 0;
            flag = kSingular;
        }
        xl2norm = std::sqrt(xl2norm * xl2norm + ul2 * ul2);
        xnorm = std::sqrt(xl2norm * xl2norm + ul * ul + u * u);

        // Update w and x.
        if (acond < trancond && flag != kInternal && qlp == 0) {
            // Plain MINRES update.
            wl2 = wl;
            wl = w;
            for (size_t i = 0; i < n; i++) w[i] = (v[i] - epln * wl2[i] - dlta_qlp * wl[i]) / gama_tmp;
            if (xnorm < maxxnorm) {
                for (size_t i = 0; i < n; i++) x[i] += tau * w[i];
            } else {
                flag = kXNorm;
            }
        } else {
            // MINRES-QLP update.
            qlp++;
            if (qlp == 1 && iters > 1) {
                // Rebuild w_{k-3}, w_{k-2}, w_{k-1} on the switch from MINRES.
                if (iters > 3)
                    for (size_t i = 0; i < n; i++) wl2[i] = gamal3 * wl2[i] + veplnl2 * wl[i] + etal * w[i];
                if (iters > 2)
                    for (size_t i = 0; i < n; i++) wl[i] = gamal_qlp * wl[i] + vepln_qlp * w[i];
                for (size_t i = 0; i < n; i++) w[i] = gama_qlp * w[i];
                for (size_t i = 0; i < n; i++) xl2[i] = x[i] - wl[i] * ul_qlp - w[i] * u_qlp;
            }
            if (iters == 1) {
                wl2 = wl;
                for (size_t i = 0; i < n; i++) { wl[i] = v[i] * sr1; w[i] = -v[i] * cr1; }
            } else if (iters == 2) {
                wl2 = wl;
                for (size_t i = 0; i < n; i++) {
                    const cplx wi = w[i];
                    wl[i] = wi * cr1 + v[i] * sr1;
                    w[i] = wi * sr1 - v[i] * cr1;
                }
            } else {
                for (size_t i = 0; i < n; i++) {
                    const cplx p_wl = wl[i], p_w = w[i];
                    const cplx nw = p_wl * sr2 - v[i] * cr2;       // rotate (w_{k-2}, v)
                    const cplx nwl2 = p_wl * cr2 + v[i] * sr2;
                    const cplx t = p_w * cr1 + nw * sr1;           // rotate (w_{k-1}, new w)
                    w[i] = p_w * sr1 - nw * cr1;
                    wl[i] = t;
                    wl2[i] = nwl2;
                    v[i] = t;
                }
            }
            for (size_t i = 0; i < n; i++) {
                xl2[i] += wl2[i] * ul2;
                x[i] = xl2[i] + wl[i] * ul + w[i] * u;
            }
        }

        // Next right rotation P_{k-1,k+1}.
        const double gamal_tmp = gamal;
        givens(gamal, eplnn, cr2, sr2, gamal);
        gamal_qlp = gamal_tmp;
        vepln_qlp = vepln;
        gama_qlp = gama;
        ul_qlp = ul;
        u_qlp = u;

        // Norm and condition estimates.
        const double abs_gama = std::fabs(gama);
        anorm = std::max({anorm, pnorm, gamal, abs_gama});
        if (iters == 1) {
            gmin = gama;
            gminl = gmin;
        } else {
            const double gminl2 = gminl;
            gminl = gmin;
            gmin = std::min({gminl2, gamal, abs_gama});
        }
        const double acondl = acond;
        acond = anorm / gmin;
        const double rnorml = rnorm;
        const double relresl = relres;
        if (flag != kSingular) rnorm = phi;
        relres = rnorm / (anorm * xnorm + beta1);
        const double rootl = std::sqrt(gbar * gbar + dltan * dltan);
        const double relaresl = rootl / anorm;
        const double epsx = anorm * xnorm * kEps;

        // Stopping tests, later tests taking precedence (code/minresqlp.h:336-364).
        if (flag == kInternal || flag == kSingular) {
            const double t1 = 1 + relres, t2 = 1 + relaresl;
            if (iters >= maxit) flag = kMaxIt;
            if (acond >= acondlim) flag = kACond;
            if (xnorm >= maxxnorm) flag = kXNorm;
            if (epsx >= beta1) flag = kEigConv;
            if (t2 <= 1) flag = kEpsLS;
            if (t1 <= 1) flag = kEps1;
            if (relaresl <= rtol) flag = kConvLS;
            if (relres <= rtol) flag = kConv;
        }
        if (flag == kConvLS || flag == kEpsLS || flag == kXNorm || flag == kACond) {
            iters--;
            acond = acondl;
            rnorm = rnorml;
            relres = relresl;
        }
    }

    QlpInfo info;
    info.flag = flag;
    info.iters = iters;
    info.qlp_iters = qlp;
    info.relres = relres;
    info.anorm = anorm;
    info.acond = acond;
    info.xnorm = xnorm;
    return info;
}

}  // namespace nqes_oracle
