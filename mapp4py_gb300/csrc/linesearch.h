// Line searches of the minimizers along x = x0 + alpha h.  Host code: each
// trial is one device energy evaluation behind Fn::F(alpha), so the search
// itself is a handful of scalars per iteration.
//
// The three searches are the reference's (ls.h): back-tracking (Armijo,
// LineSearchBackTrack::min 711-769), golden section (LineSearchGoldenSection
// ::min 340-515) and Brent's parabolic/golden method (LineSearchBrent::min
// 524-706), the last two optionally after the bracketing of
// LineSearch::bracket (214-335).  Their decision rules, constants and
// evaluation order are kept, so the sequence of trial steps - and with it
// the trajectory - is the reference's.  The caller's ls_prep (MinMDHandler::
// ls_prep, min_cg.h:230-256) supplies dfa = -f.h and max_a = max_dx/max|h|
// and handles the three early exits.
#pragma once

#include <math.h>

#include <algorithm>
#include <limits>

#include "mappg.h"

namespace mappg {

// stop codes shared with the minimizers (ls.h:9-22, plus the force stop)
enum {
    LS_S,
    LS_F_DOWNHILL,
    LS_F_GRAD0,
    LS_MIN_ALPHA,
    MIN_S_TOLERANCE,
    MIN_F_MAX_ITER,
    B_S,
    B_F_MAX_ALPHA,
    B_F_DOWNHILL,
    MIN_S_FTOL = 100
};

struct LsParams {
    int kind = MAPPG_LS_BT;
    double c = 0.4, rho = 0.5, min_alpha = 0.0;  // back-tracking (ls.cpp:456-461)
    double tol = sqrt(2.0 * std::numeric_limits<double>::epsilon());  // golden, Brent (ls.cpp:95-100,262-268)
    int max_iter = 5;
    bool bracket = true;
    double zeps = std::numeric_limits<double>::epsilon() * 1.0e-3;  // Brent
};

// Fn: double F(double alpha) leaves the system at x0 + alpha h and returns
// its energy; void reset() puts it back at x0.
template <class Fn>
struct LineSearch {
    const LsParams& p;
    Fn& fn;
    double prev_val = -1.0;  // kept across iterations of one run
    static constexpr double eps = std::numeric_limits<double>::epsilon();
    const double sqrt_eps = sqrt(std::numeric_limits<double>::epsilon());
    const double golden = 0.5 + 0.5 * sqrt(5.0);
    static constexpr double gold = 0.61803399, cgold = 0.38196601;

    LineSearch(const LsParams& p_, Fn& fn_) : p(p_), fn(fn_) {}

    // dfa < 0 and max_a > 0 (the caller's ls_prep checks); nrgy is the energy
    // at x0 on entry and at the accepted point on return
    int min(double dfa, double max_a, double& nrgy, double& alpha, int init_flag) {
        switch (p.kind) {
            case MAPPG_LS_GOLDEN: return golden_section(dfa, max_a, nrgy, alpha);
            case MAPPG_LS_BRENT: return brent(dfa, max_a, nrgy, alpha);
            default: return backtrack(dfa, max_a, nrgy, alpha, init_flag);
        }
    }

    int backtrack(double dfa, double max_a, double& nrgy, double& alpha, int init_flag) {
        const double e0 = nrgy;
        if (init_flag == 0) {
            max_a = std::min(max_a, 1.0);
        } else if (init_flag == 1) {
            // conjugate gradients: no longer than the previous step's decrease allows
            if (prev_val > 0.0 && dfa < 0.0) max_a = std::min(max_a, -prev_val / dfa);
            prev_val = -dfa;
        }
        if (max_a <= p.min_alpha) return LS_MIN_ALPHA;
        alpha = max_a;
        while (true) {
            double ideal = nrgy + alpha * p.c * dfa;
            double e = fn.F(alpha);
            if (e <= ideal) {
                if (init_flag == 1) prev_val *= alpha;
                nrgy = e;
                return LS_S;
            }
            alpha *= p.rho;
            if (alpha <= p.min_alpha) {
                nrgy = e0;
                fn.reset();
                return LS_MIN_ALPHA;
            }
        }
    }

    // a < b < c with f(b) below f(a) and f(c), starting from a = 0
    int bracket(double dfa, double max_a, double& a, double& b, double& c, double& fa, double& fb, double& fc) {
        double q = 1.0e-14 / (max_a * fabs(dfa));
        if (0.01 < q && q < 1.0)
            b = q * max_a;
        else if (q >= 1.0)
            b = max_a;
        else
            b = 0.01 * max_a;
        fb = fn.F(b);
        if (fb >= fa) {
            // first trial uphill: shrink towards 0 with a quadratic model
            c = b;
            fc = fb;
            int left = 20;
            double r = (fa - fc) / (c * dfa);
            b = c * 0.5 / (1.0 + r);
            while (fb >= fa && left && b > eps) {
                fb = fn.F(b);
                if (fb < fa) break;
                c = b;
                fc = fb;
                left--;
                r = (fa - fc) / (c * dfa);
                b = c * 0.5 / (1.0 + r);
            }
            if (fb >= fa) {
                b = sqrt_eps < max_a ? sqrt_eps : max_a;
                fb = fn.F(b);
                if (fb >= fa) return B_F_DOWNHILL;
            }
            return B_S;
        }
        // downhill: grow by the golden ratio with parabolic steps, up to max_a
        fc = fb;
        while (fb >= fc) {
            c = b + golden * (b - a);
            if (c >= max_a) {
                c = max_a;
                fc = fn.F(c);
                return B_S;
            }
            fc = fn.F(c);
            if (fc > fb) break;
            const double ulim = max_a;
            double r = (b - a) * (fb - fc);
            q = (b - c) * (fb - fa);
            double u = b - ((b - c) * q - (b - a) * r) / (2.0 * (q - r));
            if (b < u && u < c) {
                double fu = fn.F(u);
                if (fu < fc) {
                    a = b;
                    b = u;
                    fa = fb;
                    fb = fu;
                    return B_S;
                } else if (fu > fb) {
                    c = u;
                    fc = fu;
                    return B_S;
                }
                a = b;
                b = c;
                fa = fb;
                fb = fc;
            } else if (u > c) {
                u = std::min(u, ulim);
                double fu = fn.F(u);
                a = b;
                b = c;
                c = u;
                fa = fb;
                fb = fc;
                fc = fu;
            } else {
                a = b;
                b = c;
                fa = fb;
                fb = fc;
            }
        }
        return B_S;
    }

    int golden_section(double dfa, double max_a, double& nrgy, double& alpha) {
        int calc = 0;  // which of x1 (1) and x2 (2) was evaluated last
        double x0, x1, x2, x3, f1, f2;
        double a = 0.0, fa = nrgy;
        if (p.bracket) {
            double b, c, fb, fc;
            int chk = bracket(dfa, max_a, a, b, c, fa, fb, fc);
            if (chk != B_S) {
                fn.reset();
                return chk;
            }
            x0 = a;
            x3 = c;
            if (c - b > b - a) {
                x1 = b;
                x2 = b + cgold * (c - b);
                f1 = fb;
                f2 = fn.F(x2);
                calc = 2;
            } else {
                x1 = b + cgold * (a - b);
                x2 = b;
                f1 = fn.F(x1);
                f2 = fb;
                calc = 1;
            }
            int left = p.max_iter;
            while (x3 - x0 > p.tol * (x1 + x2) && x3 - x0 > eps && left) {
                if (f2 < f1) {
                    x0 = x1;
                    x1 = x2;
                    x2 = gold * x2 + cgold * x3;
                    f1 = f2;
                    f2 = fn.F(x2);
                    calc = 2;
                } else {
                    x3 = x2;
                    x2 = x1;
                    x1 = gold * x1 + cgold * x0;
                    f2 = f1;
                    f1 = fn.F(x1);
                    calc = 1;
                }
                left--;
            }
        } else {
            // the whole interval [0, max_a], without bracketing
            f1 = f2 = 0.0;
            x0 = x1 = x2 = 0.0;
            double f0 = fa;
            x3 = max_a;
            double f3 = fn.F(x3);
            int left = p.max_iter;
            bool have_left = false, have_right = false;
            while (x3 - x0 > p.tol * (x1 + x2) && x3 - x0 > eps && left) {
                double delta = cgold * (x3 - x0);
                if (!have_left) {
                    x1 = x0 + delta;
                    f1 = fn.F(x1);
                    calc = 1;
                    have_left = true;
                }
                if (!have_right) {
                    x2 = x3 - delta;
                    f2 = fn.F(x2);
                    calc = 2;
                    have_right = true;
                }
                if ((f0 < f2 && f0 < f3) || (f1 < f2 && f1 < f3)) {
                    have_left = false;
                    x3 = x2;
                    x2 = x1;
                    f3 = f2;
                    f2 = f1;
                } else {
                    have_right = false;
                    x0 = x1;
                    x1 = x2;
                    f0 = f1;
                    f1 = f2;
                }
                left--;
            }
            if (!have_left && f0 < f1) {
                if (x0 == 0.0) {
                    fn.reset();
                    alpha = 0.0;
                    return LS_MIN_ALPHA;
                }
                x1 = x0;
                f1 = fn.F(x1);
                calc = 1;
            }
            if (!have_right && f3 < f2) {
                x2 = x3;
                f2 = fn.F(x2);
                calc = 2;
            }
        }
        // leave the system at the better of x1, x2
        if (f1 < f2) {
            if (calc == 2) f1 = fn.F(x1);
            nrgy = f1;
            alpha = x1;
        } else {
            if (calc == 1) f2 = fn.F(x2);
            nrgy = f2;
            alpha = x2;
        }
        prev_val = -dfa * alpha;
        return LS_S;
    }

    int brent(double dfa, double max_a, double& nrgy, double& alpha) {
        double a = 0.0, b, fa = nrgy, fb;
        double x, fx;
        if (p.bracket) {
            int chk = bracket(dfa, max_a, a, x, b, fa, fx, fb);
            if (chk != B_S) {
                fn.reset();
                return chk;
            }
        } else {
            b = max_a;
            x = cgold * (b - a);
            fx = fn.F(x);
        }
        double d = 0.0, e = 0.0, u = 0.0, fu = 0.0;
        double w = x, v = x, fw = fx, fv = fx;
        for (int it = 0; it < p.max_iter; it++) {
            const double xm = 0.5 * (a + b);
            const double tol1 = p.tol * fabs(x) + p.zeps;
            const double tol2 = 2.0 * tol1;
            if (fabs(x - xm) <= (tol2 - 0.5 * (b - a))) {
                if (u != x) fn.F(x);
                nrgy = fx;
                alpha = x;
                prev_val = alpha;
                return LS_S;
            }
            if (fabs(e) > tol1) {
                // parabola through x, w, v
                double r = (x - w) * (fx - fv);
                double q = (x - v) * (fx - fw);
                double pp = (x - v) * q - (x - w) * r;
                q = 2.0 * (q - r);
                if (q > 0.0) pp = -pp;
                q = fabs(q);
                const double etemp = e;
                e = d;
                if (fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (a - x) || pp >= q * (b - x)) {
                    e = x >= xm ? a - x : b - x;
                    d = cgold * e;
                } else {
                    d = pp / q;
                    u = x + d;
                    if (u - a < tol2 || b - u < tol2) d = xm - x >= 0.0 ? fabs(tol1) : -fabs(tol1);
                }
            } else {
                e = x >= xm ? a - x : b - x;
                d = cgold * e;
            }
            if (fabs(d) >= tol1)
                u = x + d;
            else
                u = d >= 0.0 ? x + fabs(tol1) : x - fabs(tol1);
            fu = fn.F(u);
            if (fu <= fx) {
                if (u >= x)
                    a = x;
                else
                    b = x;
                v = w;
                w = x;
                x = u;
                fv = fw;
                fw = fx;
                fx = fu;
            } else {
                if (u < x)
                    a = u;
                else
                    b = u;
                if (fu <= fw || w == x) {
                    v = w;
                    w = u;
                    fv = fw;
                    fw = fu;
                } else if (fu <= fv || v == x || v == w) {
                    v = u;
                    fv = fu;
                }
            }
        }
        // never end above the starting energy
        if (fa < fx) {
            fn.reset();
            alpha = 0.0;
            return LS_MIN_ALPHA;
        }
        if (u != x) fn.F(x);
        nrgy = fx;
        alpha = x;
        prev_val = alpha;
        return LS_S;
    }
};

}  // namespace mappg
