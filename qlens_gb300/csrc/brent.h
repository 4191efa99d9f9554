// brent.h -- Brent's method for a minimum as a resumable state machine, so
// that many minimisations (one per batched evaluation) can advance in
// lockstep, each function value coming from a device evaluation.
//
// The steps are those of QLens::brents_min_method (pixelgrid.cpp:16849-16932):
// start at bx - CGOLD (bx - ax), parabolic interpolation through the three
// best points when its step is acceptable, golden section otherwise, steps no
// smaller than 1e-8, convergence when |x - xmid| <= 2 (tol |x| + 1e-10) -
// (b - a) / 2, at most max_iter iterations; the result is the point with the
// least value.  Driving it:
//     BrentMin b(ax, bx, tol, max_iter);
//     double x;
//     while (b.want(&x)) b.give(f(x));
//     x_min = b.xmin();
#pragma once
#include <cmath>

namespace qlpix {

class BrentMin {
public:
    BrentMin() = default;
    BrentMin(double ax, double bx, double tol, int max_iter) { reset(ax, bx, tol, max_iter); }

    void reset(double ax, double bx, double tol, int max_iter)
    {
        a_ = ax; b_ = bx; tol_ = tol; maxit_ = max_iter;
        xstep_ = 0.0; e_ = 0.0;
        x_ = w_ = wprev_ = bx - CGOLD * (bx - ax);
        iter_ = 0; evals_ = 0;
        state_ = FIRST;
        u_ = x_;
    }

    // The next point to evaluate, or false when the minimisation has ended.
    bool want(double* x)
    {
        if (state_ == FIRST) { *x = x_; return true; }
        if (state_ == DONE) return false;
        // state_ == STEP: one iteration of the loop up to the evaluation
        if (iter_ >= maxit_) { state_ = DONE; return false; }
        const double xmid = 0.5 * (a_ + b_);
        const double tol1 = tol_ * std::fabs(x_);
        const double tol2 = 2.0 * (tol1 + ZEPS);
        if (std::fabs(x_ - xmid) <= (tol2 - 0.5 * (b_ - a_))) { state_ = DONE; return false; }
        if ((w_ != wprev_) && (std::fabs(e_) > tol1)) {
            const double r = (x_ - w_) * (fx_ - fwprev_);
            double q = (x_ - wprev_) * (fx_ - fw_);
            double p = (x_ - wprev_) * q - (x_ - w_) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) p = -p;
            q = std::fabs(q);
            const double etemp = e_;
            e_ = xstep_;
            if ((std::fabs(p) >= std::fabs(0.5 * q * etemp)) || (p <= q * (a_ - x_)) || (p >= q * (b_ - x_))) {
                e_ = (x_ >= xmid) ? a_ - x_ : b_ - x_;
                xstep_ = CGOLD * e_;
            } else {
                xstep_ = p / q;
                const double u = x_ + xstep_;
                if ((u - a_ < tol2) || (b_ - u < tol2)) xstep_ = (xmid - x_) >= 0 ? std::fabs(tol1) : -std::fabs(tol1);
            }
        } else {
            e_ = (x_ >= xmid) ? a_ - x_ : b_ - x_;
            xstep_ = CGOLD * e_;
        }
        u_ = (std::fabs(xstep_) >= ROOTPREC) ? x_ + xstep_ : x_ + (xstep_ >= 0 ? ROOTPREC : -ROOTPREC);
        *x = u_;
        return true;
    }

    // The value at the point want() returned last.
    void give(double f)
    {
        evals_++;
        if (state_ == FIRST) {
            fw_ = fwprev_ = fx_ = f;
            state_ = STEP;
            return;
        }
        const double fu = f;
        if (fu <= fx_) {
            if (u_ >= x_) a_ = x_; else b_ = x_;
            wprev_ = w_; w_ = x_; x_ = u_;
            fwprev_ = fw_; fw_ = fx_; fx_ = fu;
        } else {
            if (u_ < x_) a_ = u_; else b_ = u_;
            if (fu <= fw_ || w_ == x_) {
                wprev_ = w_; fwprev_ = fw_;
                w_ = u_; fw_ = fu;
            } else if ((fu <= fwprev_) || (wprev_ == x_) || (wprev_ == w_)) {
                wprev_ = u_; fwprev_ = fu;
            }
        }
        iter_++;
    }

    double xmin() const { return x_; }
    double fmin() const { return fx_; }
    int evals() const { return evals_; }

private:
    static constexpr double CGOLD = 0.3819660, ZEPS = 1.0e-10, ROOTPREC = 1.0e-8;
    enum { FIRST, STEP, DONE } state_ = DONE;
    double a_ = 0, b_ = 0, tol_ = 0, xstep_ = 0, e_ = 0;
    double x_ = 0, w_ = 0, wprev_ = 0, u_ = 0, fx_ = 0, fw_ = 0, fwprev_ = 0;
    int maxit_ = 0, iter_ = 0, evals_ = 0;
};

}  // namespace qlpix
