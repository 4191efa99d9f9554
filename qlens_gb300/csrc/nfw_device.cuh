// nfw_device.cuh -- elliptical NFW deflection on the device by QLens's
// adaptive Gauss-Patterson quadrature, in FP64.
//
//   NFW::kappa_rsq, lens_function_xsq, kapavg_spherical_rsq   models.cpp:978-1010
//   q == 1: LensProfile::deflection_spherical_default         profile.cpp:1515-1518, 2281-2290
//   q <  1: LensProfile::deflection_numerical                 profile.cpp:2359-2375
//           alpha_x = x J_0, alpha_y = y J_1,
//           J_n = sqrt(1-eps) int_0^1 2w kappa(u (x^2 + y^2/(1-eps u)) q) / (1-eps u)^(n+1/2) dw,
//           u = w^2, eps = 1 - q^2 (LensIntegral, profile.h:441-449; profile.cpp:2703-2733, 2778-2783)
//   LensIntegral::PattersonIntegrate                          profile.cpp:3830-3876
//           levels of 1, 3, ..., 511 nested nodes; stop after level 2 once
//           |I_L - I_{L-1}| < 1e-3 |I_L| (QLens's default integral_tolerance)
//
// Both integrals share their nodes: each node's kappa is evaluated once and
// feeds J_0 and J_1, each of which keeps its own convergence test, so every
// level sum is the one the reference forms for that integral alone.  The sum
// of a level runs over the new nodes first, then the old ones, both in
// ascending order, as in the reference.  Node values of levels <= 5 (63
// nodes) are kept per thread; the rare rays that need levels 6-8 recompute
// the older values they lack, which gives the same bits (same code, no
// contraction in the units built with --fmad=false).
//
// (1-eps u)^(1/2) and ^(3/2) use sqrt (correctly rounded) rather than pow;
// kappa's atan / atanh / log are CUDA's, within a few ulp of the host libm.
#pragma once
#include "qlpix_internal.h"
#include "patterson_rule.h"

namespace qlpix {

static __constant__ double c_pat_points[QLP_PAT_N] = QLP_PAT_POINTS_INIT;
static __constant__ double c_pat_weights[QLP_PAT_NW] = QLP_PAT_WEIGHTS_INIT;

#define NFW_PAT_TOL 1e-3                 // QLens's default integral_tolerance (LensRec::tol)
#define NFW_KEEP_LEVELS 6            // levels 0..5 keep their node values
#define NFW_KEEP ((2 << (NFW_KEEP_LEVELS - 1)) - 1)   // 63

__device__ __forceinline__ double nfw_lens_function_xsq(double xsq)
{
    return ((xsq > 1.0) ? (atan(sqrt(xsq - 1)) / sqrt(xsq - 1))
                        : (xsq < 1.0) ? (atanh(sqrt(1 - xsq)) / sqrt(1 - xsq)) : 1.0);
}

__device__ __forceinline__ double nfw_kappa_rsq(double ks, double rs, double rsq)
{
    double xsq = rsq / (rs * rs);
    if (xsq < 1e-6) return -ks * (2 + log(xsq / 4));
    else if (fabs(xsq - 1) < 1e-5) return 2 * ks * (0.3333333333333333 - (xsq - 1) / 5.0);
    else return 2 * ks * (1 - nfw_lens_function_xsq(xsq)) / (xsq - 1);
}

__device__ __forceinline__ double nfw_kapavg_spherical_rsq(double ks, double rs, double rsq)
{
    double xsq = rsq / (rs * rs);
    if (xsq > 1e-5) return 2 * ks * (2 * nfw_lens_function_xsq(xsq) + log(xsq / 4)) / xsq;
    else return -ks * (1 + log(xsq / 4));
}

// The two integrands at node index i of the 511-point set.
static __device__ __noinline__ void nfw_node(const LensRec& L, double xsq, double ysq, int i, double& f0, double& f1)
{
    const double w = 0.5 + 0.5 * c_pat_points[i];
    const double u = w * w;
    const double qfac = 1 - L.epsilon * u;
    const double t = 2 * w * nfw_kappa_rsq(L.ks, L.rs, u * (xsq + ysq / qfac) * L.q);
    const double sq = sqrt(qfac);
    f0 = t / sq;
    f1 = t / (qfac * sq);
}

// The two Patterson integrals of LensIntegral::j_integral for lens-frame
// (x^2, y^2): I_n = 0.5 * sum_level(w_j f_n(node_j)) at the level where that
// integral converged to `tol` (QLens: 1e-3).  The deflection is
// alpha_x = x sqrt(1-eps) I_0, alpha_y = y sqrt(1-eps) I_1.
static __device__ void nfw_integrals(const LensRec& L, double xsq, double ysq, double tol, double& I0, double& I1)
{
    double keep0[NFW_KEEP], keep1[NFW_KEEP];   // values at nodes of levels <= 5, slot (i+1)/8 - 1
    double r0 = 0, r1 = 0, old0, old1;
    bool done0 = false, done1 = false;
    int level = 0;
    do {
        const double* wt = c_pat_weights + ((2 << level) - level - 2);   // levels 0..L-1 hold 2^(L+1)-2-L weights
        const int order = (2 << level) - 1;
        const int istep0 = (QLP_PAT_N + 1) / (order + 1);
        const int istep = 2 * istep0;
        old0 = r0; old1 = r1;
        double s0 = 0, s1 = 0;
        // new nodes (even j)
        for (int j = 0, i = istep0 - 1; j < order; j += 2, i += istep) {
            double f0, f1;
            nfw_node(L, xsq, ysq, i, f0, f1);
            if (((i + 1) & 7) == 0) { keep0[((i + 1) >> 3) - 1] = f0; keep1[((i + 1) >> 3) - 1] = f1; }
            s0 += wt[j] * f0;
            s1 += wt[j] * f1;
        }
        // old nodes (odd j)
        for (int j = 1, i = istep - 1; j < order; j += 2, i += istep) {
            double f0, f1;
            if (((i + 1) & 7) == 0) { f0 = keep0[((i + 1) >> 3) - 1]; f1 = keep1[((i + 1) >> 3) - 1]; }
            else nfw_node(L, xsq, ysq, i, f0, f1);
            s0 += wt[j] * f0;
            s1 += wt[j] * f1;
        }
        if (!done0) {
            r0 = s0;
            if ((level > 1) && (fabs(r0 - old0) < tol * fabs(r0))) done0 = true;
        }
        if (!done1) {
            r1 = s1;
            if ((level > 1) && (fabs(r1 - old1) < tol * fabs(r1))) done1 = true;
        }
    } while (++level < QLP_PAT_LEVELS && !(done0 && done1));
    I0 = 0.5 * r0;
    I1 = 0.5 * r1;
}

// The same two integrals for one ray per warp (all 32 lanes call it with the
// same arguments, converged): the lanes evaluate a level's new nodes in
// parallel into the warp's buffers v0, v1 (QLP_PAT_N doubles each, by node
// index), then every lane forms the level sums from the buffers in
// nfw_integrals' order.  The node values come from the same function and
// are added in the same order, so the result has nfw_integrals' bits, after
// about one node's latency per level instead of 2^level of them.
static __device__ void nfw_integrals_warp(const LensRec& L, double xsq, double ysq, double tol, double& I0,
                                          double& I1, double* v0, double* v1)
{
    const int lane = threadIdx.x & 31;
    double r0 = 0, r1 = 0, old0, old1;
    bool done0 = false, done1 = false;
    int level = 0;
    do {
        const double* wt = c_pat_weights + ((2 << level) - level - 2);
        const int order = (2 << level) - 1;
        const int istep0 = (QLP_PAT_N + 1) / (order + 1);
        const int istep = 2 * istep0;
        old0 = r0; old1 = r1;
        for (int q = lane; 2 * q < order; q += 32) {
            const int i = istep0 - 1 + q * istep;
            double f0, f1;
            nfw_node(L, xsq, ysq, i, f0, f1);
            v0[i] = f0;
            v1[i] = f1;
        }
        __syncwarp();
        double s0 = 0, s1 = 0;
        for (int j = 0, i = istep0 - 1; j < order; j += 2, i += istep) {
            s0 += wt[j] * v0[i];
            s1 += wt[j] * v1[i];
        }
        for (int j = 1, i = istep - 1; j < order; j += 2, i += istep) {
            s0 += wt[j] * v0[i];
            s1 += wt[j] * v1[i];
        }
        if (!done0) {
            r0 = s0;
            if ((level > 1) && (fabs(r0 - old0) < tol * fabs(r0))) done0 = true;
        }
        if (!done1) {
            r1 = s1;
            if ((level > 1) && (fabs(r1 - old1) < tol * fabs(r1))) done1 = true;
        }
        __syncwarp();
    } while (++level < QLP_PAT_LEVELS && !(done0 && done1));
    I0 = 0.5 * r0;
    I1 = 0.5 * r1;
}

// wbuf: null, or the calling warp's 2 QLP_PAT_N doubles for
// nfw_integrals_warp (then all 32 lanes call with the same arguments)
static __device__ void nfw_deflection(const LensRec& L, double x, double y, double& dx, double& dy,
                                      double* wbuf = nullptr)
{
    if (L.q == 1.0) {
        double kapavg = nfw_kapavg_spherical_rsq(L.ks, L.rs, x * x + y * y);
        dx = kapavg * x;
        dy = kapavg * y;
        return;
    }
    if ((fabs(x) < 1e-14) && (fabs(y) < 1e-14)) {
        dx = 0;
        dy = 0;
        return;
    }
    double I0, I1;
    if (wbuf) nfw_integrals_warp(L, x * x, y * y, L.tol, I0, I1, wbuf, wbuf + QLP_PAT_N);
    else nfw_integrals(L, x * x, y * y, L.tol, I0, I1);
    const double sqe = sqrt(1 - L.epsilon);
    dx = x * (sqe * I0);
    dy = y * (sqe * I1);
}

}  // namespace qlpix
