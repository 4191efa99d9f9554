// lens_device.cuh -- FP64 deflection of the lens models on the device.
// The units that must reproduce QLens's bits (raytrace.cu, sur_exact.cu,
// outside.cu) include it built with --fmad=false;
// surrogate.cu includes it with contraction (its rays carry an error bound).
#pragma once
#include "qlpix_internal.h"

namespace qlpix {

// Coefficients rho_i = f (beta i - 1) / (beta i + 1) of the Tessore series
// for i = 1 .. SPLE_RHO_TAB, the same expression as in the series loop, so a
// table filled once per CTA holds the bits the loop would compute.
#define SPLE_RHO_TAB 48
__device__ __forceinline__ double sple_rho(const LensRec& L, int i)
{
    double beta = 2.0 / (2 - L.alpha);
    double ff = (1 - L.q) / (1 + L.q);
    return ff * (beta * i - 1) / (beta * i + 1);
}

// The series' stopping test |o|^2 > 1e-16 |f|^2, |z|^2 as hypot(re, im)^2
// (std::norm).  The plain sums of squares differ from those by a few ulp, so
// they decide whenever they are clear of the threshold by a relative 1e-12;
// only a near tie evaluates the hypot form -- the decision is the same.
__device__ __forceinline__ bool sple_series_continues(double orr, double oi, double fr, double fi)
{
    const double A = orr * orr + oi * oi;
    const double t = 1e-16 * (fr * fr + fi * fi);
    if (A > t * (1.0 + 1e-12)) return true;
    if (A < t * (1.0 - 1e-12)) return false;
    const double a = hypot(orr, oi), c = hypot(fr, fi);
    return a * a > 1e-16 * (c * c);
}

// SPLE_Lens::deflection_angular_factor (models.cpp:336-351): the Tessore et
// al. (2015) series for the core-free elliptical power law, complex products
// written out as (ac - bd, ad + bc).  rho_tab: rho_1 .. rho_SPLE_RHO_TAB for
// this lens (sple_rho), or null.
__device__ __forceinline__ void sple_angular_factor(const LensRec& L, double phi, double& fr, double& fi,
                                                    const double* rho_tab)
{
    double s1, c1;
    sincos(phi, &s1, &c1);
    fr = 1.0 * c1; fi = 1.0 * s1;
    double orr = fr, oi = fi;
    double s2, c2;
    sincos(2 * phi, &s2, &c2);
    int i = 1;
    do {
        const double rho = (rho_tab && i <= SPLE_RHO_TAB) ? rho_tab[i - 1] : sple_rho(L, i);
        double pr = -(rho * c2), pi = -(rho * s2);
        double nr = pr * orr - pi * oi;
        double ni = pr * oi + pi * orr;
        orr = nr; oi = ni;
        fr += orr; fi += oi;
        i++;
    } while (sple_series_continues(orr, oi, fr, fi) && i < 1000);
}

__device__ __forceinline__ void sple_deflection(const LensRec& L, double x, double y, double& dx, double& dy,
                                                const double* rho_tab = nullptr)
{
    if (L.kind == 1) {
        // SPLE_Lens::deflection_elliptical_iso (models.cpp:208-216)
        double psi = sqrt(L.qsq * (L.ssq + x * x) + y * y);
        double u = sqrt(1 - L.qsq);
        double pre = L.bprime * L.q / u;
        dx = pre * atan(u * x / (psi + L.sprime));
        dy = pre * atanh(u * y / (psi + L.qsq * L.sprime));
    } else if (L.kind == 2) {
        // SPLE_Lens::deflection_elliptical_nocore (models.cpp:244-262)
        double R = sqrt(x * x + y * y / L.qsq);
        double phi = atan(fabs(y / (L.q * x)));
        if (x < 0) {
            if (y < 0) phi = phi - M_PI;
            else phi = M_PI - phi;
        } else if (y < 0) {
            phi = -phi;
        }
        double fr, fi;
        sple_angular_factor(L, phi, fr, fi, rho_tab);
        double scal = 2 * L.bprime * L.q / (1 + L.q) * pow(L.bprime / R, L.alpha - 1);
        dx = scal * fr;
        dy = scal * fi;
    } else {
        // LensProfile::deflection_spherical_default (profile.cpp:2281-2290)
        double rsq = x * x + y * y, kapavg;
        if (L.alpha == 1.0) kapavg = L.b * (sqrt(L.s * L.s + rsq) - L.s) / rsq;
        else kapavg = (pow(L.b, L.alpha) * (pow(rsq + L.s * L.s, 1 - L.alpha / 2) - pow(L.s, 2 - L.alpha))) / rsq;
        dx = kapavg * x;
        dy = kapavg * y;
    }
}

}  // namespace qlpix
#include "nfw_device.cuh"
namespace qlpix {

// LensProfile::deflection (profile.cpp:1782-1805); Shear::deflection (models.cpp:2266-2272).
// NFW = false compiles the kernel without the quadrature (no NFW lens in the model).
// wbuf: see nfw_deflection (null: one ray per thread).
template <bool NFW>
__device__ __forceinline__ void lens_deflection(const LensRec& L, double x, double y, double& dx, double& dy,
                                                const double* rho_tab = nullptr, double* wbuf = nullptr)
{
    if (L.type == QLP_LENS_SHEAR) {
        x -= L.xc; y -= L.yc;
        dx = x * L.shear1 + y * L.shear2;
        dy = -y * L.shear1 + x * L.shear2;
        return;
    }
    x -= L.xc;
    y -= L.yc;
    const bool rot = (L.sintheta != 0);
    if (rot) {
        double xp = x * L.costheta + y * L.sintheta;
        y = -x * L.sintheta + y * L.costheta;
        x = xp;
    }
    double ax, ay;
    if (!NFW || L.type == QLP_LENS_SPLE) sple_deflection(L, x, y, ax, ay, rho_tab);
    else nfw_deflection(L, x, y, ax, ay, wbuf);
    if (rot) {
        double xp = ax * L.costheta - ay * L.sintheta;
        ay = ax * L.sintheta + ay * L.costheta;
        ax = xp;
    }
    dx = ax; dy = ay;
}

// Sub-pixel centres (set_nsplits, pixelgrid.cpp:10898-10938): sub-pixel
// (ii, jj) of pixel (i, j) sits at (1-u0) x_i + u0 x_{i+1} with
// u0 = (1 + 2 ii) / (2 ns), likewise in y.  subpix_table forms u0 and 1 - u0
// once per CTA (any threads; a barrier before use); subpix_centre uses the
// table when ns fits it and the same expressions otherwise -- the same bits
// either way, with no FP64 divide per ray.
#define SUBPIX_TAB 32
__device__ __forceinline__ void subpix_table(int ns, double* fu, double* f1mu)
{
    for (int e = threadIdx.x; e < ns && e < SUBPIX_TAB; e += blockDim.x) {
        const double u0 = ((double)(1 + 2 * e)) / (2 * ns);
        fu[e] = u0;
        f1mu[e] = 1 - u0;
    }
}

__device__ __forceinline__ void subpix_centre(const StaticData& sd, int ns, int ii, int jj, int i, int j,
                                              const double* fu, const double* f1mu, double& px, double& py)
{
    if (ns <= SUBPIX_TAB) {
        px = f1mu[ii] * sd.xvals[i] + fu[ii] * sd.xvals[i + 1];
        py = f1mu[jj] * sd.yvals[j] + fu[jj] * sd.yvals[j + 1];
    } else {
        const double u0 = ((double)(1 + 2 * ii)) / (2 * ns);
        const double w0 = ((double)(1 + 2 * jj)) / (2 * ns);
        px = (1 - u0) * sd.xvals[i] + u0 * sd.xvals[i + 1];
        py = (1 - w0) * sd.yvals[j] + w0 * sd.yvals[j + 1];
    }
}

// QLens::deflection + QLens::find_sourcept (lenscalc.cpp:81-113, 325-330).
// rho_tab: SPLE_RHO_TAB series coefficients per lens (lens k at k *
// SPLE_RHO_TAB), or null.
template <bool NFW>
__device__ __forceinline__ void find_sourcept(const LensModel& lm, double x, double y, double& bx, double& by,
                                              const double* rho_tab = nullptr, double* wbuf = nullptr)
{
    double defx = 0, defy = 0;
    double dsx[QLP_MAX_PLANES], dsy[QLP_MAX_PLANES];
    #pragma unroll 1
    for (int i = 0; i < lm.n_planes; i++) {
        dsx[i] = 0; dsy[i] = 0;
        if (lm.zfac[i] != 0.0) {
            double xi = x, yi = y;
            #pragma unroll 1
            for (int j = 0; j < i; j++) {
                xi -= lm.beta[i - 1][j] * dsx[j];
                yi -= lm.beta[i - 1][j] * dsy[j];
            }
            #pragma unroll 1
            for (int k = 0; k < lm.nlens; k++) {
                if (lm.lens[k].plane != i) continue;
                double ax, ay;
                lens_deflection<NFW>(lm.lens[k], xi, yi, ax, ay, rho_tab ? rho_tab + k * SPLE_RHO_TAB : nullptr,
                                     wbuf);
                dsx[i] += ax; dsy[i] += ay;
            }
            dsx[i] *= lm.zfac[i];
            dsy[i] *= lm.zfac[i];
            defx += dsx[i];
            defy += dsy[i];
        }
    }
    bx = x - defx;
    by = y - defy;
}

}  // namespace qlpix
