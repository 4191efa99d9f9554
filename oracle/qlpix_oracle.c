/*
 * qlpix_oracle.c -- CPU restatement of QLens's pixel-image likelihood.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm
 * may load it; the product (qlens_gb300, libqlpix) never does.
 *
 * It restates, in plain C with OpenMP, the reference's own algorithm for a
 * Cartesian source, interpolating ray tracing and the dense inversion, step
 * by step and in the reference's floating-point evaluation order where that
 * order decides the result bit for bit (ray shooting, source-grid corners,
 * L weights, the dense PSF convolution).  Build with -ffp-contract=off so no
 * multiply-add is fused (x86-64 g++ without -march fuses none either).
 *
 * Pinned against golden vectors dumped from the compiled reference by
 * oracle/ref_harness.cpp (tests/golden/ fixtures, tests/test_oracle_golden.py).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/qlpix.h"
#include "qlpix_oracle.h"

/* mathexpr.h:10 -- QLens's (truncated) half-pi constant */
static const double QL_HALFPI = 1.57079632679;
/* mathexpr.h:14 -- QLens's (truncated) 4 pi */
static const double QL_4PI = 12.5663706144;
/* mathexpr.h:27 */
static double deg2rad(double t) { return 0.017453292519943295 * t; }

/* ------------------------------------------------------------------ */
/* lens models                                                          */
/* ------------------------------------------------------------------ */

typedef struct {
    int type, plane;
    int kind;               /* SPLE dispatch: 0 spherical, 1 elliptical iso, 2 elliptical nocore */
    double xc, yc, costheta, sintheta;
    double q, qsq, b, bprime, s, sprime, ssq, alpha;
    double shear1, shear2;
    /* NFW */
    double ks, rs, f_major_axis;
} olens;

/* LensProfile::set_angle (profile.cpp:1625-1637) with orient_major_axis_north */
static void set_angle(olens* L, double theta_deg)
{
    double theta = deg2rad(theta_deg);
    double c = cos(theta), s = sin(theta);
    L->sintheta = c;
    L->costheta = -s;
}

static int setup_lens(olens* L, const qlp_lens* d, const double* p)
{
    memset(L, 0, sizeof(*L));
    L->type = d->type;
    L->plane = d->plane;
    if (d->type == QLP_LENS_SPLE) {
        /* SPLE_Lens::initialize_parameters / update_meta_parameters (models.cpp:37-108),
           update_ellipticity_meta_parameters emode 1 (profile.cpp:1686-1689) */
        L->b = p[0]; L->alpha = p[1]; L->s = p[2]; L->q = p[3];
        if (L->s < 0) L->s = -L->s;
        set_angle(L, p[4]);
        L->xc = p[5]; L->yc = p[6];
        double f = 1.0 / sqrt(L->q);
        L->bprime = L->b * f;
        L->sprime = L->s * f;
        L->qsq = L->q * L->q;
        L->ssq = L->sprime * L->sprime;
        /* set_integration_pointers + set_model_specific_integration_pointers (profile.cpp:1509-1521, models.cpp:132-156) */
        if (L->q == 1.0) L->kind = 0;
        else if (L->alpha == 1.0) L->kind = 1;
        else if (L->s == 0.0) L->kind = 2;
        else return -1; /* cored power law with q != 1: numerical quadrature, not on this path */
    } else if (d->type == QLP_LENS_SHEAR) {
        /* Shear::initialize_parameters / update_meta_parameters (models.cpp:2140-2224) */
        double shear = p[0];
        double theta = deg2rad(p[1]);
        double theta_eff = theta + QL_HALFPI;
        L->shear1 = shear * cos(2 * theta_eff);
        L->shear2 = shear * sin(2 * theta_eff);
        L->xc = p[2]; L->yc = p[3];
    } else if (d->type == QLP_LENS_NFW || d->type == QLP_LENS_NFW_M200_C || d->type == QLP_LENS_NFW_M200_RS) {
        L->type = QLP_LENS_NFW;
        if (d->type == QLP_LENS_NFW) {
            L->ks = p[0]; L->rs = p[1];
        } else {
            /* NFW::update_meta_parameters (models.cpp:891-898) -> set_ks_rs_from_m200_c200 (pmode 1,
               models.cpp:968-976) or set_ks_c200_from_m200_rs (pmode 2, models.cpp:959-966) */
            double m200 = p[0], c200, rs_kpc;
            double rvir_kpc = pow(m200 / (200.0 * QL_4PI / 3.0 * 1e-9 * d->critical_density), 0.333333333333);
            if (d->type == QLP_LENS_NFW_M200_C) {
                c200 = p[1];
                rs_kpc = rvir_kpc / c200;
                L->rs = rs_kpc * d->kpc_to_arcsec;
            } else {
                rs_kpc = p[1];
                L->rs = rs_kpc * d->kpc_to_arcsec;
                c200 = rvir_kpc / rs_kpc;
            }
            L->ks = m200 / (QL_4PI * L->rs * L->rs * d->sigma_cr * (log(1 + c200) - c200 / (1 + c200)));
        }
        L->q = p[2];
        set_angle(L, p[3]);
        L->xc = p[4]; L->yc = p[5];
        L->f_major_axis = 1.0 / sqrt(L->q);
        L->qsq = L->q * L->q;
        return oracle_nfw_setup(L->ks, L->rs, L->q) ? 0 : -1;
    } else {
        return -1;
    }
    return 0;
}

static int n_params_of(int type)
{
    switch (type) {
        case QLP_LENS_SPLE: return 7;
        case QLP_LENS_SHEAR: return 4;
        case QLP_LENS_NFW:
        case QLP_LENS_NFW_M200_C:
        case QLP_LENS_NFW_M200_RS: return 6;
    }
    return 0;
}

/* SPLE_Lens::deflection_angular_factor (models.cpp:336-351): Tessore et al.
   2015 series with std::complex arithmetic written out; std::norm of a
   complex<double> is |z|^2 computed through std::abs (hypot). */
static void angular_factor(const olens* L, double phi, double* fre, double* fim)
{
    double beta = 2.0 / (2 - L->alpha);
    double ff = (1 - L->q) / (1 + L->q);
    double fr = 1.0 * cos(phi), fi = 1.0 * sin(phi);
    double or_ = fr, oi = fi;
    int i = 1;
    double nw, nf;
    do {
        double rho = ff * (beta * i - 1) / (beta * i + 1);
        double pr = rho * cos(2 * phi), pi = rho * sin(2 * phi);
        pr = -pr; pi = -pi;
        double nr = pr * or_ - pi * oi;
        double ni = pr * oi + pi * or_;
        or_ = nr; oi = ni;
        fr += or_; fi += oi;
        i++;
        double a = hypot(or_, oi); nw = a * a;
        double c = hypot(fr, fi);  nf = c * c;
    } while (nw > 1e-16 * nf);   /* SPLE_Lens::def_tolerance (models.cpp:19) */
    *fre = fr; *fim = fi;
}

static void sple_deflection(const olens* L, double x, double y, double* dx, double* dy)
{
    if (L->kind == 1) {
        /* SPLE_Lens::deflection_elliptical_iso (models.cpp:208-216) */
        double psi = sqrt(L->qsq * (L->ssq + x * x) + y * y);
        double u = sqrt(1 - L->qsq);
        *dx = (L->bprime * L->q / u) * atan(u * x / (psi + L->sprime));
        *dy = (L->bprime * L->q / u) * atanh(u * y / (psi + L->qsq * L->sprime));
    } else if (L->kind == 2) {
        /* SPLE_Lens::deflection_elliptical_nocore (models.cpp:244-262) */
        double R = sqrt(x * x + y * y / L->qsq);
        double phi = atan(fabs(y / (L->q * x)));
        if (x < 0) {
            if (y < 0) phi = phi - M_PI;
            else phi = M_PI - phi;
        } else if (y < 0) {
            phi = -phi;
        }
        double fre, fim;
        angular_factor(L, phi, &fre, &fim);
        double scal = 2 * L->bprime * L->q / (1 + L->q) * pow(L->bprime / R, L->alpha - 1);
        *dx = scal * fre;
        *dy = scal * fim;
    } else {
        /* LensProfile::deflection_spherical_default (profile.cpp:2281-2290) with
           SPLE_Lens::kapavg_spherical_rsq(_iso) (models.cpp:162-170) */
        double rsq = x * x + y * y, kapavg;
        if (L->alpha == 1.0) kapavg = L->b * (sqrt(L->s * L->s + rsq) - L->s) / rsq;
        else kapavg = (pow(L->b, L->alpha) * (pow(rsq + L->s * L->s, 1 - L->alpha / 2) - pow(L->s, 2 - L->alpha))) / rsq;
        *dx = kapavg * x;
        *dy = kapavg * y;
    }
}

/* LensProfile::deflection (profile.cpp:1782-1805), Shear::deflection (models.cpp:2266-2272) */
static void lens_deflection(const olens* L, double x, double y, double* dx, double* dy)
{
    if (L->type == QLP_LENS_SHEAR) {
        x -= L->xc; y -= L->yc;
        *dx = x * L->shear1 + y * L->shear2;
        *dy = -y * L->shear1 + x * L->shear2;
        return;
    }
    x -= L->xc;
    y -= L->yc;
    int rot = (L->sintheta != 0);
    if (rot) {
        double xp = x * L->costheta + y * L->sintheta;
        y = -x * L->sintheta + y * L->costheta;
        x = xp;
    }
    double ax, ay;
    if (L->type == QLP_LENS_SPLE) sple_deflection(L, x, y, &ax, &ay);
    else oracle_nfw_deflection(L->ks, L->rs, L->q, L->f_major_axis, x, y, &ax, &ay);
    if (rot) {
        double xp = ax * L->costheta - ay * L->sintheta;
        ay = ax * L->sintheta + ay * L->costheta;
        ax = xp;
    }
    *dx = ax; *dy = ay;
}

/* QLens::deflection + find_sourcept (lenscalc.cpp:81-113, 325-330) */
static void find_sourcept(const olens* lenses, int nlens, const qlp_planes* pl,
                          double x, double y, double* bx, double* by)
{
    double defx = 0, defy = 0;
    double dsx[QLP_MAX_PLANES], dsy[QLP_MAX_PLANES];
    for (int i = 0; i < pl->n_planes; i++) {
        if (pl->zfac[i] != 0.0) {
            dsx[i] = 0; dsy[i] = 0;
            double xi = x, yi = y;
            for (int j = 0; j < i; j++) {
                xi -= pl->beta[i - 1][j] * dsx[j];
                yi -= pl->beta[i - 1][j] * dsy[j];
            }
            for (int k = 0; k < nlens; k++) {
                if (lenses[k].plane != i) continue;
                double ax, ay;
                lens_deflection(&lenses[k], xi, yi, &ax, &ay);
                dsx[i] += ax; dsy[i] += ay;
            }
            dsx[i] *= pl->zfac[i];
            dsy[i] *= pl->zfac[i];
            defx += dsx[i];
            defy += dsy[i];
        } else {
            dsx[i] = 0; dsy[i] = 0;
        }
    }
    *bx = x - defx;
    *by = y - defy;
}

/* ------------------------------------------------------------------ */
/* last-evaluation state (parity dumps)                                 */
/* ------------------------------------------------------------------ */

static struct {
    int n_sub, n_mask, n_pix, M, src_nx, src_ny, nnz;
    double* srcpt;       /* [2*n_sub] */
    int* L_rowptr; int* L_index; double* L_value;
    int* active_index;   /* [src_nx*src_ny] */
    double* Lpsf;        /* [n_pix*M] */
    double* D; double* s; double* model;
    double* Fdiag;
    double grid[4];
    int nx, ny;
    double* osb_sb;              /* [nx*ny] outside-SB pass: PSF-convolved model */
    unsigned char* osb_maps;     /* [nx*ny] its mapping flags */
    double osb_penalty;
} g_last;

static void free_last(void)
{
    free(g_last.srcpt); free(g_last.L_rowptr); free(g_last.L_index); free(g_last.L_value);
    free(g_last.active_index); free(g_last.Lpsf); free(g_last.D); free(g_last.s); free(g_last.model);
    free(g_last.Fdiag); free(g_last.osb_sb); free(g_last.osb_maps);
    memset(&g_last, 0, sizeof(g_last));
}

/* ------------------------------------------------------------------ */
/* packed-lower Cholesky (pixelgrid.cpp:17071-17105, 17201-17246)       */
/* ------------------------------------------------------------------ */

static int cholesky_packed_lower(double* a, int n)
{
    long* indx = (long*)malloc(sizeof(long) * (n > 0 ? n : 1));
    indx[0] = 0;
    for (int j = 1; j < n; j++) indx[j] = indx[j - 1] + j;
    int status = 1;
    a[0] = sqrt(a[0]);
    for (int j = 1; j < n; j++) a[indx[j]] /= a[0];
    for (int i = 1; i < n; i++) {
        #pragma omp parallel for schedule(static)
        for (int j = i; j < n; j++) {
            const double* a1 = a + indx[i];
            const double* a2 = a + indx[j];
            double* a3 = a + indx[j] + i;
            for (int k = 0; k < i; k++) *a3 -= a1[k] * a2[k];
        }
        double* d = a + indx[i] + i;
        if (*d < 0) status = 0;
        *d = sqrt(fabs(*d));
        for (int j = i + 1; j < n; j++) a[indx[j] + i] /= *d;
    }
    free(indx);
    return status;
}

static void cholesky_solve_packed_lower(const double* a, const double* b, double* x, int n)
{
    long* indx = (long*)malloc(sizeof(long) * (n > 0 ? n : 1));
    indx[0] = 0;
    for (int i = 0; i < n; i++) {
        if (i > 0) indx[i] = indx[i - 1] + i;
        double sum = b[i];
        for (int k = i - 1; k >= 0; k--) sum -= a[indx[i] + k] * x[k];
        x[i] = sum / a[indx[i] + i];
    }
    for (int i = n - 1; i >= 0; i--) {
        double sum = x[i];
        for (int k = i + 1; k < n; k++) sum -= a[indx[k] + i] * x[k];
        x[i] = sum / a[indx[i] + i];
    }
    free(indx);
}

static double cholesky_logdet_packed_lower(const double* a, int n)
{
    double logdet = 0;
    long idx = 0;
    for (int i = 0; i < n; i++) {
        logdet += log(fabs(a[idx]));
        idx += i + 2;
    }
    return 2 * logdet;
}

/* repack_matrix_lower (pixelgrid.cpp:17300-17321): packed upper (row-major) -> packed lower (row-major) */
/* ---------------------------------------------------------------------------
 * Brent's method for a minimum: QLens::brents_min_method (pixelgrid.cpp:
 * 16849-16932), restated step for step (same start point, tolerances, step
 * choices and bracket updates).  Returns the point with the least value;
 * *nevals counts the function evaluations.
 * ------------------------------------------------------------------------- */
double oracle_brent_min(double (*f)(double, void*), void* user, double ax, double bx, double tol, int maxit,
                        int* nevals)
{
    const double CGOLD = 0.3819660, ZEPS = 1.0e-10, ROOTPREC = 1.0e-8;
    double a = ax, b = bx, xstep = 0.0, e = 0.0;
    double x, w, wprev, fx, fw, fwprev, u, fu, tol1, tol2, xmid;
    int n = 0;
    x = w = wprev = bx - CGOLD * (bx - ax);
    fw = fwprev = fx = f(x, user);
    n++;
    for (int iter = 0; iter < maxit; iter++) {
        xmid = 0.5 * (a + b);
        tol1 = tol * fabs(x);
        tol2 = 2.0 * (tol1 + ZEPS);
        if (fabs(x - xmid) <= (tol2 - 0.5 * (b - a))) break;
        if ((w != wprev) && (fabs(e) > tol1)) {
            double r = (x - w) * (fx - fwprev);
            double q = (x - wprev) * (fx - fw);
            double p = (x - wprev) * q - (x - w) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) p = -p;
            q = fabs(q);
            double etemp = e;
            e = xstep;
            if ((fabs(p) >= fabs(0.5 * q * etemp)) || (p <= q * (a - x)) || (p >= q * (b - x))) {
                e = (x >= xmid) ? a - x : b - x;
                xstep = CGOLD * e;
            } else {
                xstep = p / q;
                u = x + xstep;
                if ((u - a < tol2) || (b - u < tol2))
                    xstep = ((xmid - x) >= 0 ? (tol1 >= 0 ? tol1 : -tol1) : (tol1 >= 0 ? -tol1 : tol1));
            }
        } else {
            e = (x >= xmid) ? a - x : b - x;
            xstep = CGOLD * e;
        }
        if (fabs(xstep) >= ROOTPREC) u = x + xstep;
        else u = x + (xstep >= 0 ? ROOTPREC : -ROOTPREC);
        fu = f(u, user);
        n++;
        if (fu <= fx) {
            if (u >= x) a = x; else b = x;
            wprev = w; w = x; x = u;
            fwprev = fw; fw = fx; fx = fu;
        } else {
            if (u < x) a = u; else b = u;
            if (fu <= fw || w == x) {
                wprev = w; fwprev = fw;
                w = u; fw = fu;
            } else if ((fu <= fwprev) || (wprev == x) || (wprev == w)) {
                wprev = u; fwprev = fu;
            }
        }
    }
    if (nevals) *nevals = n;
    return x;
}

/* 'outside_sb_prior on' (lens.cpp:294-296 defaults: off, fraction 0.3 of the
   in-mask peak, noise multiple -1e30 i.e. unused; emask_nsplit 1, lens.cpp:498).
   emask: the extended mask [nx*ny] (NULL: every pixel). */
static struct {
    int on, emask_nsplit;
    double frac, noise_frac;
    unsigned char* emask;
    long emask_n;
} g_osb = {0, 1, 0.3, -1e30, NULL, 0};

void oracle_set_outside_sb(int on, double frac, double noise_frac, int emask_nsplit, const unsigned char* emask,
                           long n)
{
    g_osb.on = on;
    g_osb.frac = frac;
    g_osb.noise_frac = noise_frac;
    g_osb.emask_nsplit = emask_nsplit;
    free(g_osb.emask);
    g_osb.emask = NULL;
    g_osb.emask_n = 0;
    if (emask && n > 0) {
        g_osb.emask = (unsigned char*)malloc(n);
        memcpy(g_osb.emask, emask, n);
        g_osb.emask_n = n;
    }
}

static int cmp_int(const void* a, const void* b) { int x = *(const int*)a, y = *(const int*)b; return (x > y) - (x < y); }

/* The outside-surface-brightness pass (lens.cpp:13063-13158, Cartesian branch)
   after the inversion: the pixel grid switches to the extended mask
   (ImagePixelGrid::activate_extended_mask, pixelgrid.cpp:10833-10852), whose
   pixels outside the mask split emask_nsplit ways (set_nsplits 10898-10938);
   they are ray-traced and mapped onto the same source grid (assign_pixel_mappings
   12777-12910), the cells any of them maps to become the new active set (in
   cell order) holding the inverted amplitudes where the inversion had them and
   zero elsewhere (SourcePixel::update_surface_brightness 817-831,
   fill_surface_brightness_vector 833-851), the model is the dense L times
   those amplitudes in column order (convert_Lmatrix_to_dense 13717-13747,
   calculate_image_pixel_surface_brightness_dense 18268-18290), then
   PSF-convolved over the active extended-mask pixels
   (PSF_convolution_pixel_vector, direct branch 14409-14493).  A neighbour in
   the extended mask that maps nowhere has pixel index -1 there, which the
   reference reads as element -1 of its vector; it is taken as 0 here.  The
   penalty: with the peak over masked mapped pixels and threshold
   max(noise_frac sigma, frac peak), the largest |sb| >= threshold over mapped
   extended-mask pixels outside the mask adds (1 + |(sb - t)/t|)^60 - 1. */
static double outside_sb_penalty(const qlp_image* im, const qlp_psf* psf, const olens* lenses, int nlens,
                                 const qlp_planes* planes, int ns, const double* cx, const double* cy,
                                 const double* ccx, const double* ccy, int snx, int sny, const int* aidx,
                                 const double* s)
{
    const int nx = im->npixels_x, ny = im->npixels_y;
    const int ens = g_osb.emask_nsplit;
    unsigned char* em = (unsigned char*)malloc((size_t)nx * ny);
    for (long t = 0; t < (long)nx * ny; t++)
        em[t] = (g_osb.emask && t < g_osb.emask_n) ? (g_osb.emask[t] != 0) : 1;
    /* extended-mask pixels, j-outer / i-inner, and their sub-pixel offsets */
    int ne = 0;
    for (long t = 0; t < (long)nx * ny; t++) ne += em[t];
    int* epix = (int*)malloc(sizeof(int) * (ne > 0 ? ne : 1));
    long* eoff = (long*)malloc(sizeof(long) * (ne + 1));
    {
        int c = 0;
        long o = 0;
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const int t = i * ny + j;
                if (!em[t]) continue;
                const int nsp = im->in_mask[t] ? ns : ens;
                epix[c] = t;
                eoff[c++] = o;
                o += (long)nsp * nsp;
            }
        eoff[ne] = o;
    }
    const long nsub_e = eoff[ne];
    double* sp = (double*)malloc(sizeof(double) * 2 * (nsub_e > 0 ? nsub_e : 1));
    #pragma omp parallel for schedule(dynamic, 16)
    for (int e = 0; e < ne; e++) {
        const int i = epix[e] / ny, j = epix[e] % ny;
        const int nsp = im->in_mask[epix[e]] ? ns : ens;
        const double x0 = im->xvals[i], x1 = im->xvals[i + 1], y0 = im->yvals[j], y1 = im->yvals[j + 1];
        long k = eoff[e];
        for (int ii = 0; ii < nsp; ii++)
            for (int jj = 0; jj < nsp; jj++) {
                const double u0 = ((double)(1 + 2 * ii)) / (2 * nsp);
                const double w0 = ((double)(1 + 2 * jj)) / (2 * nsp);
                double bx, by;
                find_sourcept(lenses, nlens, planes, (1 - u0) * x0 + u0 * x1, (1 - w0) * y0 + w0 * y1, &bx, &by);
                sp[2 * k] = bx;
                sp[2 * k + 1] = by;
                k++;
            }
    }
    /* cells and weights per sub-pixel, as in the inversion's mapping */
    int* cell3 = (int*)malloc(sizeof(int) * 3 * (nsub_e > 0 ? nsub_e : 1));
    double* w3 = (double*)malloc(sizeof(double) * 3 * (nsub_e > 0 ? nsub_e : 1));
    unsigned char* mapped = (unsigned char*)calloc((size_t)snx * sny, 1);
    unsigned char* pmaps = (unsigned char*)calloc(ne > 0 ? ne : 1, 1);
    for (int e = 0; e < ne; e++) {
        const int nsp = im->in_mask[epix[e]] ? ns : ens;
        const double weight = 1.0 / (nsp * nsp);
        for (long t = eoff[e]; t < eoff[e + 1]; t++) {
            const double px = sp[2 * t], py = sp[2 * t + 1];
            cell3[3 * t] = -1;
            if (!(px >= cx[0] && px < cx[snx] && py >= cy[0] && py < cy[sny])) continue;
            int lo = 0, hi = snx - 1;
            while (lo < hi) { int mid = (lo + hi + 1) / 2; if (cx[mid] <= px) lo = mid; else hi = mid - 1; }
            const int ci = lo;
            lo = 0; hi = sny - 1;
            while (lo < hi) { int mid = (lo + hi + 1) / 2; if (cy[mid] <= py) lo = mid; else hi = mid - 1; }
            const int cj = lo;
            const int xn = ((px > ccx[ci] && ci < snx - 1) || ci == 0) ? ci + 1 : ci - 1;
            const int yn = ((py > ccy[cj] && cj < sny - 1) || cj == 0) ? cj + 1 : cj - 1;
            const int c0 = cj * snx + ci, c1 = cj * snx + xn, c2 = yn * snx + ci;
            cell3[3 * t] = c0; cell3[3 * t + 1] = c1; cell3[3 * t + 2] = c2;
            mapped[c0] = mapped[c1] = mapped[c2] = 1;
            pmaps[e] = 1;
            const double p0x = ccx[ci], p0y = ccy[cj], p1x = ccx[xn], p1y = ccy[cj], p2x = ccx[ci], p2y = ccy[yn];
            const double d = (p0x - p1x) * (p1y - p2y) - (p1x - p2x) * (p0y - p1y);
            w3[3 * t] = weight * (px * (p1y - p2y) + py * (p2x - p1x) + p1x * p2y - p1y * p2x) / d;
            w3[3 * t + 1] = weight * (px * (p2y - p0y) + py * (p0x - p2x) + p0y * p2x - p0x * p2y) / d;
            w3[3 * t + 2] = weight * (px * (p0y - p1y) + py * (p1x - p0x) + p0x * p1y - p0y * p1x) / d;
        }
    }
    /* model per mapped pixel: the row's entries merged per cell in CSR order,
       then summed over cells in ascending order (= ascending new active index) */
    int* pidx = (int*)malloc(sizeof(int) * nx * ny);
    for (long t = 0; t < (long)nx * ny; t++) pidx[t] = -1;
    int na = 0;
    for (int e = 0; e < ne; e++) if (pmaps[e]) pidx[epix[e]] = na++;
    double* model = (double*)malloc(sizeof(double) * (na > 0 ? na : 1));
    int* act = (int*)malloc(sizeof(int) * (na > 0 ? na : 1));
    {
        int r = 0;
        for (int e = 0; e < ne; e++) {
            if (!pmaps[e]) continue;
            act[r] = epix[e];
            const long n3 = 3 * (eoff[e + 1] - eoff[e]);
            int* cells = (int*)malloc(sizeof(int) * (n3 > 0 ? n3 : 1));
            int nc = 0;
            for (long t = eoff[e]; t < eoff[e + 1]; t++) {
                if (cell3[3 * t] < 0) continue;
                for (int u = 0; u < 3; u++) {
                    int seen = 0;
                    for (int q = 0; q < nc; q++) if (cells[q] == cell3[3 * t + u]) { seen = 1; break; }
                    if (!seen) cells[nc++] = cell3[3 * t + u];
                }
            }
            qsort(cells, nc, sizeof(int), cmp_int);
            double acc = 0;
            for (int q = 0; q < nc; q++) {
                double v = 0;
                for (long t = eoff[e]; t < eoff[e + 1]; t++) {
                    if (cell3[3 * t] < 0) continue;
                    for (int u = 0; u < 3; u++) if (cell3[3 * t + u] == cells[q]) v += w3[3 * t + u];
                }
                const int a = aidx[cells[q]];
                acc += v * (a >= 0 ? s[a] : 0.0);
            }
            model[r++] = acc;
            free(cells);
        }
    }
    /* PSF convolution over the mapped extended-mask pixels */
    double* sb = (double*)calloc((size_t)nx * ny, sizeof(double));
    {
        const int pnx = psf->nx, pny = psf->ny, nxh = pnx / 2, nyh = pny / 2;
        for (int r = 0; r < na; r++) {
            const int k = act[r] / ny, l = act[r] % ny;
            double v = 0;
            for (int pk = 0; pk < pnx; pk++) {
                const int ii = k + nxh - pk;
                if (ii < 0 || ii >= nx) continue;
                for (int pl = 0; pl < pny; pl++) {
                    const int jj = l + nyh - pl;
                    if (jj < 0 || jj >= ny) continue;
                    if (!em[ii * ny + jj]) continue;
                    const int q = pidx[ii * ny + jj];
                    if (q < 0) continue;
                    v += psf->matrix[pk * pny + pl] * model[q];
                }
            }
            sb[act[r]] = v;
        }
    }
    double max_sb = -1e30, max_ext = -1e30;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            const int t = i * ny + j;
            if (im->in_mask[t] && pidx[t] >= 0 && sb[t] > max_sb) max_sb = sb[t];
        }
    const double a = g_osb.noise_frac * im->background_pixel_noise, b = g_osb.frac * max_sb;
    const double thr = (a > b) ? a : b;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            const int t = i * ny + j;
            if (!im->in_mask[t] && em[t] && pidx[t] >= 0 && fabs(sb[t]) >= thr && fabs(sb[t]) > max_ext)
                max_ext = fabs(sb[t]);
        }
    double penalty = 0;
    if (max_ext > 0) penalty = pow(1 + fabs((max_ext - thr) / thr), 60) - 1.0;
    unsigned char* maps = (unsigned char*)calloc((size_t)nx * ny, 1);
    for (long t = 0; t < (long)nx * ny; t++) maps[t] = pidx[t] >= 0;
    free(g_last.osb_sb); free(g_last.osb_maps);
    g_last.osb_sb = sb; g_last.osb_maps = maps; g_last.nx = nx; g_last.ny = ny;
    g_last.osb_penalty = penalty;
    free(em); free(epix); free(eoff); free(sp); free(cell3); free(w3); free(mapped); free(pmaps); free(pidx);
    free(model); free(act);
    return penalty;
}

/* 'include_noise_term_in_loglike on' (lens.cpp:303 default off) */
static int g_noise_term = 0;
void oracle_set_noise_term(int on) { g_noise_term = on; }

/* 'optimize_regparam on' settings (lens.cpp:421-425 defaults) */
static struct { int on; double minlog, maxlog, tol; int maxit; } g_regopt = {0, -3.0, 5.0, 0.01, 20};

void oracle_set_regopt(int on, double minlog, double maxlog, double tol, int maxit)
{
    g_regopt.on = on; g_regopt.minlog = minlog; g_regopt.maxlog = maxlog; g_regopt.tol = tol; g_regopt.maxit = maxit;
}

static void repack_lower(const double* up, double* lo, int n)
{
    long k = 0;
    for (int i = 0; i < n; i++) {
        long rowstart = (long)i * n - (long)i * (i - 1) / 2;  /* start of row i in packed upper */
        for (int j = i; j < n; j++) {
            /* element (i,j) of the upper triangle = (j,i) of the lower */
            lo[(long)j * (j + 1) / 2 + i] = up[rowstart + (j - i)];
            k++;
        }
    }
}

/* -2 log(evidence) as a function of log10(lambda) for fixed L and R:
 * QLens::chisq_regparam_dense (pixelgrid.cpp:16526-16700), the packed branch:
 * F = F0 + lambda R, Cholesky, solve, log det, the model over the active
 * pixels, Ed = sum (model - d)^2 C^-1 over them (the reference sums it with an
 * OpenMP reduction; here in pixel order), and the regularisation prior term. */
struct regopt_ctx {
    const double *F0, *Rp, *D, *Lp, *dvec, *cvec;
    int M, npix;
    long ntot;
    double logdetR;
};

static double regopt_objective(double logreg, void* user)
{
    const struct regopt_ctx* c = (const struct regopt_ctx*)user;
    const int M = c->M;
    const double lam = pow(10, logreg);
    double* Fc = (double*)malloc(sizeof(double) * c->ntot);
    double* Fl = (double*)malloc(sizeof(double) * c->ntot);
    double* s = (double*)malloc(sizeof(double) * M);
    for (long e = 0; e < c->ntot; e++) Fc[e] = c->F0[e] + lam * c->Rp[e];
    repack_lower(Fc, Fl, M);
    cholesky_packed_lower(Fl, M);
    cholesky_solve_packed_lower(Fl, c->D, s, M);
    const double logdet = cholesky_logdet_packed_lower(Fl, M);
    double Ed = 0;
    for (int r = 0; r < c->npix; r++) {
        double m = 0;
        for (int j = 0; j < M; j++) m += c->Lp[(size_t)r * M + j] * s[j];
        const double dd = m - c->dvec[r];
        Ed += dd * dd * c->cvec[r];
    }
    double Es = 0;
    for (int i = 0; i < M; i++) {
        long rs = (long)i * M - (long)i * (i - 1) / 2;
        Es += c->Rp[rs] * (s[i] * s[i]);
        for (int j = i + 1; j < M; j++) {
            double rv = c->Rp[rs + (j - i)];
            if (rv != 0) Es += 2 * s[i] * rv * s[j];
        }
    }
    double chisq = Ed + (lam * Es - M * log(lam) - c->logdetR);
    chisq += logdet;
    free(Fc); free(Fl); free(s);
    return chisq;
}

/* ------------------------------------------------------------------ */
/* the likelihood                                                       */
/* ------------------------------------------------------------------ */

int oracle_eval(const qlp_image* im, const qlp_psf* psf, const qlp_srcgrid_opts* op,
                const qlp_lens* lensdesc, int nlens, const qlp_planes* planes_in,
                const double* lens_params, double regparam, qlp_result* out)
{
    memset(out, 0, sizeof(*out));
    free_last();
    if (!im || !im->surface_brightness || !im->in_mask || !im->xvals || !im->yvals) {
        out->m2logev = -1e30; out->status = QLP_ERR_NO_DATA; return QLP_ERR_NO_DATA;
    }
    if (!op || nlens <= 0 || nlens > QLP_MAX_LENSES || op->nsplit < 1) { out->status = QLP_ERR_ARG; return QLP_ERR_ARG; }
    qlp_planes planes;
    if (planes_in) planes = *planes_in;
    else { memset(&planes, 0, sizeof(planes)); planes.n_planes = 1; planes.zfac[0] = 1.0; }

    olens lenses[QLP_MAX_LENSES];
    {
        int off = 0;
        for (int k = 0; k < nlens; k++) {
            const double* p = lens_params ? lens_params + off : lensdesc[k].p;
            if (setup_lens(&lenses[k], &lensdesc[k], p) != 0) { out->status = QLP_ERR_ARG; return QLP_ERR_ARG; }
            off += n_params_of(lensdesc[k].type);
        }
    }
    if (regparam <= 0) regparam = op->regparam;
    const int nx = im->npixels_x, ny = im->npixels_y;
    const int ns = op->nsplit, nsub = ns * ns;

    /* masked pixels in the reference's j-outer / i-inner order (setup_ray_tracing_arrays, pixelgrid.cpp:9996-10005) */
    int n_mask = 0;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) if (im->in_mask[i * ny + j]) n_mask++;
    int* mpix = (int*)malloc(sizeof(int) * (n_mask > 0 ? n_mask : 1));
    {
        int c = 0;
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) if (im->in_mask[i * ny + j]) mpix[c++] = i * ny + j;
    }
    const int n_sub = n_mask * nsub;
    double* sp = (double*)malloc(sizeof(double) * 2 * (n_sub > 0 ? n_sub : 1));

    /* sub-pixel centres (set_nsplits, pixelgrid.cpp:10898-10938) and ray shooting
       (calculate_sourcepts_and_areas, pixelgrid.cpp:10410-10441) */
    #pragma omp parallel for schedule(dynamic, 16)
    for (int m = 0; m < n_mask; m++) {
        int i = mpix[m] / ny, j = mpix[m] % ny;
        double x0 = im->xvals[i], x1 = im->xvals[i + 1];
        double y0 = im->yvals[j], y1 = im->yvals[j + 1];
        int k = 0;
        for (int ii = 0; ii < ns; ii++)
            for (int jj = 0; jj < ns; jj++) {
                double u0 = ((double)(1 + 2 * ii)) / (2 * ns);
                double w0 = ((double)(1 + 2 * jj)) / (2 * ns);
                double px = (1 - u0) * x0 + u0 * x1;
                double py = (1 - w0) * y0 + w0 * y1;
                double bx, by;
                find_sourcept(lenses, nlens, &planes, px, py, &bx, &by);
                sp[2 * ((long)m * nsub + k)] = bx;
                sp[2 * ((long)m * nsub + k) + 1] = by;
                k++;
            }
    }

    /* source-grid bounds: find_optimal_sourcegrid (pixelgrid.cpp:10998-11080) + srcgrid_size_scale (lens.cpp:12459-12470) */
    double gxmin, gxmax, gymin, gymax;
    if (op->auto_sourcegrid) {
        gxmin = 1e30; gxmax = -1e30; gymin = 1e30; gymax = -1e30;
        int use_nt = op->noise_threshold > 0;
        for (int m = 0; m < n_mask; m++) {
            int i = mpix[m] / ny, j = mpix[m] % ny;
            if (use_nt) {
                double noise = im->covinv_map ? 1.0 / sqrt(im->covinv_map[i * ny + j]) : im->background_pixel_noise;
                if (im->surface_brightness[i * ny + j] <= op->noise_threshold * noise) continue;
            }
            double xs = 0, ys = 0;
            for (int k = 0; k < nsub; k++) { xs += sp[2 * ((long)m * nsub + k)]; ys += sp[2 * ((long)m * nsub + k) + 1]; }
            xs /= nsub; ys /= nsub;
            if (xs < gxmin) { if (xs > op->limit_xmin) gxmin = xs; else if (gxmin > op->limit_xmin) gxmin = op->limit_xmin; }
            if (xs > gxmax) { if (xs < op->limit_xmax) gxmax = xs; else if (gxmax < op->limit_xmax) gxmax = op->limit_xmax; }
            if (ys < gymin) { if (ys > op->limit_ymin) gymin = ys; else if (gymin > op->limit_ymin) gymin = op->limit_ymin; }
            if (ys > gymax) { if (ys < op->limit_ymax) gymax = ys; else if (gymax < op->limit_ymax) gymax = op->limit_ymax; }
        }
        double xw = 0.1 * (gxmax - gxmin), yw = 0.1 * (gymax - gymin);
        gxmin -= xw / 2; gxmax += xw / 2; gymin -= yw / 2; gymax += yw / 2;
        if (op->size_scale != 0) {
            double xwa = op->size_scale * (gxmax - gxmin), ywa = op->size_scale * (gymax - gymin);
            double xc = (gxmax + gxmin) / 2, yc = (gymax + gymin) / 2;
            gxmin = xc - xwa / 2; gxmax = xc + xwa / 2; gymin = yc - ywa / 2; gymax = yc + ywa / 2;
        }
    } else {
        gxmin = op->xmin; gxmax = op->xmax; gymin = op->ymin; gymax = op->ymax;
    }
    g_last.grid[0] = gxmin; g_last.grid[1] = gxmax; g_last.grid[2] = gymin; g_last.grid[3] = gymax;
    const int snx = op->npixels_x, sny = op->npixels_y;
    g_last.src_nx = snx; g_last.src_ny = sny;
    g_last.srcpt = sp; g_last.n_sub = n_sub; g_last.n_mask = n_mask;
    if (snx < 2 || sny < 2) {
        free(mpix);
        out->m2logev = 2e30; out->status = QLP_ERR_GRID_TOO_SMALL; return QLP_ERR_GRID_TOO_SMALL;
    }

    /* SourcePixelGrid::create_pixel_grid (pixelgrid.cpp:401-472): corners by accumulation;
       SourcePixel ctor (761-783): centre = mean of 4 corners */
    double* cx = (double*)malloc(sizeof(double) * (snx + 1));
    double* cy = (double*)malloc(sizeof(double) * (sny + 1));
    {
        double xstep = (gxmax - gxmin) / snx, ystep = (gymax - gymin) / sny, x, y;
        int i;
        for (i = 0, x = gxmin; i <= snx; i++, x += xstep) cx[i] = x;
        for (i = 0, y = gymin; i <= sny; i++, y += ystep) cy[i] = y;
    }
    double* ccx = (double*)malloc(sizeof(double) * snx);
    double* ccy = (double*)malloc(sizeof(double) * sny);
    for (int i = 0; i < snx; i++) ccx[i] = (cx[i] + cx[i] + cx[i + 1] + cx[i + 1]) / 4.0;
    for (int j = 0; j < sny; j++) ccy[j] = (cy[j] + cy[j + 1] + cy[j] + cy[j + 1]) / 4.0;

    /* per sub-pixel: containing cell + x/y interpolation neighbours
       (bisection_search_interpolate + assign_source_mapping_flags_interpolate, pixelgrid.cpp:2291-2432) */
    int* cell3 = (int*)malloc(sizeof(int) * 3 * (n_sub > 0 ? n_sub : 1));
    unsigned char* mapped = (unsigned char*)calloc((size_t)snx * sny, 1);
    unsigned char* pixmaps = (unsigned char*)calloc(n_mask > 0 ? n_mask : 1, 1);
    for (long t = 0; t < n_sub; t++) {
        double px = sp[2 * t], py = sp[2 * t + 1];
        cell3[3 * t] = -1;
        if (!(px >= cx[0] && px < cx[snx] && py >= cy[0] && py < cy[sny])) continue;
        int lo = 0, hi = snx - 1;
        while (lo < hi) { int mid = (lo + hi + 1) / 2; if (cx[mid] <= px) lo = mid; else hi = mid - 1; }
        int ci = lo;
        lo = 0; hi = sny - 1;
        while (lo < hi) { int mid = (lo + hi + 1) / 2; if (cy[mid] <= py) lo = mid; else hi = mid - 1; }
        int cj = lo;
        int xn, yn;
        if ((px > ccx[ci] && ci < snx - 1) || ci == 0) xn = ci + 1; else xn = ci - 1;
        if ((py > ccy[cj] && cj < sny - 1) || cj == 0) yn = cj + 1; else yn = cj - 1;
        cell3[3 * t] = cj * snx + ci;
        cell3[3 * t + 1] = cj * snx + xn;
        cell3[3 * t + 2] = yn * snx + ci;
        mapped[cj * snx + ci] = 1; mapped[cj * snx + xn] = 1; mapped[yn * snx + ci] = 1;
        pixmaps[t / nsub] = 1;
    }
    /* assign_active_indices (pixelgrid.cpp:3576-3626): mapped cells, j-outer / i-inner */
    int* aidx = (int*)malloc(sizeof(int) * snx * sny);
    int M = 0;
    for (int c = 0; c < snx * sny; c++) aidx[c] = mapped[c] ? M++ : -1;
    g_last.active_index = aidx;
    g_last.M = M;
    /* active image pixels (assign_pixel_mappings, pixelgrid.cpp:12881-12910) */
    int npix = 0;
    for (int m = 0; m < n_mask; m++) if (pixmaps[m]) npix++;
    int* apix = (int*)malloc(sizeof(int) * (npix > 0 ? npix : 1));   /* mask-list position */
    int* pixindex = (int*)malloc(sizeof(int) * nx * ny);
    for (int t = 0; t < nx * ny; t++) pixindex[t] = -1;
    {
        int c = 0;
        for (int m = 0; m < n_mask; m++) if (pixmaps[m]) { apix[c] = m; pixindex[mpix[m]] = c; c++; }
    }
    g_last.n_pix = npix;
    out->n_active_pixels = npix;
    out->n_active_src = M;
    if (M == 0) {
        free(mpix); free(cx); free(cy); free(ccx); free(ccy); free(cell3); free(mapped); free(pixmaps);
        free(apix); free(pixindex);
        out->m2logev = 2e30; out->status = QLP_ERR_NO_SOURCE_PIXELS; return QLP_ERR_NO_SOURCE_PIXELS;
    }

    /* pre-PSF L in CSR (assign_Lmatrix 13196-13321, calculate_Lmatrix_interpolate 2501-2527) */
    int* rowptr = (int*)malloc(sizeof(int) * (npix + 1));
    rowptr[0] = 0;
    for (int r = 0; r < npix; r++) {
        int m = apix[r], cnt = 0;
        for (int k = 0; k < nsub; k++) if (cell3[3 * ((long)m * nsub + k)] >= 0) cnt += 3;
        rowptr[r + 1] = rowptr[r] + cnt;
    }
    const int nnz = rowptr[npix];
    int* Lidx = (int*)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    double* Lval = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    const double weight = 1.0 / nsub;
    #pragma omp parallel for schedule(static)
    for (int r = 0; r < npix; r++) {
        int m = apix[r], e = rowptr[r];
        for (int k = 0; k < nsub; k++) {
            long t = (long)m * nsub + k;
            if (cell3[3 * t] < 0) continue;
            double p0x, p0y, p1x, p1y, p2x, p2y;
            int c0 = cell3[3 * t], c1 = cell3[3 * t + 1], c2 = cell3[3 * t + 2];
            p0x = ccx[c0 % snx]; p0y = ccy[c0 / snx];
            p1x = ccx[c1 % snx]; p1y = ccy[c1 / snx];
            p2x = ccx[c2 % snx]; p2y = ccy[c2 / snx];
            double px = sp[2 * t], py = sp[2 * t + 1];
            double d = (p0x - p1x) * (p1y - p2y) - (p1x - p2x) * (p0y - p1y);
            Lidx[e] = aidx[c0];
            Lval[e] = weight * (px * (p1y - p2y) + py * (p2x - p1x) + p1x * p2y - p1y * p2x) / d;
            Lidx[e + 1] = aidx[c1];
            Lval[e + 1] = weight * (px * (p2y - p0y) + py * (p0x - p2x) + p0y * p2x - p0x * p2y) / d;
            Lidx[e + 2] = aidx[c2];
            Lval[e + 2] = weight * (px * (p0y - p1y) + py * (p1x - p0x) + p0x * p1y - p0y * p1x) / d;
            e += 3;
        }
    }
    g_last.L_rowptr = rowptr; g_last.L_index = Lidx; g_last.L_value = Lval; g_last.nnz = nnz;
    out->L_nnz = nnz;

    /* dense L (convert_Lmatrix_to_dense, pixelgrid.cpp:13717-13747) */
    double* Ld = (double*)calloc((size_t)npix * M, sizeof(double));
    #pragma omp parallel for schedule(static)
    for (int r = 0; r < npix; r++)
        for (int e = rowptr[r]; e < rowptr[r + 1]; e++) Ld[(size_t)r * M + Lidx[e]] += Lval[e];

    /* PSF convolution, direct dense path (PSF_convolution_Lmatrix_dense, pixelgrid.cpp:14092-14176) */
    double* Lp = (double*)calloc((size_t)npix * M, sizeof(double));
    {
        const int pnx = psf->nx, pny = psf->ny, nxh = pnx / 2, nyh = pny / 2;
        #pragma omp parallel for schedule(static)
        for (int r = 0; r < npix; r++) {
            int k = mpix[apix[r]] / ny, l = mpix[apix[r]] % ny;
            double* out_row = Lp + (size_t)r * M;
            for (int pk = 0; pk < pnx; pk++) {
                int ii = k + nxh - pk;
                if (ii < 0 || ii >= nx) continue;
                for (int pl = 0; pl < pny; pl++) {
                    int jj = l + nyh - pl;
                    if (jj < 0 || jj >= ny) continue;
                    int q = pixindex[ii * ny + jj];
                    if (q < 0) continue;   /* not (in mask and mapped) */
                    double pv = psf->matrix[pk * pny + pl];
                    const double* in_row = Ld + (size_t)q * M;
                    for (int s2 = 0; s2 < M; s2++) out_row[s2] += pv * in_row[s2];
                }
            }
        }
    }
    free(Ld);
    g_last.Lpsf = Lp;

    /* data vector, noise (fill_surface_brightness_vector 11428; create_lensing_matrices_from_Lmatrix_dense 15590-15736) */
    const int use_noise_map = im->covinv_map != NULL;
    const double cov_inverse = (im->background_pixel_noise == 0) ? 1 : 1.0 / (im->background_pixel_noise * im->background_pixel_noise);
    double* dvec = (double*)malloc(sizeof(double) * npix);
    double* cvec = (double*)malloc(sizeof(double) * npix);
    for (int r = 0; r < npix; r++) {
        int t = mpix[apix[r]];
        dvec[r] = im->surface_brightness[t];
        cvec[r] = use_noise_map ? im->covinv_map[t] : cov_inverse;
    }
    double* D = (double*)calloc(M, sizeof(double));
    double* Lt = (double*)malloc(sizeof(double) * (size_t)M * npix);
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < M; i++) {
        for (int j = 0; j < npix; j++) {
            double sb_adj = dvec[j] - 0.0;
            D[i] += Lp[(size_t)j * M + i] * sb_adj * cvec[j];
            Lt[(size_t)i * npix + j] = Lp[(size_t)j * M + i];
        }
    }
    /* F = L^T C^-1 L, packed upper, naive dot products (pixelgrid.cpp:15682-15710) */
    const long ntot = (long)M * (M + 1) / 2;
    double* Fp = (double*)malloc(sizeof(double) * ntot);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < M; i++) {
        long rowstart = (long)i * M - (long)i * (i - 1) / 2;
        const double* l1 = Lt + (size_t)i * npix;
        for (int j = i; j < M; j++) {
            const double* l2 = Lt + (size_t)j * npix;
            double f = 0;
            if (use_noise_map) {
                for (int l = 0; l < npix; l++) f += l1[l] * l2[l] * cvec[l];
            } else {
                for (int l = 0; l < npix; l++) f += l1[l] * l2[l];
                f *= cov_inverse;
            }
            Fp[rowstart + (j - i)] = f;
        }
    }
    free(Lt);

    /* curvature regularisation R = Hx^T Hx + Hy^T Hy (generate_hmatrices 2968-3071,
       generate_Rmatrix_from_hmatrices 3073-3240); entries are small integers, so
       the order of accumulation does not matter */
    double logdetR = 0, Es = 0, regterms = 0;
    double* Rp = NULL;  /* packed upper */
    if (op->regularization) {
        Rp = (double*)calloc(ntot, sizeof(double));
        for (int l = 0; l < 2; l++) {
            for (int cj = 0; cj < sny; cj++)
                for (int ci = 0; ci < snx; ci++) {
                    int a = aidx[cj * snx + ci];
                    if (a < 0) continue;
                    int idx[3]; double h[3]; int nh = 0;
                    idx[nh] = a; h[nh++] = -2;
                    int n1i = (l == 0) ? ci + 1 : ci, n1j = (l == 0) ? cj : cj + 1;
                    int n2i = (l == 0) ? ci - 1 : ci, n2j = (l == 0) ? cj : cj - 1;
                    if (n1i < snx && n1j < sny && aidx[n1j * snx + n1i] >= 0) { idx[nh] = aidx[n1j * snx + n1i]; h[nh++] = 1; }
                    if (n2i >= 0 && n2j >= 0 && aidx[n2j * snx + n2i] >= 0) { idx[nh] = aidx[n2j * snx + n2i]; h[nh++] = 1; }
                    for (int u = 0; u < nh; u++)
                        for (int v = u; v < nh; v++) {
                            int r1 = idx[u], r2 = idx[v];
                            if (r1 > r2) { int tmp = r1; r1 = r2; r2 = tmp; }
                            Rp[(long)r1 * M - (long)r1 * (r1 - 1) / 2 + (r2 - r1)] += h[u] * h[v];
                        }
                }
        }
        /* Rmatrix_determinant_dense (pixelgrid.cpp:18176-18191) */
        double* Rl = (double*)malloc(sizeof(double) * ntot);
        repack_lower(Rp, Rl, M);
        if (!cholesky_packed_lower(Rl, M)) {
            free(Rl);
            out->status = QLP_ERR_NOT_SPD;
        } else {
            logdetR = cholesky_logdet_packed_lower(Rl, M);
            free(Rl);
        }
        /* optimize_regparam: lambda = 10^x with x from Brent's method over the
           objective above (optimize_regularization_parameter, pixelgrid.cpp:
           15865-15890); the inversion below then runs at that lambda, which
           reproduces the best trial's amplitudes and log det F */
        if (g_regopt.on && M > 0 && out->status == 0) {
            struct regopt_ctx rc = {Fp, Rp, D, Lp, dvec, cvec, M, npix, ntot, logdetR};
            int nev = 0;
            const double x = oracle_brent_min(regopt_objective, &rc, g_regopt.minlog, g_regopt.maxlog, g_regopt.tol,
                                              g_regopt.maxit, &nev);
            regparam = pow(10, x);
            out->regopt_evals = nev;
        }
        /* add_regularization_term_to_dense_Fmatrix (pixelgrid.cpp:15781-15819) */
        for (long e = 0; e < ntot; e++) Fp[e] += regparam * Rp[e];
    }
    double* Fdiag = (double*)malloc(sizeof(double) * M);
    for (int i = 0; i < M; i++) Fdiag[i] = Fp[(long)i * M - (long)i * (i - 1) / 2];
    g_last.Fdiag = Fdiag;

    /* invert_lens_mapping_dense (pixelgrid.cpp:17346-17396) */
    double* Fl = (double*)malloc(sizeof(double) * ntot);
    repack_lower(Fp, Fl, M);
    free(Fp);
    double* s = (double*)malloc(sizeof(double) * M);
    int spd = cholesky_packed_lower(Fl, M);
    cholesky_solve_packed_lower(Fl, D, s, M);
    double logdetF = cholesky_logdet_packed_lower(Fl, M);
    free(Fl);
    if (!spd) out->status = QLP_ERR_NOT_SPD;

    /* model image (calculate_image_pixel_surface_brightness_dense, pixelgrid.cpp:18268-18290) */
    double* model = (double*)malloc(sizeof(double) * npix);
    #pragma omp parallel for schedule(static)
    for (int r = 0; r < npix; r++) {
        double acc = 0;
        for (int j = 0; j < M; j++) acc += Lp[(size_t)r * M + j] * s[j];
        model[r] = acc;
    }

    /* regularisation prior term, sparse branch (pixelgrid.cpp:15852-15860) */
    if (op->regularization && regparam != 0) {
        for (int i = 0; i < M; i++) {
            long rs = (long)i * M - (long)i * (i - 1) / 2;
            Es += Rp[rs] * (s[i] * s[i]);
            for (int j = i + 1; j < M; j++) {
                double rv = Rp[rs + (j - i)];
                if (rv != 0) Es += 2 * s[i] * rv * s[j];
            }
        }
        regterms = regparam * Es - M * log(regparam) - logdetR;
    }
    free(Rp);

    /* chi^2 over the mask, x-outer / y-inner (lens.cpp:12950-13016) */
    double chisq0 = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            int t = i * ny + j;
            if (!im->in_mask[t]) continue;
            double ci_ = use_noise_map ? im->covinv_map[t] : cov_inverse;
            int r = pixindex[t];
            if (r >= 0) { double dd = model[r] - im->surface_brightness[t]; chisq0 += dd * dd * ci_; }
            else { double dd = im->surface_brightness[t]; chisq0 += dd * dd * ci_; }
        }
    double loglike = 0;
    if (op->regularization && M > 0) {
        if (regparam != 0) loglike += regterms;
        loglike += logdetF;
    }
    loglike += chisq0;
    /* the pixel noise term (lens.cpp:13033-13043): minus log C^-1 of each active
       pixel in turn (noise map) or of the uniform noise times the masked-pixel
       count, plus the masked-pixel count times log(2 pi) */
    if (g_noise_term) {
        if (use_noise_map) {
            for (int r = 0; r < npix; r++) loglike -= log(cvec[r]);
        } else {
            loglike -= n_mask * log(cov_inverse);
        }
        loglike += n_mask * log(6.28318530717958647692);
    }
    if (g_osb.on && out->status == 0)
        loglike += outside_sb_penalty(im, psf, lenses, nlens, &planes, ns, cx, cy, ccx, ccy, snx, sny, aidx, s);

    out->chisq0 = chisq0;
    out->logdet_F = logdetF;
    out->logdet_R = logdetR;
    out->Es_times_two = Es;
    out->regterms = regterms;
    out->m2logev = loglike;
    out->regparam = regparam;
    g_last.D = D; g_last.s = s; g_last.model = model;

    free(mpix); free(cx); free(cy); free(ccx); free(ccy); free(cell3); free(mapped); free(pixmaps);
    free(apix); free(pixindex); free(dvec); free(cvec);
    return out->status;
}

int oracle_n_params(const qlp_lens* lenses, int nlens)
{
    int n = 0;
    for (int k = 0; k < nlens; k++) n += n_params_of(lenses[k].type);
    return n;
}

/* Copy a dumped array of the last evaluation; returns its element count. */
long oracle_get(const char* name, void* buf, long cap)
{
    const void* src = NULL; long n = 0; size_t es = 8;
    if (!strcmp(name, "srcpt")) { src = g_last.srcpt; n = 2L * g_last.n_sub; }
    else if (!strcmp(name, "L_rowptr")) { src = g_last.L_rowptr; n = g_last.n_pix + 1; es = 4; }
    else if (!strcmp(name, "L_index")) { src = g_last.L_index; n = g_last.nnz; es = 4; }
    else if (!strcmp(name, "L_value")) { src = g_last.L_value; n = g_last.nnz; }
    else if (!strcmp(name, "active_index")) { src = g_last.active_index; n = (long)g_last.src_nx * g_last.src_ny; es = 4; }
    else if (!strcmp(name, "Lpsf")) { src = g_last.Lpsf; n = (long)g_last.n_pix * g_last.M; }
    else if (!strcmp(name, "D")) { src = g_last.D; n = g_last.M; }
    else if (!strcmp(name, "s")) { src = g_last.s; n = g_last.M; }
    else if (!strcmp(name, "model")) { src = g_last.model; n = g_last.n_pix; }
    else if (!strcmp(name, "F_diag")) { src = g_last.Fdiag; n = g_last.M; }
    else if (!strcmp(name, "grid")) { src = g_last.grid; n = 4; }
    else if (!strcmp(name, "osb_sb")) { src = g_last.osb_sb; n = g_last.osb_sb ? (long)g_last.nx * g_last.ny : 0; }
    else if (!strcmp(name, "osb_maps")) { src = g_last.osb_maps; n = g_last.osb_maps ? (long)g_last.nx * g_last.ny : 0; es = 1; }
    else if (!strcmp(name, "osb_penalty")) { src = &g_last.osb_penalty; n = 1; }
    else return -1;
    if (buf && src) memcpy(buf, src, es * (size_t)(n < cap ? n : cap));
    return n;
}

int oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
