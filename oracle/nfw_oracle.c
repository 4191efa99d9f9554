/*
 * nfw_oracle.c -- elliptical NFW deflection by adaptive Gauss-Patterson
 * quadrature, restated from QLens.  TEST INFRASTRUCTURE ONLY (the checker;
 * see qlpix_oracle.c).
 *
 * Reference (file:line):
 *   NFW::kappa_rsq, lens_function_xsq, kapavg_spherical_rsq  models.cpp:978-1010
 *   LensProfile::set_integration_pointers (q == 1 -> spherical)  profile.cpp:1510-1524
 *   LensProfile::deflection_spherical_default                  profile.cpp:2281-2290
 *   LensProfile::deflection_numerical                          profile.cpp:2359-2375
 *   LensIntegral::initialize (epsilon = 1 - q^2, fsqinv = q for emode 1)  profile.h:441-449
 *   LensIntegral::j_integral, j_integrand_prime                profile.cpp:2703-2733, 2778-2783
 *   LensIntegral::PattersonIntegrate                           profile.cpp:3830-3876
 * QLens's default integral_tolerance is 1e-3 (lens.cpp:556), handed to
 * every lens as its Patterson tolerance (lens.cpp:1338, profile.cpp:1480-1486);
 * Gauss_NN = 60 < 511, so an unconverged integral keeps its 511-point value.
 *
 * Evaluation order follows the reference expression by expression (compile
 * with -ffp-contract=off) so that, with the same libm, results agree bit for
 * bit with the compiled reference.
 */
#include <math.h>
#include "qlpix_oracle.h"
#include "../qlens_gb300/csrc/patterson_rule.h"

#define NFW_PAT_TOL 1e-3

int oracle_nfw_setup(double ks, double rs, double q)
{
    (void)ks;
    return (rs > 0 && q > 0 && q <= 1) ? 1 : 0;
}

static double lens_function_xsq(double xsq)
{
    return ((xsq > 1.0) ? (atan(sqrt(xsq - 1)) / sqrt(xsq - 1))
                        : (xsq < 1.0) ? (atanh(sqrt(1 - xsq)) / sqrt(1 - xsq)) : 1.0);
}

static double kappa_rsq(double ks, double rs, double rsq)
{
    double xsq = rsq / (rs * rs);
    if (xsq < 1e-6) return -ks * (2 + log(xsq / 4));
    else if (fabs(xsq - 1) < 1e-5) return 2 * ks * (0.3333333333333333 - (xsq - 1) / 5.0);
    else return 2 * ks * (1 - lens_function_xsq(xsq)) / (xsq - 1);
}

static double kapavg_spherical_rsq(double ks, double rs, double rsq)
{
    double xsq = rsq / (rs * rs);
    if (xsq > 1e-5)
        return 2 * ks * (2 * lens_function_xsq(xsq) + log(xsq / 4)) / xsq;
    else
        return -ks * (1 + log(xsq / 4));
}

typedef struct {
    double ks, rs, xsqval, ysqval, epsilon, fsqinv, nval_plus_half;
} jint;

static double j_integrand_prime(const jint* J, double w)
{
    double u = w * w;
    double qfac = 1 - J->epsilon * u;
    return (2 * w * kappa_rsq(J->ks, J->rs, u * (J->xsqval + J->ysqval / qfac) * J->fsqinv) / pow(qfac, J->nval_plus_half));
}

/* PattersonIntegrate on [0, 1]: level L uses the nodes (j+1)*2^(8-L)-1 of the
   511-point set; new nodes (even j) are evaluated and summed first, then the
   old ones (odd j) from the stored values, in ascending order. */
static double patterson_0_1(const jint* J)
{
    double funcs[QLP_PAT_N];
    double result = 0, result_old;
    const double absum = 0.5, abdif = 0.5;
    int level = 0;
    do {
        const double* wt = qlp_pat_weights_host + qlp_pat_offset[level];
        result_old = result;
        int order = (2 << level) - 1;
        int istep = (QLP_PAT_N + 1) / (order + 1);
        int istart = istep - 1;
        istep *= 2;
        result = 0;
        int i, j;
        for (j = 0, i = istart; j < order; j += 2, i += istep) {
            funcs[i] = j_integrand_prime(J, absum + abdif * qlp_pat_points_host[i]);
            result += wt[j] * funcs[i];
        }
        for (j = 1, i = istep - 1; j < order; j += 2, i += istep) result += wt[j] * funcs[i];
        if ((level > 1) && (fabs(result - result_old) < NFW_PAT_TOL * fabs(result))) break;
    } while (++level < QLP_PAT_LEVELS);
    return abdif * result;
}

void oracle_nfw_deflection(double ks, double rs, double q, double f_major_axis,
                           double x, double y, double* dx, double* dy)
{
    (void)f_major_axis;
    if (q == 1.0) {
        double kapavg = kapavg_spherical_rsq(ks, rs, x * x + y * y);
        *dx = kapavg * x;
        *dy = kapavg * y;
        return;
    }
    if ((fabs(x) < 1e-14) && (fabs(y) < 1e-14)) {
        *dx = 0;
        *dy = 0;
        return;
    }
    jint J;
    J.ks = ks; J.rs = rs;
    J.xsqval = x * x;
    J.ysqval = y * y;
    J.epsilon = 1 - q * q;
    J.fsqinv = q;                      /* emode 1 */
    J.nval_plus_half = 0 + 0.5;
    *dx = x * (sqrt(1 - J.epsilon) * patterson_0_1(&J));
    J.nval_plus_half = 1 + 0.5;
    *dy = y * (sqrt(1 - J.epsilon) * patterson_0_1(&J));
}
