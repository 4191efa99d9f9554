/* qlpix_oracle.h -- CPU restatement of QLens's pixel-image likelihood.
 * Test infrastructure only (see qlpix_oracle.c). */
#ifndef QLPIX_ORACLE_H
#define QLPIX_ORACLE_H
#include "../include/qlpix.h"
#ifdef __cplusplus
extern "C" {
#endif
int oracle_eval(const qlp_image* im, const qlp_psf* psf, const qlp_srcgrid_opts* op,
                const qlp_lens* lenses, int nlens, const qlp_planes* planes,
                const double* lens_params, double regparam, qlp_result* out);
int oracle_n_params(const qlp_lens* lenses, int nlens);
long oracle_get(const char* name, void* buf, long cap);
int oracle_threads(void);
void oracle_set_noise_term(int on);
void oracle_set_outside_sb(int on, double frac, double noise_frac, int emask_nsplit, const unsigned char* emask,
                           long n);
void oracle_set_regopt(int on, double minlog, double maxlog, double tol, int maxit);
double oracle_brent_min(double (*f)(double, void*), void* user, double ax, double bx, double tol, int maxit,
                        int* nevals);
/* NFW with numerical (Gauss-Patterson) deflection, oracle/nfw_oracle.c */
int oracle_nfw_setup(double ks, double rs, double q);
void oracle_nfw_deflection(double ks, double rs, double q, double f_major_axis,
                           double x, double y, double* dx, double* dy);
#ifdef __cplusplus
}
#endif
#endif
