/* nfw_oracle.c -- NFW deflection by adaptive Gauss-Patterson quadrature
 * (placeholder until the quadrature restatement lands). Test infrastructure only. */
#include "qlpix_oracle.h"
int oracle_nfw_setup(double ks, double rs, double q) { (void)ks; (void)rs; (void)q; return 0; }
void oracle_nfw_deflection(double ks, double rs, double q, double f, double x, double y, double* dx, double* dy)
{ (void)ks; (void)rs; (void)q; (void)f; (void)x; (void)y; *dx = 0; *dy = 0; }
