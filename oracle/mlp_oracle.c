/*
 * mlp_oracle.c -- CPU reference of the NFW surrogate network's forward pass,
 * loss and parameter gradients, in double precision.  TEST INFRASTRUCTURE
 * ONLY: the GPU training kernels (qlens_gb300/csrc/surrogate.cu) are checked
 * against it; the product never calls it.
 *
 * Network (the layout the GPU kernels use): 3 inputs -> 4 hidden layers of
 * 128 tanh units -> 2 linear outputs.  Parameters, flattened in this order:
 *   W0 [3][128], b0 [128], W1 [128][128], b1, W2 [128][128], b2,
 *   W3 [128][128], b3, W4 [128][2], b4 [2]        (W[l] is [in][out])
 * Loss: mean over the batch of sum_o (y_o - t_o)^2.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define H 128
#define NIN 3
#define NOUT 2
#define NLAYER 5

static const int dims[NLAYER + 1] = {NIN, H, H, H, H, NOUT};

int oracle_mlp_n_params(void)
{
    int n = 0;
    for (int l = 0; l < NLAYER; l++) n += dims[l] * dims[l + 1] + dims[l + 1];
    return n;
}

/* x [batch][3], t [batch][2]; p parameters; grad (may be NULL) gets dL/dp;
   y (may be NULL) gets the outputs [batch][2].  Returns the loss. */
double oracle_mlp_loss_grad(const double* p, int batch, const double* x, const double* t, double* grad, double* y)
{
    const double* W[NLAYER];
    const double* b[NLAYER];
    double* gW[NLAYER];
    double* gb[NLAYER];
    size_t off = 0;
    for (int l = 0; l < NLAYER; l++) {
        W[l] = p + off;
        if (grad) gW[l] = grad + off;
        off += (size_t)dims[l] * dims[l + 1];
        b[l] = p + off;
        if (grad) gb[l] = grad + off;
        off += dims[l + 1];
    }
    if (grad) memset(grad, 0, sizeof(double) * off);
    double* act[NLAYER + 1];
    for (int l = 0; l <= NLAYER; l++) act[l] = (double*)malloc(sizeof(double) * (size_t)batch * dims[l]);
    memcpy(act[0], x, sizeof(double) * (size_t)batch * NIN);
    for (int l = 0; l < NLAYER; l++) {
        const int ni = dims[l], no = dims[l + 1];
        for (int s = 0; s < batch; s++)
            for (int j = 0; j < no; j++) {
                double z = b[l][j];
                for (int k = 0; k < ni; k++) z += act[l][(size_t)s * ni + k] * W[l][(size_t)k * no + j];
                act[l + 1][(size_t)s * no + j] = (l < NLAYER - 1) ? tanh(z) : z;
            }
    }
    double loss = 0;
    double* d = (double*)malloc(sizeof(double) * (size_t)batch * H);
    double* dn = (double*)malloc(sizeof(double) * (size_t)batch * H);
    for (int s = 0; s < batch; s++)
        for (int o = 0; o < NOUT; o++) {
            const double e = act[NLAYER][(size_t)s * NOUT + o] - t[(size_t)s * NOUT + o];
            loss += e * e;
            d[(size_t)s * NOUT + o] = 2.0 * e / batch;     /* dL/dz of the output layer */
        }
    loss /= batch;
    if (y) memcpy(y, act[NLAYER], sizeof(double) * (size_t)batch * NOUT);
    if (grad) {
        for (int l = NLAYER - 1; l >= 0; l--) {
            const int ni = dims[l], no = dims[l + 1];
            for (int k = 0; k < ni; k++)
                for (int j = 0; j < no; j++) {
                    double g = 0;
                    for (int s = 0; s < batch; s++) g += act[l][(size_t)s * ni + k] * d[(size_t)s * no + j];
                    gW[l][(size_t)k * no + j] = g;
                }
            for (int j = 0; j < no; j++) {
                double g = 0;
                for (int s = 0; s < batch; s++) g += d[(size_t)s * no + j];
                gb[l][j] = g;
            }
            if (l == 0) break;
            for (int s = 0; s < batch; s++)
                for (int k = 0; k < ni; k++) {
                    double g = 0;
                    for (int j = 0; j < no; j++) g += d[(size_t)s * no + j] * W[l][(size_t)k * no + j];
                    const double a = act[l][(size_t)s * ni + k];
                    dn[(size_t)s * ni + k] = g * (1.0 - a * a);   /* through tanh */
                }
            double* tmp = d; d = dn; dn = tmp;
        }
    }
    free(d); free(dn);
    for (int l = 0; l <= NLAYER; l++) free(act[l]);
    return loss;
}
