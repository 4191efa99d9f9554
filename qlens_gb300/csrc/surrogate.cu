// surrogate.cu -- the learned part: an MLP surrogate of the elliptical NFW
// deflection, trained on the GPU on output of the Gauss-Patterson quadrature
// (nfw_device.cuh) and run on the tensor cores inside the ray shooting, with
// the quadrature as fallback wherever the surrogate's error bound is exceeded.
//
// What is learned.  For the lens-frame point (x, y), the quadrature gives
// alpha_x = x ks G_0(X, Y, q), alpha_y = y ks G_1(X, Y, q) with X = x/rs,
// Y = y/rs (LensProfile::deflection_numerical, profile.cpp:2359-2375; G_n =
// sqrt(1-eps) J_n / ks, eps = 1 - q^2, is dimensionless because
// kappa(r^2; ks, rs) = ks kappa_hat(r^2/rs^2), models.cpp:978-984).  The
// network maps the inputs (log R, phi, q), R = sqrt(X^2 + Y^2),
// phi = atan2(|Y|, |X|) -- log rs is absorbed exactly by that scaling -- to
// s_n = log(G_n / B) / (1 - q), B = the spherical mean convergence kapavg_hat
// at the elliptical radius xi^2 = q X^2 + Y^2 / q (NFW::kapavg_spherical_rsq,
// models.cpp:1001-1010, in FP64): log(G_n / B) is a bounded residual that
// vanishes at q = 1 (where G_n = B exactly), so dividing by 1 - q leaves an
// O(1) smooth target and makes the surrogate exact in the spherical limit.
// Deflection only: the pixel likelihood ray-traces, it never needs the
// Hessian.
//
// Network: 3 -> 4 x 128 tanh -> 2 (50,306 parameters, the layout of
// oracle/mlp_oracle.c).  Training (k_sur_*): FP32 SIMT GEMMs for the
// forward pass, the backward pass and the weight gradients (split over the
// batch, reduced in a fixed order), Adam; the loss weights each sample by its
// squared dimensionless deflection, since the error the gate tests is |alpha|
// times the relative error.  Inference (sur_mlp_wg): 128 rays per warpgroup =
// the 128 TMEM lanes, two warpgroups per persistent CTA; layer 0 (3 -> 128) on
// the CUDA cores, layers 1-3 (128 x 128) as tcgen05 kind::f16 MMAs with the
// activations in TMEM (A operand, F16 hi + lo) and the weights resident in
// shared memory (B operand, F16 hi + lo), three products per K step; the
// output layer on the CUDA cores.
//
// Error bound.  After training the surrogate is compared with the quadrature
// (tolerance 1e-10) on 32 jittered points of every cell of a 64 x 16 x 16 grid
// over (log R, phi, q); three times the largest relative error of G_0, G_1 in
// a cell is that cell's bound.  A ray uses the surrogate only if
// ks |G| |(x, y)| times its cell's bound is below the gate (2e-5 arcsec by
// default) and its inputs lie inside the trained domain; every other ray
// takes the quadrature.
#include <cuda.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include "qlpix_ctx.h"
#include "lens_device.cuh"
#include "tc_common.cuh"

namespace qlpix {

#define SUR_H 128
#define SUR_W0 0
#define SUR_B0 (SUR_W0 + 3 * SUR_H)
#define SUR_W1 (SUR_B0 + SUR_H)
#define SUR_B1 (SUR_W1 + SUR_H * SUR_H)
#define SUR_W2 (SUR_B1 + SUR_H)
#define SUR_B2 (SUR_W2 + SUR_H * SUR_H)
#define SUR_W3 (SUR_B2 + SUR_H)
#define SUR_B3 (SUR_W3 + SUR_H * SUR_H)
#define SUR_W4 (SUR_B3 + SUR_H)
#define SUR_B4 (SUR_W4 + 2 * SUR_H)
#define SUR_NP (SUR_B4 + 2)

// trained domain
#define SUR_RHO_LO (-9.210340371976184)   // log 1e-4
#define SUR_RHO_HI (5.298317366548036)    // log 200
#define SUR_Q_LO 0.45
#define SUR_NB_RHO 64
#define SUR_NB_PHI 16
#define SUR_NB_Q 16
#define SUR_NBINS (SUR_NB_RHO * SUR_NB_PHI * SUR_NB_Q)
#define SUR_VAL_PER_BIN 32
#define SUR_BOUND_SAFETY 3.0
#define SUR_TARGET_TOL 1e-10

// ---------------------------------------------------------------------------
// shared pieces: inputs, baseline, activation
// ---------------------------------------------------------------------------
// tanh(x) = 1 - 2 / (1 + e^2x), the quotient by the SFU reciprocal (within
// 2 ulp; e^2x beyond 2^126 gives 1 exactly).  Training and inference share it.
__device__ __forceinline__ float sur_tanh(float x)
{
    return 1.0f - __fdividef(2.0f, 1.0f + __expf(2.0f * x));
}

// s tanh(x) from a = 2 log2(e) x (the inference's parameters carry the
// factor): s - 2 s / (1 + 2^a) with the SFU's base-2 exponential and
// reciprocal, one FMA for the rest
__device__ __forceinline__ float sur_tanh_a(float a, float s)
{
    float e, r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(a));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
    return __fmaf_rn(-2.0f * s, r, s);
}

struct SurIn {
    float f0, f1, f2;   // normalised inputs
    int bin;            // error-bound cell, -1 outside the domain
    double B;           // baseline
    double B_rel;       // bound on B's relative error (0: FP64)
};

// The baseline B = kapavg_hat(xi^2) (ks = rs = 1) in FP32 where xi^2 >= 0.5:
// there 2 F + log(xi^2 / 4) cancels by at most a factor 6, and FP32 sqrt,
// atan / atanh and log (within a few ulp) keep B within SUR_B32_REL of the
// FP64 value (measured on CPU over xi^2 in [0.5, 1e6]: 9e-7 at most).  The
// ray adds SUR_B32_REL to its cell's error bound.  Smaller xi^2 (rays within
// about one scale radius) keep the FP64 form, whose small-radius branch
// cancels.
#define SUR_B32_MIN 0.5
#define SUR_B32_REL 5e-6
__device__ __forceinline__ float sur_B32(float x)
{
    float F;
    if (x > 1.0f) {
        const float s = sqrtf(x - 1.0f);
        F = atanf(s) / s;
    } else if (x < 1.0f) {
        const float s = sqrtf(1.0f - x);
        F = atanhf(s) / s;
    } else {
        F = 1.0f;
    }
    return 2.0f * (2.0f * F + logf(0.25f * x)) / x;
}

__host__ __device__ __forceinline__ int sur_cell(double rho, double phi, double q)
{
    if (!(rho >= SUR_RHO_LO && rho < SUR_RHO_HI && q >= SUR_Q_LO && q < 1.0)) return -1;
    // (multiplications by the cells per unit: no FP64 divide per ray)
    int ir = (int)((rho - SUR_RHO_LO) * (SUR_NB_RHO / (SUR_RHO_HI - SUR_RHO_LO)));
    int ip = (int)(phi * (SUR_NB_PHI / (0.5 * M_PI)));
    int iq = (int)((q - SUR_Q_LO) * (SUR_NB_Q / (1.0 - SUR_Q_LO)));
    ir = ir < 0 ? 0 : (ir >= SUR_NB_RHO ? SUR_NB_RHO - 1 : ir);
    ip = ip < 0 ? 0 : (ip >= SUR_NB_PHI ? SUR_NB_PHI - 1 : ip);
    iq = iq < 0 ? 0 : (iq >= SUR_NB_Q ? SUR_NB_Q - 1 : iq);
    return (ir * SUR_NB_PHI + ip) * SUR_NB_Q + iq;
}

// X = x/rs, Y = y/rs in the lens frame (either sign), q < 1
__device__ __forceinline__ SurIn sur_inputs(double X, double Y, double q)
{
    SurIn s;
    const double ax = fabs(X), ay = fabs(Y);
    const double R2 = ax * ax + ay * ay;
    const double rho = 0.5 * log(R2);
    const double phi = atan2(ay, ax);
    const double hr = 0.5 * (SUR_RHO_HI - SUR_RHO_LO), mr = 0.5 * (SUR_RHO_HI + SUR_RHO_LO);
    const double hq = 0.5 * (1.0 - SUR_Q_LO), mq = 0.5 * (1.0 + SUR_Q_LO);
    // outside the domain (or at the centre) the network still runs on clamped
    // inputs, but the ray takes the quadrature
    s.f0 = (float)fmin(fmax((rho - mr) / hr, -2.0), 2.0);
    s.f1 = (float)(phi * (4.0 / M_PI) - 1.0);
    s.f2 = (float)fmin(fmax((q - mq) * (1.0 / hq), -2.0), 2.0);
    s.bin = sur_cell(rho, phi, q);
    s.B = nfw_kapavg_spherical_rsq(1.0, 1.0, q * ax * ax + ay * ay / q);
    s.B_rel = 0.0;
    return s;
}

__device__ __forceinline__ uint64_t sur_hash(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ double sur_unif(uint64_t seed, uint64_t i, int j)
{
    return (double)(sur_hash(seed * 0x100000001B3ull + i * 4 + j) >> 11) * (1.0 / 9007199254740992.0);
}

// One sample at (rho, phi, q): network inputs, the quadrature's G_0, G_1
// (tolerance 1e-10) and the baseline.
__device__ void sur_point(double rho, double phi, double q, float* f, double* G, double* B)
{
    const double R = exp(rho);
    const double X = R * cos(phi), Y = R * sin(phi);
    LensRec L;
    memset(&L, 0, sizeof(L));
    L.type = QLP_LENS_NFW;
    L.ks = 1.0; L.rs = 1.0; L.q = q; L.qsq = q * q; L.epsilon = 1 - L.qsq;
    double I0, I1;
    nfw_integrals(L, X * X, Y * Y, SUR_TARGET_TOL, I0, I1);
    const double sqe = sqrt(1 - L.epsilon);
    G[0] = sqe * I0;
    G[1] = sqe * I1;
    const SurIn s = sur_inputs(X, Y, q);
    f[0] = s.f0; f[1] = s.f1; f[2] = s.f2;
    *B = s.B;
}

// Samples: mode 0 uniform over the domain, mode 1 SUR_VAL_PER_BIN jittered
// points per error-bound cell (sample i belongs to cell i / SUR_VAL_PER_BIN).
// Writes the inputs X [n][3], the raw targets T [n][2] (s_0, s_1), when G is
// not null G [n][2], the baselines Bv [n] and q [n], and when Wt is not null
// the squared dimensionless deflection (the training weight before scaling).
__global__ void k_sur_samples(int n, uint64_t seed, int mode, float* __restrict__ Xf, float* __restrict__ Tf,
                              double* __restrict__ G, double* __restrict__ Bv, double* __restrict__ Qv,
                              float* __restrict__ Wt)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double rho, phi, q;
        const double u0 = sur_unif(seed, i, 0), u1 = sur_unif(seed, i, 1), u2 = sur_unif(seed, i, 2);
        if (mode == 0) {
            rho = SUR_RHO_LO + u0 * (SUR_RHO_HI - SUR_RHO_LO);
            phi = u1 * 0.5 * M_PI;
            q = SUR_Q_LO + u2 * (1.0 - SUR_Q_LO);
        } else {
            const int b = i / SUR_VAL_PER_BIN;
            const int iq = b % SUR_NB_Q, ip = (b / SUR_NB_Q) % SUR_NB_PHI, ir = b / (SUR_NB_Q * SUR_NB_PHI);
            rho = SUR_RHO_LO + (ir + u0) * (SUR_RHO_HI - SUR_RHO_LO) / SUR_NB_RHO;
            phi = (ip + u1) * 0.5 * M_PI / SUR_NB_PHI;
            q = SUR_Q_LO + (iq + u2) * (1.0 - SUR_Q_LO) / SUR_NB_Q;
        }
        if (q >= 1.0) q = 0.999999;
        float f[3];
        double g[2], b;
        sur_point(rho, phi, q, f, g, &b);
        Xf[3 * (size_t)i] = f[0]; Xf[3 * (size_t)i + 1] = f[1]; Xf[3 * (size_t)i + 2] = f[2];
        Tf[2 * (size_t)i] = (float)(log(g[0] / b) / (1.0 - q));
        Tf[2 * (size_t)i + 1] = (float)(log(g[1] / b) / (1.0 - q));
        if (G) { G[2 * (size_t)i] = g[0]; G[2 * (size_t)i + 1] = g[1]; Bv[i] = b; Qv[i] = q; }
        if (Wt) {   // |alpha| / (ks rs) squared: where an error in G matters most
            const double R = exp(rho), c = cos(phi), sn = sin(phi);
            Wt[i] = (float)(R * R * (g[0] * g[0] * c * c + g[1] * g[1] * sn * sn));
        }
    }
}

// given points (rho, phi, q): inputs, quadrature G and baselines
__global__ void k_sur_points(int n, const double* __restrict__ rpq, float* __restrict__ Xf, double* __restrict__ G,
                             double* __restrict__ Bv)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double q = rpq[3 * (size_t)i + 2];
        if (q >= 1.0) q = 0.999999;
        float f[3];
        double g[2], b;
        sur_point(rpq[3 * (size_t)i], rpq[3 * (size_t)i + 1], q, f, g, &b);
        Xf[3 * (size_t)i] = f[0]; Xf[3 * (size_t)i + 1] = f[1]; Xf[3 * (size_t)i + 2] = f[2];
        G[2 * (size_t)i] = g[0]; G[2 * (size_t)i + 1] = g[1];
        Bv[i] = b;
    }
}

// targets to zero mean, unit variance per output; weights to wfloor + wscale w
__global__ void k_sur_affine(int n, float* __restrict__ T, float mu0, float mu1, float is0, float is1,
                             float* __restrict__ Wt, float wscale, float wfloor)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        T[2 * (size_t)i] = (T[2 * (size_t)i] - mu0) * is0;
        T[2 * (size_t)i + 1] = (T[2 * (size_t)i + 1] - mu1) * is1;
        Wt[i] = wfloor + Wt[i] * wscale;
    }
}

// ---------------------------------------------------------------------------
// training: FP32 SIMT GEMM C[M][N] = op(A)[M][K] op(B)[K][N] with generic
// strides, 64x64 tiles, 256 threads, 4x4 outputs per thread, and epilogues
//   EPI_STORE      C = acc
//   EPI_TANH       C = tanh(acc + bias)       hidden layer, forward
//   EPI_BIAS       C = acc + bias             output layer, forward
//   EPI_DTANH      C = acc * (1 - Aux^2)      backward through tanh
// gridDim.z > 1 splits K: split z writes C + z * M * N.
// ---------------------------------------------------------------------------
#define EPI_STORE 0
#define EPI_TANH 1
#define EPI_BIAS 2
#define EPI_DTANH 3

template <int EPI>
__global__ void __launch_bounds__(256) k_sur_gemm(int M, int N, int K, const float* __restrict__ A, int a_rs, int a_cs,
                                                  const float* __restrict__ B, int b_rs, int b_cs,
                                                  float* __restrict__ C, const float* __restrict__ bias,
                                                  const float* __restrict__ aux)
{
    __shared__ float As[16][64 + 4];
    __shared__ float Bs[16][64 + 4];
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int ksplit = (K + gridDim.z - 1) / gridDim.z;
    const int kbeg = blockIdx.z * ksplit, kend = min(K, kbeg + ksplit);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4] = {};
    for (int k0 = kbeg; k0 < kend; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            const int kk = e >> 6, mm = e & 63;
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < kend) ? A[(size_t)gm * a_rs + (size_t)gk * a_cs] : 0.f;
            const int gn = n0 + mm;
            Bs[kk][mm] = (gn < N && gk < kend) ? B[(size_t)gk * b_rs + (size_t)gn * b_cs] : 0.f;
        }
        __syncthreads();
        #pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            float a[4], b[4];
            #pragma unroll
            for (int u = 0; u < 4; u++) { a[u] = As[kk][ty * 4 + u]; b[u] = Bs[kk][tx * 4 + u]; }
            #pragma unroll
            for (int u = 0; u < 4; u++)
                #pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] = __fmaf_rn(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
    float* Cz = C + (size_t)blockIdx.z * M * N;
    #pragma unroll
    for (int u = 0; u < 4; u++)
        #pragma unroll
        for (int v = 0; v < 4; v++) {
            const int gm = m0 + ty * 4 + u, gn = n0 + tx * 4 + v;
            if (gm >= M || gn >= N) continue;
            float x = acc[u][v];
            if (EPI == EPI_TANH) x = sur_tanh(x + bias[gn]);
            else if (EPI == EPI_BIAS) x = x + bias[gn];
            else if (EPI == EPI_DTANH) { const float a = aux[(size_t)gm * N + gn]; x = x * (1.f - a * a); }
            Cz[(size_t)gm * N + gn] = x;
        }
}

// out[i] = sum_z part[z][i] in order (deterministic split-K reduction)
__global__ void k_sur_reduce(int n, int nz, const float* __restrict__ part, float* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int z = 0; z < nz; z++) s += part[(size_t)z * n + i];
        out[i] = s;
    }
}

// bias gradients: column sums of D [rows][n], one block per column, fixed order
__global__ void __launch_bounds__(256) k_sur_colsum(int rows, int n, const float* __restrict__ D, float* __restrict__ out)
{
    __shared__ float red[256];
    const int c = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) s += D[(size_t)r * n + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

// output-layer gradient dL/dy = 2 w (y - t) / batch (w = 1 without weights);
// per-block partial sums of w (y - t)^2
__global__ void __launch_bounds__(256) k_sur_mse(int batch, const float* __restrict__ Y, const float* __restrict__ T,
                                                 const float* __restrict__ W, float* __restrict__ dY,
                                                 double* __restrict__ part)
{
    __shared__ double red[256];
    double s = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * batch; i += gridDim.x * blockDim.x) {
        const float w = W ? W[i >> 1] : 1.f;
        const float e = Y[i] - T[i];
        dY[i] = 2.f * w * e / batch;
        s += (double)w * e * e;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_sur_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                           float* __restrict__ m2, float lr, float b1, float b2, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = b;
        p[i] -= lr * (a * c1) / (sqrtf(b * c2) + 1e-8f);
    }
}

// ---------------------------------------------------------------------------
// inference on the tensor cores
// ---------------------------------------------------------------------------
// Layers 1-3 (128 x 128) run as tcgen05 kind::f16 MMAs -- M = 128 rays,
// N = 128 outputs, K = 128 inputs -- with both operands split into an F16
// high part and an F16 remainder (hi*hi + hi*lo + lo*hi: ~22 significant
// bits, as 3xTF32, at the F16 tensor rate).  The activations (tanh, |h| <= 1)
// enter scaled by 2^SUR_ACT_EXP and each layer's weights by 2^s_l (largest
// entry near 2^14), so both parts stay in F16's normal range; the epilogue
// multiplies the accumulator by 2^-(SUR_ACT_EXP + s_l) (exact), times the
// factor 2 log2(e) of tanh's base-2 form.
//   B (weights): resident in shared memory for the kernel's life -- the F16
//     image [3 layers][hi, lo][2 K blocks][128 output rows][64 inputs] in the
//     128-byte swizzled K-major layout the MMA descriptor reads (192 KB),
//     built once after training (k_sur_prep) and copied in by bulk copies;
//   A (activations): in TMEM, two F16 per 32-bit column (even k in the low
//     half), hi and lo 64 columns each;
//   D: 128 FP32 columns of TMEM.
// Persistent CTAs, one per SM, two ray groups of 256 threads (8 warps): each
// owns 256 TMEM columns (D | A_hi | A_lo) and runs 128-ray groups of its
// own, so one group's epilogues and FP64 lens work overlap the other's MMAs.
// Two threads share a ray (warps w and w + 4 of a group read the same TMEM
// lane quadrant): each runs the epilogues of half the hidden units, which
// doubles the warps on the SIMT-bound epilogues (tanh, the F16 split, TMEM
// loads and stores) for the same TMEM.
#define SUR_SMALL (3 * SUR_H + 4 * SUR_H + 2 * SUR_H + 2 + 3)   // W0, b0..b3, W4, b4, unscale of layers 1..3
#define SUR_OPB (SUR_H * SUR_H * 2)                              // one F16 part of one layer: 32 KB
#define SUR_WIMG (3 * 2 * SUR_OPB)                               // 192 KB
#define SUR_ACT_EXP 14
#define SUR_SMEM (SUR_WIMG + 1024 + SUR_SMALL * 4)
#define SUR_THREADS 512
#define SUR_RG 256                                               // threads of a ray group

__device__ __forceinline__ void mma_f16_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                           uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
        "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tmem_st_16cols_u(uint32_t taddr, const uint32_t* v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}

__device__ __forceinline__ void tmem_st_32cols_u(uint32_t taddr, const uint32_t* v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]),
        "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]),
        "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}

// 64 FP32 columns of the warp's 32 TMEM lanes in one load (one wait for all
// of them: the epilogue of a thread's 64 hidden units waits once per layer)
__device__ __forceinline__ void tmem_ld_64cols(uint32_t taddr, float* v)
{
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    #pragma unroll
    for (int i = 0; i < 64; i++) v[i] = __uint_as_float(r[i]);
}

// (a, b) -> packed F16 high parts and packed F16 remainders, a in the low half
__device__ __forceinline__ void f16_split2(float a, float b, uint32_t& hi, uint32_t& lo)
{
    const __half2 h = __floats2half2_rn(a, b);              // a in the low half
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// named barrier of one ray group (ids 1, 2; 0 is __syncthreads)
__device__ __forceinline__ void wg_sync(int wg) { asm volatile("bar.sync %0, 256;" ::"r"(1 + wg) : "memory"); }

// true on every thread of the ray group if p holds on any of them
__device__ __forceinline__ bool wg_any(int wg, bool p)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred pi, po;\n\t"
        "setp.ne.u32 pi, %1, 0;\n\t"
        "bar.red.or.pred po, %2, 256, pi;\n\t"
        "selp.u32 %0, 1, 0, po;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)p), "r"(1 + wg)
        : "memory");
    return r != 0;
}

// Per-ray-group state of the tensor-core MLP.
struct SurWG {
    const unsigned char* w;   // weight image in shared memory (1024-aligned)
    const float* small;       // SUR_SMALL floats in shared memory
    uint64_t* mma_bar;        // this group's MMA-completion barrier
    volatile int* abort;
    float2* xo;               // this group's [2 halves][128 rays] partial outputs
    float4* xin;              // this group's [128 rays] network inputs (the first half's, for the second)
    uint32_t tmem;            // this group's columns: D [0,128), A_hi [128,192), A_lo [192,256)
    uint32_t phase;           // completed layers (mbarrier parity)
    int wg;                   // ray group
    int half;                 // hidden units [64 half, 64 half + 64) of the thread's ray
};

// The 256 threads of a ray group call this together, two per ray (row
// threadIdx.x % 128), each with its ray's inputs; both return the network's
// two outputs.  ok is cleared if a bounded wait ran out.
__device__ void sur_mlp_wg(SurWG& S, float f0, float f1, float f2, float& t0, float& t1, bool& ok)
{
    const int tid = threadIdx.x & 127, warp = tid >> 5;
    const uint32_t row = S.tmem + (((uint32_t)(warp * 32)) << 16);   // this warp's 32 lanes
    const int u0 = 64 * S.half;                                        // this thread's hidden units
    const float* W0 = S.small;
    const float* bb = S.small + 3 * SUR_H;          // b0, b1, b2, b3
    const float* W4 = S.small + 7 * SUR_H;
    const float* b4 = S.small + 9 * SUR_H;
    const float* unscale = S.small + 9 * SUR_H + 2;
    const float ascale = (float)(1 << SUR_ACT_EXP);
    // layer 0 on the CUDA cores, straight into TMEM as the next A operand
    #pragma unroll 1
    for (int c = u0; c < u0 + 64; c += 32) {
        uint32_t hi[16], lo[16];
        #pragma unroll
        for (int j = 0; j < 16; j++) {
            const int u = c + 2 * j;          // a pair of units: 8-byte loads of their weights and biases
            const float2 w0 = *reinterpret_cast<const float2*>(W0 + u);
            const float2 w1 = *reinterpret_cast<const float2*>(W0 + SUR_H + u);
            const float2 w2 = *reinterpret_cast<const float2*>(W0 + 2 * SUR_H + u);
            const float2 b0 = *reinterpret_cast<const float2*>(bb + u);
            const float h0 = sur_tanh_a(__fmaf_rn(w2.x, f2, __fmaf_rn(w1.x, f1, __fmaf_rn(w0.x, f0, b0.x))), ascale);
            const float h1 = sur_tanh_a(__fmaf_rn(w2.y, f2, __fmaf_rn(w1.y, f1, __fmaf_rn(w0.y, f0, b0.y))), ascale);
            f16_split2(h0, h1, hi[j], lo[j]);
        }
        tmem_st_16cols_u(row + 128 + c / 2, hi);
        tmem_st_16cols_u(row + 192 + c / 2, lo);
    }
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    float o0 = 0.f, o1 = 0.f;
    for (int l = 1; l <= 3; l++) {
        tc_fence_before();
        wg_sync(S.wg);
        tc_fence_after();
        if ((threadIdx.x & (SUR_RG - 1)) == 0) {
            const uint32_t idesc = idesc_f16_128x128();
            const unsigned char* wl = S.w + (size_t)(l - 1) * 2 * SUR_OPB;
            #pragma unroll
            for (int kb = 0; kb < 2; kb++) {
                const uint64_t b_hi = sdesc_sw128(smem_u32(wl + kb * (SUR_OPB / 2)));
                const uint64_t b_lo = sdesc_sw128(smem_u32(wl + SUR_OPB + kb * (SUR_OPB / 2)));
                #pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    // 16 inputs per MMA: 32 bytes of a weight row, 8 TMEM columns of A
                    const uint32_t ka = (uint32_t)(kb * 32 + kk * 8);
                    const uint64_t off = (uint64_t)((kk * 32) >> 4);
                    mma_f16_ta(S.tmem, S.tmem + 128 + ka, b_hi + off, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
                    mma_f16_ta(S.tmem, S.tmem + 128 + ka, b_lo + off, idesc, 1u);
                    mma_f16_ta(S.tmem, S.tmem + 192 + ka, b_hi + off, idesc, 1u);
                }
            }
            mma_commit(S.mma_bar);
        }
        __syncwarp();
        const bool done = mbar_wait_bounded(S.mma_bar, S.phase & 1, S.abort, false);
        tc_fence_after();
        S.phase++;
        if (!done || *S.abort) ok = false;
        // epilogue: unscale, bias, tanh; layers 1-2 back into TMEM as A, layer 3 into the output layer
        const float us = unscale[l - 1];
        const float* bl = bb + l * SUR_H;
        float va[64];
        tmem_ld_64cols(row + u0, va);
        const float sc = (l < 3) ? ascale : 1.0f;          // layers 1-2 feed the next MMA, scaled
        #pragma unroll
        for (int cc = 0; cc < 64; cc += 32) {
            const int c = u0 + cc;
            float* v = va + cc;
            #pragma unroll
            for (int j = 0; j < 32; j += 4) {
                const float4 b4v = *reinterpret_cast<const float4*>(bl + c + j);
                v[j] = sur_tanh_a(__fmaf_rn(v[j], us, b4v.x), sc);
                v[j + 1] = sur_tanh_a(__fmaf_rn(v[j + 1], us, b4v.y), sc);
                v[j + 2] = sur_tanh_a(__fmaf_rn(v[j + 2], us, b4v.z), sc);
                v[j + 3] = sur_tanh_a(__fmaf_rn(v[j + 3], us, b4v.w), sc);
            }
            if (l < 3) {
                uint32_t hi[16], lo[16];
                #pragma unroll
                for (int j = 0; j < 16; j++) f16_split2(v[2 * j], v[2 * j + 1], hi[j], lo[j]);
                tmem_st_16cols_u(row + 128 + c / 2, hi);
                tmem_st_16cols_u(row + 192 + c / 2, lo);
            } else {
                #pragma unroll
                for (int j = 0; j < 32; j++) {
                    const float2 w = *reinterpret_cast<const float2*>(W4 + 2 * (c + j));
                    o0 = __fmaf_rn(v[j], w.x, o0);
                    o1 = __fmaf_rn(v[j], w.y, o1);
                }
            }
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    // the two halves' output sums, added in the same order on both threads
    S.xo[S.half * 128 + tid] = make_float2(o0, o1);
    wg_sync(S.wg);
    const float2 a = S.xo[tid], b = S.xo[128 + tid];
    t0 = (a.x + b.x) + b4[0];
    t1 = (a.y + b.y) + b4[1];
}

// CTA set-up of the persistent MLP kernels (all SUR_THREADS threads): the
// weight image into shared memory by bulk copies, the small parameters, the
// barriers and 512 TMEM columns; returns false if the weights did not arrive
// within the bounded wait.
__device__ __forceinline__ bool sur_cta_begin(SurWG& S, unsigned char* smem_raw, const unsigned char* __restrict__ wimg,
                                              const float* __restrict__ small_g, uint64_t* w_bar, uint64_t* mma_bar,
                                              uint32_t* tmem_slot, volatile int* abort, float2* xo)
{
    unsigned char* w = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float* small = reinterpret_cast<float*>(w + SUR_WIMG);
    const int wg = threadIdx.x / SUR_RG;
    if (threadIdx.x == 0) {
        mbar_init(w_bar, 1);
        mbar_init(&mma_bar[0], 1);
        mbar_init(&mma_bar[1], 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(w_bar, SUR_WIMG);
        for (int k = 0; k < 6; k++)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(w + k * SUR_OPB)),
                "l"(wimg + (size_t)k * SUR_OPB), "r"((uint32_t)SUR_OPB), "r"(smem_u32(w_bar))
                : "memory");
    }
    for (int i = threadIdx.x; i < SUR_SMALL; i += blockDim.x) small[i] = small_g[i];
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    S.w = w;
    S.small = small;
    S.mma_bar = &mma_bar[wg];
    S.abort = abort;
    S.tmem = *tmem_slot + (uint32_t)(wg * 256);
    S.phase = 0;
    S.wg = wg;
    S.half = (threadIdx.x >> 7) & 1;
    S.xo = xo + wg * 256;
    S.xin = reinterpret_cast<float4*>(xo + 2 * 256) + wg * 128;
    return mbar_wait_bounded(w_bar, 0, abort, false);
}

__device__ __forceinline__ void sur_cta_end(const SurWG& S, uint32_t tmem_base)
{
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512) : "memory");
    }
}

// Batch inference for the error-bound table and the tests: T[i] = net(X[i]),
// persistent over 128-point groups.
__global__ void __launch_bounds__(SUR_THREADS, 1) k_sur_infer(int n, const float* __restrict__ X,
                                                              float* __restrict__ T,
                                                              const unsigned char* __restrict__ wimg,
                                                              const float* __restrict__ small_g, int* status)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t w_bar, mma_bar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    __shared__ float2 xo[2 * 256 + 2 * 2 * 128];   // partial outputs, then the inputs
    SurWG S;
    bool ok = sur_cta_begin(S, smem_raw, wimg, small_g, &w_bar, mma_bar, &tmem_slot, &abort_flag, xo);
    const int tid = threadIdx.x & 127;
    for (int grp = blockIdx.x * 2 + S.wg; grp * 128 < n; grp += gridDim.x * 2) {
        if (wg_any(S.wg, !ok || abort_flag)) { ok = false; break; }
        const int i = grp * 128 + tid;
        float f0 = 0.f, f1 = 0.f, f2 = 0.f;
        if (i < n) { f0 = X[3 * (size_t)i]; f1 = X[3 * (size_t)i + 1]; f2 = X[3 * (size_t)i + 2]; }
        float t0, t1;
        sur_mlp_wg(S, f0, f1, f2, t0, t1, ok);
        if (i < n && S.half == 0) { T[2 * (size_t)i] = t0; T[2 * (size_t)i + 1] = t1; }
    }
    if (!ok && tid == 0) atomicExch(status, QLP_ERR_TIMEOUT);
    sur_cta_end(S, tmem_slot);
}

// Ray shooting with NFW lenses on the surrogate: k_raytrace's lens equation
// (QLens::find_sourcept, lenscalc.cpp:81-113), persistent over 128-ray groups,
// one group per warpgroup at a time.  At every NFW lens with q < 1 the 128
// threads of the warpgroup run the network together (unless no ray of the
// group can pass the gate, then none does); a ray whose bound exceeds
// `thresh` (or whose inputs leave the domain) takes the quadrature instead --
// right here, or, for the lens `defer_lens` (the only NFW lens, on the last
// plane), later in k_nfw_fallback at full occupancy (its lens-frame position
// is queued and its contribution left out here).  out->pad counts the
// fallbacks.
// Per-CTA tables of the ray shooting: per-lens reciprocals (a multiply per
// ray instead of an FP64 divide), the constants of a core-free SIE, and the
// sub-pixel fractions.  Any threads fill them; a barrier precedes their use.
struct SurTabs {
    double inv_rs[QLP_MAX_LENSES], inv_q[QLP_MAX_LENSES];
    double sie_u[QLP_MAX_LENSES], sie_pre[QLP_MAX_LENSES];
    double frac_u[SUBPIX_TAB], frac_1mu[SUBPIX_TAB];
    // an NFW lens's constants in FP32 for the surrogate's per-ray arithmetic:
    // 1/rs, q, 1/q, ks, cos and sin of its angle, and the network's q feature
    float f_inv_rs[QLP_MAX_LENSES], f_q[QLP_MAX_LENSES], f_inv_q[QLP_MAX_LENSES], f_ks[QLP_MAX_LENSES];
    float f_cos[QLP_MAX_LENSES], f_sin[QLP_MAX_LENSES], f_feat_q[QLP_MAX_LENSES];
    int qbin[QLP_MAX_LENSES];    // the error cell's q index (sur_cell's), -1 outside the trained q range
};

// sur_cell from the network's FP32 inputs and the lens's q index (the cell
// indices in log R and phi by the same multiplications in FP32: a ray within
// rounding of a cell boundary may take the neighbouring cell's bound, both
// estimated from points on either side of it)
__device__ __forceinline__ int sur_cell_f(float rho, float phi, int qbin)
{
    if (qbin < 0 || !(rho >= (float)SUR_RHO_LO && rho < (float)SUR_RHO_HI)) return -1;
    int ir = (int)((rho - (float)SUR_RHO_LO) * (float)(SUR_NB_RHO / (SUR_RHO_HI - SUR_RHO_LO)));
    int ip = (int)(phi * (float)(SUR_NB_PHI / (0.5 * M_PI)));
    ir = ir < 0 ? 0 : (ir >= SUR_NB_RHO ? SUR_NB_RHO - 1 : ir);
    ip = ip < 0 ? 0 : (ip >= SUR_NB_PHI ? SUR_NB_PHI - 1 : ip);
    return (ir * SUR_NB_PHI + ip) * SUR_NB_Q + qbin;
}

__device__ __forceinline__ void sur_tabs_fill(const EvalParams* __restrict__ ep, int nsplit, SurTabs& T)
{
    if (threadIdx.x < QLP_MAX_LENSES && threadIdx.x < ep->lm.nlens) {
        const LensRec& L = ep->lm.lens[threadIdx.x];
        T.inv_rs[threadIdx.x] = (L.type == QLP_LENS_NFW) ? 1.0 / L.rs : 0.0;
        T.inv_q[threadIdx.x] = (L.type == QLP_LENS_NFW) ? 1.0 / L.q : 0.0;
        // SIE without core (sple_deflection kind 1, s = 0)
        const bool sie0 = L.type == QLP_LENS_SPLE && L.kind == 1 && L.sprime == 0.0 && L.ssq == 0.0;
        T.sie_u[threadIdx.x] = sie0 ? sqrt(1 - L.qsq) : 0.0;
        T.sie_pre[threadIdx.x] = sie0 ? L.bprime * L.q / sqrt(1 - L.qsq) : 0.0;
        const bool nfw = L.type == QLP_LENS_NFW;
        T.f_inv_rs[threadIdx.x] = nfw ? (float)(1.0 / L.rs) : 0.f;
        T.f_q[threadIdx.x] = (float)L.q;
        T.f_inv_q[threadIdx.x] = nfw ? (float)(1.0 / L.q) : 0.f;
        T.f_ks[threadIdx.x] = (float)L.ks;
        T.f_cos[threadIdx.x] = (float)L.costheta;
        T.f_sin[threadIdx.x] = (float)L.sintheta;
        const double hq = 0.5 * (1.0 - SUR_Q_LO), mq = 0.5 * (1.0 + SUR_Q_LO);
        T.f_feat_q[threadIdx.x] = (float)fmin(fmax((L.q - mq) * (1.0 / hq), -2.0), 2.0);
        int iq = -1;
        if (L.q >= SUR_Q_LO && L.q < 1.0) {
            iq = (int)((L.q - SUR_Q_LO) * (SUR_NB_Q / (1.0 - SUR_Q_LO)));
            iq = iq < 0 ? 0 : (iq >= SUR_NB_Q ? SUR_NB_Q - 1 : iq);
        }
        T.qbin[threadIdx.x] = iq;
    }
    subpix_table(nsplit, T.frac_u, T.frac_1mu);
}

// sub-pixel t's centre
__device__ __forceinline__ void sur_ray_pos(const StaticData& sd, const SurTabs& T, int t, double& px, double& py)
{
    const int ns = sd.nsplit, nsub = sd.nsub;
    const int m = t / nsub, k = t - m * nsub;
    const int pix = sd.mpix[m];
    const int i = pix / sd.ny, j = pix - i * sd.ny;
    const int ii = k / ns, jj = k - ii * ns;
    subpix_centre(sd, ns, ii, jj, i, j, T.frac_u, T.frac_1mu, px, py);
}

// SPLE_Lens::deflection_elliptical_iso with s = 0 (T.sie_u[k] != 0): both
// components share the reciprocal u / psi
__device__ __forceinline__ void sur_sie0(const LensRec& L, const SurTabs& T, int k, double xi, double yi,
                                         double& ax, double& ay)
{
    double x = xi - L.xc, y = yi - L.yc;
    const bool rot = (L.sintheta != 0);
    if (rot) {
        const double xp = x * L.costheta + y * L.sintheta;
        y = -x * L.sintheta + y * L.costheta;
        x = xp;
    }
    const double r = T.sie_u[k] / sqrt(L.qsq * x * x + y * y);
    double bx = T.sie_pre[k] * atan(x * r), by = T.sie_pre[k] * atanh(y * r);
    if (rot) {
        const double xp = bx * L.costheta - by * L.sintheta;
        by = bx * L.sintheta + by * L.costheta;
        bx = xp;
    }
    ax = bx; ay = by;
}

// The deflection of NFW lens k at (xi, yi) on its plane through the
// surrogate, for the 128 rays of a warpgroup (every thread calls, converged;
// `valid` false for padding rays).  LensProfile::deflection's shift, rotate,
// deflect, rotate back.  A ray that fails the gate takes the quadrature
// inline, or, for the deferred lens, is queued for k_nfw_fallback (deflection
// 0 here).  Adds the ray's error bound to eps (twice the plane factor times
// |alpha| times the relative bound) and counts fallbacks in fb.
struct SurRayOut {
    int* fb_count; int* fb_ray; double* fb_xy;
};

// Relative error allowance of the FP32 arithmetic around the network
// (inputs, B, G, alpha and its rotation, each within a few ulp: well below
// 1e-6), added to every surrogate ray's bound
#define SUR_F32_REL 2e-6f

__device__ __forceinline__ void sur_nfw(SurWG& S, bool& ok, const LensRec& L, int k, const SurTabs& T,
                                        const float* __restrict__ bound, double thresh, double zabs, bool valid,
                                        int t, int defer_lens, const SurRayOut& q, int& fb, double& eps,
                                        double xi, double yi, double& ax, double& ay)
{
    // the per-ray work is the first half's; the second half takes the
    // network's inputs from shared memory (after the group's reduction
    // below).  The lens-frame position is formed in FP64 (a difference of
    // nearby coordinates), everything after it in FP32: the network's own
    // error, bounded per cell at 1e-5 and more, dwarfs FP32 rounding, and
    // SUR_F32_REL covers it in the bound.
    const int tid = threadIdx.x & 127;
    const bool first = S.half == 0;
    double x = 0, y = 0;
    float xf = 0.f, yf = 0.f, bnd = 0.f, B = 0.f;
    bool rot = false, centre = false, inb = false, maybe = false;
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    const float thr = (float)thresh;
    if (first) {
        x = xi - L.xc; y = yi - L.yc;
        rot = (L.sintheta != 0);
        if (rot) {
            const double xp = x * L.costheta + y * L.sintheta;
            y = -x * L.sintheta + y * L.costheta;
            x = xp;
        }
        xf = (float)x; yf = (float)y;
        centre = (fabsf(xf) < 1e-14f) && (fabsf(yf) < 1e-14f);
        // the network's inputs (log R, polar angle, q), its error cell, and
        // the baseline B at xi^2 = q X^2 + Y^2 / q
        const float Xa = fabsf(xf * T.f_inv_rs[k]), Ya = fabsf(yf * T.f_inv_rs[k]);
        const float rho = 0.5f * __logf(__fmaf_rn(Xa, Xa, Ya * Ya));
        const float phi = atan2f(Ya, Xa);
        const float hr = (float)(0.5 * (SUR_RHO_HI - SUR_RHO_LO)), mr = (float)(0.5 * (SUR_RHO_HI + SUR_RHO_LO));
        f0 = fminf(fmaxf((rho - mr) / hr, -2.0f), 2.0f);
        f1 = phi * (float)(4.0 / M_PI) - 1.0f;
        f2 = T.f_feat_q[k];
        const int bin = sur_cell_f(rho, phi, T.qbin[k]);
        inb = bin >= 0;
        const float xi2 = T.f_q[k] * Xa * Xa + Ya * Ya * T.f_inv_q[k];
        float brel = 0.f;
        if (xi2 >= (float)SUR_B32_MIN) {
            B = sur_B32(xi2);
            brel = (float)SUR_B32_REL;
        } else {                                   // small radius: the FP64 form (its series cancels)
            const double Xd = x * T.inv_rs[k], Yd = y * T.inv_rs[k];
            B = (float)nfw_kapavg_spherical_rsq(1.0, 1.0, L.q * Xd * Xd + Yd * Yd * T.inv_q[k]);
        }
        // the cell's bound on the relative error of G, plus B's and the FP32 arithmetic's
        bnd = inb ? bound[bin] + brel + SUR_F32_REL : 0.f;
        // before the network: |alpha| ~ ks B |(x, y)| (G is within a few tens of
        // percent of B), so a group none of whose rays can pass the gate skips
        // the network and sends every ray to the quadrature (squares compared)
        const float gb = T.f_ks[k] * B * bnd;
        maybe = valid && !centre && inb && gb * gb * (xf * xf + yf * yf) <= 2.25f * thr * thr;
        S.xin[tid] = make_float4(f0, f1, f2, 0.f);
    }
    float bxf = 0.f, byf = 0.f;
    bool use = false;
    if (wg_any(S.wg, maybe)) {
        if (!first) {
            const float4 v = S.xin[tid];
            f0 = v.x; f1 = v.y; f2 = v.z;
        }
        float t0, t1;
        sur_mlp_wg(S, f0, f1, f2, t0, t1, ok);
        if (first) {
            const float oq = 1.0f - T.f_q[k];
            const float kb = T.f_ks[k] * B;
            bxf = xf * (kb * expf(oq * t0));
            byf = yf * (kb * expf(oq * t1));
            const float m2 = bxf * bxf + byf * byf;
            use = ok && !centre && inb && m2 * bnd * bnd <= thr * thr;
            // |alpha| rounded up by far more than its error
            if (use) eps += 2.0 * zabs * (double)(sqrtf(m2) * 1.000001f * bnd);
        }
    }
    if (!first) { ax = 0; ay = 0; return; }
    if (use) {
        if (rot) {
            const float xp = bxf * T.f_cos[k] - byf * T.f_sin[k];
            byf = bxf * T.f_sin[k] + byf * T.f_cos[k];
            bxf = xp;
        }
        ax = (double)bxf; ay = (double)byf;
        return;
    }
    double bx = 0, by = 0;
    if (valid) {
        fb++;
        if (k == defer_lens) {
            const int e = atomicAdd(q.fb_count, 1);
            q.fb_ray[e] = t;
            q.fb_xy[2 * (size_t)e] = x;
            q.fb_xy[2 * (size_t)e + 1] = y;
        } else {
            nfw_deflection(L, x, y, bx, by);
            if (rot) {
                const double xp = bx * L.costheta - by * L.sintheta;
                by = bx * L.sintheta + by * L.costheta;
                bx = xp;
            }
        }
    }
    ax = bx; ay = by;
}

// PRE = false: the whole lens equation per ray (any model).  PRE = true: the
// model has one NFW lens (defer_lens) on the last plane and k_ray_pre has
// already traced every other lens: spx/spy hold the source points without
// that lens's deflection and nfw_xy the rays' positions on its plane, so
// this kernel runs only the surrogate and subtracts its deflection.
template <bool PRE>
__global__ void __launch_bounds__(SUR_THREADS, 1) k_raytrace_sur(StaticData sd_, const EvalParams* __restrict__ ep,
                                                                 double* __restrict__ spx, double* __restrict__ spy,
                                                                 const double* __restrict__ nfw_xy,
                                                                 const unsigned char* __restrict__ wimg,
                                                                 const float* __restrict__ small_g,
                                                                 const float* __restrict__ bound, double thresh,
                                                                 int defer_lens, SurRayOut q,
                                                                 float* __restrict__ sur_eps, GridState* gs,
                                                                 EvalOut* out)
{
    const StaticData sd = eval_shape(sd_);
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t w_bar, mma_bar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    __shared__ __align__(16) LensModel lm;
    __shared__ SurTabs T;
    __shared__ int n_fb;
    __shared__ float2 xo[2 * 256 + 2 * 2 * 128];   // partial outputs, then the inputs
    if ((int)blockIdx.x * 2 * 128 >= sd.n_sub) return;     // launched for the slot's capacity
    {
        const double* src = reinterpret_cast<const double*>(&ep->lm);
        double* dst = reinterpret_cast<double*>(&lm);
        for (int k = threadIdx.x; k < (int)(sizeof(LensModel) / sizeof(double)); k += blockDim.x) dst[k] = src[k];
        if (threadIdx.x == 0) n_fb = 0;
        sur_tabs_fill(ep, sd.nsplit, T);     // (sur_cta_begin's barrier orders these with their readers)
    }
    SurWG S;
    bool ok = sur_cta_begin(S, smem_raw, wimg, small_g, &w_bar, mma_bar, &tmem_slot, &abort_flag, xo);
    const int tid = threadIdx.x & 127;
    int fb = 0;
    for (int grp = blockIdx.x * 2 + S.wg; grp * 128 < sd.n_sub; grp += gridDim.x * 2) {
        if (wg_any(S.wg, !ok || abort_flag)) { ok = false; break; }
        const int t = grp * 128 + tid;
        // both threads of a ray trace it; the first half stores it, queues
        // its fallback and counts it
        const bool valid = t < sd.n_sub && S.half == 0;
        // bound on this ray's source-point error against the plain path:
        // rounding (this unit contracts multiply-adds, and deflections are
        // summed in another order) plus, per surrogate deflection, twice its
        // plane factor times its bound
        double eps = 1e-12;
        if (PRE) {
            const LensRec& L = lm.lens[defer_lens];
            const double z = lm.zfac[L.plane];
            double xi = 0, yi = 0, sx = 0, sy = 0;
            if (valid) {
                xi = nfw_xy[2 * (size_t)t];
                yi = nfw_xy[2 * (size_t)t + 1];
                sx = spx[t];
                sy = spy[t];
            }
            double ax, ay;
            sur_nfw(S, ok, L, defer_lens, T, bound, thresh, fabs(z), valid, t, defer_lens, q, fb, eps, xi, yi,
                    ax, ay);
            if (valid) {
                spx[t] = sx - z * ax;
                spy[t] = sy - z * ay;
                sur_eps[t] = (float)eps;
            }
            continue;
        }
        double px = 0, py = 0;
        if (valid) sur_ray_pos(sd, T, t, px, py);
        double defx = 0, defy = 0;
        double dsx[QLP_MAX_PLANES], dsy[QLP_MAX_PLANES];
        for (int p = 0; p < lm.n_planes; p++) {
            dsx[p] = 0; dsy[p] = 0;
            if (lm.zfac[p] == 0.0) continue;
            double xi = px, yi = py;
            for (int jp = 0; jp < p; jp++) {
                xi -= lm.beta[p - 1][jp] * dsx[jp];
                yi -= lm.beta[p - 1][jp] * dsy[jp];
            }
            for (int k = 0; k < lm.nlens; k++) {
                const LensRec& L = lm.lens[k];
                if (L.plane != p) continue;
                double ax, ay;
                if (L.type == QLP_LENS_NFW && L.q != 1.0)
                    sur_nfw(S, ok, L, k, T, bound, thresh, fabs(lm.zfac[p]), valid, t, defer_lens, q, fb, eps, xi,
                            yi, ax, ay);
                else if (S.half != 0)
                    ax = ay = 0;       // (the second half only joins the network's evaluations)
                else if (T.sie_u[k] != 0.0)
                    sur_sie0(L, T, k, xi, yi, ax, ay);
                else
                    lens_deflection<true>(L, xi, yi, ax, ay);
                dsx[p] += ax; dsy[p] += ay;
            }
            dsx[p] *= lm.zfac[p];
            dsy[p] *= lm.zfac[p];
            defx += dsx[p];
            defy += dsy[p];
        }
        if (valid) {
            spx[t] = px - defx;
            spy[t] = py - defy;
            sur_eps[t] = (float)eps;
        }
    }
    if (fb) atomicAdd(&n_fb, fb);
    sur_cta_end(S, tmem_slot);
    if (threadIdx.x == 0) {
        if (n_fb) atomicAdd(&out->pad, n_fb);
        if (!ok) atomicExch(&gs->status, QLP_ERR_TIMEOUT);
    }
}

// The FP64 part of the rays of a model whose one NFW lens (nfw_lens) sits on
// the last plane: every other lens of every plane, a thread per ray at full
// occupancy (GB300's FP64 pipe needs many warps in flight; the fused kernel
// holds eight per SM).  Writes the source points without the NFW lens's
// deflection and the rays' positions on its plane (nfw_xy) for
// k_raytrace_sur<true>.
__global__ void __launch_bounds__(256) k_ray_pre(StaticData sd_, const EvalParams* __restrict__ ep, int nfw_lens,
                                                 double* __restrict__ spx, double* __restrict__ spy,
                                                 double* __restrict__ nfw_xy)
{
    const StaticData sd = eval_shape(sd_);
    __shared__ __align__(16) LensModel lm;
    __shared__ double rho_tab[QLP_MAX_LENSES * SPLE_RHO_TAB];
    __shared__ SurTabs T;
    {
        const double* src = reinterpret_cast<const double*>(&ep->lm);
        double* dst = reinterpret_cast<double*>(&lm);
        for (int k = threadIdx.x; k < (int)(sizeof(LensModel) / sizeof(double)); k += blockDim.x) dst[k] = src[k];
        sur_tabs_fill(ep, sd.nsplit, T);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < lm.nlens * SPLE_RHO_TAB; e += blockDim.x) {
        const LensRec& L = lm.lens[e / SPLE_RHO_TAB];
        rho_tab[e] = (L.type == QLP_LENS_SPLE && L.kind == 2) ? sple_rho(L, e % SPLE_RHO_TAB + 1) : 0.0;
    }
    __syncthreads();
    const int P = lm.lens[nfw_lens].plane;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < sd.n_sub; t += gridDim.x * blockDim.x) {
        double px, py;
        sur_ray_pos(sd, T, t, px, py);
        double defx = 0, defy = 0, xP = px, yP = py;
        double dsx[QLP_MAX_PLANES], dsy[QLP_MAX_PLANES];
        for (int p = 0; p < lm.n_planes; p++) {
            dsx[p] = 0; dsy[p] = 0;
            if (lm.zfac[p] == 0.0) continue;
            double xi = px, yi = py;
            for (int jp = 0; jp < p; jp++) {
                xi -= lm.beta[p - 1][jp] * dsx[jp];
                yi -= lm.beta[p - 1][jp] * dsy[jp];
            }
            if (p == P) { xP = xi; yP = yi; }
            for (int k = 0; k < lm.nlens; k++) {
                const LensRec& L = lm.lens[k];
                if (L.plane != p || k == nfw_lens) continue;
                double ax, ay;
                if (T.sie_u[k] != 0.0) sur_sie0(L, T, k, xi, yi, ax, ay);
                else lens_deflection<false>(L, xi, yi, ax, ay, rho_tab + k * SPLE_RHO_TAB);
                dsx[p] += ax; dsy[p] += ay;
            }
            dsx[p] *= lm.zfac[p];
            dsy[p] *= lm.zfac[p];
            defx += dsx[p];
            defy += dsy[p];
        }
        spx[t] = px - defx;
        spy[t] = py - defy;
        nfw_xy[2 * (size_t)t] = xP;
        nfw_xy[2 * (size_t)t + 1] = yP;
    }
}

// The queued fallbacks of k_raytrace_sur: quadrature deflection of lens
// `lens` at the queued lens-frame points, rotated back, scaled by its plane's
// factor and subtracted from the rays' source points.
__global__ void k_nfw_fallback(const EvalParams* __restrict__ ep, int lens, const int* __restrict__ fb_count,
                               const int* __restrict__ fb_ray, const double* __restrict__ fb_xy,
                               double* __restrict__ spx, double* __restrict__ spy)
{
    const int n = *fb_count;
    const LensRec& L = ep->lm.lens[lens];
    const double z = ep->lm.zfac[L.plane];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        double bx, by;
        nfw_deflection(L, fb_xy[2 * (size_t)e], fb_xy[2 * (size_t)e + 1], bx, by);
        if (L.sintheta != 0) {
            const double xp = bx * L.costheta - by * L.sintheta;
            by = bx * L.sintheta + by * L.costheta;
            bx = xp;
        }
        const int t = fb_ray[e];
        spx[t] -= z * bx;
        spy[t] -= z * by;
    }
}

// ---------------------------------------------------------------------------
// host side: one trained network per device, shared by every context
// ---------------------------------------------------------------------------
struct SurState {
    bool ready = false;
    float* params = nullptr;          // training layout
    unsigned char* wimg = nullptr;    // SUR_WIMG: layers 1-3 as the MMA's shared-memory image (k_sur_prep)
    float* small = nullptr;           // SUR_SMALL
    float* bound = nullptr;           // SUR_NBINS
    qlp_surrogate_report rep{};
};
static std::mutex g_sur_mu;
static SurState g_sur[64];

// The inference copies: layers 1-3 as the F16 hi/lo image the MMAs read from
// shared memory -- byte offset of weight (out n, in k) of layer l, part h:
// (2 l + h) SUR_OPB + (k / 64) (SUR_OPB / 2) + 128 n + 16 ((k % 64) / 8 XOR n % 8)
// + 2 (k % 8), the 128-byte swizzled K-major layout -- each layer scaled by
// 2^sexp[l]; and the small parameters, with the target normalisation folded
// into the output layer, the unscale factors 2^-(SUR_ACT_EXP + sexp[l]), and
// the factor 2 log2(e) of tanh's base-2 form on W0, the hidden biases and the
// unscale factors.
__global__ void k_sur_prep(const float* __restrict__ p, unsigned char* __restrict__ wimg, float* __restrict__ small,
                           float mu0, float mu1, float sg0, float sg1, int3 sexp)
{
    const int n = 3 * SUR_H * SUR_H;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int l = e / (SUR_H * SUR_H), r = e % (SUR_H * SUR_H), o = r / SUR_H, i = r % SUR_H;
        const int se = (l == 0) ? sexp.x : (l == 1) ? sexp.y : sexp.z;
        const float w = ldexpf(p[SUR_W1 + l * (SUR_H * SUR_H + SUR_H) + i * SUR_H + o], se);
        const __half h = __float2half_rn(w);
        const __half lo = __float2half_rn(w - __half2float(h));
        const size_t off = (size_t)(i / 64) * (SUR_OPB / 2) + (size_t)o * 128 +
                           (size_t)((((i % 64) / 8) ^ (o % 8)) * 16) + (size_t)(i % 8) * 2;
        *reinterpret_cast<__half*>(wimg + (size_t)(2 * l) * SUR_OPB + off) = h;
        *reinterpret_cast<__half*>(wimg + (size_t)(2 * l + 1) * SUR_OPB + off) = lo;
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < SUR_SMALL; e += gridDim.x * blockDim.x) {
        // (W0, the hidden biases and the unscale factors carry the factor
        // 2 log2(e) of tanh(x) = 1 - 2 / (1 + 2^(2 log2(e) x)): the
        // epilogues' FMA yields the exponent directly)
        const float c2 = (float)(2.0 * 1.4426950408889634);
        float v;
        if (e < 3 * SUR_H) v = p[SUR_W0 + e] * c2;
        else if (e < 7 * SUR_H) {
            const int l = (e - 3 * SUR_H) / SUR_H, u = (e - 3 * SUR_H) % SUR_H;
            v = p[SUR_B0 + l * (SUR_H * SUR_H + SUR_H) + u] * c2;
        } else if (e < 9 * SUR_H) v = p[SUR_W4 + (e - 7 * SUR_H)] * (((e - 7 * SUR_H) & 1) ? sg1 : sg0);
        else if (e < 9 * SUR_H + 2)
            v = p[SUR_B4 + (e - 9 * SUR_H)] * ((e & 1) ? sg1 : sg0) + ((e & 1) ? mu1 : mu0);   // un-normalised s
        else {
            const int l = e - (9 * SUR_H + 2);
            v = ldexpf(1.0f, -(SUR_ACT_EXP + ((l == 0) ? sexp.x : (l == 1) ? sexp.y : sexp.z))) * c2;
        }
        small[e] = v;
    }
}

// per-cell bound: SUR_BOUND_SAFETY x the largest relative error of G_0, G_1 among the cell's samples
__global__ void k_sur_bound(int nbins, const float* __restrict__ Tnet, const double* __restrict__ G,
                            const double* __restrict__ Bv, const double* __restrict__ Qv, float* __restrict__ bound,
                            double* __restrict__ stats)
{
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
        double mx = 0;
        for (int s = 0; s < SUR_VAL_PER_BIN; s++) {
            const size_t i = (size_t)b * SUR_VAL_PER_BIN + s;
            for (int o = 0; o < 2; o++) {
                const double g = Bv[i] * exp((1.0 - Qv[i]) * Tnet[2 * i + o]);
                const double e = fabs(g - G[2 * i + o]) / fabs(G[2 * i + o]);
                mx = fmax(mx, e);
            }
        }
        bound[b] = (float)(SUR_BOUND_SAFETY * mx);
        stats[b] = mx;
    }
}

// Persistent MLP kernels: one CTA per SM at most, two 128-point groups per CTA at a time.
static int sur_grid(int n)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    const int pairs = (n + 255) / 256;
    return std::max(1, std::min(pairs, sms));
}

#define SCK(x)                                                                    \
    do {                                                                          \
        cudaError_t e__ = (x);                                                    \
        if (e__ != cudaSuccess) {                                                 \
            set_error("%s (%d)", "surrogate: CUDA error", (int)e__);              \
            rc = QLP_ERR_CUDA;                                                    \
            goto done;                                                            \
        }                                                                         \
    } while (0)

static const int g_dims[6] = {3, SUR_H, SUR_H, SUR_H, SUR_H, 2};

static void sur_offsets(size_t* off, size_t* boff)
{
    size_t p = 0;
    for (int l = 0; l < 5; l++) {
        off[l] = p;
        p += (size_t)g_dims[l] * g_dims[l + 1];
        boff[l] = p;
        p += g_dims[l + 1];
    }
}

// One forward + backward pass of the training kernels: activations in act
// (6 x bs x 128), gradient into grad.  W (per-sample loss weights) may be null.
static void sur_fwd_bwd(cudaStream_t s, const float* P, const float* xb, const float* tb, const float* W, int bs,
                        float* act, float* dz, float* dz2, float* gpart, int KS, float* grad, double* lpart,
                        int mse_blocks)
{
    size_t off[5], boff[5];
    sur_offsets(off, boff);
    float* a[6];
    for (int l = 0; l < 6; l++) a[l] = act + (size_t)l * bs * SUR_H;
    const float* in = xb;
    for (int l = 0; l < 5; l++) {
        dim3 g((g_dims[l + 1] + 63) / 64, (bs + 63) / 64, 1);
        if (l < 4)
            k_sur_gemm<EPI_TANH><<<g, 256, 0, s>>>(bs, g_dims[l + 1], g_dims[l], in, g_dims[l], 1, P + off[l],
                                                   g_dims[l + 1], 1, a[l + 1], P + boff[l], nullptr);
        else
            k_sur_gemm<EPI_BIAS><<<g, 256, 0, s>>>(bs, 2, SUR_H, in, SUR_H, 1, P + off[l], 2, 1, a[5], P + boff[l],
                                                   nullptr);
        in = a[l + 1];
    }
    k_sur_mse<<<mse_blocks, 256, 0, s>>>(bs, a[5], tb, W, dz, lpart);
    // backward: dcur = dL/dz of layer l; weight gradient a[l]^T dcur, bias gradient colsum(dcur)
    float* dcur = dz;
    float* dnext = dz2;
    for (int l = 4; l >= 0; l--) {
        const float* al = (l == 0) ? xb : a[l];
        const int ni = g_dims[l], no = g_dims[l + 1];
        dim3 gw((no + 63) / 64, (ni + 63) / 64, KS);
        k_sur_gemm<EPI_STORE><<<gw, 256, 0, s>>>(ni, no, bs, al, 1, ni, dcur, no, 1, gpart, nullptr, nullptr);
        k_sur_reduce<<<(ni * no + 255) / 256, 256, 0, s>>>(ni * no, KS, gpart, grad + off[l]);
        k_sur_colsum<<<no, 256, 0, s>>>(bs, no, dcur, grad + boff[l]);
        if (l == 0) break;
        // dz_prev = (dcur W_l^T) * (1 - a[l]^2)
        dim3 gb((ni + 63) / 64, (bs + 63) / 64, 1);
        k_sur_gemm<EPI_DTANH><<<gb, 256, 0, s>>>(bs, ni, no, dcur, no, 1, P + off[l], 1, no, dnext, nullptr, a[l]);
        std::swap(dcur, dnext);
    }
}

int surrogate_train(int device, const qlp_surrogate_opts* o, qlp_surrogate_report* rep)
{
    std::lock_guard<std::mutex> lock(g_sur_mu);
    if (device < 0 || device >= 64) return QLP_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return QLP_ERR_NO_DEVICE;
    SurState& st = g_sur[device];
    const int ntr = std::max(o->n_train, 4096), bs = std::min(std::max(o->batch, 256), ntr);
    const int steps = std::max(o->steps, 1);
    const int nval = SUR_NBINS * SUR_VAL_PER_BIN;
    const int KS = std::max(1, bs / 256);              // split-K for the weight gradients
    const int mse_blocks = 64;
    cudaStream_t s = nullptr;
    float *X = nullptr, *T = nullptr, *Wtr = nullptr, *Xv = nullptr, *Tv = nullptr, *Tnet = nullptr, *act = nullptr;
    float *dz = nullptr, *dz2 = nullptr, *grad = nullptr, *gpart = nullptr, *m1 = nullptr, *m2 = nullptr;
    double *Gv = nullptr, *Bv = nullptr, *Qv = nullptr, *lpart = nullptr, *stats = nullptr;
    int* dstatus = nullptr;
    int rc = QLP_OK;
    float mu[2] = {0.f, 0.f}, sg[2] = {1.f, 1.f};
    double last_loss = 0;
    size_t off[5], boff[5];
    sur_offsets(off, boff);
    const auto t_start = std::chrono::steady_clock::now();
    SCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    if (!st.params) {
        SCK(cudaMalloc(&st.params, sizeof(float) * SUR_NP));
        SCK(cudaMalloc(&st.wimg, SUR_WIMG));
        SCK(cudaMalloc(&st.small, sizeof(float) * SUR_SMALL));
        SCK(cudaMalloc(&st.bound, sizeof(float) * SUR_NBINS));
    }
    st.ready = false;
    SCK(cudaMalloc(&X, sizeof(float) * 3 * (size_t)ntr));
    SCK(cudaMalloc(&T, sizeof(float) * 2 * (size_t)ntr));
    SCK(cudaMalloc(&Wtr, sizeof(float) * (size_t)ntr));
    SCK(cudaMalloc(&Xv, sizeof(float) * 3 * (size_t)nval));
    SCK(cudaMalloc(&Tv, sizeof(float) * 2 * (size_t)nval));
    SCK(cudaMalloc(&Tnet, sizeof(float) * 2 * (size_t)nval));
    SCK(cudaMalloc(&Gv, sizeof(double) * 2 * (size_t)nval));
    SCK(cudaMalloc(&Bv, sizeof(double) * (size_t)nval));
    SCK(cudaMalloc(&Qv, sizeof(double) * (size_t)nval));
    SCK(cudaMalloc(&act, sizeof(float) * 6 * (size_t)bs * SUR_H));
    SCK(cudaMalloc(&dz, sizeof(float) * (size_t)bs * SUR_H));
    SCK(cudaMalloc(&dz2, sizeof(float) * (size_t)bs * SUR_H));
    SCK(cudaMalloc(&grad, sizeof(float) * SUR_NP));
    SCK(cudaMalloc(&gpart, sizeof(float) * (size_t)KS * SUR_H * SUR_H));
    SCK(cudaMalloc(&m1, sizeof(float) * SUR_NP));
    SCK(cudaMalloc(&m2, sizeof(float) * SUR_NP));
    SCK(cudaMalloc(&lpart, sizeof(double) * mse_blocks));
    SCK(cudaMalloc(&stats, sizeof(double) * SUR_NBINS));
    SCK(cudaMalloc(&dstatus, sizeof(int)));
    SCK(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
    {   // Glorot-uniform initial weights, zero biases (host RNG, seeded)
        std::vector<float> h(SUR_NP, 0.f);
        uint64_t z = o->seed * 0x2545F4914F6CDD1Dull + 1;
        auto rnd = [&]() { z ^= z << 13; z ^= z >> 7; z ^= z << 17; return (double)(z >> 11) / 9007199254740992.0; };
        for (int l = 0; l < 5; l++) {
            const double a = sqrt(6.0 / (g_dims[l] + g_dims[l + 1]));
            for (size_t i = 0; i < (size_t)g_dims[l] * g_dims[l + 1]; i++) h[off[l] + i] = (float)((2 * rnd() - 1) * a);
        }
        SCK(cudaMemcpyAsync(st.params, h.data(), sizeof(float) * SUR_NP, cudaMemcpyHostToDevice, s));
        SCK(cudaMemsetAsync(m1, 0, sizeof(float) * SUR_NP, s));
        SCK(cudaMemsetAsync(m2, 0, sizeof(float) * SUR_NP, s));
        SCK(cudaStreamSynchronize(s));
    }
    // training and validation samples from the quadrature
    k_sur_samples<<<(ntr + 127) / 128, 128, 0, s>>>(ntr, o->seed, 0, X, T, nullptr, nullptr, nullptr, Wtr);
    k_sur_samples<<<(nval + 127) / 128, 128, 0, s>>>(nval, o->seed ^ 0x5DEECE66Dull, 1, Xv, Tv, Gv, Bv, Qv,
                                                      nullptr);
    SCK(cudaGetLastError());
    {   // target mean and spread, mean weight (host, double), then normalise on the device
        std::vector<float> ht(2 * (size_t)ntr), hw(ntr);
        SCK(cudaMemcpyAsync(ht.data(), T, sizeof(float) * ht.size(), cudaMemcpyDeviceToHost, s));
        SCK(cudaMemcpyAsync(hw.data(), Wtr, sizeof(float) * hw.size(), cudaMemcpyDeviceToHost, s));
        SCK(cudaStreamSynchronize(s));
        double wmean = 0;
        for (int i = 0; i < ntr; i++) wmean += hw[i];
        wmean = std::max(wmean / ntr, 1e-30);
        for (int o2 = 0; o2 < 2; o2++) {
            double a = 0, b = 0;
            for (int i = 0; i < ntr; i++) { const double v = ht[2 * (size_t)i + o2]; a += v; b += v * v; }
            a /= ntr;
            mu[o2] = (float)a;
            sg[o2] = (float)std::max(sqrt(std::max(b / ntr - a * a, 0.0)), 1e-6);
        }
        // loss weight: 0.1 + 0.9 |alpha|^2 / mean |alpha|^2 -- the deflection
        // error the gate tests is |alpha| times the relative error the loss sees
        k_sur_affine<<<(ntr + 255) / 256, 256, 0, s>>>(ntr, T, mu[0], mu[1], 1.f / sg[0], 1.f / sg[1], Wtr,
                                                        (float)(0.9 / wmean), 0.1f);
    }
    {
        const float b1 = 0.9f, b2 = 0.999f;
        double p1 = 1, p2 = 1;
        for (int it = 0; it < steps; it++) {
            const size_t base = ((size_t)it * bs) % (size_t)(ntr - bs + 1);
            sur_fwd_bwd(s, st.params, X + 3 * base, T + 2 * base, Wtr + base, bs, act, dz, dz2, gpart, KS, grad,
                        lpart, mse_blocks);
            // Adam: linear warm-up over the first 2 % of the steps, then a
            // cosine decay of the learning rate to 0.1 % of o->lr
            p1 *= b1; p2 *= b2;
            const double frac = (double)it / steps;
            const double warm = std::min(1.0, (it + 1) / (0.02 * steps + 1));
            const float lr = (float)(o->lr * warm * (0.001 + 0.999 * 0.5 * (1 + cos(M_PI * frac))));
            k_sur_adam<<<(SUR_NP + 255) / 256, 256, 0, s>>>(SUR_NP, st.params, grad, m1, m2, lr, b1, b2,
                                                            (float)(1.0 / (1 - p1)), (float)(1.0 / (1 - p2)));
        }
        double hp[64];
        SCK(cudaMemcpyAsync(hp, lpart, sizeof(double) * mse_blocks, cudaMemcpyDeviceToHost, s));
        SCK(cudaStreamSynchronize(s));
        for (int b = 0; b < mse_blocks; b++) last_loss += hp[b];
        last_loss /= bs;
    }
    SCK(cudaGetLastError());
    // inference copies, then the error-bound table from the tensor-core path
    {   // per-layer power-of-two scale: the largest weight of layers 1-3 near 2^14 in F16
        std::vector<float> hp(SUR_NP);
        SCK(cudaMemcpyAsync(hp.data(), st.params, sizeof(float) * SUR_NP, cudaMemcpyDeviceToHost, s));
        SCK(cudaStreamSynchronize(s));
        int se[3];
        for (int l = 0; l < 3; l++) {
            float mx = 0.f;
            for (int e = 0; e < SUR_H * SUR_H; e++) mx = std::max(mx, std::fabs(hp[SUR_W1 + l * (SUR_H * SUR_H + SUR_H) + e]));
            int ex = 0;
            std::frexp(std::max(mx, 1e-30f), &ex);       // mx < 2^ex
            se[l] = 14 - ex;
        }
        k_sur_prep<<<64, 256, 0, s>>>(st.params, st.wimg, st.small, mu[0], mu[1], sg[0], sg[1],
                                      make_int3(se[0], se[1], se[2]));
    }
    SCK(cudaStreamSynchronize(s));
    SCK(cudaFuncSetAttribute(k_sur_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, SUR_SMEM));
    SCK(cudaFuncSetAttribute(k_raytrace_sur<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SUR_SMEM));
    SCK(cudaFuncSetAttribute(k_raytrace_sur<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SUR_SMEM));
    k_sur_infer<<<sur_grid(nval), SUR_THREADS, SUR_SMEM, s>>>(nval, Xv, Tnet, st.wimg, st.small, dstatus);
    k_sur_bound<<<(SUR_NBINS + 255) / 256, 256, 0, s>>>(SUR_NBINS, Tnet, Gv, Bv, Qv, st.bound, stats);
    SCK(cudaGetLastError());
    {
        std::vector<double> hs(SUR_NBINS);
        int hstat = 0;
        SCK(cudaMemcpyAsync(hs.data(), stats, sizeof(double) * SUR_NBINS, cudaMemcpyDeviceToHost, s));
        SCK(cudaMemcpyAsync(&hstat, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
        SCK(cudaStreamSynchronize(s));
        if (hstat != 0) {
            set_error("%s (%d)", "surrogate: tensor-core inference timed out", hstat);
            rc = QLP_ERR_TIMEOUT;
            goto done;
        }
        double mx = 0, sum = 0;
        int below = 0;
        for (double v : hs) { mx = std::max(mx, v); sum += v; below += (SUR_BOUND_SAFETY * v <= 1e-5); }
        st.rep.final_loss = last_loss;
        st.rep.val_max_rel = mx;
        st.rep.val_mean_rel = sum / SUR_NBINS;
        st.rep.cells_below_1e5 = (double)below / SUR_NBINS;
        st.rep.n_params = SUR_NP;
        st.rep.n_train = ntr;
        st.rep.steps = steps;
        st.rep.train_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
        st.ready = true;
        if (rep) *rep = st.rep;
    }
done:
    void* bufs[] = {X, T, Wtr, Xv, Tv, Tnet, Gv, Bv, Qv, act, dz, dz2, grad, gpart, m1, m2, lpart, stats, dstatus};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (s) cudaStreamDestroy(s);
    return rc;
}

bool surrogate_ready(int device) { return device >= 0 && device < 64 && g_sur[device].ready; }

// One forward + backward pass of the training kernels on a given batch and
// parameter vector, unweighted (the gradient test).  grad: SUR_NP floats.
int surrogate_grad_check(int device, const float* params, const float* x, const float* t, int batch, double* loss,
                         float* grad_out)
{
    if (cudaSetDevice(device) != cudaSuccess) return QLP_ERR_NO_DEVICE;
    const int bs = batch, KS = std::max(1, bs / 256), mse_blocks = 64;
    float *P = nullptr, *X = nullptr, *T = nullptr, *act = nullptr, *dz = nullptr, *dz2 = nullptr, *grad = nullptr,
          *gpart = nullptr;
    double* lpart = nullptr;
    int rc = QLP_OK;
    double hp[64];
    cudaStream_t s = nullptr;
    SCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    SCK(cudaMalloc(&P, sizeof(float) * SUR_NP));
    SCK(cudaMalloc(&X, sizeof(float) * 3 * (size_t)bs));
    SCK(cudaMalloc(&T, sizeof(float) * 2 * (size_t)bs));
    SCK(cudaMalloc(&act, sizeof(float) * 6 * (size_t)bs * SUR_H));
    SCK(cudaMalloc(&dz, sizeof(float) * (size_t)bs * SUR_H));
    SCK(cudaMalloc(&dz2, sizeof(float) * (size_t)bs * SUR_H));
    SCK(cudaMalloc(&grad, sizeof(float) * SUR_NP));
    SCK(cudaMalloc(&gpart, sizeof(float) * (size_t)KS * SUR_H * SUR_H));
    SCK(cudaMalloc(&lpart, sizeof(double) * mse_blocks));
    SCK(cudaMemcpyAsync(P, params, sizeof(float) * SUR_NP, cudaMemcpyHostToDevice, s));
    SCK(cudaMemcpyAsync(X, x, sizeof(float) * 3 * (size_t)bs, cudaMemcpyHostToDevice, s));
    SCK(cudaMemcpyAsync(T, t, sizeof(float) * 2 * (size_t)bs, cudaMemcpyHostToDevice, s));
    sur_fwd_bwd(s, P, X, T, nullptr, bs, act, dz, dz2, gpart, KS, grad, lpart, mse_blocks);
    SCK(cudaGetLastError());
    SCK(cudaMemcpyAsync(hp, lpart, sizeof(double) * mse_blocks, cudaMemcpyDeviceToHost, s));
    SCK(cudaMemcpyAsync(grad_out, grad, sizeof(float) * SUR_NP, cudaMemcpyDeviceToHost, s));
    SCK(cudaStreamSynchronize(s));
    {
        double l = 0;
        for (int b = 0; b < mse_blocks; b++) l += hp[b];
        *loss = l / bs;
    }
done:
    void* bufs[] = {P, X, T, act, dz, dz2, grad, gpart, lpart};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (s) cudaStreamDestroy(s);
    return rc;
}

// At n points (rho, phi, q): t = log(G/B) through the tensor-core inference
// path, the quadrature's G, the baselines and each point's cell bound.
int surrogate_eval(int device, const double* rpq, int n, double* t_net, double* G_quad, double* B, double* bound_out)
{
    if (!surrogate_ready(device)) {
        set_error("%s (%d)", "surrogate not trained on this device", device);
        return QLP_ERR_ARG;
    }
    if (cudaSetDevice(device) != cudaSuccess) return QLP_ERR_NO_DEVICE;
    SurState& st = g_sur[device];
    int rc = QLP_OK;
    cudaStream_t s = nullptr;
    float *X = nullptr, *T = nullptr;
    double *P = nullptr, *G = nullptr, *Bd = nullptr;
    int* dstatus = nullptr;
    int hstat = 0;
    std::vector<float> ht(2 * (size_t)n), hb(SUR_NBINS);
    SCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    SCK(cudaMalloc(&X, sizeof(float) * 3 * (size_t)n + 16));
    SCK(cudaMalloc(&T, sizeof(float) * 2 * (size_t)n + 16));
    SCK(cudaMalloc(&P, sizeof(double) * 3 * (size_t)n + 16));
    SCK(cudaMalloc(&G, sizeof(double) * 2 * (size_t)n + 16));
    SCK(cudaMalloc(&Bd, sizeof(double) * (size_t)n + 16));
    SCK(cudaMalloc(&dstatus, sizeof(int)));
    SCK(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
    SCK(cudaMemcpyAsync(P, rpq, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, s));
    k_sur_points<<<(n + 127) / 128, 128, 0, s>>>(n, P, X, G, Bd);
    k_sur_infer<<<sur_grid(n), SUR_THREADS, SUR_SMEM, s>>>(n, X, T, st.wimg, st.small, dstatus);
    SCK(cudaGetLastError());
    SCK(cudaMemcpyAsync(ht.data(), T, sizeof(float) * 2 * (size_t)n, cudaMemcpyDeviceToHost, s));
    SCK(cudaMemcpyAsync(hb.data(), st.bound, sizeof(float) * SUR_NBINS, cudaMemcpyDeviceToHost, s));
    if (G_quad) SCK(cudaMemcpyAsync(G_quad, G, sizeof(double) * 2 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (B) SCK(cudaMemcpyAsync(B, Bd, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
    SCK(cudaMemcpyAsync(&hstat, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCK(cudaStreamSynchronize(s));
    if (hstat) {
        rc = QLP_ERR_TIMEOUT;
        goto done;
    }
    for (int i = 0; i < n; i++) {   // t = (1 - q) s
        const double rho = rpq[3 * (size_t)i], phi = rpq[3 * (size_t)i + 1];
        double q = rpq[3 * (size_t)i + 2];
        if (q >= 1.0) q = 0.999999;
        t_net[2 * (size_t)i] = (1.0 - q) * ht[2 * (size_t)i];
        t_net[2 * (size_t)i + 1] = (1.0 - q) * ht[2 * (size_t)i + 1];
        if (bound_out) {
            const int c = sur_cell(rho, phi, q);
            bound_out[i] = (c < 0) ? INFINITY : (double)hb[c];
        }
    }
done:
    void* bufs[] = {X, T, P, G, Bd, dstatus};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (s) cudaStreamDestroy(s);
    return rc;
}

// ray shooting through the surrogate (ctx.cpp selects it)
int launch_raytrace_sur(const StaticData& sd, Work& w, double thresh, int defer_lens, cudaStream_t st)
{
    if (sd.n_sub == 0) return QLP_OK;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!surrogate_ready(dev)) {
        set_error("%s (%d)", "no trained NFW surrogate on this device", dev);
        return QLP_ERR_ARG;
    }
    SurState& S = g_sur[dev];
    cudaMemsetAsync(w.fb_count, 0, sizeof(int), st);
    const SurRayOut q{w.fb_count, w.fb_ray, w.fb_xy};
    int n = 1;
    if (defer_lens >= 0) {
        // one NFW lens, on the last plane: the other lenses first, at full occupancy
        k_ray_pre<<<(sd.n_sub + 255) / 256, 256, 0, st>>>(sd, w.ep, defer_lens, w.spx, w.spy, w.nfw_xy);
        k_raytrace_sur<true><<<sur_grid(sd.n_sub), SUR_THREADS, SUR_SMEM, st>>>(
            sd, w.ep, w.spx, w.spy, w.nfw_xy, S.wimg, S.small, S.bound, thresh, defer_lens, q, w.sur_eps, w.gs,
            w.out);
        n++;
    } else {
        k_raytrace_sur<false><<<sur_grid(sd.n_sub), SUR_THREADS, SUR_SMEM, st>>>(
            sd, w.ep, w.spx, w.spy, nullptr, S.wimg, S.small, S.bound, thresh, defer_lens, q, w.sur_eps, w.gs,
            w.out);
    }
    if (defer_lens >= 0) {
        const int blocks = std::min((sd.n_sub + 255) / 256, 152 * 8);
        k_nfw_fallback<<<blocks, 256, 0, st>>>(w.ep, defer_lens, w.fb_count, w.fb_ray, w.fb_xy, w.spx, w.spy);
        n++;
    }
    count_launches(n);
    return QLP_OK;
}

}  // namespace qlpix
