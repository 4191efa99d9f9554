// qlpix_internal.h -- device-side data structures shared by the kernels and
// the host runtime of libqlpix.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "../../include/qlpix.h"

namespace qlpix {

// One lens, reduced to the constants its deflection needs.  Filled on the
// host with the same libm calls QLens makes in update_meta_parameters
// (models.cpp:101-108, 2212-2224; profile.cpp:1625-1689).
struct LensRec {
    int type;        // QLP_LENS_*
    int plane;       // lens-redshift plane
    int kind;        // SPLE: 0 spherical, 1 elliptical alpha=1, 2 elliptical core-free
    int nfw_mode;    // NFW: 0 quadrature, 1 surrogate
    double xc, yc, costheta, sintheta;
    double q, qsq, b, bprime, s, sprime, ssq, alpha;
    double shear1, shear2;
    double ks, rs, f_major_axis, epsilon;   // NFW
    double tol;                             // NFW: the quadrature's relative tolerance (QLens integral_tolerance)
};

struct LensModel {
    int nlens;
    int n_planes;
    double zfac[QLP_MAX_PLANES];
    double beta[QLP_MAX_PLANES][QLP_MAX_PLANES];
    LensRec lens[QLP_MAX_LENSES];
};

// Mask and source-grid size of one evaluation.  Kept in device memory (in
// the slot's EvalParams): a batch with uneven masks and grids replays one
// launch sequence sized for the slot's capacity, and the kernels take the
// actual sizes from here.
struct InstShape {
    const int* mpix;          // n_mask masked pixels, j-outer / i-inner order
    int n_mask, n_sub;        // masked pixels, sub-pixels
    int snx, sny;             // source-grid cells
};

// What changes from one evaluation to the next: the lens model (meta
// parameters computed on the host), the regularisation parameter and the
// mask / source-grid size.  Kept in
// device memory, one copy per slot, so that one captured launch sequence (a
// CUDA graph) serves every evaluation a slot runs.
struct EvalParams {
    LensModel lm;
    double regparam;
    InstShape shape;
};

// Source-grid state computed on the device each evaluation.
struct GridState {
    double xmin, xmax, ymin, ymax;    // bounds after auto-sizing
    double ext[4];                    // the extremes of the per-pixel mean source points they came from
                                      // (x min, x max, y min, y max; before the clamp and widening)
    int snx, sny;                     // cells
    int M;                            // active source cells
    int N;                            // active image pixels
    int nnz;                          // pre-PSF L nonzeros
    int status;                       // QLP_* status raised on the device
    int not_spd_F, not_spd_R;         // first failing pivot + 1 (0 = fine)
};

// Scalars of one evaluation, written by the final assembly kernel.
struct EvalOut {
    double chisq0, logdet_F, logdet_R, Es_times_two, regterms, m2logev;
    double f_regopt;                   // the lambda optimisation's objective: chi^2 over the active
                                       // pixels + regularisation terms + log det F
    int n_active_pixels, n_active_src, L_nnz, status, refine_iters;
    int pad;                           // rays that took the NFW quadrature instead of the surrogate
    int n_exact;                       // surrogate rays traced again exactly near a grid decision
    double osb_penalty;                // the outside-surface-brightness prior's penalty (0 when off)
};

// The outside-surface-brightness prior (QLens 'outside_sb_prior'): static
// tables of the extended mask, uploaded once per setting.
struct OsbStatic {
    const unsigned char* emask;        // nx*ny extended mask
    const unsigned char* inmask;       // nx*ny the context's mask
    const int* epix;                   // ne extended-mask pixels, j-outer / i-inner
    const int* eoff;                   // ne+1 sub-pixel offsets (mask pixels split nsplit ways, others ens)
    int ne, nsub_e, ens;
    double frac, noise_frac, bg_noise; // threshold max(noise_frac bg_noise, frac peak)
};
// ... and its per-slot workspace
struct OsbWork {
    double* sp;                        // 2 nsub_e source points
    int* cell3;  double* w3;           // 3 nsub_e
    double* model;  int* act;  double* sb;   // nx*ny
};

#define PSFX_LEXP 28               // grid of the L entries in the PSF-to-X products: 2^-28

struct StaticData {            // per-context, uploaded once
    int nx, ny;                // image pixels
    int n_mask;                // masked pixels
    int nsplit, nsub;          // split factor, sub-pixels per pixel
    int n_sub;                 // n_mask * nsub
    int pnx, pny;              // PSF size
    int use_noise_map;
    double cov_inverse;        // uniform 1/sigma^2 when !use_noise_map
    int noise_term;            // add the pixel-noise normalisation to -2 log(evidence)
    const double* xvals;       // nx+1
    const double* yvals;       // ny+1
    const double* data;        // nx*ny
    const double* covinv;      // nx*ny (filled with cov_inverse when uniform)
    const int* mpix;           // n_mask: i*ny+j, j-outer / i-inner order
    const double* psf;         // pnx*pny
    // fixed-point PSF-to-X sums of the mixed path (sqrt(C^-1) is applied to
    // the sum): every product psf x L is the exact integer product of the tap
    // on the grid 2^-(fix_exp_x - PSFX_LEXP) (psf_int, |psf_int| summing to at
    // most 2^30) and the L entry on the grid 2^-PSFX_LEXP (|L| <= 4: at most
    // 2^30), so a sum -- one entry per tap at most -- stays below 2^61
    int fix_exp_x;
    // the PSF on its grid, x fastest: psf_int[pl * pnx + pk] =
    // round(psf[pk * pny + pl] * 2^(fix_exp_x - PSFX_LEXP))
    const int* psf_int;
    // F16 operands of the mixed path's SYRK: X scaled by 2^x_exp puts its
    // largest possible entry (4 sum|psf| max sqrt(C^-1)) at or below 2^14
    int x_exp;
    // device address of this evaluation's InstShape: the kernels take mpix,
    // n_mask, n_sub and the source-grid size from there (the host-side copy
    // of those fields only sizes the launches)
    const InstShape* shape;
};

#ifdef __CUDACC__
__device__ __forceinline__ StaticData eval_shape(StaticData s)
{
    const InstShape* p = s.shape;
    s.mpix = p->mpix;
    s.n_mask = p->n_mask;
    s.n_sub = p->n_sub;
    return s;
}
#endif

struct SrcOpts {
    int snx, sny;
    int auto_grid;
    double xmin, xmax, ymin, ymax;
    double lxmin, lxmax, lymin, lymax;
    double noise_threshold, size_scale;
    int regularization;
    double regparam;
};

#ifdef __CUDACC__
__device__ __forceinline__ SrcOpts eval_grid(SrcOpts o, const StaticData& s)
{
    o.snx = s.shape->snx;
    o.sny = s.shape->sny;
    return o;
}
#endif

// Per-evaluation device workspace (sized for the largest case at creation).
struct Work {
    double* spx;  double* spy;         // n_sub source points
    double* cx;   double* cy;          // snx+1, sny+1 cell corners
    double* ccx;  double* ccy;         // snx, sny cell centres
    int* cell3;   double* w3;          // 3 per sub-pixel
    int* mapped;                       // snx*sny flags
    int* active_index;                 // snx*sny
    int* pixmaps;                      // n_mask: # mapped sub-pixels (0 = pixel unmapped)
    int* rowidx;                       // n_mask: active row or -1
    int* pixindex;                     // nx*ny: active row or -1
    int* rowpix;                       // n_mask: image pixel of each active row
    int* rowptr;                       // N+1
    int* Lidx;    double* Lval;        // pre-PSF L, CSR
    int* cidx;    double* cval; int* ccnt;   // compressed rows (duplicates summed), same capacity
    double* Lpsf;                      // N x ldL, FP64
    unsigned char* lnz;                // plain path: nonzero flags of L' per (64-column block, 16-row chunk)
    int lnz_chunks;                    // row chunks per column block in lnz
    int ldL;                           // leading dimension of Lpsf (>= M_max)
    double* dvec; double* cvec;        // N: data and C^-1 per active row
    double* D;                         // M
    double* F;                         // M x ldF (lower triangle)
    double* R;                         // M x ldF (lower triangle)
    int ldF;
    double* s;   double* tmp;          // M
    double* model;                     // N
    double* partial;                   // reduction scratch
    double* gpart;  int* gpart_cnt;    // source-grid bounds: per-block partials (1024 blocks at most)
    int* cpart;                        // compaction: per-block counts (3 x 1025)
    double* linv;                      // 64x64 inverse of the current diagonal Cholesky block
    GridState* gs;
    EvalOut* out;                      // this slot's result (copied to the host after each evaluation)
    EvalParams* ep;                    // this slot's per-evaluation parameters
    // rays whose NFW deflection the surrogate hands to the quadrature (n_sub capacity)
    int* fb_ray;  double* fb_xy;  int* fb_count;
    double* nfw_xy;                    // 2 n_sub: rays' positions on the NFW lens's plane (k_ray_pre)
    float* sur_eps;                    // n_sub: bound on each ray's source-point error on the surrogate path
    int* xlist;  int* xcount;          // n_sub, 1: rays the surrogate path traces again exactly
    double* F0;                        // plain path, lambda optimisation: L'^T C^-1 L' before lambda R
};

// Device address of the regularisation parameter of a slot's EvalParams.
inline const double* regparam_dev(const Work& w)
{
    return reinterpret_cast<const double*>(reinterpret_cast<const char*>(w.ep) + offsetof(EvalParams, regparam));
}

// ---- kernels (launch wrappers implemented in the .cu files) ----
void launch_raytrace(const StaticData& sd, bool nfw, Work& w, int threads, cudaStream_t st);
void launch_grid(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st);
void launch_locate(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st);
void launch_compact(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st);
void launch_build_L(const StaticData& sd, const SrcOpts& so, Work& w, cudaStream_t st);
void launch_rowpix(const StaticData& sd, Work& w, cudaStream_t st);
void launch_psf(const StaticData& sd, const SrcOpts& so, Work& w, int M_max, cudaStream_t st);
void op_Ls(Work& w, int N_cap, const double* s, double* t, cudaStream_t st);
void op_conv(const StaticData& sd, Work& w, int N_cap, bool transpose, const double* in, const double* scale_in,
             double* out, double* img, const int2* pixT, cudaStream_t st);
void launch_dvec(const StaticData& sd, Work& w, int N_max, cudaStream_t st);
void launch_D(Work& w, int N_max, int M_max, cudaStream_t st);
void launch_syrk_fp64(const StaticData& sd, Work& w, int N_max, int M_max, cudaStream_t st);
// parts: REG_F adds lambda R to F, REG_R writes R (both: the plain evaluation)
#define REG_F 1
#define REG_R 2
void launch_regularization(const SrcOpts& so, Work& w, int M_max, const double* regp, int parts, cudaStream_t st);
int  launch_cholesky_fp64(double* A, int ld, int M_max, const GridState* gs, int which, double* linv,
                          cudaStream_t st);
void launch_logdet(const double* A, int ld, int M_max, Work& w, int which, cudaStream_t st);
void launch_solve_fp64(Work& w, int M_max, cudaStream_t st);
void launch_model_chi2(const StaticData& sd, const SrcOpts& so, Work& w, int N_max, int M_max,
                       const double* regp, cudaStream_t st, bool model_ready = false);
void launch_outside_sb(const StaticData& sd, const SrcOpts& so, const OsbStatic& os, const OsbWork& ow, bool nfw,
                       Work& w, cudaStream_t st);
void init_kernel_attributes();
long long kernel_launch_counter();
void count_launches(int n);

}  // namespace qlpix

#define QLP_CUDA_CHECK(x) do { cudaError_t e__ = (x); if (e__ != cudaSuccess) return e__; } while (0)
