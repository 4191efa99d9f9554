// qlpix_ctx.h -- the context object behind qlp_ctx* (host runtime).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "qlpix_internal.h"

#define QLP_N_STAGES 6
#define QLP_MAX_SLOTS 64

namespace qlpix {

// One evaluation lane: a stream and the full per-evaluation workspace.  A
// batch spreads its instances over several slots so that the sequential
// parts of one evaluation (Cholesky pivots, triangular solves) overlap the
// parallel parts of others.
struct Slot {
    cudaStream_t stream = nullptr;
    Work w{};
    void* mixed = nullptr;          // mixed-precision workspace (mixed.cu)
    int M_cap = 0;                  // capacity in source cells (multiple of 64)
    int N_cap = 0;                  // capacity in masked pixels
    int nsub_cap = 0;
    int snx_cap = 0, sny_cap = 0;
    int npix_pad = 0;               // image pixels with a PSF-half-width border: (nx + 2 (pnx/2)) (ny + 2 (pny/2))
    int img_nx = 0, img_ny = 0;     // image and PSF sizes (the PSF-to-X band layout)
    int psf_nx = 0, psf_ny = 0;
    bool fp64_mats = false;         // F and R in FP64 allocated
    cudaEvent_t done = nullptr;
    // second stream of the slot: R's factorisation runs beside F's
    cudaStream_t side = nullptr;
    cudaEvent_t side_fork = nullptr, side_join = nullptr;
    // the launch sequence captured as a CUDA graph, sized for the slot's
    // capacity (any mask and source grid that fit), valid for one
    // (precision, capacity, NFW, NFW mode, lambda optimisation) combination and
    // graph generation; with the lambda optimisation on, `graph` holds the
    // lambda-independent part and `graph_trial` one lambda trial
    cudaGraphExec_t graph = nullptr;
    int graph_key[7] = {0, 0, 0, 0, 0, 0, 0};
    long long graph_gen = 0;
    long long graph_launches = 0;   // kernels per replay
    cudaGraphExec_t graph_trial = nullptr;
    int trial_key[7] = {0, 0, 0, 0, 0, 0, 0};
    long long trial_gen = 0;
    long long trial_launches = 0;
    OsbWork osb{};                  // outside-surface-brightness pass (allocated when the prior is on)
    int osb_nsub = 0;               // its capacity in sub-pixels
};

}  // namespace qlpix

struct qlp_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int precision = QLP_FP64;
    int max_slots = 16;                   // schedule: evaluations in flight
    int ray_threads = 256;                // schedule: ray-shooting CTA size
    int psfx_threads = 256;               // schedule: k_psf_x CTA size
    int psfx_split = 1;                   // schedule: row chunks / bands per source cell in the PSF-to-X build
    int psfx_mode = -1;                   // schedule: PSF-to-X kernel, 0 active-row chunks, 1 image-row
                                          // bands (-1: chosen from the PSF size at creation)

    // lens model
    std::vector<qlp_lens> lenses;
    std::vector<qlp_fit_param> fit;    // qlp_set_fit_params
    qlp_planes planes{};

    // host copies of the static inputs
    int nx = 0, ny = 0;
    std::vector<int> mpix;                // masked pixels of the image mask (j-outer, i-inner)
    qlp_srcgrid_opts opts{};

    // device copies
    double* d_xvals = nullptr;
    double* d_yvals = nullptr;
    double* d_data = nullptr;
    double* d_covinv = nullptr;
    double* d_psf = nullptr;
    int* d_psf_int = nullptr;      // the PSF on the PSF-to-X fixed-point grid (StaticData::psf_int)
    int* d_mpix = nullptr;

    // extra masks for batched evaluation (device mpix lists, concatenated)
    std::vector<int> mask_off, mask_cnt;
    int* d_inst_mpix = nullptr;

    qlpix::StaticData sd{};
    qlpix::SrcOpts so{};
    std::vector<qlpix::Slot> slots;       // slots[0] serves qlp_eval

    qlpix::EvalOut* h_out = nullptr;      // pinned, one per batch instance
    int h_out_cap = 0;
    qlpix::EvalOut* h_trial = nullptr;    // pinned, one per slot: results of lambda trials
    std::vector<double> regopt_lam;       // per batch instance: the lambda of its result
    std::vector<int> regopt_evals;        // per batch instance: lambda trials run
    cudaEvent_t ev[QLP_N_STAGES + 1] = {};
    cudaEvent_t fork = nullptr, join = nullptr;
    std::vector<cudaEvent_t> ev_pool;     // (QLP_N_STAGES+1) per batched instance
    qlpix::EvalParams* h_ep = nullptr;    // pinned, one per batch instance
    int h_ep_cap = 0;
    int use_graphs = 1;                   // batched evaluation replays captured graphs
    int refine = 1;                       // FP64 refinement sweeps of the mixed path's amplitudes
    // regularisation-parameter optimisation (QLens 'optimize_regparam on'):
    // Brent's method over log10(lambda), QLens's defaults
    int regopt = 0;
    double regopt_minlog = -3.0, regopt_maxlog = 5.0, regopt_tol = 0.01;
    int regopt_maxit = 20;
    int nfw_mode = QLP_NFW_QUADRATURE;    // NFW deflection: quadrature or trained surrogate
    double nfw_threshold = 2e-5;          // surrogate error bound (arcsec) above which a ray falls back
    double nfw_tol = 1e-3;                // the NFW quadrature's tolerance (QLens integral_tolerance)
    // outside-surface-brightness prior (QLens 'outside_sb_prior'): settings,
    // device tables of the extended mask, background noise of the image
    int osb_on = 0;
    qlpix::OsbStatic osb{};
    unsigned char* d_emask = nullptr;
    unsigned char* d_inmask = nullptr;
    int* d_epix = nullptr;
    int* d_eoff = nullptr;
    double bg_noise = 0;
    long long graph_gen = 1;              // bumped whenever captured graphs go stale
    long long last_h2d = 0, last_d2h = 0; // bytes moved by the last call
    float stage_ms[QLP_N_STAGES] = {};
    float device_ms = 0;
    long long last_launches = 0;
};

namespace qlpix {
int ctx_init(qlp_ctx* c, const qlp_image* im, const qlp_psf* psf, const qlp_srcgrid_opts* opts);
void ctx_free(qlp_ctx* c);
int ctx_eval(qlp_ctx* c, const double* lens_params, double regparam, qlp_result* out);
int ctx_set_masks(qlp_ctx* c, const unsigned char* masks, int n_masks);
int ctx_eval_batch(qlp_ctx* c, const double* params, const double* regparams, const qlp_instance* inst, int n,
                   qlp_result* out);
int ctx_dump(qlp_ctx* c, double* srcpt_xy, int* L_rowptr, int* L_index, double* L_value, int* active_index,
             double* D, double* s, double* model);
int ctx_dump_Lpsf(qlp_ctx* c, int rows, double* out);
int make_lens_rec(LensRec& L, const qlp_lens& d, const double* p);
int fit_set(qlp_ctx* c, const qlp_fit_param* fp, int n);
int fit_loglike_batch(qlp_ctx* c, const double* x, int n, double* loglike, qlp_result* out);
int fit_terms(const qlp_fit_param* fp, int n, const double* x, double* t, int* penalised, double* terms);
bool is_nfw_type(int type);
int n_params_of(int type);
void set_error(const char* fmt, const char* a, int code);
// mixed.cu
int mixed_init(Slot& slot);
void mixed_free(Slot& slot);
// launch sequences of one evaluation: the whole of it, or, for the
// regularisation-parameter optimisation, its lambda-independent part and one
// lambda trial
#define PIPE_ALL 0
#define PIPE_PRE 1
#define PIPE_TRIAL 2
int mixed_ensure_f0(Slot& slot);
int run_inversion_mixed(const qlp_ctx* c, Slot& slot, const StaticData& sd, const SrcOpts& so, const double* regp,
                        int part, cudaStream_t st,
                        cudaEvent_t* ev);
// autotune.cpp
int ctx_get_schedule(const qlp_ctx* c, qlp_schedule* out);
// outside.cu / ctx.cpp: the outside-surface-brightness prior
int ctx_set_outside_sb(qlp_ctx* c, int on, double frac, double noise_frac, const unsigned char* emask, int ens);
int ctx_set_schedule(qlp_ctx* c, const qlp_schedule* s);
int ctx_autotune(qlp_ctx* c, const double* params, const double* lambdas, const qlp_instance* inst, int n, int reps,
                 qlp_tune_report* rep);
void ctx_trim_slots(qlp_ctx* c, int keep);
// surrogate.cu
int surrogate_train(int device, const qlp_surrogate_opts* o, qlp_surrogate_report* rep);
bool surrogate_ready(int device);
int surrogate_grad_check(int device, const float* params, const float* x, const float* t, int batch, double* loss,
                         float* grad);
int surrogate_eval(int device, const double* rpq, int n, double* t_net, double* G_quad, double* B, double* bound);
int launch_raytrace_sur(const StaticData& sd, Work& w, double thresh, int defer_lens, cudaStream_t st);
int launch_surrogate_exact(const StaticData& sd, const SrcOpts& so, Work& w, double eps_g, int step,
                           cudaStream_t st);
}  // namespace qlpix
