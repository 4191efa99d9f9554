// ctx.cpp -- context set-up, evaluation slots, and the per-evaluation launch
// sequence.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <vector>
#include <algorithm>
#include "qlpix_ctx.h"
#include "brent.h"

namespace qlpix {

void psf_init_attributes();
void linalg_init_attributes();
void sparseops_init_attributes();
void sur_exact_init_attributes();

static int cuda_fail(cudaError_t e, const char* where)
{
    set_error("CUDA error in %s: %d", where, (int)e);
    return (e == cudaErrorMemoryAllocation) ? QLP_ERR_NOMEM : QLP_ERR_CUDA;
}

#define CK(x, where) do { cudaError_t e__ = (x); if (e__ != cudaSuccess) return cuda_fail(e__, where); } while (0)

template <typename T>
static cudaError_t dalloc(T** p, size_t n)
{
    return cudaMalloc((void**)p, sizeof(T) * (n > 0 ? n : 1));
}

static int round64(int x) { return (x + 63) & ~63; }

// Masked pixels in the order QLens lists them (setup_ray_tracing_arrays,
// pixelgrid.cpp:9996-10005: j outer, i inner).
static std::vector<int> masked_list(const unsigned char* mask, int nx, int ny)
{
    std::vector<int> v;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
            if (mask[i * ny + j]) v.push_back(i * ny + j);
    return v;
}

static void free_work(Work& w)
{
    void* ptrs[] = {w.spx, w.spy, w.cx, w.cy, w.ccx, w.ccy, w.cell3, w.w3, w.mapped, w.active_index, w.pixmaps,
                    w.rowidx, w.pixindex, w.rowpix, w.rowptr, w.Lidx, w.Lval, w.cidx, w.cval, w.ccnt, w.Lpsf,
                    w.dvec, w.cvec, w.D, w.F, w.R, w.s, w.tmp, w.model, w.partial, w.linv, w.gs, w.out, w.ep,
                    w.fb_ray, w.fb_xy, w.fb_count, w.F0, w.gpart, w.gpart_cnt, w.cpart, w.lnz, w.sur_eps, w.xlist, w.xcount, w.nfw_xy};
    for (void* p : ptrs) if (p) cudaFree(p);
    memset(&w, 0, sizeof(w));
}

static void drop_graph(Slot& s)
{
    if (s.graph) cudaGraphExecDestroy(s.graph);
    s.graph = nullptr;
    s.graph_gen = 0;
    if (s.graph_trial) cudaGraphExecDestroy(s.graph_trial);
    s.graph_trial = nullptr;
    s.trial_gen = 0;
}

static void free_slot(Slot& s)
{
    drop_graph(s);
    mixed_free(s);
    free_work(s.w);
    OsbWork& o = s.osb;
    void* op[] = {o.sp, o.cell3, o.w3, o.model, o.act, o.sb};
    for (void* p : op) if (p) cudaFree(p);
    o = OsbWork{};
    s.osb_nsub = 0;
    s.M_cap = s.N_cap = s.nsub_cap = s.snx_cap = s.sny_cap = 0;
    s.fp64_mats = false;
}

// Workspace of one slot for up to n_mask masked pixels (nsub sub-pixels each)
// and Mcells source cells.  The FP64 F and R are allocated on first use.
static int alloc_work(qlp_ctx* c, Slot& s, int n_mask, int nsub, int Mcells, int snx_max, int sny_max)
{
    free_slot(s);
    Work& w = s.w;
    const int Mc = round64(std::max(Mcells, 64));
    const size_t n_sub = (size_t)n_mask * nsub;
    const size_t nnz = 3 * n_sub;
    CK(dalloc(&w.spx, n_sub), "alloc"); CK(dalloc(&w.spy, n_sub), "alloc");
    CK(dalloc(&w.cx, snx_max + 1), "alloc"); CK(dalloc(&w.cy, sny_max + 1), "alloc");
    CK(dalloc(&w.ccx, snx_max), "alloc"); CK(dalloc(&w.ccy, sny_max), "alloc");
    CK(dalloc(&w.cell3, 3 * n_sub), "alloc"); CK(dalloc(&w.w3, 3 * n_sub), "alloc");
    CK(dalloc(&w.mapped, Mcells), "alloc"); CK(dalloc(&w.active_index, Mcells), "alloc");
    CK(dalloc(&w.pixmaps, n_mask), "alloc"); CK(dalloc(&w.rowidx, n_mask), "alloc");
    CK(dalloc(&w.pixindex, (size_t)c->nx * c->ny), "alloc");
    CK(dalloc(&w.rowpix, n_mask), "alloc");
    CK(dalloc(&w.rowptr, n_mask + 1), "alloc");
    CK(dalloc(&w.Lidx, nnz), "alloc"); CK(dalloc(&w.Lval, nnz), "alloc");
    CK(dalloc(&w.cidx, nnz), "alloc"); CK(dalloc(&w.cval, nnz), "alloc"); CK(dalloc(&w.ccnt, n_mask), "alloc");
    w.ldL = Mc;
    CK(dalloc(&w.dvec, n_mask), "alloc"); CK(dalloc(&w.cvec, n_mask), "alloc");
    w.ldF = Mc;
    CK(dalloc(&w.D, Mc), "alloc");
    CK(dalloc(&w.s, Mc), "alloc"); CK(dalloc(&w.tmp, Mc), "alloc");
    CK(dalloc(&w.model, n_mask), "alloc");
    const size_t part = std::max((size_t)((n_mask + 255) / 256 + 1) * Mc, (size_t)Mc * 4);
    CK(dalloc(&w.partial, part), "alloc");
    CK(dalloc(&w.gpart, 4 * 1024), "alloc"); CK(dalloc(&w.gpart_cnt, 1024), "alloc");
    CK(dalloc(&w.cpart, 3 * 1025), "alloc");
    CK(dalloc(&w.linv, (size_t)Mc * 64), "alloc");
    CK(dalloc(&w.gs, 1), "alloc"); CK(dalloc(&w.out, 1), "alloc"); CK(dalloc(&w.ep, 1), "alloc");
    CK(dalloc(&w.fb_ray, n_sub), "alloc"); CK(dalloc(&w.fb_xy, 2 * n_sub), "alloc"); CK(dalloc(&w.fb_count, 1), "alloc");
    CK(dalloc(&w.sur_eps, n_sub), "alloc");
    CK(dalloc(&w.xlist, n_sub), "alloc"); CK(dalloc(&w.xcount, 1), "alloc");
    CK(dalloc(&w.nfw_xy, 2 * n_sub), "alloc");
    s.M_cap = Mc;
    s.N_cap = n_mask;
    s.npix_pad = (c->nx + 2 * (c->sd.pnx / 2)) * (c->ny + 2 * (c->sd.pny / 2));
    s.img_nx = c->nx; s.img_ny = c->ny;
    s.psf_nx = c->sd.pnx; s.psf_ny = c->sd.pny;
    s.nsub_cap = nsub;
    s.snx_cap = snx_max;
    s.sny_cap = sny_max;
    return QLP_OK;
}

// Dense FP64 L', F and R: only the plain path uses them.
static int ensure_fp64_mats(Slot& s)
{
    if (s.fp64_mats) return QLP_OK;
    CK(dalloc(&s.w.Lpsf, (size_t)s.N_cap * s.M_cap), "alloc L'");
    CK(cudaMemset(s.w.Lpsf, 0, sizeof(double) * (size_t)s.N_cap * s.M_cap), "memset");
    s.w.lnz_chunks = (s.N_cap + 15) / 16;
    CK(dalloc(&s.w.lnz, (size_t)s.w.lnz_chunks * (s.M_cap / 64)), "alloc L' flags");
    CK(dalloc(&s.w.F, (size_t)s.M_cap * s.M_cap), "alloc F");
    CK(dalloc(&s.w.R, (size_t)s.M_cap * s.M_cap), "alloc R");
    s.fp64_mats = true;
    return QLP_OK;
}

// Make slot k exist with at least the given capacities.
static int ensure_slot(qlp_ctx* c, int k, int n_mask, int cells, int snx, int sny)
{
    while ((int)c->slots.size() <= k) c->slots.emplace_back();
    Slot& s = c->slots[k];
    if (!s.stream) CK(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "stream");
    if (!s.done) CK(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "event");
    if (!s.side) CK(cudaStreamCreateWithFlags(&s.side, cudaStreamNonBlocking), "stream");
    if (!s.side_fork) CK(cudaEventCreateWithFlags(&s.side_fork, cudaEventDisableTiming), "event");
    if (!s.side_join) CK(cudaEventCreateWithFlags(&s.side_join, cudaEventDisableTiming), "event");
    const int nsub = c->sd.nsub;
    if (s.N_cap >= n_mask && s.M_cap >= round64(std::max(cells, 64)) && s.snx_cap >= snx && s.sny_cap >= sny &&
        s.nsub_cap == nsub)
        return QLP_OK;
    return alloc_work(c, s, std::max(n_mask, s.N_cap), nsub, std::max(cells, s.M_cap), std::max(snx, s.snx_cap),
                      std::max(sny, s.sny_cap));
}

int ctx_init(qlp_ctx* c, const qlp_image* im, const qlp_psf* psf, const qlp_srcgrid_opts* opts)
{
    c->nx = im->npixels_x;
    c->ny = im->npixels_y;
    c->opts = *opts;
    const int nx = c->nx, ny = c->ny, npx = nx * ny;
    c->mpix = masked_list(im->in_mask, nx, ny);
    CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking), "stream");
    c->stream = c->own_stream;
    for (int i = 0; i <= QLP_N_STAGES; i++) CK(cudaEventCreate(&c->ev[i]), "event");
    CK(cudaEventCreate(&c->fork), "event");
    CK(cudaEventCreate(&c->join), "event");

    std::vector<double> covinv(npx);
    const bool noise_map = im->covinv_map != nullptr;
    const double cov_inverse = (im->background_pixel_noise == 0) ? 1.0
                               : 1.0 / (im->background_pixel_noise * im->background_pixel_noise);
    for (int t = 0; t < npx; t++) covinv[t] = noise_map ? im->covinv_map[t] : cov_inverse;
    CK(dalloc(&c->d_xvals, nx + 1), "alloc"); CK(dalloc(&c->d_yvals, ny + 1), "alloc");
    CK(dalloc(&c->d_data, npx), "alloc"); CK(dalloc(&c->d_covinv, npx), "alloc");
    CK(dalloc(&c->d_psf, (size_t)psf->nx * psf->ny), "alloc");
    CK(dalloc(&c->d_mpix, c->mpix.size()), "alloc");
    CK(cudaMemcpy(c->d_xvals, im->xvals, sizeof(double) * (nx + 1), cudaMemcpyHostToDevice), "h2d");
    CK(cudaMemcpy(c->d_yvals, im->yvals, sizeof(double) * (ny + 1), cudaMemcpyHostToDevice), "h2d");
    CK(cudaMemcpy(c->d_data, im->surface_brightness, sizeof(double) * npx, cudaMemcpyHostToDevice), "h2d");
    CK(cudaMemcpy(c->d_covinv, covinv.data(), sizeof(double) * npx, cudaMemcpyHostToDevice), "h2d");
    CK(cudaMemcpy(c->d_psf, psf->matrix, sizeof(double) * psf->nx * psf->ny, cudaMemcpyHostToDevice), "h2d");
    if (!c->mpix.empty())
        CK(cudaMemcpy(c->d_mpix, c->mpix.data(), sizeof(int) * c->mpix.size(), cudaMemcpyHostToDevice), "h2d");

    StaticData& sd = c->sd;
    sd.nx = nx; sd.ny = ny;
    sd.n_mask = (int)c->mpix.size();
    sd.nsplit = opts->nsplit;
    sd.nsub = opts->nsplit * opts->nsplit;
    sd.n_sub = sd.n_mask * sd.nsub;
    sd.pnx = psf->nx; sd.pny = psf->ny;
    // default PSF-to-X schedule: the dense window of image rows pays off once
    // the footprint work dominates (measured: 31x31 PSFs gain, 21x21 lose on
    // an annular mask); the autotuner can override it
    if (c->psfx_mode < 0) c->psfx_mode = (psf->nx * psf->ny >= 500) ? 1 : 0;
    sd.use_noise_map = noise_map ? 1 : 0;
    sd.cov_inverse = cov_inverse;
    c->bg_noise = im->background_pixel_noise;
    sd.xvals = c->d_xvals; sd.yvals = c->d_yvals; sd.data = c->d_data; sd.covinv = c->d_covinv;
    sd.mpix = c->d_mpix; sd.psf = c->d_psf;
    {
        double psum = 0, cmax = 0;
        for (int t = 0; t < psf->nx * psf->ny; t++) psum += fabs(psf->matrix[t]);
        for (int t = 0; t < npx; t++) cmax = std::max(cmax, covinv[t]);
        const double xmax = 4.0 * std::max(psum, 1e-30) * std::max(sqrt(cmax), 1e-30);
        sd.x_exp = std::max(-60, std::min(60, (int)floor(log2(16384.0 / xmax))));
        // the taps on the grid 2^-T with sum |tap| <= 2^30 (each rounded tap
        // then stays below 2^31)
        const int T = std::max(0, std::min(70, 30 - (int)ceil(log2(std::max(psum, 1e-30)))));
        sd.fix_exp_x = T + PSFX_LEXP;
        const int pnx = psf->nx, pny = psf->ny;
        std::vector<int> pi((size_t)pnx * pny);
        for (int pl = 0; pl < pny; pl++)
            for (int pk = 0; pk < pnx; pk++)
                pi[(size_t)pl * pnx + pk] = (int)llrint(ldexp(psf->matrix[(size_t)pk * pny + pl], T));
        CK(dalloc(&c->d_psf_int, pi.size()), "alloc");
        CK(cudaMemcpy(c->d_psf_int, pi.data(), sizeof(int) * pi.size(), cudaMemcpyHostToDevice), "h2d");
        sd.psf_int = c->d_psf_int;
    }

    SrcOpts& so = c->so;
    so.snx = opts->npixels_x; so.sny = opts->npixels_y;
    so.auto_grid = opts->auto_sourcegrid;
    so.xmin = opts->xmin; so.xmax = opts->xmax; so.ymin = opts->ymin; so.ymax = opts->ymax;
    so.lxmin = opts->limit_xmin; so.lxmax = opts->limit_xmax; so.lymin = opts->limit_ymin; so.lymax = opts->limit_ymax;
    so.noise_threshold = opts->noise_threshold;
    so.size_scale = opts->size_scale;
    so.regularization = opts->regularization;
    so.regparam = opts->regparam;

    psf_init_attributes();
    linalg_init_attributes();
    sparseops_init_attributes();
    sur_exact_init_attributes();
    int snx = std::max(so.snx, 2), sny = std::max(so.sny, 2);
    return ensure_slot(c, 0, sd.n_mask, snx * sny, snx, sny);
}

void ctx_free(qlp_ctx* c)
{
    for (Slot& s : c->slots) {
        free_slot(s);
        if (s.stream) cudaStreamDestroy(s.stream);
        if (s.done) cudaEventDestroy(s.done);
        if (s.side) cudaStreamDestroy(s.side);
        if (s.side_fork) cudaEventDestroy(s.side_fork);
        if (s.side_join) cudaEventDestroy(s.side_join);
    }
    c->slots.clear();
    void* ptrs[] = {c->d_xvals, c->d_yvals, c->d_data, c->d_covinv, c->d_psf, c->d_psf_int, c->d_mpix, c->d_inst_mpix,
                    c->d_emask, c->d_inmask, c->d_epix, c->d_eoff};
    for (void* p : ptrs) if (p) cudaFree(p);
    if (c->h_out) cudaFreeHost(c->h_out);
    if (c->h_ep) cudaFreeHost(c->h_ep);
    if (c->h_trial) cudaFreeHost(c->h_trial);
    for (int i = 0; i <= QLP_N_STAGES; i++) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->join) cudaEventDestroy(c->join);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
}

static int build_lens_model(qlp_ctx* c, const double* lens_params, LensModel& lm)
{
    if (c->lenses.empty()) { set_error("%s (%d)", "no lens model set", 0); return QLP_ERR_ARG; }
    memset(&lm, 0, sizeof(lm));
    lm.nlens = (int)c->lenses.size();
    lm.n_planes = c->planes.n_planes;
    for (int i = 0; i < QLP_MAX_PLANES; i++) {
        lm.zfac[i] = c->planes.zfac[i];
        for (int j = 0; j < QLP_MAX_PLANES; j++) lm.beta[i][j] = c->planes.beta[i][j];
    }
    int off = 0;
    for (int k = 0; k < lm.nlens; k++) {
        const qlp_lens& d = c->lenses[k];
        const double* p = lens_params ? lens_params + off : d.p;
        int r = make_lens_rec(lm.lens[k], d, p);
        lm.lens[k].tol = c->nfw_tol;
        if (r != QLP_OK) { set_error("%s (lens %d)", "unsupported lens parameters", k); return r; }
        off += n_params_of(d.type);
    }
    return QLP_OK;
}

static bool model_has_nfw(const qlp_ctx* c)
{
    for (const qlp_lens& l : c->lenses)
        if (is_nfw_type(l.type)) return true;
    return false;
}

// The launch sequence of one evaluation on stream st with the workspace of
// `slot`; sd / so size the launches (the evaluation's own mask and source
// grid, or the slot's capacity when the sequence is captured for replay).
// Everything that changes between evaluations (lens model, regularisation
// parameter, mask and source-grid size) is read from the slot's EvalParams in
// device memory, so one captured sequence serves every evaluation the slot
// runs.  ev (QLP_N_STAGES+1 events, or null) brackets the stages.  part:
// PIPE_ALL the whole evaluation; PIPE_PRE / PIPE_TRIAL the lambda-independent
// part and one lambda trial of the regularisation-parameter optimisation.
static int run_pipeline(qlp_ctx* c, Slot& slot, const StaticData& sd_in, const SrcOpts& so_in, cudaStream_t st,
                        cudaEvent_t* ev, int part)
{
    StaticData sd = sd_in;
    SrcOpts so = so_in;
    Work& w = slot.w;
    sd.shape = &w.ep->shape;
    const int Mc = slot.M_cap;
    const int N_max = sd.n_mask;
    const double* regp = regparam_dev(w);
    const bool mixed = (c->precision == QLP_MIXED);
    if (part == PIPE_TRIAL) {
        if (mixed) {
            int r = run_inversion_mixed(c, slot, sd, so, regp, PIPE_TRIAL, st, nullptr);
            if (r != QLP_OK) return r;
        } else {
            const size_t bytes = sizeof(double) * (size_t)w.ldF * Mc;
            cudaMemsetAsync(&w.gs->not_spd_F, 0, sizeof(int), st);
            cudaMemcpyAsync(w.F, w.F0, bytes, cudaMemcpyDeviceToDevice, st);
            launch_regularization(so, w, Mc, regp, REG_F, st);
            launch_cholesky_fp64(w.F, w.ldF, Mc, w.gs, 0, w.linv, st);
            launch_logdet(w.F, w.ldF, Mc, w, 0, st);
            launch_solve_fp64(w, Mc, st);
        }
        launch_model_chi2(sd, so, w, N_max, Mc, regp, st, mixed);
        if (c->osb_on) launch_outside_sb(sd, so, c->osb, slot.osb, model_has_nfw(c), w, st);
        return QLP_OK;
    }
    cudaMemsetAsync(w.out, 0, sizeof(EvalOut), st);
    if (ev) cudaEventRecord(ev[0], st);
    if (c->nfw_mode == QLP_NFW_SURROGATE && model_has_nfw(c)) {
        // a single NFW lens on the last plane: its quadrature fallbacks can run
        // afterwards in their own kernel (nothing downstream needs them)
        int defer = -1, n_nfw = 0;
        for (int k = 0; k < (int)c->lenses.size(); k++)
            if (is_nfw_type(c->lenses[k].type)) { n_nfw++; defer = k; }
        if (n_nfw != 1 || c->lenses[defer].plane != c->planes.n_planes - 1) defer = -1;
        int r = launch_raytrace_sur(sd, w, c->nfw_threshold, defer, st);
        if (r != QLP_OK) return r;
    } else {
        launch_raytrace(sd, model_has_nfw(c), w, c->ray_threads, st);
    }
    if (ev) cudaEventRecord(ev[1], st);
    launch_grid(sd, so, w, st);
    if (c->nfw_mode == QLP_NFW_SURROGATE && model_has_nfw(c)) {
        // rays whose surrogate error could flip a grid decision are traced
        // again exactly: first those that could set the grid's extremes (and
        // the grid is laid out again), then those near a cell's lines
        double zmax = 0;
        for (int p = 0; p < c->planes.n_planes; p++) zmax = std::max(zmax, std::fabs(c->planes.zfac[p]));
        const double eps_g = 2.0 * c->nfw_threshold * zmax + 1e-12;
        launch_surrogate_exact(sd, so, w, eps_g, 0, st);
        launch_grid(sd, so, w, st);
        launch_surrogate_exact(sd, so, w, eps_g, 1, st);
    }
    launch_locate(sd, so, w, st);
    launch_compact(sd, so, w, st);
    launch_build_L(sd, so, w, st);
    launch_rowpix(sd, w, st);
    if (ev) cudaEventRecord(ev[2], st);
    launch_dvec(sd, w, N_max, st);
    if (mixed) {
        int r = run_inversion_mixed(c, slot, sd, so, regp, part, st, ev);
        if (r != QLP_OK) return r;
        if (part == PIPE_PRE) return QLP_OK;
    } else {
        int r = ensure_fp64_mats(slot);
        if (r != QLP_OK) return r;
        launch_psf(sd, so, w, Mc, st);
        launch_D(w, N_max, Mc, st);
        if (ev) cudaEventRecord(ev[3], st);
        launch_syrk_fp64(sd, w, N_max, Mc, st);
        if (ev) cudaEventRecord(ev[4], st);
        if (part == PIPE_PRE)
            cudaMemcpyAsync(w.F0, w.F, sizeof(double) * (size_t)w.ldF * Mc, cudaMemcpyDeviceToDevice, st);
        launch_regularization(so, w, Mc, regp, part == PIPE_PRE ? REG_R : (REG_F | REG_R), st);
        if (so.regularization) {
            launch_cholesky_fp64(w.R, w.ldF, Mc, w.gs, 1, w.linv, st);
            launch_logdet(w.R, w.ldF, Mc, w, 1, st);
        }
        if (part == PIPE_PRE) return QLP_OK;
        launch_cholesky_fp64(w.F, w.ldF, Mc, w.gs, 0, w.linv, st);
        launch_logdet(w.F, w.ldF, Mc, w, 0, st);
        launch_solve_fp64(w, Mc, st);
    }
    if (ev) cudaEventRecord(ev[5], st);
    launch_model_chi2(sd, so, w, N_max, Mc, regp, st, mixed);
    if (c->osb_on) launch_outside_sb(sd, so, c->osb, slot.osb, model_has_nfw(c), w, st);
    if (ev) cudaEventRecord(ev[6], st);
    return QLP_OK;
}

// Make the slot's workspace ready for the pipeline without allocating during
// a stream capture.
static int ensure_osb(qlp_ctx* c, Slot& s)
{
    if (!c->osb_on || (s.osb.sp && s.osb_nsub >= c->osb.nsub_e)) return QLP_OK;
    OsbWork& o = s.osb;
    cudaFree(o.sp); cudaFree(o.cell3); cudaFree(o.w3); cudaFree(o.model); cudaFree(o.act); cudaFree(o.sb);
    o = OsbWork{};
    const size_t n = (size_t)std::max(c->osb.nsub_e, 1), np = (size_t)c->nx * c->ny;
    CK(dalloc(&o.sp, 2 * n), "alloc osb");
    CK(cudaMalloc((void**)&o.cell3, sizeof(int) * 3 * n), "alloc osb");
    CK(dalloc(&o.w3, 3 * n), "alloc osb");
    CK(dalloc(&o.model, np), "alloc osb");
    CK(cudaMalloc((void**)&o.act, sizeof(int) * np), "alloc osb");
    CK(dalloc(&o.sb, np), "alloc osb");
    s.osb_nsub = c->osb.nsub_e;
    return QLP_OK;
}

static int prepare_slot(qlp_ctx* c, Slot& s)
{
    {
        int e = ensure_osb(c, s);
        if (e != QLP_OK) return e;
    }
    const bool regopt = c->regopt && c->so.regularization;
    if (c->precision == QLP_MIXED) return regopt ? mixed_ensure_f0(s) : mixed_init(s);
    int r = ensure_fp64_mats(s);
    if (r == QLP_OK && regopt && !s.w.F0) CK(dalloc(&s.w.F0, (size_t)s.M_cap * s.M_cap), "alloc F0");
    return r;
}

// Capture the slot's launch sequence, sized for its capacity, as a graph.
static int capture_graph(qlp_ctx* c, Slot& s, const StaticData& sd, const SrcOpts& so, const int key[7], int part)
{
    const bool trial = (part == PIPE_TRIAL);
    cudaGraphExec_t& slot_graph = trial ? s.graph_trial : s.graph;
    if (slot_graph) cudaGraphExecDestroy(slot_graph);
    slot_graph = nullptr;
    int r = prepare_slot(c, s);
    if (r != QLP_OK) return r;
    const long long l0 = kernel_launch_counter();
    CK(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal), "capture");
    r = run_pipeline(c, s, sd, so, s.stream, nullptr, part);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s.stream, &g);
    const long long n = kernel_launch_counter() - l0;
    count_launches((int)-n);            // nothing ran yet: replays count them
    if (r != QLP_OK) { if (g) cudaGraphDestroy(g); return r; }
    if (e != cudaSuccess || !g) return cuda_fail(e, "stream capture");
    e = cudaGraphInstantiate(&slot_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { slot_graph = nullptr; return cuda_fail(e, "graph instantiate"); }
    for (int i = 0; i < 7; i++) (trial ? s.trial_key : s.graph_key)[i] = key[i];
    (trial ? s.trial_gen : s.graph_gen) = c->graph_gen;
    (trial ? s.trial_launches : s.graph_launches) = n;
    return QLP_OK;
}

// One evaluation on slot s: upload its parameters, run (replay or launch) the
// sequence, copy its result to *h_dst -- all asynchronous on the slot stream.
static int issue_eval(qlp_ctx* c, Slot& s, const StaticData& sd, const SrcOpts& so, const EvalParams* h_ep,
                      EvalOut* h_dst, cudaEvent_t* ev, int part = PIPE_ALL)
{
    if (part == PIPE_TRIAL)      // a lambda trial changes lambda only
        CK(cudaMemcpyAsync(&s.w.ep->regparam, &h_ep->regparam, sizeof(double), cudaMemcpyHostToDevice, s.stream),
           "h2d");
    else
        CK(cudaMemcpyAsync(s.w.ep, h_ep, sizeof(EvalParams), cudaMemcpyHostToDevice, s.stream), "h2d");
    if (c->use_graphs && ev == nullptr) {
        // one graph per slot for every mask and source grid that fits its
        // capacity: the launches are sized for the capacity, the kernels read
        // the actual sizes from the EvalParams just uploaded
        StaticData sdc = sd;
        sdc.n_mask = s.N_cap;
        sdc.n_sub = s.N_cap * sd.nsub;
        SrcOpts soc = so;
        soc.snx = s.snx_cap;
        soc.sny = s.sny_cap;
        const int key[7] = {c->precision, s.N_cap, s.snx_cap, s.sny_cap, model_has_nfw(c) ? 1 : 0, c->nfw_mode,
                            part};
        const bool trial = (part == PIPE_TRIAL);
        const cudaGraphExec_t have = trial ? s.graph_trial : s.graph;
        const int* have_key = trial ? s.trial_key : s.graph_key;
        bool ok = have && (trial ? s.trial_gen : s.graph_gen) == c->graph_gen;
        for (int i = 0; ok && i < 7; i++) ok = (have_key[i] == key[i]);
        if (!ok) {
            int r = capture_graph(c, s, sdc, soc, key, part);
            if (r != QLP_OK) return r;
        }
        CK(cudaGraphLaunch(trial ? s.graph_trial : s.graph, s.stream), "graph launch");
        count_launches((int)(trial ? s.trial_launches : s.graph_launches));
    } else {
        int r = prepare_slot(c, s);
        if (r != QLP_OK) return r;
        r = run_pipeline(c, s, sd, so, s.stream, ev, part);
        if (r != QLP_OK) return r;
    }
    if (part != PIPE_PRE)
        CK(cudaMemcpyAsync(h_dst, s.w.out, sizeof(EvalOut), cudaMemcpyDeviceToHost, s.stream), "d2h");
    return QLP_OK;
}

static void fill_result(const EvalOut& o, qlp_result* out)
{
    memset(out, 0, sizeof(*out));
    out->chisq0 = o.chisq0;
    out->logdet_F = o.logdet_F;
    out->logdet_R = o.logdet_R;
    out->Es_times_two = o.Es_times_two;
    out->regterms = o.regterms;
    out->m2logev = o.m2logev;
    out->n_active_pixels = o.n_active_pixels;
    out->n_active_src = o.n_active_src;
    out->L_nnz = o.L_nnz;
    out->status = o.status;
    out->refine_iters = o.refine_iters;
    out->nfw_fallbacks = o.pad;
    out->nfw_exact_rays = o.n_exact;
    out->outside_sb_penalty = o.osb_penalty;
}

static int ensure_results(qlp_ctx* c, int n)
{
    if (!c->h_trial) CK(cudaMallocHost((void**)&c->h_trial, sizeof(EvalOut) * QLP_MAX_SLOTS), "pinned");
    if ((int)c->regopt_lam.size() < n) { c->regopt_lam.resize(n); c->regopt_evals.resize(n); }
    if (c->h_out_cap < n) {
        if (c->h_out) cudaFreeHost(c->h_out);
        c->h_out = nullptr;
        CK(cudaMallocHost((void**)&c->h_out, sizeof(EvalOut) * n), "pinned");
        c->h_out_cap = n;
    }
    if (c->h_ep_cap < n) {
        if (c->h_ep) cudaFreeHost(c->h_ep);
        c->h_ep = nullptr;
        CK(cudaMallocHost((void**)&c->h_ep, sizeof(EvalParams) * n), "pinned");
        c->h_ep_cap = n;
    }
    return QLP_OK;
}

// The regularisation-parameter optimisation of the batch instances inst[j]
// (j = 0 .. k-1), instance inst[j] on slot j (QLens's 'optimize_regparam on':
// QLens::optimize_regularization_parameter, pixelgrid.cpp:15865-15890).  Each
// slot runs its instance's lambda-independent part once, then Brent's method
// over log10(lambda) (brent.h) advances all instances in lockstep: one lambda
// trial per instance per round, launched on every slot before the host waits
// for them.  The trial with the least objective (QLens::chisq_regparam_dense,
// pixelgrid.cpp:16526-16700: chi^2 over the active pixels + regularisation
// terms + log det F) gives the instance's result, as the reference keeps the
// amplitudes and log det F of its best trial; its lambda goes to regopt_lam.
static int regopt_wave(qlp_ctx* c, const std::vector<int>& inst, const std::vector<StaticData>& sds,
                       const std::vector<SrcOpts>& sos)
{
    const int k = (int)inst.size();
    for (int j = 0; j < k; j++) {
        int r = issue_eval(c, c->slots[j], sds[j], sos[j], &c->h_ep[inst[j]], nullptr, nullptr, PIPE_PRE);
        if (r != QLP_OK) return r;
    }
    std::vector<BrentMin> br(k);
    std::vector<double> best(k, INFINITY);
    std::vector<char> act(k);
    for (int j = 0; j < k; j++) br[j].reset(c->regopt_minlog, c->regopt_maxlog, c->regopt_tol, c->regopt_maxit);
    while (true) {
        bool any = false;
        for (int j = 0; j < k; j++) {
            double x;
            act[j] = br[j].want(&x);
            if (!act[j]) continue;
            EvalParams& ep = c->h_ep[inst[j]];
            ep.regparam = pow(10.0, x);
            int r = issue_eval(c, c->slots[j], sds[j], sos[j], &ep, &c->h_trial[j], nullptr, PIPE_TRIAL);
            if (r != QLP_OK) return r;
            any = true;
        }
        if (!any) break;
        for (int j = 0; j < k; j++)
            if (act[j]) CK(cudaStreamSynchronize(c->slots[j].stream), "lambda trial");
        for (int j = 0; j < k; j++) {
            if (!act[j]) continue;
            const double f = c->h_trial[j].f_regopt;
            if (f < best[j]) {
                best[j] = f;
                c->h_out[inst[j]] = c->h_trial[j];
                c->regopt_lam[inst[j]] = c->h_ep[inst[j]].regparam;
            }
            br[j].give(f);
        }
    }
    for (int j = 0; j < k; j++) c->regopt_evals[inst[j]] = br[j].evals();
    return QLP_OK;
}

// Single evaluation: slot 0, launched directly (not replayed) so that the
// stage events bracket each part of the pipeline.
int ctx_eval(qlp_ctx* c, const double* lens_params, double regparam, qlp_result* out)
{
    memset(out, 0, sizeof(*out));
    cudaSetDevice(c->device);
    if (c->so.snx < 2 || c->so.sny < 2) {
        out->m2logev = 2e30; out->status = QLP_ERR_GRID_TOO_SMALL;
        return QLP_ERR_GRID_TOO_SMALL;
    }
    int r = ensure_results(c, 1);
    if (r != QLP_OK) return r;
    EvalParams& ep = c->h_ep[0];
    r = build_lens_model(c, lens_params, ep.lm);
    if (r != QLP_OK) { out->status = r; return r; }
    ep.regparam = (regparam > 0) ? regparam : c->opts.regparam;
    ep.shape = InstShape{c->sd.mpix, c->sd.n_mask, c->sd.n_sub, c->so.snx, c->so.sny};
    Slot& s = c->slots[0];
    long long l0 = kernel_launch_counter();
    cudaStream_t st = c->stream;
    CK(cudaEventRecord(c->fork, st), "event");
    CK(cudaStreamWaitEvent(s.stream, c->fork, 0), "wait");
    if (c->regopt && c->so.regularization) {
        // lambda optimisation: the pre part and the trials, timed as a whole
        CK(cudaEventRecord(c->ev[0], s.stream), "event");
        r = regopt_wave(c, {0}, {c->sd}, {c->so});
        if (r != QLP_OK) { out->status = r; return r; }
        for (int i = 1; i <= QLP_N_STAGES; i++) CK(cudaEventRecord(c->ev[i], s.stream), "event");
        CK(cudaEventRecord(s.done, s.stream), "event");
        CK(cudaStreamWaitEvent(st, s.done, 0), "wait");
        CK(cudaStreamSynchronize(st), "eval");
        c->last_launches = kernel_launch_counter() - l0;
        c->last_h2d = sizeof(EvalParams) + sizeof(double) * c->regopt_evals[0];
        c->last_d2h = sizeof(EvalOut) * c->regopt_evals[0];
        for (int i = 0; i < QLP_N_STAGES; i++) c->stage_ms[i] = 0;
        cudaEventElapsedTime(&c->device_ms, c->ev[0], c->ev[QLP_N_STAGES]);
        fill_result(c->h_out[0], out);
        if (c->precision == QLP_MIXED) out->refine_iters = c->refine;
        out->regparam = c->regopt_lam[0];
        out->regopt_evals = c->regopt_evals[0];
        return out->status;
    }
    r = issue_eval(c, s, c->sd, c->so, &ep, &c->h_out[0], c->ev);
    if (r != QLP_OK) { out->status = r; return r; }
    CK(cudaEventRecord(s.done, s.stream), "event");
    CK(cudaStreamWaitEvent(st, s.done, 0), "wait");
    CK(cudaGetLastError(), "launch");
    CK(cudaStreamSynchronize(st), "eval");
    c->last_launches = kernel_launch_counter() - l0;
    c->last_h2d = sizeof(EvalParams);
    c->last_d2h = sizeof(EvalOut);
    for (int i = 0; i < QLP_N_STAGES; i++) cudaEventElapsedTime(&c->stage_ms[i], c->ev[i], c->ev[i + 1]);
    cudaEventElapsedTime(&c->device_ms, c->ev[0], c->ev[QLP_N_STAGES]);
    fill_result(c->h_out[0], out);
    if (c->precision == QLP_MIXED) out->refine_iters = c->refine;
    out->regparam = ep.regparam;
    return out->status;
}

// Free the workspaces of slots keep, keep+1, ... (slot 0 always stays).
void ctx_trim_slots(qlp_ctx* c, int keep)
{
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (int k = std::max(keep, 1); k < (int)c->slots.size(); k++) free_slot(c->slots[k]);
}

int ctx_set_masks(qlp_ctx* c, const unsigned char* masks, int n_masks)
{
    cudaSetDevice(c->device);
    std::vector<int> all;
    c->mask_off.clear(); c->mask_cnt.clear();
    size_t npx = (size_t)c->nx * c->ny;
    for (int k = 0; k < n_masks; k++) {
        std::vector<int> v = masked_list(masks + k * npx, c->nx, c->ny);
        c->mask_off.push_back((int)all.size());
        c->mask_cnt.push_back((int)v.size());
        all.insert(all.end(), v.begin(), v.end());
    }
    // captured graphs stay valid: the mask pointers travel in EvalParams
    if (c->d_inst_mpix) { cudaFree(c->d_inst_mpix); c->d_inst_mpix = nullptr; }
    CK(dalloc(&c->d_inst_mpix, all.size()), "alloc");
    if (!all.empty())
        CK(cudaMemcpy(c->d_inst_mpix, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice), "h2d");
    return QLP_OK;
}

// Batched evaluation: instance i runs on slot i % S, each slot on its own
// stream, forked from and joined back into the context stream, with one host
// synchronisation for the whole batch.
int ctx_eval_batch(qlp_ctx* c, const double* params, const double* regparams, const qlp_instance* inst, int n,
                   qlp_result* out)
{
    cudaSetDevice(c->device);
    if (n == 0) return QLP_OK;
    const int np = [&] { int s = 0; for (auto& l : c->lenses) s += n_params_of(l.type); return s; }();
    int nmask_max = (int)c->mpix.size(), cells_max = c->so.snx * c->so.sny, snx_max = c->so.snx, sny_max = c->so.sny;
    for (int i = 0; i < n && inst; i++) {
        if (inst[i].mask_id >= (int)c->mask_cnt.size()) {
            set_error("%s %d", "bad mask id", inst[i].mask_id);
            return QLP_ERR_ARG;
        }
        if (inst[i].mask_id >= 0 && c->osb_on) {
            set_error("%s %d", "the outside-surface-brightness prior uses the image mask; refused mask id",
                      inst[i].mask_id);
            return QLP_ERR_ARG;
        }
        if (inst[i].mask_id >= 0) nmask_max = std::max(nmask_max, c->mask_cnt[inst[i].mask_id]);
        if (inst[i].src_npixels_x < 2 || inst[i].src_npixels_y < 2) continue;
        cells_max = std::max(cells_max, inst[i].src_npixels_x * inst[i].src_npixels_y);
        snx_max = std::max(snx_max, inst[i].src_npixels_x);
        sny_max = std::max(sny_max, inst[i].src_npixels_y);
    }
    // slot count: bounded by the batch, the configured maximum and memory
    int S = std::min(n, std::max(1, std::min(c->max_slots, QLP_MAX_SLOTS)));
    for (int k = 0; k < S; k++) {
        int r = ensure_slot(c, k, nmask_max, cells_max, std::max(snx_max, 2), std::max(sny_max, 2));
        if (r == QLP_OK && c->precision == QLP_MIXED) r = mixed_init(c->slots[k]);
        if (r != QLP_OK) {
            if (k == 0) return r;
            free_slot(c->slots[k]);
            cudaGetLastError();
            S = k;
            break;
        }
    }
    int r = ensure_results(c, n);
    if (r != QLP_OK) return r;
    const bool timed = !c->use_graphs && !(c->regopt && c->so.regularization);  // stage events: direct launches
    const int ne = QLP_N_STAGES + 1;
    while (timed && (int)c->ev_pool.size() < ne * n) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e), "event");
        c->ev_pool.push_back(e);
    }
    cudaStream_t st0 = c->stream;
    long long l0 = kernel_launch_counter();
    CK(cudaEventRecord(c->fork, st0), "event");
    for (int k = 0; k < S; k++) CK(cudaStreamWaitEvent(c->slots[k].stream, c->fork, 0), "wait");
    std::vector<int> pre(n, QLP_OK);
    int rc = QLP_OK;
    // lambda optimisation: instances go in waves of S, one per slot
    const bool regopt = c->regopt && c->so.regularization;
    std::vector<int> wave;
    std::vector<StaticData> wave_sd;
    std::vector<SrcOpts> wave_so;
    for (int i = 0; i < n; i++) {
        Slot& s = c->slots[i % S];
        EvalParams& ep = c->h_ep[i];
        int ri = build_lens_model(c, params + (size_t)i * np, ep.lm);
        ep.regparam = (regparams && regparams[i] > 0) ? regparams[i] : c->opts.regparam;
        StaticData sd = c->sd;
        SrcOpts so = c->so;
        if (inst) {
            if (inst[i].mask_id >= 0) {
                const int mask_id = inst[i].mask_id;
                sd.mpix = c->d_inst_mpix + c->mask_off[mask_id];
                sd.n_mask = c->mask_cnt[mask_id];
                sd.n_sub = sd.n_mask * sd.nsub;
            }
            if (inst[i].src_npixels_x > 0) { so.snx = inst[i].src_npixels_x; so.sny = inst[i].src_npixels_y; }
        }
        if (ri == QLP_OK && (so.snx < 2 || so.sny < 2)) ri = QLP_ERR_GRID_TOO_SMALL;
        ep.shape = InstShape{sd.mpix, sd.n_mask, sd.n_sub, so.snx, so.sny};
        c->regopt_lam[i] = ep.regparam;
        c->regopt_evals[i] = 0;
        if (ri == QLP_OK && regopt) {
            wave.push_back(i);
            wave_sd.push_back(sd);
            wave_so.push_back(so);
        } else if (ri == QLP_OK) {
            ri = issue_eval(c, s, sd, so, &ep, &c->h_out[i], timed ? &c->ev_pool[(size_t)ne * i] : nullptr);
        }
        if (regopt && ((int)wave.size() == S || (i == n - 1 && !wave.empty()))) {
            const int rw = regopt_wave(c, wave, wave_sd, wave_so);
            if (rw != QLP_OK) return rw;
            wave.clear(); wave_sd.clear(); wave_so.clear();
        }
        pre[i] = ri;
        if (ri != QLP_OK && rc == QLP_OK) rc = ri;
    }
    for (int k = 0; k < S; k++) {
        CK(cudaEventRecord(c->slots[k].done, c->slots[k].stream), "event");
        CK(cudaStreamWaitEvent(st0, c->slots[k].done, 0), "wait");
    }
    CK(cudaEventRecord(c->join, st0), "event");
    CK(cudaGetLastError(), "launch");
    CK(cudaStreamSynchronize(st0), "batch");
    c->last_launches = kernel_launch_counter() - l0;
    c->last_h2d = (long long)n * sizeof(EvalParams);
    c->last_d2h = (long long)n * sizeof(EvalOut);
    for (int k = 0; k < QLP_N_STAGES; k++) c->stage_ms[k] = 0;
    for (int i = 0; timed && i < n; i++) {
        if (pre[i] != QLP_OK) continue;
        for (int k = 0; k < QLP_N_STAGES; k++) {
            float t = 0;
            cudaEventElapsedTime(&t, c->ev_pool[(size_t)ne * i + k], c->ev_pool[(size_t)ne * i + k + 1]);
            c->stage_ms[k] += t;
        }
    }
    cudaEventElapsedTime(&c->device_ms, c->fork, c->join);
    for (int i = 0; i < n; i++) {
        if (pre[i] != QLP_OK) {
            memset(&out[i], 0, sizeof(out[i]));
            out[i].status = pre[i];
            out[i].m2logev = (pre[i] == QLP_ERR_GRID_TOO_SMALL) ? 2e30 : 0;
            continue;
        }
        fill_result(c->h_out[i], &out[i]);
        if (c->precision == QLP_MIXED) out[i].refine_iters = c->refine;
        out[i].regparam = c->regopt_lam[i];
        out[i].regopt_evals = c->regopt_evals[i];
    }
    return rc;
}

// The outside-surface-brightness prior's tables: the extended-mask pixels in
// the reference's j-outer / i-inner order with their sub-pixel offsets (the
// mask's pixels split nsplit ways, the others ens ways, set_nsplits,
// pixelgrid.cpp:10898-10938).
int ctx_set_outside_sb(qlp_ctx* c, int on, double frac, double noise_frac, const unsigned char* emask, int ens)
{
    cudaSetDevice(c->device);
    if (on && (ens < 1 || ens > 16 || !(frac >= 0))) {
        set_error("%s (%d)", "bad outside-surface-brightness settings", ens);
        return QLP_ERR_ARG;
    }
    c->graph_gen++;                    // the pass is part of the captured sequence
    c->osb_on = 0;
    if (!on) return QLP_OK;
    const int nx = c->nx, ny = c->ny;
    std::vector<unsigned char> em((size_t)nx * ny, 1), in((size_t)nx * ny, 0);
    if (emask) for (size_t t = 0; t < em.size(); t++) em[t] = emask[t] ? 1 : 0;
    for (int p : c->mpix) in[p] = 1;
    std::vector<int> epix, eoff;
    long o = 0;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const int t = i * ny + j;
            if (!em[t]) continue;
            const int ns = in[t] ? c->sd.nsplit : ens;
            epix.push_back(t);
            eoff.push_back((int)o);
            o += (long)ns * ns;
        }
    eoff.push_back((int)o);
    if (o > (1L << 30)) { set_error("%s (%d)", "extended mask too large", 0); return QLP_ERR_ARG; }
    void* old[] = {c->d_emask, c->d_inmask, c->d_epix, c->d_eoff};
    for (void* p : old) if (p) cudaFree(p);
    c->d_emask = c->d_inmask = nullptr;
    c->d_epix = c->d_eoff = nullptr;
    CK(cudaMalloc((void**)&c->d_emask, em.size()), "alloc");
    CK(cudaMalloc((void**)&c->d_inmask, in.size()), "alloc");
    CK(cudaMalloc((void**)&c->d_epix, sizeof(int) * std::max<size_t>(epix.size(), 1)), "alloc");
    CK(cudaMalloc((void**)&c->d_eoff, sizeof(int) * eoff.size()), "alloc");
    CK(cudaMemcpy(c->d_emask, em.data(), em.size(), cudaMemcpyHostToDevice), "h2d");
    CK(cudaMemcpy(c->d_inmask, in.data(), in.size(), cudaMemcpyHostToDevice), "h2d");
    if (!epix.empty()) CK(cudaMemcpy(c->d_epix, epix.data(), sizeof(int) * epix.size(), cudaMemcpyHostToDevice), "h2d");
    CK(cudaMemcpy(c->d_eoff, eoff.data(), sizeof(int) * eoff.size(), cudaMemcpyHostToDevice), "h2d");
    OsbStatic& os = c->osb;
    os.emask = c->d_emask;
    os.inmask = c->d_inmask;
    os.epix = c->d_epix;
    os.eoff = c->d_eoff;
    os.ne = (int)epix.size();
    os.nsub_e = (int)o;
    os.ens = ens;
    os.frac = frac;
    os.noise_frac = noise_frac;
    os.bg_noise = c->bg_noise;
    c->osb_on = 1;
    return QLP_OK;
}

int ctx_dump(qlp_ctx* c, double* srcpt_xy, int* L_rowptr, int* L_index, double* L_value, int* active_index,
             double* D, double* s, double* model)
{
    cudaSetDevice(c->device);
    Work& w = c->slots[0].w;
    GridState gs;
    CK(cudaMemcpy(&gs, w.gs, sizeof(gs), cudaMemcpyDeviceToHost), "d2h");
    const int nsub = c->sd.n_sub;
    if (srcpt_xy) {
        std::vector<double> x(nsub), y(nsub);
        CK(cudaMemcpy(x.data(), w.spx, sizeof(double) * nsub, cudaMemcpyDeviceToHost), "d2h");
        CK(cudaMemcpy(y.data(), w.spy, sizeof(double) * nsub, cudaMemcpyDeviceToHost), "d2h");
        for (int t = 0; t < nsub; t++) { srcpt_xy[2 * t] = x[t]; srcpt_xy[2 * t + 1] = y[t]; }
    }
    if (L_rowptr) CK(cudaMemcpy(L_rowptr, w.rowptr, sizeof(int) * (gs.N + 1), cudaMemcpyDeviceToHost), "d2h");
    if (L_index) CK(cudaMemcpy(L_index, w.Lidx, sizeof(int) * gs.nnz, cudaMemcpyDeviceToHost), "d2h");
    if (L_value) CK(cudaMemcpy(L_value, w.Lval, sizeof(double) * gs.nnz, cudaMemcpyDeviceToHost), "d2h");
    if (active_index)
        CK(cudaMemcpy(active_index, w.active_index, sizeof(int) * gs.snx * gs.sny, cudaMemcpyDeviceToHost), "d2h");
    if (D) CK(cudaMemcpy(D, w.D, sizeof(double) * gs.M, cudaMemcpyDeviceToHost), "d2h");
    if (s) CK(cudaMemcpy(s, w.s, sizeof(double) * gs.M, cudaMemcpyDeviceToHost), "d2h");
    if (model) CK(cudaMemcpy(model, w.model, sizeof(double) * gs.N, cudaMemcpyDeviceToHost), "d2h");
    return QLP_OK;
}

int ctx_dump_Lpsf(qlp_ctx* c, int rows, double* out)
{
    cudaSetDevice(c->device);
    Work& w = c->slots[0].w;
    GridState gs;
    CK(cudaMemcpy(&gs, w.gs, sizeof(gs), cudaMemcpyDeviceToHost), "d2h");
    if (rows > gs.N) rows = gs.N;
    if (rows <= 0 || gs.M <= 0 || !w.Lpsf) return QLP_OK;
    CK(cudaMemcpy2D(out, sizeof(double) * gs.M, w.Lpsf, sizeof(double) * w.ldL, sizeof(double) * gs.M, rows,
                    cudaMemcpyDeviceToHost), "d2h");
    return QLP_OK;
}

}  // namespace qlpix
