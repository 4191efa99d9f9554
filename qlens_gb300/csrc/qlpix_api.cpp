// qlpix_api.cpp -- host runtime and C ABI of libqlpix (see include/qlpix.h).
//
// The host side keeps QLens's set-up semantics: the image pixel grid and mask
// of ImagePixelData/ImagePixelGrid (pixelgrid.cpp:9622-9700, 9940-10099), the
// lens meta-parameters of update_meta_parameters (profile.cpp:1625-1689,
// models.cpp:101-108, 2212-2224) evaluated with the host libm exactly as the
// reference evaluates them, and the sentinel returns of
// QLens::invert_image_surface_brightness_map (lens.cpp:12293-13195).
// Everything per evaluation runs on one CUDA stream with no host round trip
// until the final scalars are copied back.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <atomic>
#include <algorithm>
#include "qlpix_internal.h"
#include "qlpix_ctx.h"
#include "brent.h"

namespace qlpix {

static std::atomic<long long> g_launches{0};
void count_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long kernel_launch_counter() { return g_launches.load(); }

static thread_local std::string t_err;
void set_error(const char* fmt, const char* a, int code)
{
    char buf[512];
    snprintf(buf, sizeof(buf), fmt, a, code);
    t_err = buf;
}

static const double QL_HALFPI = 1.57079632679;                 // mathexpr.h:10
static double deg2rad(double t) { return 0.017453292519943295 * t; }  // mathexpr.h:27

int n_params_of(int type)
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

bool is_nfw_type(int type)
{
    return type == QLP_LENS_NFW || type == QLP_LENS_NFW_M200_C || type == QLP_LENS_NFW_M200_RS;
}

static const double QL_4PI = 12.5663706144;                    // mathexpr.h:14

// ks and rs of an NFW lens given by its mass: NFW::set_ks_rs_from_m200_c200
// (pmode 1) and NFW::set_ks_c200_from_m200_rs (pmode 2), models.cpp:959-976,
// in the reference's operation order (pow(., 0.333333333333), not cbrt).
static int nfw_from_mass(const qlp_lens& d, const double* p, double& ks, double& rs)
{
    const double m200 = p[0];
    if (!(m200 > 0) || !(d.sigma_cr > 0) || !(d.kpc_to_arcsec > 0) || !(d.critical_density > 0)) return QLP_ERR_ARG;
    const double rvir_kpc = pow(m200 / (200.0 * QL_4PI / 3.0 * 1e-9 * d.critical_density), 0.333333333333);
    double c200, rs_kpc;
    if (d.type == QLP_LENS_NFW_M200_C) {
        c200 = p[1];
        if (!(c200 > 0)) return QLP_ERR_ARG;
        rs_kpc = rvir_kpc / c200;
        rs = rs_kpc * d.kpc_to_arcsec;
    } else {
        rs_kpc = p[1];
        if (!(rs_kpc > 0)) return QLP_ERR_ARG;
        rs = rs_kpc * d.kpc_to_arcsec;
        c200 = rvir_kpc / rs_kpc;
    }
    ks = m200 / (QL_4PI * rs * rs * d.sigma_cr * (log(1 + c200) - c200 / (1 + c200)));
    return QLP_OK;
}

// LensProfile::set_angle with orient_major_axis_north (profile.cpp:1625-1637)
static void set_angle(LensRec& L, double theta_deg)
{
    double theta = deg2rad(theta_deg);
    double c = cos(theta), s = sin(theta);
    L.sintheta = c;
    L.costheta = -s;
}

int make_lens_rec(LensRec& L, const qlp_lens& d, const double* p)
{
    memset(&L, 0, sizeof(L));
    int type = d.type;
    L.type = type;
    L.plane = d.plane;
    double nfw_p[2];
    if (type == QLP_LENS_NFW_M200_C || type == QLP_LENS_NFW_M200_RS) {
        // the device sees an ordinary (ks, rs) NFW lens
        int r = nfw_from_mass(d, p, nfw_p[0], nfw_p[1]);
        if (r != QLP_OK) return r;
        type = L.type = QLP_LENS_NFW;
    }
    if (type == QLP_LENS_SPLE) {
        L.b = p[0]; L.alpha = p[1]; L.s = p[2]; L.q = p[3];
        if (L.s < 0) L.s = -L.s;
        if (!(L.q > 0) || L.q > 1) return QLP_ERR_ARG;
        set_angle(L, p[4]);
        L.xc = p[5]; L.yc = p[6];
        double f = 1.0 / sqrt(L.q);         // emode 1 (profile.cpp:1686-1689)
        L.bprime = L.b * f;
        L.sprime = L.s * f;
        L.qsq = L.q * L.q;
        L.ssq = L.sprime * L.sprime;
        if (L.q == 1.0) L.kind = 0;
        else if (L.alpha == 1.0) L.kind = 1;
        else if (L.s == 0.0) L.kind = 2;
        else return QLP_ERR_ARG;           // cored power law, q<1: quadrature, not supported here
    } else if (type == QLP_LENS_SHEAR) {
        double theta_eff = deg2rad(p[1]) + QL_HALFPI;
        L.shear1 = p[0] * cos(2 * theta_eff);
        L.shear2 = p[0] * sin(2 * theta_eff);
        L.xc = p[2]; L.yc = p[3];
    } else if (type == QLP_LENS_NFW) {
        if (d.type == QLP_LENS_NFW) { L.ks = p[0]; L.rs = p[1]; }
        else { L.ks = nfw_p[0]; L.rs = nfw_p[1]; }
        L.q = p[2];
        if (!(L.q > 0) || L.q > 1 || !(L.rs > 0)) return QLP_ERR_ARG;
        set_angle(L, p[3]);
        L.xc = p[4]; L.yc = p[5];
        L.f_major_axis = 1.0 / sqrt(L.q);
        L.qsq = L.q * L.q;
        L.epsilon = 1 - L.qsq;
    } else {
        return QLP_ERR_ARG;
    }
    return QLP_OK;
}

template <typename T>
static cudaError_t dalloc(T** p, size_t n)
{
    return cudaMalloc((void**)p, sizeof(T) * (n > 0 ? n : 1));
}

}  // namespace qlpix

namespace qlpix {
int spd_solve_logdet_noalloc(const double* F, int n, int ld, const double* D, double* s, double* logdet,
                             void* stream, std::string& err);
}

using namespace qlpix;

static int fail(int code, const char* msg)
{
    t_err = msg;
    return code;
}

extern "C" {

void qlp_srcgrid_defaults(qlp_srcgrid_opts* o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->nsplit = 2;                      // default_imgpixel_nsplit (lens.cpp:497)
    o->npixels_x = o->npixels_y = 20;
    o->auto_sourcegrid = 1;             // lens.cpp:390
    o->xmin = -1; o->xmax = 1; o->ymin = -1; o->ymax = 1;   // lens.cpp:377
    o->limit_xmin = -1e30; o->limit_xmax = 1e30; o->limit_ymin = -1e30; o->limit_ymax = 1e30;
    o->noise_threshold = 0;             // lens.cpp:433
    o->size_scale = 0;                  // pixelgrid.cpp:561
    o->regularization = 1;              // curvature (lens.cpp:403)
    o->regparam = 100;                  // pixelgrid.cpp:558
}

const char* qlp_last_error(void) { return t_err.c_str(); }

int qlp_set_fit_params(qlp_ctx* c, const qlp_fit_param* fp, int n)
{
    if (!c || (n > 0 && !fp) || n < 0) return fail(QLP_ERR_ARG, "bad fit parameters");
    if (fit_set(c, fp, n) != QLP_OK) return fail(QLP_ERR_ARG, "bad fit parameter (target, transform or prior)");
    return QLP_OK;
}

int qlp_fit_terms(const qlp_fit_param* fp, int n, const double* x, double* transformed, int* penalised,
                  double* terms)
{
    if (!fp || n < 1 || !x || !transformed || !penalised || !terms) return fail(QLP_ERR_ARG, "bad arguments");
    return fit_terms(fp, n, x, transformed, penalised, terms);
}

int qlp_fit_loglike_batch(qlp_ctx* c, const double* x, int n, double* loglike, qlp_result* out)
{
    if (!c || !x || n < 1 || !loglike) return fail(QLP_ERR_ARG, "bad arguments");
    if (c->fit.empty()) return fail(QLP_ERR_ARG, "no fit parameters set (qlp_set_fit_params)");
    return fit_loglike_batch(c, x, n, loglike, out);
}

long long qlp_last_launch_count(const qlp_ctx* ctx) { return ctx ? ctx->last_launches : 0; }

qlp_ctx* qlp_create(const qlp_image* im, const qlp_psf* psf, const qlp_srcgrid_opts* opts, int device, int* status)
{
    int st_dummy;
    if (!status) status = &st_dummy;
    *status = QLP_OK;
    if (!im || !im->xvals || !im->yvals || !im->surface_brightness || !im->in_mask) {
        *status = fail(QLP_ERR_NO_DATA, "no image data");
        return nullptr;
    }
    if (!psf || !psf->matrix || psf->nx < 1 || psf->ny < 1 || !opts || opts->nsplit < 1 ||
        im->npixels_x < 1 || im->npixels_y < 1) {
        *status = fail(QLP_ERR_ARG, "bad image/psf/options");
        return nullptr;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
        *status = fail(QLP_ERR_NO_DEVICE, "no CUDA device available");
        return nullptr;
    }
    qlp_ctx* c = new qlp_ctx();
    c->device = device;
    cudaSetDevice(device);
    int code = ctx_init(c, im, psf, opts);
    if (code != QLP_OK) {
        ctx_free(c);
        delete c;
        *status = code;
        return nullptr;
    }
    return c;
}

int qlp_set_lens_model(qlp_ctx* c, const qlp_lens* lenses, int nlens, const qlp_planes* planes)
{
    if (!c || !lenses || nlens <= 0 || nlens > QLP_MAX_LENSES) return fail(QLP_ERR_ARG, "bad lens model");
    c->lenses.assign(lenses, lenses + nlens);
    memset(&c->planes, 0, sizeof(c->planes));
    if (planes) c->planes = *planes;
    else { c->planes.n_planes = 1; c->planes.zfac[0] = 1.0; }
    if (c->planes.n_planes < 1 || c->planes.n_planes > QLP_MAX_PLANES) return fail(QLP_ERR_ARG, "bad planes");
    for (int k = 0; k < nlens; k++)
        if (lenses[k].plane < 0 || lenses[k].plane >= c->planes.n_planes || n_params_of(lenses[k].type) == 0)
            return fail(QLP_ERR_ARG, "bad lens type or plane");
    c->graph_gen++;     // captured graphs select kernels by the lens list (NFW, deferred fallback)
    return QLP_OK;
}

int qlp_set_batch_slots(qlp_ctx* c, int slots)
{
    if (!c || slots < 1 || slots > QLP_MAX_SLOTS) return fail(QLP_ERR_ARG, "bad slot count");
    c->max_slots = slots;
    return QLP_OK;
}

int qlp_set_graphs(qlp_ctx* c, int on)
{
    if (!c) return fail(QLP_ERR_ARG, "null context");
    c->use_graphs = on ? 1 : 0;
    return QLP_OK;
}

int qlp_set_regparam_optimization(qlp_ctx* c, int on, double minlog, double maxlog, double tol, int max_iter)
{
    if (!c) return fail(QLP_ERR_ARG, "null context");
    if (on && !(minlog < maxlog && tol > 0 && max_iter >= 1)) return fail(QLP_ERR_ARG, "bad lambda optimisation range");
    c->regopt = on ? 1 : 0;
    if (on) {
        c->regopt_minlog = minlog;
        c->regopt_maxlog = maxlog;
        c->regopt_tol = tol;
        c->regopt_maxit = max_iter;
    }
    c->graph_gen++;     // the captured sequences split into a lambda-independent part and trials
    return QLP_OK;
}

int qlp_brent_min(double (*f)(double, void*), void* user, double ax, double bx, double tol, int max_iter,
                  double* xmin, int* evals)
{
    if (!f || !xmin || !(ax < bx) || max_iter < 0) return fail(QLP_ERR_ARG, "bad Brent arguments");
    qlpix::BrentMin b(ax, bx, tol, max_iter);
    double x;
    while (b.want(&x)) b.give(f(x, user));
    *xmin = b.xmin();
    if (evals) *evals = b.evals();
    return QLP_OK;
}

int qlp_get_schedule(const qlp_ctx* c, qlp_schedule* out)
{
    if (!c || !out) return fail(QLP_ERR_ARG, "null argument");
    return ctx_get_schedule(c, out);
}

int qlp_set_schedule(qlp_ctx* c, const qlp_schedule* s)
{
    if (!c || !s) return fail(QLP_ERR_ARG, "null argument");
    if (ctx_set_schedule(c, s) != QLP_OK) return fail(QLP_ERR_ARG, "schedule value outside its candidate set");
    return QLP_OK;
}

int qlp_autotune(qlp_ctx* c, const double* params, const double* lambdas, const qlp_instance* inst, int n, int reps,
                 qlp_tune_report* rep)
{
    if (!c || !params) return fail(QLP_ERR_ARG, "null argument");
    return ctx_autotune(c, params, lambdas, inst, n, reps, rep);
}

int qlp_set_refinement(qlp_ctx* c, int sweeps)
{
    if (!c || sweeps < 0 || sweeps > 4) return fail(QLP_ERR_ARG, "refinement sweeps must be 0..4");
    c->refine = sweeps;
    c->graph_gen++;     // the sweeps are part of the captured sequence
    return QLP_OK;
}

int qlp_set_noise_term(qlp_ctx* c, int on)
{
    if (!c) return fail(QLP_ERR_ARG, "null context");
    c->sd.noise_term = on ? 1 : 0;
    c->graph_gen++;     // the flag is a launch argument of the captured final reduction
    return QLP_OK;
}

int qlp_set_outside_sb_prior(qlp_ctx* c, int on, double frac_threshold, double noise_frac,
                             const unsigned char* emask, int emask_nsplit)
{
    if (!c) return fail(QLP_ERR_ARG, "null context");
    return ctx_set_outside_sb(c, on, frac_threshold, noise_frac, emask, emask_nsplit);
}

int qlp_last_transfer_bytes(const qlp_ctx* c, long long* h2d, long long* d2h)
{
    if (!c || !h2d || !d2h) return fail(QLP_ERR_ARG, "bad arguments");
    *h2d = c->last_h2d;
    *d2h = c->last_d2h;
    return QLP_OK;
}

void qlp_surrogate_defaults(qlp_surrogate_opts* o)
{
    if (!o) return;
    o->n_train = 1 << 20;
    o->batch = 16384;
    o->steps = 30000;
    o->lr = 3e-3;
    o->seed = 1;
}

int qlp_nfw_surrogate_train(int device, const qlp_surrogate_opts* opts, qlp_surrogate_report* rep)
{
    qlp_surrogate_opts d;
    qlp_surrogate_defaults(&d);
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(QLP_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= n) return fail(QLP_ERR_ARG, "bad device");
    return surrogate_train(device, opts ? opts : &d, rep);
}

int qlp_set_nfw_tolerance(qlp_ctx* c, double tol)
{
    if (!c || !(tol < 1)) return fail(QLP_ERR_ARG, "bad NFW quadrature tolerance");
    c->nfw_tol = (tol > 0) ? tol : 1e-3;
    return QLP_OK;
}

int qlp_set_nfw_mode(qlp_ctx* c, int mode, double threshold_arcsec)
{
    if (!c || (mode != QLP_NFW_QUADRATURE && mode != QLP_NFW_SURROGATE)) return fail(QLP_ERR_ARG, "bad NFW mode");
    if (mode == QLP_NFW_SURROGATE && !surrogate_ready(c->device))
        return fail(QLP_ERR_ARG, "no trained NFW surrogate on this device (qlp_nfw_surrogate_train)");
    c->nfw_mode = mode;
    c->nfw_threshold = (threshold_arcsec > 0) ? threshold_arcsec : 2e-5;
    c->graph_gen++;     // the gate is a launch argument of the captured ray shooting
    return QLP_OK;
}

int qlp_surrogate_grad_check(int device, const float* params, const float* x, const float* t, int batch,
                             double* loss, float* grad)
{
    if (!params || !x || !t || !loss || !grad || batch < 1) return fail(QLP_ERR_ARG, "bad arguments");
    return surrogate_grad_check(device, params, x, t, batch, loss, grad);
}

int qlp_surrogate_eval(int device, const double* rpq, int n, double* t, double* G, double* B, double* bound)
{
    if (!rpq || !t || n < 1) return fail(QLP_ERR_ARG, "bad arguments");
    return surrogate_eval(device, rpq, n, t, G, B, bound);
}

int qlp_n_params(const qlp_ctx* c)
{
    if (!c) return 0;
    int n = 0;
    for (auto& l : c->lenses) n += n_params_of(l.type);
    return n;
}

int qlp_set_precision(qlp_ctx* c, int mode)
{
    if (!c || (mode != QLP_FP64 && mode != QLP_MIXED)) return fail(QLP_ERR_ARG, "bad precision mode");
    c->precision = mode;
    return QLP_OK;
}

int qlp_set_stream(qlp_ctx* c, void* stream)
{
    if (!c) return fail(QLP_ERR_ARG, "null context");
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return QLP_OK;
}

int qlp_eval(qlp_ctx* c, const double* lens_params, double regparam, qlp_result* out)
{
    if (!c || !out) return fail(QLP_ERR_ARG, "null argument");
    const int r = ctx_eval(c, lens_params, regparam, out);
    if (r != QLP_OK && out->status == QLP_OK) out->status = r;   // a failure before any result
    return r;
}

int qlp_set_instance_masks(qlp_ctx* c, const unsigned char* masks, int n_masks)
{
    if (!c || (n_masks > 0 && !masks) || n_masks < 0) return fail(QLP_ERR_ARG, "bad masks");
    return ctx_set_masks(c, masks, n_masks);
}

int qlp_eval_batch(qlp_ctx* c, const double* params, const double* regparams, const qlp_instance* inst, int n,
                   qlp_result* out)
{
    if (!c || !out || n < 0 || (n > 0 && !params)) return fail(QLP_ERR_ARG, "bad batch arguments");
    const int r = ctx_eval_batch(c, params, regparams, inst, n, out);
    // a failure of the batch itself (not of one instance's likelihood) leaves
    // no valid result: every instance reports it
    if (r != QLP_OK && r != QLP_ERR_NOT_SPD && r != QLP_ERR_NO_SOURCE_PIXELS && r != QLP_ERR_GRID_TOO_SMALL)
        for (int i = 0; i < n; i++) {
            memset(&out[i], 0, sizeof(out[i]));
            out[i].status = r;
        }
    return r;
}

int qlp_dump(qlp_ctx* c, double* srcpt_xy, int* L_rowptr, int* L_index, double* L_value, int* active_index,
             double* D, double* s, double* model)
{
    if (!c) return fail(QLP_ERR_ARG, "null context");
    return ctx_dump(c, srcpt_xy, L_rowptr, L_index, L_value, active_index, D, s, model);
}

int qlp_dump_Lpsf(qlp_ctx* c, int rows, double* out)
{
    if (!c || !out || rows < 0) return fail(QLP_ERR_ARG, "bad arguments");
    return ctx_dump_Lpsf(c, rows, out);
}

int qlp_stage_times(qlp_ctx* c, float* ms, int n)
{
    if (!c || !ms || n < QLP_N_STAGES) return fail(QLP_ERR_ARG, "bad arguments");
    for (int i = 0; i < QLP_N_STAGES; i++) ms[i] = c->stage_ms[i];
    return QLP_OK;
}

int qlp_last_device_time(qlp_ctx* c, float* ms)
{
    if (!c || !ms) return fail(QLP_ERR_ARG, "bad arguments");
    *ms = c->device_ms;
    return QLP_OK;
}

int qlp_spd_solve_logdet_noalloc(const double* F, int n, int ld, const double* D, double* s, double* logdet,
                                 void* stream)
{
    std::string err;
    int rc = spd_solve_logdet_noalloc(F, n, ld, D, s, logdet, stream, err);
    if (rc != QLP_OK) t_err = err;
    return rc;
}

void qlp_destroy(qlp_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    ctx_free(c);
    delete c;
}

}  // extern "C"
