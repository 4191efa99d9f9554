// fitparam.cpp -- the sampler-facing likelihood of QLens's fit drivers:
// QLens::fitmodel_loglike_extended_source (lens.cpp:10657-10748) over the
// library's evaluation.
//
// A fit parameter vector (what simplex, Powell, T-Walk and the nested
// samplers move) is mapped to the lens parameters by QLens's ParamSettings
// (params.h): each fit parameter is inverse-transformed
// (ParamSettings::inverse_transform_parameters, params.h:722-743), checked
// against its penalty limits (1e30 outside, lens.cpp:10671-10680), written
// into its slot of the lens-parameter vector (or the regularisation
// parameter), and after the evaluation
//   -log L = (-2 log evidence) / 2 + prior terms (params.h:810-840, with the
//            fit parameters as drawn) + Jacobian terms (params.h:884-893,
//            with the transformed ones).
// Transforms: none, log10, linear, ratio.  QLens's Gaussian transform
// (through its own erfinv, GregsMathHdr.cpp:439) is refused with
// QLP_ERR_ARG.  Priors: uniform, log, Gaussian; prior_norm is QLens's
// ParamSettings::prior_norms[i] (set_prior_norms, params.h:862-878), which
// the caller computes from its prior limits.
#include <cmath>
#include <cstring>
#include <vector>
#include "qlpix_internal.h"
#include "qlpix_ctx.h"

namespace qlpix {

// Inverse transform and penalty check of one fit vector; false: penalised.
static bool fit_transform(const std::vector<qlp_fit_param>& fp, const double* x, double* t)
{
    const int n = (int)fp.size();
    bool ratio_later = false;
    for (int i = 0; i < n; i++) {
        switch (fp[i].transform) {
            case QLP_TRANSFORM_NONE: t[i] = x[i]; break;
            case QLP_TRANSFORM_LOG: t[i] = pow(10.0, x[i]); break;
            case QLP_TRANSFORM_LINEAR: t[i] = (x[i] - fp[i].b) / fp[i].a; break;
            case QLP_TRANSFORM_RATIO:
                if (fp[i].ratio_param < i) t[i] = x[i] * t[fp[i].ratio_param];
                else ratio_later = true;
                break;
        }
    }
    if (ratio_later)
        for (int i = 0; i < n; i++)
            if (fp[i].transform == QLP_TRANSFORM_RATIO) t[i] = x[i] * t[fp[i].ratio_param];
    for (int i = 0; i < n; i++)
        if (fp[i].use_penalty_limits && (t[i] < fp[i].penalty_lo || t[i] > fp[i].penalty_hi)) return false;
    return true;
}

// Prior terms (with the fit parameters x) and Jacobian terms (with the
// transformed ones t), added to loglike in QLens's order.
static double fit_prior_jacobian(const std::vector<qlp_fit_param>& fp, const double* x, const double* t,
                                 double loglike)
{
    const int n = (int)fp.size();
    double tot = 0;
    for (int i = 0; i < n; i++) {
        if (fp[i].prior == QLP_PRIOR_UNIFORM) continue;
        tot += log(fp[i].prior_norm);
        if (fp[i].prior == QLP_PRIOR_LOG) tot += log(x[i]);
        else if (fp[i].prior == QLP_PRIOR_GAUSS) {
            const double d = (x[i] - fp[i].prior_pos) / fp[i].prior_sig;
            tot += d * d / 2.0;
        }
    }
    loglike += tot;
    for (int i = 0; i < n; i++) {
        if (!fp[i].include_jacobian) continue;
        if (fp[i].transform == QLP_TRANSFORM_LOG) loglike -= log(t[i]);
        else if (fp[i].transform == QLP_TRANSFORM_RATIO) loglike += log(t[fp[i].ratio_param]);
    }
    return loglike;
}

int fit_set(qlp_ctx* c, const qlp_fit_param* fp, int n)
{
    const int np = [&] { int s = 0; for (auto& l : c->lenses) s += n_params_of(l.type); return s; }();
    for (int i = 0; i < n; i++) {
        const qlp_fit_param& f = fp[i];
        if (f.target < QLP_FIT_REGPARAM || f.target >= np) return QLP_ERR_ARG;
        if (f.transform < QLP_TRANSFORM_NONE || f.transform > QLP_TRANSFORM_RATIO) return QLP_ERR_ARG;
        if (f.transform == QLP_TRANSFORM_LINEAR && f.a == 0) return QLP_ERR_ARG;
        if (f.transform == QLP_TRANSFORM_RATIO && (f.ratio_param < 0 || f.ratio_param >= n || f.ratio_param == i ||
                                                   fp[f.ratio_param].transform == QLP_TRANSFORM_RATIO))
            return QLP_ERR_ARG;
        if (f.prior < QLP_PRIOR_UNIFORM || f.prior > QLP_PRIOR_GAUSS) return QLP_ERR_ARG;
        if (f.prior != QLP_PRIOR_UNIFORM && !(f.prior_norm > 0)) return QLP_ERR_ARG;
        if (f.prior == QLP_PRIOR_GAUSS && !(f.prior_sig > 0)) return QLP_ERR_ARG;
    }
    c->fit.assign(fp, fp + n);
    return QLP_OK;
}

int fit_loglike_batch(qlp_ctx* c, const double* x, int n, double* loglike, qlp_result* out)
{
    const int nf = (int)c->fit.size();
    if (nf == 0) return QLP_ERR_ARG;
    const int np = [&] { int s = 0; for (auto& l : c->lenses) s += n_params_of(l.type); return s; }();
    std::vector<double> base(np);
    {
        int o = 0;
        for (auto& l : c->lenses) {
            for (int k = 0; k < n_params_of(l.type); k++) base[o + k] = l.p[k];
            o += n_params_of(l.type);
        }
    }
    std::vector<double> t((size_t)n * nf), P, lam;
    std::vector<int> live;                        // vectors that pass their penalty limits
    for (int i = 0; i < n; i++) {
        if (!fit_transform(c->fit, x + (size_t)i * nf, &t[(size_t)i * nf])) continue;
        live.push_back(i);
        std::vector<double> p = base;
        double reg = c->opts.regparam;
        for (int k = 0; k < nf; k++) {
            const double v = t[(size_t)i * nf + k];
            if (c->fit[k].target == QLP_FIT_REGPARAM) reg = v;
            else p[c->fit[k].target] = v;
        }
        P.insert(P.end(), p.begin(), p.end());
        lam.push_back(reg);
    }
    std::vector<qlp_result> res(live.size());
    int rc = QLP_OK;
    if (!live.empty()) {
        rc = ctx_eval_batch(c, P.data(), lam.data(), nullptr, (int)live.size(), res.data());
        if (rc != QLP_OK && rc != QLP_ERR_NOT_SPD && rc != QLP_ERR_NO_SOURCE_PIXELS && rc != QLP_ERR_GRID_TOO_SMALL &&
            rc != QLP_ERR_ARG)
            return rc;
    }
    size_t k = 0;
    for (int i = 0; i < n; i++) {
        qlp_result r;
        memset(&r, 0, sizeof(r));
        double ll = 1e30;                                    // QLens's penalty (lens.cpp:10677)
        if (k < live.size() && live[k] == i) {
            r = res[k++];
            if (r.status == QLP_ERR_ARG) ll = 1e30;            // a lens the model rejects: update_model's penalty
            else ll = fit_prior_jacobian(c->fit, x + (size_t)i * nf, &t[(size_t)i * nf], r.m2logev / 2);
        }
        if (out) out[i] = r;
        loglike[i] = ll;
    }
    return QLP_OK;
}

int fit_terms(const qlp_fit_param* fp, int n, const double* x, double* t, int* penalised, double* terms)
{
    std::vector<qlp_fit_param> f(fp, fp + n);
    const bool ok = fit_transform(f, x, t);
    *penalised = ok ? 0 : 1;
    *terms = ok ? fit_prior_jacobian(f, x, t, 0.0) : 0.0;
    return QLP_OK;
}

}  // namespace qlpix
