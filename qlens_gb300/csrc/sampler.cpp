// sampler.cpp -- sampler-side batching: the speculative first-accept search.
//
// The reference's samplers evaluate one candidate at a time inside a
// rejection loop: the nested sampler draws points until one beats the worst
// live point (UCMC::MonoSample, mcmchdr.cpp:3063-3098 and 3192-3248), and the
// Metropolis-type samplers (UCMC::MetHas, mcmchdr.cpp:439-483) keep their
// state until a proposal is accepted.  While candidates are being rejected the
// sampler's state does not change, so the next K candidates can be drawn
// before any of them is evaluated, evaluated together in one batched call, and
// examined in draw order: the first accepted one is the one the one-at-a-time
// loop would have accepted, provided that everything random about candidate i
// is drawn when it is proposed.  The candidates drawn after it are discarded
// and the caller's random state is wound back to just after the accepted
// draw (the rewind callback), so the run continues exactly as the serial loop
// would have.  With MPI the reference does the same across process groups,
// one candidate per group, accepting the first in group order
// (mcmchdr.cpp:3076-3090).
//
// K adapts to the acceptance rate seen so far (kept by the caller in
// qlp_search_state): the smallest K whose chance of holding an accepted
// candidate is 90%, within [k_min, k_max].
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>
#include "qlpix_ctx.h"

using namespace qlpix;

namespace {

using BatchEval = std::function<int(const double* params, const double* regparams, int n, qlp_result* out)>;

int batch_size(const qlp_search_state* st, int k_min, int k_max)
{
    const double p = st->accept_rate;
    int k = k_max;
    if (p > 0 && p < 1) k = (int)std::ceil(std::log(0.1) / std::log1p(-p));
    else if (p >= 1) k = 1;
    return std::max(k_min, std::min(k_max, k));
}

int search(const BatchEval& eval, int np, qlp_propose_fn propose, qlp_accept_fn accept, qlp_rewind_fn rewind,
           void* user, int k_min, int k_max, long max_candidates, qlp_search_state* st, long* accepted)
{
    if (!propose || !accept || !st || !accepted || np < 0 || k_min < 1 || k_max < k_min || max_candidates < 1) {
        set_error("%s (%d)", "bad speculative search arguments", 0);
        return QLP_ERR_ARG;
    }
    *accepted = -1;
    std::vector<double> P((size_t)k_max * std::max(np, 1)), lam(k_max);
    std::vector<qlp_result> res(k_max);
    long next = 0;                                    // index of the next candidate to propose
    while (next < max_candidates) {
        int k = batch_size(st, k_min, k_max);
        k = (int)std::min<long>(k, max_candidates - next);
        for (int i = 0; i < k; i++) {
            lam[i] = 0.0;
            if (propose(user, next + i, &P[(size_t)i * np], &lam[i]) != 0) {
                set_error("%s (%d)", "the proposal callback stopped the search", 0);
                return QLP_ERR_ARG;
            }
        }
        const int e = eval(P.data(), lam.data(), k, res.data());
        if (e != QLP_OK && e != QLP_ERR_NOT_SPD && e != QLP_ERR_NO_SOURCE_PIXELS && e != QLP_ERR_GRID_TOO_SMALL)
            return e;
        st->proposed += k;
        st->evaluated += k;
        st->batches++;
        for (int i = 0; i < k; i++) {
            const int a = accept(user, next + i, &res[i]);
            if (a < 0) {
                set_error("%s (%d)", "the acceptance callback stopped the search", a);
                return QLP_ERR_ARG;
            }
            // examined candidates update the rate: i + 1 trials, one success
            if (a > 0) {
                st->accepted++;
                st->examined += i + 1;
                st->accept_rate = (double)st->accepted / (double)st->examined;
                *accepted = next + i;
                if (i + 1 < k && rewind) rewind(user, next + i + 1);     // candidates past it are discarded
                st->discarded += k - (i + 1);
                return QLP_OK;
            }
        }
        st->examined += k;
        st->accept_rate = (double)std::max<long>(st->accepted, 0) / (double)st->examined;
        next += k;
    }
    return QLP_OK;                                    // no candidate accepted within max_candidates
}

}  // namespace

extern "C" {

int qlp_speculative_search(qlp_ctx* c, qlp_propose_fn propose, qlp_accept_fn accept, qlp_rewind_fn rewind,
                           void* user, int k_min, int k_max, long max_candidates, qlp_search_state* st,
                           long* accepted)
{
    if (!c) return QLP_ERR_ARG;
    const int np = qlp_n_params(c);
    BatchEval ev = [c](const double* p, const double* lam, int n, qlp_result* out) {
        return ctx_eval_batch(c, p, lam, nullptr, n, out);
    };
    return search(ev, np, propose, accept, rewind, user, k_min, k_max, max_candidates, st, accepted);
}

int qlp_speculative_search_fn(qlp_batch_eval_fn eval, void* eval_user, int n_params, qlp_propose_fn propose,
                              qlp_accept_fn accept, qlp_rewind_fn rewind, void* user, int k_min, int k_max,
                              long max_candidates, qlp_search_state* st, long* accepted)
{
    if (!eval) return QLP_ERR_ARG;
    BatchEval ev = [eval, eval_user](const double* p, const double* lam, int n, qlp_result* out) {
        return eval(eval_user, p, lam, n, out);
    };
    return search(ev, n_params, propose, accept, rewind, user, k_min, k_max, max_candidates, st, accepted);
}

}  // extern "C"
