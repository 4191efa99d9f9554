// autotune.cpp -- the launch-schedule autotuner of the batched path.
//
// A schedule (qlp_schedule) holds the knobs that change how the batched
// evaluation is launched but not what it computes: evaluations in flight
// (slots), the CTA size of the FP64 ray shooting, and the CTA size and
// image-row split of the mixed path's PSF-to-X build.  Every kernel sums in a
// fixed order whatever its CTA size or split, so all schedules give the same
// bits -- the tuner checks that on the caller's sample -- and only the time
// differs.  The best schedule depends on the workload (mask size, source-grid
// size, PSF size, lens model), which is why it is measured rather than fixed:
// the tuner runs the caller's own sample batch, times it on the device
// (fork/join events of the batch, best of `reps`), and walks the knobs one at
// a time (coordinate descent), keeping a candidate only if it is faster.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include "qlpix_ctx.h"

using namespace qlpix;

namespace {

struct Knob {
    int qlp_schedule::*field;
    std::vector<int> values;
};

void apply(qlp_ctx* c, const qlp_schedule& s)
{
    c->max_slots = s.slots;
    c->ray_threads = s.ray_threads;
    c->psfx_threads = s.psfx_threads;
    c->psfx_split = s.psfx_split;
    c->psfx_mode = s.psfx_mode;
    c->graph_gen++;          // captured graphs hold the old launch shapes
}

bool same(const qlp_schedule& a, const qlp_schedule& b)
{
    return a.slots == b.slots && a.ray_threads == b.ray_threads && a.psfx_threads == b.psfx_threads &&
           a.psfx_split == b.psfx_split && a.psfx_mode == b.psfx_mode;
}

}  // namespace

namespace qlpix {

int ctx_get_schedule(const qlp_ctx* c, qlp_schedule* out)
{
    out->slots = c->max_slots;
    out->ray_threads = c->ray_threads;
    out->psfx_threads = c->psfx_threads;
    out->psfx_split = c->psfx_split;
    out->psfx_mode = c->psfx_mode;
    return QLP_OK;
}

int ctx_set_schedule(qlp_ctx* c, const qlp_schedule* s)
{
    if (s->slots < 1 || s->slots > QLP_MAX_SLOTS) return QLP_ERR_ARG;
    if (s->ray_threads != 64 && s->ray_threads != 128 && s->ray_threads != 256) return QLP_ERR_ARG;
    if (s->psfx_threads != 128 && s->psfx_threads != 256 && s->psfx_threads != 512) return QLP_ERR_ARG;
    if (s->psfx_split != 1 && s->psfx_split != 2 && s->psfx_split != 4) return QLP_ERR_ARG;
    if (s->psfx_mode != 0 && s->psfx_mode != 1) return QLP_ERR_ARG;
    apply(c, *s);
    return QLP_OK;
}

int ctx_autotune(qlp_ctx* c, const double* params, const double* lambdas, const qlp_instance* inst, int n, int reps,
                 qlp_tune_report* rep)
{
    if (n <= 0 || reps < 1) {
        set_error("%s (%d)", "autotune needs a sample batch and reps >= 1", n);
        return QLP_ERR_ARG;
    }
    qlp_schedule start;
    ctx_get_schedule(c, &start);
    const int saved_graphs = c->use_graphs;
    c->use_graphs = 1;                 // tune the path the batches run
    std::vector<qlp_result> res(n), ref(n);
    bool have_ref = false;
    qlp_tune_report r;
    memset(&r, 0, sizeof(r));

    // one trial: warm-up batch (captures the graphs), then the best of reps
    auto measure = [&](const qlp_schedule& s, double* ms) -> int {
        apply(c, s);
        int e = ctx_eval_batch(c, params, lambdas, inst, n, res.data());
        if (e != QLP_OK && e != QLP_ERR_NOT_SPD && e != QLP_ERR_NO_SOURCE_PIXELS && e != QLP_ERR_GRID_TOO_SMALL)
            return e;
        double best = INFINITY;
        for (int k = 0; k < reps; k++) {
            e = ctx_eval_batch(c, params, lambdas, inst, n, res.data());
            if (e != QLP_OK && e != QLP_ERR_NOT_SPD && e != QLP_ERR_NO_SOURCE_PIXELS &&
                e != QLP_ERR_GRID_TOO_SMALL)
                return e;
            best = std::min(best, (double)c->device_ms);
        }
        if (!have_ref) {
            ref = res;
            have_ref = true;
        } else {
            for (int i = 0; i < n; i++)
                if (memcmp(&res[i].m2logev, &ref[i].m2logev, sizeof(double)) != 0 || res[i].status != ref[i].status) {
                    set_error("%s (%d)", "autotune: schedules disagree on the result of sample", i);
                    return QLP_ERR_ARG;
                }
        }
        *ms = best;
        if (r.n_trials < QLP_TUNE_MAX_TRIALS) {
            r.trial[r.n_trials] = s;
            r.trial_ms[r.n_trials] = best;
            r.n_trials++;
        }
        return QLP_OK;
    };

    qlp_schedule best = start;
    double best_ms = 0;
    int e = measure(best, &best_ms);
    if (e != QLP_OK) {
        apply(c, start);
        c->use_graphs = saved_graphs;
        return e;
    }
    r.start_ms = best_ms;
    const std::vector<Knob> knobs = {
        {&qlp_schedule::slots, {8, 16, 32, 48, 64}},
        {&qlp_schedule::psfx_mode, {0, 1}},
        {&qlp_schedule::psfx_threads, {128, 256, 512}},
        {&qlp_schedule::psfx_split, {1, 2, 4}},
        {&qlp_schedule::ray_threads, {64, 128, 256}},
    };
    for (const Knob& k : knobs) {
        const qlp_schedule base = best;
        for (int v : k.values) {
            qlp_schedule s = base;
            s.*(k.field) = v;
            if (same(s, base)) continue;
            // a batch of n never uses more than n slots
            if (k.field == &qlp_schedule::slots && std::min(s.slots, n) == std::min(base.slots, n)) continue;
            double ms = 0;
            e = measure(s, &ms);
            if (e == QLP_ERR_NOMEM) { cudaGetLastError(); continue; }   // that many slots do not fit
            if (e != QLP_OK) {
                apply(c, start);
                c->use_graphs = saved_graphs;
                return e;
            }
            if (ms < best_ms) {
                best = s;
                best_ms = ms;
            }
        }
    }
    apply(c, best);
    ctx_trim_slots(c, best.slots);     // release the workspaces of slots the schedule no longer uses
    c->use_graphs = saved_graphs;
    r.best = best;
    r.best_ms = best_ms;
    if (rep) *rep = r;
    return QLP_OK;
}

}  // namespace qlpix
