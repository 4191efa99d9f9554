"""The launch-schedule autotuner (qlp_autotune): it times the caller's sample
batch under candidate schedules (slots, ray-shooting CTA size, PSF-to-X CTA
size and split) and keeps the fastest.  No schedule changes a result, which
the tuner itself checks on the sample and these tests check across explicitly
set schedules, for uniform and uneven batches."""
import numpy as np
import pytest

from goldens import Golden

pytestmark = pytest.mark.gpu

CANDIDATES = {"slots": {1, 2, 3, 4, 8, 16, 32, 48, 64}, "ray_threads": {64, 128, 256},
              "psfx_threads": {128, 256, 512}, "psfx_split": {1, 2, 4}, "psfx_mode": {0, 1}}


def _ctx(g, precision):
    from qlens_gb300 import PixelLikelihood
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    return pl


def _draws(g, n, seed):
    rng = np.random.default_rng(seed)
    P = np.tile(np.array(g.params()), (n, 1))
    P[:, 0] *= rng.uniform(0.95, 1.05, n)
    P[:, 3] = rng.uniform(0.6, 0.95, n)
    return P


KEYS = ("m2logev", "chisq0", "logdet_F", "logdet_R", "n_active_src", "L_nnz", "status")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_schedules_give_identical_results(precision):
    from qlens_gb300 import abi
    g = Golden("powerlaw")
    pl = _ctx(g, abi.QLP_MIXED if precision == "mixed" else abi.QLP_FP64)
    P = _draws(g, 6, 3)
    ref = None
    for sched in ({"slots": 2, "ray_threads": 256, "psfx_threads": 256, "psfx_split": 1, "psfx_mode": 0},
                  {"slots": 4, "ray_threads": 64, "psfx_threads": 512, "psfx_split": 4, "psfx_mode": 1},
                  {"slots": 3, "ray_threads": 128, "psfx_threads": 128, "psfx_split": 2, "psfx_mode": 0},
                  {"slots": 2, "ray_threads": 256, "psfx_threads": 256, "psfx_split": 1, "psfx_mode": 1}):
        pl.set_schedule(**sched)
        assert pl.schedule() == sched
        res = pl.eval_batch(P)
        if ref is None:
            ref = res
        for a, b in zip(res, ref):
            for k in KEYS:
                assert a[k] == b[k], (sched, k, a[k], b[k])
    with pytest.raises(Exception):
        pl.set_schedule(psfx_split=3)
    with pytest.raises(Exception):
        pl.set_schedule(psfx_mode=2)
    pl.close()


def test_autotune_uneven_batch():
    from qlens_gb300 import abi, synthetic
    g = Golden("tiny_sie")
    pl = _ctx(g, abi.QLP_MIXED)
    xv, yv = g.arr["xvals"], g.arr["yvals"]
    masks = np.stack([synthetic.annulus_mask(xv, yv, 0.2, r).ravel() for r in (0.8, 1.0, 1.2)])
    pl.set_instance_masks(masks)
    rng = np.random.default_rng(8)
    n = 24
    P = _draws(g, n, 5)
    ids = rng.integers(0, 3, n)
    sizes = np.stack([rng.integers(5, 11, n)] * 2, axis=1)
    lam = 10.0 ** rng.uniform(0, 2, n)
    before = pl.eval_batch(P, regparams=lam, mask_ids=ids, src_sizes=sizes)
    rep = pl.autotune(P, regparams=lam, mask_ids=ids, src_sizes=sizes, reps=2)
    print("autotune:", rep["best"], "%.3f -> %.3f ms in %d trials" % (rep["start_ms"], rep["best_ms"], rep["n_trials"]))
    assert rep["n_trials"] >= 5
    assert rep["best_ms"] <= rep["start_ms"]
    assert rep["best"] == pl.schedule()
    for k, v in rep["best"].items():
        assert v in CANDIDATES[k], (k, v)
    assert min(t["ms"] for t in rep["trials"]) == rep["best_ms"]
    after = pl.eval_batch(P, regparams=lam, mask_ids=ids, src_sizes=sizes)
    for a, b in zip(before, after):
        for k in KEYS:
            assert a[k] == b[k], (k, a[k], b[k])
    pl.close()
