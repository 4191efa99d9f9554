"""Sampler-side batching on the device: QLens's nested sampler (restated in
qlens_gb300/samplers.py) over the pixel likelihood of the tiny_sie golden,
with three free lens parameters, run one candidate at a time and with the
speculative batched search (qlp_speculative_search over qlp_eval_batch).
The two runs must be the same run -- every dead point and likelihood value
identical, the same tries and ln Z -- and the batched one faster."""
import time

import numpy as np
import pytest

from goldens import Golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_nested_sampler_batched_equals_serial(precision):
    from qlens_gb300 import PixelLikelihood
    from qlens_gb300.samplers import NestedSampler, PixelTarget
    g = Golden("tiny_sie")
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    base = np.array(g.params())
    free = [0, 3, 4]                                   # b, q, theta of the SIE
    lo = base[free] * np.array([0.9, 0.85, 0.8])
    hi = base[free] * np.array([1.1, 1.15, 1.2])
    hi[1] = min(hi[1], 0.99)
    runs, times = {}, {}
    for batch in [(1, 1), (1, 16)]:
        ns = NestedSampler(PixelTarget(pl, base, free), lo, hi, n_live=16, seed=7, batch=batch)
        pl.eval_batch(np.tile(base, (2, 1)))           # warm-up (graph capture)
        t0 = time.perf_counter()
        runs[batch] = ns.run(max_dead=60)
        times[batch] = time.perf_counter() - t0
    a, b = runs[(1, 1)], runs[(1, 16)]
    print("serial %.3f s, batched %.3f s; %d dead points, %d tries, %d evaluated in %d batches; lnZ %.6f" % (
        times[(1, 1)], times[(1, 16)], b["count"], b["tries"], b["search"]["evaluated"], b["search"]["batches"],
        b["lnZ"]))
    assert a["count"] == b["count"] == 60
    assert a["tries"] == b["tries"] and a["lnZ"] == b["lnZ"]
    for (xa, la, _), (xb, lb, _) in zip(a["dead"], b["dead"]):
        assert np.array_equal(xa, xb) and la == lb
    assert b["search"]["batches"] < a["search"]["batches"]
    assert times[(1, 16)] < times[(1, 1)]
    pl.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_twalk_batched_equals_serial(precision):
    """QLens's T-Walk (restated in qlens_gb300/samplers.py) over the same
    pixel likelihood: its proposals batched through qlp_eval_batch give the
    one-at-a-time run (every chain state, -log L and R identical) in fewer
    device calls."""
    from qlens_gb300 import PixelLikelihood
    from qlens_gb300.samplers import PixelTarget, TWalk
    g = Golden("tiny_sie")
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    base = np.array(g.params())
    free = [0, 3, 4]
    lo = base[free] * np.array([0.95, 0.9, 0.9])
    hi = base[free] * np.array([1.05, 1.1, 1.1])
    hi[1] = min(hi[1], 0.99)
    runs, times = {}, {}
    for batch in [(1, 1), (1, 16)]:
        tw = TWalk(PixelTarget(pl, base, free), lo, hi, seed=5, batch=batch)
        pl.eval_batch(np.tile(base, (2, 1)))
        t0 = time.perf_counter()
        runs[batch] = tw.run(max_iter=300)
        times[batch] = time.perf_counter() - t0
    a, b = runs[(1, 1)], runs[(1, 16)]
    print("T-Walk: serial %.3f s, batched %.3f s; %d iterations, %d accepted, %d calls -> %d" % (
        times[(1, 1)], times[(1, 16)], b["iterations"], len(b["chain"]), a["search"]["batches"],
        b["search"]["batches"]))
    assert a["iterations"] == b["iterations"] == 300
    assert a["loglike"] == b["loglike"] and a["count"] == b["count"] and a["R"] == b["R"]
    assert all(np.array_equal(x, y) for x, y in zip(a["chains"], b["chains"]))
    assert b["search"]["batches"] < a["search"]["batches"]
    pl.close()
