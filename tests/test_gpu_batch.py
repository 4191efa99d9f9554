"""Batched evaluation (qlp_eval_batch): graph replay, slot reuse, uneven
per-instance masks and source grids.

* a batch replayed from captured CUDA graphs, the same batch launched kernel
  by kernel, and one qlp_eval per vector give identical results (the same
  kernels on the same inputs, fixed reduction orders);
* instances with their own mask and source-grid size (the cfg3 layout) agree
  with the oracle run on that mask and grid, 1e-6 relative in -2 log(evidence)
  (plain FP64) -- as nested-sampling live points evaluated in one call;
* replacing the instance masks re-captures the graphs.
"""
import numpy as np
import pytest

from goldens import Golden

pytestmark = pytest.mark.gpu

REL = 1e-6


def _ctx(g, precision):
    from qlens_gb300 import PixelLikelihood
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    return pl


def _draws(g, n, seed):
    rng = np.random.default_rng(seed)
    base = np.array(g.params())
    P = np.tile(base, (n, 1))
    P[:, 0] *= rng.uniform(0.95, 1.05, n)
    P[:, 3] = rng.uniform(0.6, 0.95, n)
    P[:, 4] += rng.uniform(-20, 20, n)
    P[:, 7] = rng.uniform(0.0, 0.1, n)
    return P


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_direct_and_single(precision):
    from qlens_gb300 import abi
    g = Golden("powerlaw")
    pl = _ctx(g, abi.QLP_MIXED if precision == "mixed" else abi.QLP_FP64)
    pl.set_batch_slots(3)                  # 7 evaluations on 3 slots: every graph is replayed
    P = _draws(g, 7, 5)
    pl.set_graphs(True)
    a = pl.eval_batch(P)
    a2 = pl.eval_batch(P[::-1].copy())[::-1]
    pl.set_graphs(False)
    b = pl.eval_batch(P)
    singles = [pl.invert_image_surface_brightness_map(p) for p in P]
    for ra, ra2, rb, rs in zip(a, a2, b, singles):
        assert ra["status"] == rb["status"] == rs["status"] == 0
        for k in ("m2logev", "chisq0", "logdet_F", "logdet_R"):
            assert ra[k] == rb[k] == rs[k] == ra2[k], k
    h2d, d2h = pl.last_transfer_bytes()
    assert h2d > 0 and d2h > 0
    pl.close()


def _instance_inputs(g, radii, inner):
    from qlens_gb300 import synthetic
    xv, yv = g.arr["xvals"], g.arr["yvals"]
    return np.stack([synthetic.annulus_mask(xv, yv, inner, r).ravel() for r in radii])


def test_uneven_masks_and_grids_vs_oracle():
    from oracle import oracle as O
    from qlens_gb300 import abi
    g = Golden("tiny_sie")
    pl = _ctx(g, abi.QLP_FP64)
    pl.set_batch_slots(4)
    masks = _instance_inputs(g, [0.8, 1.0, 1.2], 0.2)
    pl.set_instance_masks(masks)
    P = _draws(g, 6, 9)
    mask_ids = [0, 1, 2, 1, -1, 0]
    sizes = [(8, 8), (6, 7), (10, 9), (8, 8), (0, 0), (5, 5)]
    res = pl.eval_batch(P, mask_ids=mask_ids, src_sizes=sizes)
    for i in range(len(P)):
        mk = g.arr["mask"] if mask_ids[i] < 0 else masks[mask_ids[i]]
        img = abi.ImageBuffers(g.arr["xvals"], g.arr["yvals"], g.arr["data"], mk, None,
                               g.sc["background_pixel_noise"])
        o = abi.srcgrid_defaults()
        for name, _ in abi.qlp_srcgrid_opts._fields_:
            setattr(o, name, getattr(g.opts, name))
        if sizes[i][0] > 0:
            o.npixels_x, o.npixels_y = sizes[i]
        ro = O.evaluate(img, g.psf, o, g.lenses, lens_params=P[i])
        r = res[i]
        assert r["status"] == ro["status"] == 0, (i, r["status"], ro["status"])
        assert r["n_active_pixels"] == ro["n_active_pixels"] and r["n_active_src"] == ro["n_active_src"]
        assert abs(r["m2logev"] - ro["m2logev"]) <= REL * abs(ro["m2logev"]), (i, r["m2logev"], ro["m2logev"])
    # new masks: the captured graphs must follow them
    masks2 = _instance_inputs(g, [1.1, 0.9, 0.7], 0.25)
    pl.set_instance_masks(masks2)
    res2 = pl.eval_batch(P[:3], mask_ids=[0, 1, 2], src_sizes=sizes[:3])
    for i in range(3):
        img = abi.ImageBuffers(g.arr["xvals"], g.arr["yvals"], g.arr["data"], masks2[i], None,
                               g.sc["background_pixel_noise"])
        o = abi.srcgrid_defaults()
        for name, _ in abi.qlp_srcgrid_opts._fields_:
            setattr(o, name, getattr(g.opts, name))
        o.npixels_x, o.npixels_y = sizes[i]
        ro = O.evaluate(img, g.psf, o, g.lenses, lens_params=P[i])
        assert abs(res2[i]["m2logev"] - ro["m2logev"]) <= REL * abs(ro["m2logev"])
    pl.close()


def test_batch_with_nfw_and_two_planes():
    """Graph replay with the quadrature kernel and the plane recursion."""
    from oracle import oracle as O
    from qlens_gb300 import abi
    g = Golden("twoplane")
    pl = _ctx(g, abi.QLP_FP64)
    pl.set_batch_slots(2)
    rng = np.random.default_rng(4)
    P = np.tile(np.array(g.params()), (5, 1))
    P[:, 11] *= rng.uniform(0.6, 1.4, 5)
    P[:, 13] = rng.uniform(0.55, 0.95, 5)
    res = pl.eval_batch(P)
    for i in range(5):
        ro = O.evaluate(g.image, g.psf, g.opts, g.lenses, lens_params=P[i], planes=g.planes())
        assert res[i]["status"] == 0
        assert abs(res[i]["m2logev"] - ro["m2logev"]) <= REL * abs(ro["m2logev"])
    pl.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_uneven_graph_replay_matches_direct(precision):
    """One graph per slot serves every mask and source grid that fits the
    slot: launched for the capacity, the kernels take the actual sizes from
    the evaluation's parameters in device memory."""
    from qlens_gb300 import abi
    g = Golden("tiny_sie")
    pl = _ctx(g, abi.QLP_MIXED if precision == "mixed" else abi.QLP_FP64)
    pl.set_batch_slots(3)
    pl.set_instance_masks(_instance_inputs(g, [0.8, 1.0, 1.2], 0.2))
    P = _draws(g, 9, 13)
    ids = [0, 1, 2, 2, 1, 0, -1, 1, 2]
    sizes = [(8, 8), (6, 7), (10, 9), (5, 5), (9, 6), (7, 7), (0, 0), (8, 5), (6, 6)]
    lam = [10.0, 3.0, 30.0, 10.0, 50.0, 1.0, 10.0, 7.0, 20.0]
    pl.set_graphs(True)
    a = pl.eval_batch(P, regparams=lam, mask_ids=ids, src_sizes=sizes)
    a2 = pl.eval_batch(P, regparams=lam, mask_ids=ids, src_sizes=sizes)
    pl.set_graphs(False)
    b = pl.eval_batch(P, regparams=lam, mask_ids=ids, src_sizes=sizes)
    for i, (ra, ra2, rb) in enumerate(zip(a, a2, b)):
        assert ra["status"] == rb["status"] == 0, (i, ra["status"], rb["status"])
        for k in ("m2logev", "chisq0", "logdet_F", "logdet_R", "n_active_pixels", "n_active_src", "L_nnz"):
            assert ra[k] == rb[k] == ra2[k], (i, k, ra[k], rb[k])
    pl.close()
