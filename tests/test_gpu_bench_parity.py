"""Parity at the sizes the benchmark times.

The reference goldens at these sizes (cfg2_draw: one draw of the 200x200
power-law workload, M = 2840; cfg5_m200: the two-plane subhalo workload at its
sampling on a 160x160 image, the subhalo given by its mass) join the plain
FP64 and mixed parity cases of test_gpu_parity.py / test_gpu_mixed.py.  Here
the paths are compared on many draws of the benchmarked workloads themselves:

* plain FP64 against the oracle on two draws of the 200x200 power-law
  workload: identical L indices, -2 log(evidence) within 1e-6 relative;
* the mixed path against the plain FP64 path on 16 draws of that workload;
* mixed precision with the NFW surrogate against the plain FP64 path with the
  NFW quadrature on 16 draws of the two-plane subhalo workload (the posterior
  region around the mock's subhalo of 1e9 M_sun, per-vector source grids
  32x32-64x64), batched as the benchmark runs it, and the surrogate path's L
  indices against the plain path's;

each with the stated bound |delta log L| < 0.1, i.e. |delta(-2 log ev)| < 0.2,
and the largest difference printed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M2_TOL = 0.2      # |delta(-2 log evidence)| = 2 |delta log L|
REL = 1e-6


def _ctx(wl, precision):
    from qlens_gb300 import PixelLikelihood
    pl = PixelLikelihood(wl.xvals, wl.yvals, wl.data, wl.mask, wl.psf, covinv=None, bg_noise=wl.noise,
                         nsplit=wl.nsplit, src_npixels=wl.src_npixels, regparam=wl.regparam, precision=precision)
    pl.set_lens_model(wl.lenses, wl.zfac, wl.beta)
    return pl


def test_cfg2_fp64_vs_oracle():
    from oracle import oracle as O
    from qlens_gb300 import abi, synthetic
    wl = synthetic.cfg2()
    pl = _ctx(wl, abi.QLP_FP64)
    img = abi.ImageBuffers(wl.xvals, wl.yvals, wl.data, wl.mask, None, wl.noise)
    psf = abi.PSFBuffer(wl.psf)
    o = abi.srcgrid_defaults()
    o.nsplit = wl.nsplit
    o.npixels_x, o.npixels_y = wl.src_npixels
    o.regparam = wl.regparam
    n_sub = wl.n_mask * wl.nsplit ** 2
    for p in wl.draw(np.random.default_rng(41), 2):
        r = pl.invert_image_surface_brightness_map(p)
        ro = O.evaluate(img, psf, o, wl.lenses, lens_params=p)
        assert r["status"] == ro["status"] == 0
        assert r["n_active_src"] == ro["n_active_src"] and r["L_nnz"] == ro["L_nnz"]
        d = pl.dump(n_sub, r)
        assert np.array_equal(d["L_rowptr"], O.get("L_rowptr"))
        assert np.array_equal(d["L_index"], O.get("L_index"))
        rel = abs(r["m2logev"] - ro["m2logev"]) / abs(ro["m2logev"])
        print("cfg2 draw: M=%d fp64 %.10f oracle %.10f rel %.2e" % (r["n_active_src"], r["m2logev"],
                                                                    ro["m2logev"], rel))
        assert rel < REL
    pl.close()


def test_cfg2_mixed_vs_fp64_16_draws():
    from qlens_gb300 import abi, synthetic
    wl = synthetic.cfg2()
    P = wl.draw(np.random.default_rng(43), 16)
    p64 = _ctx(wl, abi.QLP_FP64)
    p64.set_batch_slots(8)
    a = p64.eval_batch(P)
    p64.close()
    pmx = _ctx(wl, abi.QLP_MIXED)
    pmx.set_batch_slots(16)
    b = pmx.eval_batch(P)
    pmx.close()
    d = []
    for ra, rb in zip(a, b):
        assert ra["status"] == rb["status"] == 0
        assert ra["n_active_src"] == rb["n_active_src"]
        d.append(abs(ra["m2logev"] - rb["m2logev"]))
    print("cfg2, 16 draws (M %d-%d): |delta(-2 log ev)| max %.3e mean %.3e" % (
        min(r["n_active_src"] for r in a), max(r["n_active_src"] for r in a), max(d), np.mean(d)))
    assert max(d) < M2_TOL


@pytest.fixture(scope="module")
def surrogate():
    from qlens_gb300 import pixlike
    return pixlike.train_nfw_surrogate()


def test_cfg5_surrogate_mixed_vs_fp64_quadrature_16_draws(surrogate):
    """The benchmark's own batch (the posterior region of the two-plane
    subhalo workload, per-vector source grids): surrogate rays near a grid
    decision are traced exactly, so the active sets and L sizes equal the
    plain path's and |delta log L| stays within the bound on every draw."""
    from qlens_gb300 import abi, synthetic
    wl = synthetic.cfg5()
    rng = np.random.default_rng(47)
    P = wl.draw(rng, 16)
    _ids, sizes, _lam = wl.draw_instances(rng, 16)
    p64 = _ctx(wl, abi.QLP_FP64)
    p64.set_batch_slots(8)
    a = p64.eval_batch(P, src_sizes=sizes)
    p64.close()
    pmx = _ctx(wl, abi.QLP_MIXED)
    pmx.set_nfw_mode(abi.QLP_NFW_SURROGATE)
    pmx.set_batch_slots(16)
    b = pmx.eval_batch(P, src_sizes=sizes)
    pmx.close()
    d = []
    for ra, rb in zip(a, b):
        assert ra["status"] == rb["status"] == 0
        assert ra["nfw_fallbacks"] == 0
        assert ra["n_active_src"] == rb["n_active_src"] and ra["L_nnz"] == rb["L_nnz"]
        d.append(abs(ra["m2logev"] - rb["m2logev"]))
    print("cfg5, 16 draws (sides %s, M %d-%d, fallbacks/eval %.0f, exact rays/eval %.0f): "
          "|delta(-2 log ev)| max %.3e mean %.3e" % (
              list(sizes[:, 0]), min(r["n_active_src"] for r in a), max(r["n_active_src"] for r in a),
              np.mean([r["nfw_fallbacks"] for r in b]), np.mean([r["nfw_exact_rays"] for r in b]), max(d), np.mean(d)))
    assert max(d) < M2_TOL


def test_cfg5_surrogate_lensing_matrix_indices(surrogate):
    """Single evaluations: with the surrogate (FP64 elsewhere) the pre-PSF L
    has the plain path's row pointers and column indices exactly; only its
    weights move, by the surrogate's deflection error."""
    from qlens_gb300 import abi, synthetic
    wl = synthetic.cfg5(batch_sides=(44, 44))
    P = wl.draw(np.random.default_rng(53), 3)
    n_sub = wl.n_mask * wl.nsplit ** 2
    q = _ctx(wl, abi.QLP_FP64)
    s = _ctx(wl, abi.QLP_FP64)
    s.set_nfw_mode(abi.QLP_NFW_SURROGATE)
    for p in P:
        rq = q.invert_image_surface_brightness_map(p)
        dq = q.dump(n_sub, rq)
        rs = s.invert_image_surface_brightness_map(p)
        ds = s.dump(n_sub, rs)
        assert np.array_equal(dq["L_rowptr"], ds["L_rowptr"])
        assert np.array_equal(dq["L_index"], ds["L_index"])
        assert np.array_equal(dq["active_index"], ds["active_index"])
        print("exact rays %d; weight difference max %.2e; |delta log L| %.3e" % (
            rs["nfw_exact_rays"], np.abs(dq["L_value"] - ds["L_value"]).max(), abs(rq["m2logev"] - rs["m2logev"]) / 2))
        assert abs(rq["m2logev"] - rs["m2logev"]) < M2_TOL
    q.close()
    s.close()
