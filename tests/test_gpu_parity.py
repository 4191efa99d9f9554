"""GPU parity of the plain FP64 path against the reference goldens and the oracle.

Tolerances (plain FP64 path):
  * pre-PSF L sparsity and source indices: identical (bit-exact integers);
  * source points and L weights: the device's atan/atanh/pow may differ from
    glibc's in the last bit, so they are compared to 1e-13 relative, and the
    fraction of bit-identical source points is reported;
  * -2 log(evidence), chi^2, log det F, log det R: 1e-6 relative (the
    reference's bar), measured agreement is ~1e-12.
"""
import numpy as np
import pytest

from goldens import CASES, Golden

pytestmark = pytest.mark.gpu

REL = 1e-6


def _gpu():
    from qlens_gb300 import PixelLikelihood
    return PixelLikelihood


def _run(g, params=None, precision=0):
    PL = _gpu()
    pl = PL.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    r = pl.invert_image_surface_brightness_map(params)
    return pl, r


def _srcpt_tol(g):
    """Bound on |source point difference| / coordinate scale.

    SPLE and shear: a few ulp (CUDA's and glibc's atan / atanh / pow differ in
    the last bit).  NFW: QLens's convergence kappa = 2 ks (1 - F(x)) / (x^2 - 1),
    F = atan(sqrt(x^2-1))/sqrt(x^2-1) or atanh(sqrt(1-x^2))/sqrt(1-x^2), cancels
    as x^2 -> 1 (the reference switches to its series only within 1e-5 of 1),
    so a one-ulp difference in atan / atanh becomes up to ~1e5 ulp of kappa at
    quadrature nodes near the scale radius; the integrals average it down
    (measured: 1.5e-14 of the coordinate scale)."""
    return 1e-12 if any(l["type"].startswith("nfw") for l in g.lenses) else 1e-14


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_golden_scalars(name):
    g = Golden(name)
    pl, r = _run(g)
    assert r["status"] == 0
    assert r["n_active_pixels"] == int(g.sc["n_active_pixels"])
    assert r["n_active_src"] == int(g.sc["n_active_src"])
    assert r["L_nnz"] == int(g.sc["L_nnz"])
    assert _rel(r["m2logev"], g.sc["m2logev"]) < REL
    assert _rel(r["chisq0"], g.sc["chisq0"]) < REL
    assert _rel(r["logdet_F"], g.sc["logdetF"]) < REL
    assert _rel(r["logdet_R"], g.sc["logdetR"]) < REL
    pl.close()


@pytest.mark.parametrize("name", CASES)
def test_golden_lensing_matrix(name):
    g = Golden(name)
    pl, r = _run(g)
    d = pl.dump(g.n_sub, r)
    rx, gx = g.sample("srcpt_x", d["srcpt"][0::2])
    ry, gy = g.sample("srcpt_y", d["srcpt"][1::2])
    ref_sp = np.stack([rx, ry], 1).ravel()
    got_sp = np.stack([gx, gy], 1).ravel()
    # beta = theta - alpha: a last-bit difference of alpha is an absolute error
    # on the scale of the coordinates, so bound it against that scale
    err = np.abs(got_sp - ref_sp)
    assert err.max() <= _srcpt_tol(g) * np.abs(ref_sp).max()
    same = np.mean(got_sp == ref_sp)
    print("%s: %.4f%% of source-point coordinates bit-identical" % (name, 100 * same))
    # identical L sparsity and indices
    assert np.array_equal(d["active_index"], g.arr["active_index"])
    assert np.array_equal(d["L_rowptr"], g.arr["L_rowptr"])
    assert np.array_equal(d["L_index"], g.arr["L_index"])
    # a last-bit change of a source point moves a weight by ~|dw/dx| ulp(x) ~ 1e-15
    rv, gv = g.sample("L_value", d["L_value"])
    assert np.allclose(gv, rv, rtol=1e-12, atol=1e-13 * _srcpt_tol(g) / 1e-14)
    assert np.allclose(d["s"], g.arr["s"], rtol=1e-6, atol=1e-9 * np.abs(g.arr["s"]).max())
    assert np.allclose(d["model"], g.arr["model"], rtol=1e-6, atol=1e-9 * np.abs(g.arr["model"]).max())
    M = r["n_active_src"]
    rows = g.arr["Lpsf_rows"].reshape(-1, M)
    Lp = pl.dump_Lpsf(rows.shape[0], M)
    assert np.allclose(Lp, rows, rtol=1e-12, atol=1e-15)
    pl.close()


def test_random_parameters_vs_oracle():
    from oracle import oracle as O
    g = Golden("powerlaw")
    rng = np.random.default_rng(11)
    PL = _gpu()
    pl = PL.from_opts(g.image, g.psf, g.opts)
    pl.set_lens_model(g.lenses, *g.zbeta())
    base = np.array(g.params())
    for trial in range(6):
        p = base.copy()
        p[0] *= rng.uniform(0.95, 1.05)              # b
        p[1] = rng.uniform(0.9, 1.2)                 # slope
        p[3] = rng.uniform(0.6, 0.95)                # q
        p[4] += rng.uniform(-20, 20)                 # theta
        p[7] = rng.uniform(0.0, 0.1)                 # shear
        r = pl.invert_image_surface_brightness_map(p)
        ro = O.evaluate(g.image, g.psf, g.opts, g.lenses, lens_params=p)
        assert r["status"] == ro["status"] == 0
        assert r["n_active_src"] == ro["n_active_src"] and r["L_nnz"] == ro["L_nnz"]
        assert _rel(r["m2logev"], ro["m2logev"]) < REL, (trial, r["m2logev"], ro["m2logev"])
        assert np.array_equal(pl.dump(g.n_sub, r)["L_index"], O.get("L_index"))
    pl.close()


@pytest.mark.parametrize("name", ["nfw", "twoplane"])
def test_random_nfw_parameters_vs_oracle(name):
    """Elliptical (and one spherical) NFW by Gauss-Patterson quadrature, single
    and two lens planes, against the oracle on the same parameter vectors."""
    from oracle import oracle as O
    g = Golden(name)
    rng = np.random.default_rng(23)
    PL = _gpu()
    pl = PL.from_opts(g.image, g.psf, g.opts)
    pl.set_lens_model(g.lenses, *g.zbeta())
    base = np.array(g.params())
    n_sub = g.n_sub
    for trial in range(5):
        p = base.copy()
        p[11] *= rng.uniform(0.5, 1.5)               # ks
        p[12] *= rng.uniform(0.6, 1.6)               # rs
        p[13] = 1.0 if trial == 4 else rng.uniform(0.5, 0.95)   # q (1: spherical branch)
        p[14] += rng.uniform(-40, 40)                # theta
        p[15] += rng.uniform(-0.1, 0.1)              # xc
        p[16] += rng.uniform(-0.1, 0.1)              # yc
        r = pl.invert_image_surface_brightness_map(p)
        ro = O.evaluate(g.image, g.psf, g.opts, g.lenses, lens_params=p, planes=g.planes())
        assert r["status"] == ro["status"] == 0
        assert r["n_active_src"] == ro["n_active_src"] and r["L_nnz"] == ro["L_nnz"]
        assert _rel(r["m2logev"], ro["m2logev"]) < REL, (trial, r["m2logev"], ro["m2logev"])
        d = pl.dump(n_sub, r)
        sp = O.get("srcpt")
        assert np.abs(d["srcpt"] - sp).max() <= _srcpt_tol(g) * np.abs(sp).max()
        assert np.array_equal(d["L_index"], O.get("L_index"))
    pl.close()


def test_sentinels():
    g = Golden("fixed_grid")
    g.opts.xmin, g.opts.xmax, g.opts.ymin, g.opts.ymax = 50.0, 51.0, 50.0, 51.0
    pl, r = _run(g)
    assert r["m2logev"] == 2e30 and r["n_active_src"] == 0
    pl.close()
    g = Golden("tiny_sie")
    g.opts.npixels_x = 1
    pl, r = _run(g)
    assert r["m2logev"] == 2e30
    pl.close()


def test_launch_count_and_stage_times():
    g = Golden("tiny_sie")
    pl, r = _run(g)
    assert pl.last_launch_count() > 10
    t = pl.stage_times()
    assert all(x >= 0 for x in t) and sum(t) > 0
    pl.close()
