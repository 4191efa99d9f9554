"""The learned NFW deflection: an MLP trained on the GPU on output of the
project's own Gauss-Patterson quadrature, run on the tensor cores inside the
ray shooting, with the quadrature as fallback.

* the training kernels' loss and gradients agree with the CPU oracle
  (oracle/mlp_oracle.c) on the same parameters and batch;
* the trained network through the tensor-core inference path reproduces the
  quadrature (tolerance 1e-10) on fresh points, and where the gate accepts it
  the deflection error stays at the gate's scale;
* the likelihood with the surrogate agrees with the quadrature path (which
  matches the reference goldens to 1e-6) within the mixed-precision bound
  |delta log L| < 0.1;
* the gain: on the two-plane subhalo workload the ray shooting is faster
  with the surrogate than with the quadrature alone, at the same source
  points to within the gate.
"""
import numpy as np
import pytest

from goldens import Golden

pytestmark = pytest.mark.gpu

NP = 50306
M2_TOL = 0.2            # |delta(-2 log evidence)|, i.e. |delta log L| < 0.1
GATE = 2e-5             # default gate (arcsec)


def _layer_slices():
    dims = [3, 128, 128, 128, 128, 2]
    out, o = [], 0
    for a, b in zip(dims[:-1], dims[1:]):
        out.append(("W", slice(o, o + a * b)))
        o += a * b
        out.append(("b", slice(o, o + b)))
        o += b
    assert o == NP
    return out


def test_training_gradients_match_oracle():
    from oracle import oracle as O
    from qlens_gb300 import pixlike
    rng = np.random.default_rng(11)
    dims = [3, 128, 128, 128, 128, 2]
    parts = []
    for a, b in zip(dims[:-1], dims[1:]):
        parts.append(rng.uniform(-1, 1, a * b) * np.sqrt(6.0 / (a + b)))
        parts.append(rng.normal(0, 0.05, b))
    p = np.concatenate(parts).astype(np.float32)
    x = rng.uniform(-1, 1, (512, 3)).astype(np.float32)
    t = rng.normal(0, 1, (512, 2)).astype(np.float32)
    loss_g, grad_g = pixlike.surrogate_grad_check(p, x, t)
    loss_o, grad_o, _ = O.mlp_loss_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    assert abs(loss_g - loss_o) <= 1e-4 * abs(loss_o), (loss_g, loss_o)
    for name, sl in _layer_slices():
        go, gg = grad_o[sl], grad_g[sl].astype(np.float64)
        err = np.linalg.norm(gg - go) / max(np.linalg.norm(go), 1e-30)
        assert err < 2e-3, (name, sl, err)


@pytest.fixture(scope="module")
def trained():
    from qlens_gb300 import pixlike
    rep = pixlike.train_nfw_surrogate(steps=20000, n_train=1 << 20, batch=16384)
    print("surrogate:", rep)
    return rep


def test_surrogate_report(trained):
    assert trained["n_params"] == NP
    assert trained["final_loss"] < 1e-3
    assert trained["val_mean_rel"] < 1e-3
    assert 0.0 < trained["cells_below_1e5"] <= 1.0


def test_gated_error_within_threshold(trained):
    from qlens_gb300 import pixlike
    rng = np.random.default_rng(21)
    n = 40000
    rho = rng.uniform(np.log(1e-4), np.log(200.0), n)
    phi = rng.uniform(0, 0.5 * np.pi, n)
    q = rng.uniform(0.45, 0.999, n)
    t, G, B, bound = pixlike.surrogate_eval(np.stack([rho, phi, q], axis=1))
    Gn = B[:, None] * np.exp(t)
    rel = np.abs(Gn - G) / np.abs(G)
    print("relative error of G: median %.2e  99%% %.2e  max %.2e" % (
        np.median(rel), np.quantile(rel, 0.99), rel.max()))
    assert np.median(rel) < 1e-4
    assert np.all(np.isfinite(bound))
    R = np.exp(rho)
    c, s = np.cos(phi), np.sin(phi)
    for ks, rs in [(0.3, 5.0), (0.1, 15.0), (0.2, 0.1)]:
        x, y = rs * R * c, rs * R * s
        ax, ay = ks * x * G[:, 0], ks * y * G[:, 1]
        ex, ey = ks * x * (Gn[:, 0] - G[:, 0]), ks * y * (Gn[:, 1] - G[:, 1])
        mag = np.hypot(ax, ay)
        acc = mag * bound <= GATE
        err = np.hypot(ex, ey)[acc]
        print("ks %.2f rs %.2f: accepted %.3f, worst accepted error %.2e arcsec, above gate %d" % (
            ks, rs, acc.mean(), err.max() if err.size else 0.0, int((err > GATE).sum())))
        assert err.size == 0 or err.max() <= 5 * GATE
        assert (err > GATE).sum() <= 1e-3 * max(err.size, 1)


def _nfw_q_index(lenses):
    o = 0
    for l in lenses:
        if l["type"].startswith("nfw"):
            return o + 2
        o += len(l["params"])
    raise ValueError("no NFW lens")


@pytest.mark.parametrize("name", ["nfw", "twoplane", "cfg5_m200"])
def test_likelihood_with_surrogate(trained, name):
    from qlens_gb300 import PixelLikelihood, abi
    g = Golden(name)
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=abi.QLP_FP64)
    pl.set_lens_model(g.lenses, *g.zbeta())
    rq = pl.invert_image_surface_brightness_map()
    assert rq["status"] == 0
    assert abs(rq["m2logev"] - g.sc["m2logev"]) <= 1e-6 * abs(g.sc["m2logev"])
    assert rq["nfw_fallbacks"] == 0
    pl.set_nfw_mode(abi.QLP_NFW_SURROGATE)
    rs = pl.invert_image_surface_brightness_map()
    assert rs["status"] == 0
    d = rs["m2logev"] - rq["m2logev"]
    print("%s: surrogate -2logev %.6f quadrature %.6f diff %.2e, fallbacks %d" % (
        name, rs["m2logev"], rq["m2logev"], d, rs["nfw_fallbacks"]))
    assert abs(d) < M2_TOL
    # a batch across NFW axis ratios, graphs replayed, against the quadrature
    P = np.tile(np.array(g.params()), (4, 1))
    P[:, _nfw_q_index(g.lenses)] = [0.6, 0.7, 0.8, 0.9]
    bs = pl.eval_batch(P)
    pl.set_nfw_mode(abi.QLP_NFW_QUADRATURE)
    bq = pl.eval_batch(P)
    for a, b in zip(bs, bq):
        assert a["status"] == b["status"] == 0
        print("  q batch: diff %.2e fallbacks %d" % (a["m2logev"] - b["m2logev"], a["nfw_fallbacks"]))
        assert abs(a["m2logev"] - b["m2logev"]) < M2_TOL
        assert b["nfw_fallbacks"] == 0
    pl.close()


def test_surrogate_gain(trained):
    """What the network gains: the ray-shooting stage of the two-plane subhalo
    workload (300x300, 4x4 split, NFW subhalo on the second plane) with and
    without it, single evaluations launched kernel by kernel with CUDA events
    around the stage, at the same source points to within the gate."""
    from qlens_gb300 import PixelLikelihood, abi, synthetic
    wl = synthetic.cfg5_fixed()
    kw = dict(covinv=None, bg_noise=wl.noise, nsplit=wl.nsplit, src_npixels=wl.src_npixels, regparam=wl.regparam)
    pl = PixelLikelihood(wl.xvals, wl.yvals, wl.data, wl.mask, wl.psf, precision=abi.QLP_MIXED, **kw)
    pl.set_lens_model(wl.lenses, wl.zfac, wl.beta)
    n_sub = wl.n_mask * wl.nsplit ** 2
    P = wl.draw(np.random.default_rng(31), 4)
    times = {}
    pts = {}
    for mode in (abi.QLP_NFW_QUADRATURE, abi.QLP_NFW_SURROGATE):
        pl.set_nfw_mode(mode)
        pl.invert_image_surface_brightness_map(P[0])        # warm-up
        tt, sp = [], []
        for p in P:
            r = pl.invert_image_surface_brightness_map(p)
            assert r["status"] == 0
            tt.append(pl.stage_times()[0])
            sp.append(pl.dump(n_sub, r)["srcpt"].copy())
        times[mode], pts[mode] = tt, sp
    tq, tsur = sum(times[abi.QLP_NFW_QUADRATURE]), sum(times[abi.QLP_NFW_SURROGATE])
    worst = max(np.abs(a - b).max() for a, b in zip(pts[abi.QLP_NFW_QUADRATURE], pts[abi.QLP_NFW_SURROGATE]))
    print("ray shooting: quadrature %.3f ms, surrogate %.3f ms (x%.2f); worst source-point difference %.2e" % (
        tq / len(P), tsur / len(P), tq / tsur, worst))
    # the surrogate is trained on the quadrature at tolerance 1e-10, the
    # likelihood path integrates to QLens's 1e-3: their difference is the
    # gate plus the looser quadrature's own error
    assert worst <= 1e-4
    assert tsur < tq
    pl.close()
