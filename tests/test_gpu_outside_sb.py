"""The outside-surface-brightness prior on the device (qlp_set_outside_sb_prior)
against the reference goldens and the oracle: the plain FP64 path within
1e-6 relative (penalty included), the mixed path within the stated bound
where no penalty is paid and within 1e-3 relative on the penalty (its 60th
power magnifies the amplitudes' mixed-precision error 60-fold); single
evaluations, graph-replayed batches and the lambda optimisation."""
import numpy as np
import pytest

from goldens import Golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = ["osb_tiny_sie", "osb_powerlaw"]


def _pl(g, precision):
    from qlens_gb300 import PixelLikelihood
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    pl.set_outside_sb_prior(True, g.sc["outside_sb_prior_threshold"], g.sc["outside_sb_prior_noise_frac"],
                            g.arr["emask"].reshape(g.nx, g.ny), int(g.sc["emask_nsplit"]))
    return pl


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_outside_sb_vs_reference(name, precision):
    g = Golden(name)
    base = Golden(name.replace("osb_", ""))
    pen_ref = g.sc["m2logev"] - base.sc["m2logev"]
    pl = _pl(g, precision)
    r = pl.invert_image_surface_brightness_map()
    assert r["status"] == 0
    print("%s %s: -2logev %.10g (ref %.10g), penalty %.10g (ref %.10g)" % (
        name, "fp64" if precision == 0 else "mixed", r["m2logev"], g.sc["m2logev"], r["outside_sb_penalty"], pen_ref))
    if precision == 0:
        assert abs(r["m2logev"] - g.sc["m2logev"]) <= 1e-6 * abs(g.sc["m2logev"])
        assert abs(r["outside_sb_penalty"] - pen_ref) <= 1e-6 * max(abs(pen_ref), 1.0)
    else:
        assert abs(r["outside_sb_penalty"] - pen_ref) <= 1e-3 * max(abs(pen_ref), 1.0) + 1e-9
        assert abs((r["m2logev"] - r["outside_sb_penalty"]) - base.sc["m2logev"]) < 0.2
    # batches replayed from captured graphs carry the pass
    P = np.tile(np.array(g.params()), (3, 1))
    for b in pl.eval_batch(P):
        assert b["status"] == 0
        assert abs(b["m2logev"] - r["m2logev"]) <= 1e-12 * abs(r["m2logev"]) + (0 if precision == 0 else 1e-6)
    # switched off: the plain evaluation again
    pl.set_outside_sb_prior(False)
    r0 = pl.invert_image_surface_brightness_map()
    assert r0["outside_sb_penalty"] == 0.0
    assert abs(r0["m2logev"] - base.sc["m2logev"]) <= (1e-6 * abs(base.sc["m2logev"]) if precision == 0 else 0.2)
    pl.close()


def test_outside_sb_random_draws_vs_oracle():
    """Lens parameters away from the golden's: the plain path against the
    oracle with the prior on (every pixel in the extended mask)."""
    g = Golden("osb_tiny_sie")
    from qlens_gb300 import PixelLikelihood
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=0)
    pl.set_lens_model(g.lenses, *g.zbeta())
    pl.set_outside_sb_prior(True, 0.15, -1e30, None, 1)
    rng = np.random.default_rng(4)
    p0 = np.array(g.params())
    for _ in range(4):
        p = p0 * (1 + rng.uniform(-0.03, 0.03, p0.size))
        r = pl.invert_image_surface_brightness_map(p)
        o = O.evaluate(g.image, g.psf, g.opts, g.lenses, lens_params=p, planes=g.planes(),
                       outside_sb=dict(frac=0.15, noise_frac=-1e30, emask_nsplit=1, emask=None))
        assert r["status"] == o["status"] == 0
        pen_o = float(O.get("osb_penalty")[0])
        print("penalty %.10g oracle %.10g" % (r["outside_sb_penalty"], pen_o))
        assert abs(r["outside_sb_penalty"] - pen_o) <= 1e-6 * max(abs(pen_o), 1.0)
        assert abs(r["m2logev"] - o["m2logev"]) <= 1e-6 * abs(o["m2logev"])
    pl.close()


def test_outside_sb_with_lambda_optimisation():
    g = Golden("osb_powerlaw")
    pl = _pl(g, 0)
    pl.set_regparam_optimization(True)
    r = pl.invert_image_surface_brightness_map()
    o = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), regopt=(-3.0, 5.0, 0.01, 20),
                   outside_sb=dict(frac=g.sc["outside_sb_prior_threshold"], noise_frac=-1e30, emask_nsplit=1,
                                   emask=g.arr["emask"]))
    assert r["status"] == 0
    assert abs(r["regparam"] - o["regparam"]) <= 1e-6 * o["regparam"]
    assert abs(r["m2logev"] - o["m2logev"]) <= 1e-6 * abs(o["m2logev"])
    pl.close()
