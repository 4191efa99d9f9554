"""The pixel-noise normalisation (QLens 'include_noise_term_in_loglike on',
lens.cpp:13033-13043) on the device against the oracle, with a noise map
(tiny_sie) and with uniform noise (noise_tiny_sie), through the plain FP64
path (1e-6 relative) and the mixed path (|delta log L| < 0.1), single
evaluations and a graph-replayed batch."""
import numpy as np
import pytest

from goldens import Golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = ["tiny_sie", "noise_tiny_sie"]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_noise_term_vs_oracle(name, precision):
    from qlens_gb300 import PixelLikelihood
    g = Golden(name)
    want = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), noise_term=True)
    want_off = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=precision)
    pl.set_lens_model(g.lenses, *g.zbeta())
    off = pl.invert_image_surface_brightness_map()
    pl.set_noise_term(True)
    on = pl.invert_image_surface_brightness_map()
    assert off["status"] == on["status"] == 0
    tol = 1e-6 * abs(want["m2logev"]) if precision == 0 else 0.2
    assert abs(on["m2logev"] - want["m2logev"]) <= tol, (on["m2logev"], want["m2logev"])
    # the term itself is the same sum in both precisions
    term, term_o = on["m2logev"] - off["m2logev"], want["m2logev"] - want_off["m2logev"]
    assert abs(term - term_o) <= 1e-9 * abs(term_o), (term, term_o)
    # a batch replayed from captured graphs carries it too
    P = np.tile(np.array(g.params()), (3, 1))
    for r in pl.eval_batch(P):
        assert r["status"] == 0
        assert abs(r["m2logev"] - on["m2logev"]) <= (1e-12 * abs(on["m2logev"]) if precision == 0 else 0.2)
    pl.set_noise_term(False)
    again = pl.invert_image_surface_brightness_map()
    assert abs(again["m2logev"] - off["m2logev"]) <= 1e-12 * abs(off["m2logev"]) + (0 if precision == 0 else 1e-9)
    pl.close()


def test_noise_term_with_lambda_optimisation_and_outside_prior():
    """The options together, as a fit script would set them: the noise term,
    the lambda optimisation and the outside-surface-brightness prior, plain
    FP64 against the oracle with the same three settings."""
    from qlens_gb300 import PixelLikelihood
    g = Golden("osb_tiny_sie")
    osb = dict(frac=g.sc["outside_sb_prior_threshold"], noise_frac=g.sc["outside_sb_prior_noise_frac"],
               emask_nsplit=int(g.sc["emask_nsplit"]), emask=g.arr["emask"])
    want = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), noise_term=True,
                      regopt=(-3.0, 5.0, 0.01, 20), outside_sb=osb)
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=0)
    pl.set_lens_model(g.lenses, *g.zbeta())
    pl.set_noise_term(True)
    pl.set_regparam_optimization(True)
    pl.set_outside_sb_prior(True, osb["frac"], osb["noise_frac"], osb["emask"].reshape(g.nx, g.ny),
                            osb["emask_nsplit"])
    r = pl.invert_image_surface_brightness_map()
    assert r["status"] == want["status"] == 0
    assert abs(r["regparam"] - want["regparam"]) <= 1e-6 * want["regparam"]
    assert abs(r["m2logev"] - want["m2logev"]) <= 1e-6 * abs(want["m2logev"]), (r["m2logev"], want["m2logev"])
    b = pl.eval_batch(np.tile(np.array(g.params()), (2, 1)))
    for x in b:
        assert abs(x["m2logev"] - r["m2logev"]) <= 1e-9 * abs(r["m2logev"])
    pl.close()
