"""QLens's 'include_noise_term_in_loglike on' (lens.cpp:13033-13043): the
pixel-noise normalisation added to -2 log(evidence), in the oracle.

The golden noise_tiny_sie is the tiny_sie script with the option on and
uniform noise (no noise map; with a noise map the reference reads the pixel
C^-1 vector after clear_pixel_matrices has freed it).  In that configuration
the reference builds D with an OpenMP-private copy of 1/sigma^2 that is never
initialised (pixelgrid.cpp:15637-15653, 'private(...,covinv)'): its D, source
amplitudes and model image are zero, so its chi^2 is the data's own.  The
noise term is pinned from the reference's scalars with those zero amplitudes:
-2 log ev - chi^2 - (log det F - log det R - M log lambda).
"""
import math

import numpy as np

from goldens import Golden
from oracle import oracle as O


def _implied_noise_term(g):
    sc = g.sc
    return sc["m2logev"] - sc["chisq0"] - (sc["logdetF"] - sc["logdetR"] - sc["n_active_src"] * math.log(sc["regparam"]))


def test_reference_run_has_zero_amplitudes():
    g = Golden("noise_tiny_sie")
    assert int(g.sc["use_noise_map"]) == 0
    assert np.all(g.arr["D"] == 0) and np.all(g.arr["s"] == 0) and np.all(g.arr["model"] == 0)
    # chi^2 of a zero model: the data's own over the mask
    d = g.arr["data"][g.arr["mask"].astype(bool)]
    c = 1.0 / g.sc["background_pixel_noise"] ** 2
    assert abs(np.sum(d * d) * c - g.sc["chisq0"]) <= 1e-10 * g.sc["chisq0"]


def test_oracle_noise_term_uniform_noise_vs_reference():
    g = Golden("noise_tiny_sie")
    off = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    on = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), noise_term=True)
    assert off["status"] == on["status"] == 0
    # the rest of the evaluation is the same, and agrees with the reference's
    for k, ref in (("logdet_F", "logdetF"), ("logdet_R", "logdetR")):
        assert on[k] == off[k]
        assert abs(on[k] - g.sc[ref]) <= 1e-11 * abs(g.sc[ref])
    assert on["chisq0"] == off["chisq0"]
    term = on["m2logev"] - off["m2logev"]
    ref = _implied_noise_term(g)
    assert abs(term - ref) <= 1e-9 * abs(ref), (term, ref)
    n_mask = int(g.arr["mask"].sum())
    c = 1.0 / g.sc["background_pixel_noise"] ** 2
    assert abs(term - n_mask * (math.log(2 * math.pi) - math.log(c))) <= 1e-9 * abs(ref)


def test_oracle_noise_term_noise_map():
    """With a noise map the sum runs over the active pixels' C^-1 (lens.cpp:13036-13038)
    while the log(2 pi) count is all masked pixels."""
    g = Golden("tiny_sie")
    assert int(g.sc["use_noise_map"]) == 1
    off = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    on = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), noise_term=True)
    assert abs(off["m2logev"] - g.sc["m2logev"]) <= 1e-11 * abs(g.sc["m2logev"])
    act = g.arr["active_pixels"]
    n_mask = int(g.arr["mask"].sum())
    want = -np.sum(np.log(g.arr["covinv"][act])) + n_mask * math.log(2 * math.pi)
    assert abs((on["m2logev"] - off["m2logev"]) - want) <= 1e-9 * abs(want)
