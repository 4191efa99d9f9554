"""The outside-surface-brightness prior (QLens 'outside_sb_prior on',
lens.cpp:13063-13158) in the oracle, against goldens from the compiled
reference: its pass over the extended mask (ray tracing, mapping, model,
PSF convolution) bit for bit, and -2 log(evidence) with the penalty.

osb_tiny_sie: extended mask 3 rings past the annulus, threshold 0.15 of the
in-mask peak -- the model leaks past it, a penalty of about 1.6e6.
osb_powerlaw: 2 rings, the default 0.3 -- no penalty.  The reference's own
run of the pass is dumped by the harness replaying the calls of
lens.cpp:13067-13086 after the inversion.
"""
import numpy as np
import pytest

from goldens import Golden
from oracle import oracle as O

CASES = ["osb_tiny_sie", "osb_powerlaw"]


def osb_settings(g):
    return dict(frac=g.sc["outside_sb_prior_threshold"], noise_frac=g.sc["outside_sb_prior_noise_frac"],
                emask_nsplit=int(g.sc["emask_nsplit"]), emask=g.arr["emask"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_outside_pass_vs_reference(name):
    g = Golden(name)
    assert int(g.sc["outside_sb_prior"]) == 1
    r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), outside_sb=osb_settings(g))
    assert r["status"] == 0
    assert np.array_equal(O.get("osb_maps"), g.arr["osb_maps"])
    assert np.array_equal(O.get("osb_sb"), g.arr["osb_sb"])
    assert r["m2logev"] == g.sc["m2logev"]
    base = Golden(name.replace("osb_", ""))
    pen = float(O.get("osb_penalty")[0])
    assert abs((g.sc["m2logev"] - base.sc["m2logev"]) - pen) <= 1e-9 * max(abs(pen), 1.0)
    if name == "osb_tiny_sie":
        assert pen > 1e5
    else:
        assert pen == 0.0


def test_oracle_outside_pass_edges():
    """Every pixel in the extended mask (the reference's default before any
    mask editing), a 2-way split outside the mask, and a threshold from the
    pixel noise: the pass stays consistent with its definition."""
    g = Golden("osb_tiny_sie")
    base = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(),
                   outside_sb=dict(frac=0.15, noise_frac=-1e30, emask_nsplit=2, emask=None))
    sb, maps = O.get("osb_sb"), O.get("osb_maps").astype(bool)
    m = g.arr["mask"].astype(bool)
    assert maps.sum() > int(g.arr["osb_maps"].sum())          # the whole frame maps where the grid reaches
    peak = sb[m & maps].max()
    out = np.abs(sb[(~m) & maps])
    t = 0.15 * peak
    over = out[out >= t]
    want = (1 + abs((over.max() - t) / t)) ** 60 - 1 if over.size else 0.0
    assert abs((r["m2logev"] - base["m2logev"]) - want) <= 1e-9 * max(want, 1.0)
    # a noise-based threshold far above every pixel: no penalty
    r2 = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(),
                    outside_sb=dict(frac=0.0, noise_frac=1e6, emask_nsplit=1, emask=None))
    assert r2["m2logev"] == base["m2logev"]
