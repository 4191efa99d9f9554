"""The fit drivers' likelihood: QLens::fitmodel_loglike_extended_source
(lens.cpp:10657-10748) over the library's evaluation (qlp_set_fit_params,
qlp_fit_loglike_batch, qlp_fit_terms).

CPU: the host side -- inverse transforms, penalty limits, prior and Jacobian
terms -- against a restatement of QLens's ParamSettings written here from
params.h (inverse_transform_parameters :722-743, add_prior_terms_to_loglike
:810-840, add_jacobian_terms_to_loglike :884-893).
GPU: -log L of fit vectors equals m2logev / 2 of the same lens parameters plus
those terms, penalised vectors give QLens's 1e30, and the regularisation
parameter can be a fit parameter.
"""
import math

import numpy as np
import pytest

from goldens import Golden

NONE, LOG, LINEAR, RATIO = 0, 1, 2, 3
UNIFORM, LOGP, GAUSS = 0, 1, 2

# tiny_sie's lens vector: sple b, alpha, s, q, theta, xc, yc, shear g, theta_g, xc, yc
SPEC = [
    dict(target=0, transform=LOG, include_jacobian=1, use_penalty_limits=1, penalty_lo=0.3, penalty_hi=1.5),
    dict(target=3, transform=NONE, prior=GAUSS, prior_pos=0.72, prior_sig=0.05, prior_norm=0.6),
    dict(target=4, transform=LINEAR, a=0.5, b=3.0),
    dict(target=7, transform=RATIO, ratio_param=0, include_jacobian=1),
    dict(target=-1, transform=LOG, include_jacobian=1, prior=LOGP, prior_norm=2.3),
]


def restated_terms(spec, x):
    """(transformed, penalised, prior + Jacobian terms) as QLens computes them."""
    n = len(spec)
    t = [0.0] * n
    later = False
    for i, f in enumerate(spec):
        tr = f.get("transform", NONE)
        if tr == NONE:
            t[i] = x[i]
        elif tr == LOG:
            t[i] = 10.0 ** x[i]
        elif tr == LINEAR:
            t[i] = (x[i] - f["b"]) / f["a"]
        elif tr == RATIO:
            if f["ratio_param"] < i:
                t[i] = x[i] * t[f["ratio_param"]]
            else:
                later = True
    if later:
        for i, f in enumerate(spec):
            if f.get("transform", NONE) == RATIO:
                t[i] = x[i] * t[f["ratio_param"]]
    for i, f in enumerate(spec):
        if f.get("use_penalty_limits") and not (f["penalty_lo"] <= t[i] <= f["penalty_hi"]):
            return t, True, 0.0
    tot = 0.0
    for i, f in enumerate(spec):
        pr = f.get("prior", UNIFORM)
        if pr == UNIFORM:
            continue
        tot += math.log(f["prior_norm"])
        if pr == LOGP:
            tot += math.log(x[i])
        elif pr == GAUSS:
            tot += ((x[i] - f["prior_pos"]) / f["prior_sig"]) ** 2 / 2.0
    ll = tot
    for i, f in enumerate(spec):
        if not f.get("include_jacobian"):
            continue
        tr = f.get("transform", NONE)
        if tr == LOG:
            ll -= math.log(t[i])
        elif tr == RATIO:
            ll += math.log(t[f["ratio_param"]])
    return t, False, ll


def _vectors():
    rng = np.random.default_rng(3)
    X = np.column_stack([np.log10(rng.uniform(0.5, 0.9, 12)), rng.uniform(0.62, 0.82, 12),
                         0.5 * rng.uniform(30, 50, 12) + 3.0, rng.uniform(0.02, 0.06, 12),
                         rng.uniform(0.3, 1.2, 12)])
    X[3, 0] = np.log10(1.7)        # outside b's penalty limits
    return X


def test_host_terms_match_restatement():
    from qlens_gb300 import pixlike
    for x in _vectors():
        t, pen, terms = pixlike.fit_terms(SPEC, x)
        rt, rpen, rterms = restated_terms(SPEC, list(x))
        assert pen == rpen
        assert np.array_equal(t, np.array(rt))
        if not pen:
            assert terms == rterms


def test_ratio_after_its_reference():
    """A ratio whose reference comes later in the list is resolved after the loop."""
    from qlens_gb300 import pixlike
    spec = [dict(target=7, transform=RATIO, ratio_param=1), dict(target=0, transform=LOG)]
    x = [0.05, np.log10(0.8)]
    t, pen, _ = pixlike.fit_terms(spec, x)
    rt, _, _ = restated_terms(spec, x)
    assert not pen and np.array_equal(t, np.array(rt))


@pytest.mark.gpu
def test_fit_loglike_on_the_device():
    from qlens_gb300 import PixelLikelihood, QLP_FP64
    g = Golden("tiny_sie")
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=QLP_FP64)
    pl.set_lens_model(g.lenses)
    pl.set_fit_params(SPEC)
    X = _vectors()
    ll, res = pl.fit_loglike_batch(X)
    base = np.array(g.params())
    for x, l, r in zip(X, ll, res):
        t, pen, terms = restated_terms(SPEC, list(x))
        if pen:
            assert l == 1e30 and r["status"] == 0 and r["n_active_src"] == 0
            continue
        p = base.copy()
        p[0], p[3], p[4], p[7] = t[0], t[1], t[2], t[3]
        direct = pl.invert_image_surface_brightness_map(p, regparam=t[4])
        assert direct["status"] == 0 and r["status"] == 0
        assert r["regparam"] == t[4]
        # the same terms added in another order: equal to the last bits
        assert abs(l - (direct["m2logev"] / 2 + terms)) <= 1e-12 * abs(l)
    pl.close()
