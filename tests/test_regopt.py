"""Regularisation-parameter optimisation (QLens's 'optimize_regparam on'),
host side: the oracle's Brent search pinned to goldens the compiled reference
produced with the option on (tests/golden/regopt_*.npz), and the library's
Brent state machine (brent.h, qlp_brent_min) step for step against the
oracle's restatement of QLens::brents_min_method."""
import math

import numpy as np
import pytest

from goldens import REGOPT_CASES, Golden
from oracle import oracle as O


@pytest.mark.parametrize("name", REGOPT_CASES)
def test_oracle_regopt_vs_reference(name):
    g = Golden(name)
    assert g.regopt is not None
    r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes(), regopt=g.regopt)
    assert r["status"] == 0
    # the reference sums the trial chi^2 with an OpenMP reduction (4 threads
    # for the goldens); the oracle sums in pixel order, so the Brent steps can
    # differ in the last bits
    assert abs(r["regparam"] - g.sc["regparam"]) <= 1e-9 * g.sc["regparam"]
    for k, ref in (("m2logev", "m2logev"), ("chisq0", "chisq0"), ("logdet_F", "logdetF"), ("logdet_R", "logdetR")):
        assert abs(r[k] - g.sc[ref]) <= 1e-11 * abs(g.sc[ref]), (k, r[k], g.sc[ref])
    assert 5 <= r["regopt_evals"] <= 21
    # the inversion at the chosen lambda: amplitudes and model image
    assert np.allclose(O.get("s"), g.arr["s"], rtol=1e-9, atol=1e-12)
    assert np.allclose(O.get("model"), g.arr["model"], rtol=1e-9, atol=1e-12)
    # and it beats the fixed lambda of the same script
    base = Golden(name.replace("regopt_", ""))
    assert g.sc["m2logev"] < base.sc["m2logev"]


FUNCS = [
    ("quadratic", lambda x: (x - 1.3) ** 2 + 2.0, -3.0, 5.0, 0.01, 20),
    ("quartic", lambda x: (x + 0.7) ** 4 - x, -3.0, 5.0, 0.01, 20),
    ("wiggly", lambda x: math.sin(3 * x) + 0.1 * (x - 2) ** 2, -3.0, 5.0, 1e-4, 30),
    ("edge", lambda x: math.exp(-x), -3.0, 5.0, 0.01, 20),            # minimum at the bracket's end
    ("flat", lambda x: 1.0, -3.0, 5.0, 0.01, 20),
    ("evidence-like", lambda x: 1e3 * math.log1p(math.exp(2 * (x - 1))) - 800 * x, -3.0, 5.0, 0.01, 20),
    ("few-iterations", lambda x: (x - 0.2) ** 2, -3.0, 5.0, 1e-8, 4),
]


@pytest.mark.parametrize("name,f,ax,bx,tol,maxit", FUNCS, ids=[f[0] for f in FUNCS])
def test_library_brent_matches_reference_steps(name, f, ax, bx, tol, maxit):
    from qlens_gb300 import pixlike
    xo, no, po = O.brent_min(f, ax, bx, tol, maxit)
    xl, nl, pl = pixlike.brent_min(f, ax, bx, tol, maxit)
    assert pl == po, (name, pl, po)
    assert xl == xo and nl == no == len(po)
    assert f(xl) == min(f(p) for p in po)
