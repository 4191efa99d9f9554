"""T-Walk (UCMC::TWalk, mcmchdr.cpp:820-1210) restated in
qlens_gb300/samplers.py with its proposals batched through the speculative
search (qlp_speculative_search_fn; no device needed).  The batched run must be
the one-candidate-at-a-time run: every chain state, -log L value, acceptance
count and R value identical, with fewer likelihood calls."""
import numpy as np
import pytest


def _gauss(X):
    X = np.atleast_2d(X)
    return 0.5 * np.sum(((X - np.array([0.3, 0.6, 0.45])) / np.array([0.05, 0.08, 0.04])) ** 2, axis=1)


def _run(batch, seed=3, iters=2000, **kw):
    from qlens_gb300.samplers import FunctionTarget, TWalk
    tw = TWalk(FunctionTarget(_gauss, 3), [0, 0, 0], [1, 1, 1], seed=seed, batch=batch, **kw)
    return tw.run(max_iter=iters)


@pytest.mark.parametrize("batch", [(1, 32), (4, 16)])
def test_batched_equals_serial(batch):
    a, b = _run((1, 1)), _run(batch)
    assert a["iterations"] == b["iterations"] == 2000
    assert a["loglike"] == b["loglike"] and a["count"] == b["count"] and a["mult"] == b["mult"]
    assert all(np.array_equal(x, y) for x, y in zip(a["chains"], b["chains"]))
    assert a["R"] == b["R"]
    assert len(a["chain"]) == len(b["chain"])
    for (ta, ma, xa, la), (tb, mb, xb, lb) in zip(a["chain"], b["chain"]):
        assert ta == tb and ma == mb and la == lb and np.array_equal(xa, xb)
    assert b["search"]["batches"] < a["search"]["batches"]
    print("serial: %d calls; batched %s: %d calls for %d candidates evaluated" % (
        a["search"]["batches"], batch, b["search"]["batches"], b["search"]["evaluated"]))


def test_stops_by_the_reference_rule():
    """The run stops at an R check (every n_chains iterations) once every
    parameter's R is below tol -- batched exactly as serial."""
    a, b = _run((1, 1), iters=20000, tol=1.2), _run((1, 32), iters=20000, tol=1.2)
    assert a["iterations"] == b["iterations"] < 20000
    assert (a["iterations"] + 1) % a["n_chains"] == 0
    assert a["R"][-1] < 1.2 and a["R"] == b["R"]
    assert a["loglike"] == b["loglike"]


def test_samples_the_target():
    """A long run's accepted points (weighted by how long each chain state
    lasted) sit on the Gaussian target."""
    r = _run((1, 32), iters=30000, tol=1.0 + 1e-9)
    X = np.array([x for _, _, x, _ in r["chain"]])
    assert len(X) > 5000
    assert np.all(np.abs(X.mean(0) - [0.3, 0.6, 0.45]) < 0.02)
    assert np.all(np.abs(X.std(0) / np.array([0.05, 0.08, 0.04]) - 1.0) < 0.25)


def test_moves_stay_reproducible_and_respect_the_cube():
    """Proposals outside the unit cube are never evaluated as accepted
    points; every chain stays inside it."""
    r = _run((1, 8), iters=1000)
    for x in r["chains"]:
        assert np.all((x >= 0) & (x <= 1))
