"""Sampler-side batching, host side: the speculative first-accept search
(qlp_speculative_search_fn) under the nested sampler that restates QLens's
UCMC::MonoSample (mcmchdr.cpp:2901-3400), with a likelihood computed on the
CPU.

* the batched run is the one-candidate-at-a-time run: the same dead points,
  likelihood values, try counts and ln Z, bit for bit, at several batch
  bounds (the draws after an accepted candidate are discarded and the
  generator wound back);
* the search contract itself: candidates proposed in index order, examined
  in index order up to the accepted one, rewind called once with the index
  after it;
* ln Z of a Gaussian likelihood in a box agrees with the analytic value.
"""
import ctypes as C
import math

import numpy as np
import pytest

from qlens_gb300 import abi
from qlens_gb300.samplers import (ACCEPT_FN, BATCH_EVAL_FN, PROPOSE_FN, REWIND_FN, FunctionTarget, NestedSampler,
                                  qlp_search_state, _bind)
from qlens_gb300.pixlike import load_library

MU = np.array([0.7, -1.2])


def gauss_nll(X):
    d = np.atleast_2d(X) - MU
    return 0.5 * np.sum(d * d, axis=1)


def _run(batch, seed=3, n_live=60):
    ns = NestedSampler(FunctionTarget(gauss_nll, 2), [-5, -5], [5, 5], n_live, seed=seed, batch=batch)
    return ns.run()


def test_batched_run_equals_serial_run():
    ref = _run((1, 1))
    assert ref["search"]["discarded"] == 0
    for batch in [(1, 8), (4, 32), (16, 16)]:
        r = _run(batch)
        assert r["count"] == ref["count"] and r["tries"] == ref["tries"]
        assert r["lnZ"] == ref["lnZ"]
        for (xa, la, pa), (xb, lb, pb) in zip(r["dead"], ref["dead"]):
            assert np.array_equal(xa, xb) and la == lb and pa == pb
        assert np.array_equal(r["live"][0], ref["live"][0])
        s = r["search"]
        assert s["evaluated"] == s["examined"] + s["discarded"]
        assert s["examined"] == ref["tries"] and s["batches"] < ref["search"]["batches"]


def test_lnZ_gaussian_in_box():
    r = _run((1, 32), seed=11, n_live=200)
    want = math.log(2 * math.pi / 100.0)        # prior density 1/100 over the box
    assert abs(r["lnZ"] - want) < 0.5, (r["lnZ"], want)
    w = np.concatenate([r["w_dead"], r["w_live"]])
    assert abs(w.sum() - 1.0) < 0.05
    X = np.concatenate([np.stack([d[0] for d in r["dead"]]), r["live"][0]])
    mean = (w[:, None] * X).sum(0) / w.sum()
    assert np.all(np.abs(mean - MU) < 0.3)


def test_search_contract():
    L = load_library()
    _bind(L)
    log = []
    values = [5.0, 4.0, 3.0, 0.5, 2.0, 0.1, 7.0, 8.0]   # accepted: the first below 1.0, index 3

    def propose(_u, i, p, lam):
        log.append(("p", i))
        p[0] = float(i)
        return 0

    def accept(_u, i, res):
        log.append(("a", i))
        return 1 if res.contents.m2logev < 1.0 else 0

    def rewind(_u, nxt):
        log.append(("r", nxt))

    def ev(_u, params, lam, n, out):
        for k in range(n):
            out[k] = abi.qlp_result()
            out[k].m2logev = values[int(params[k])]
        return 0

    st = qlp_search_state()
    idx = C.c_long()
    cbs = (BATCH_EVAL_FN(ev), PROPOSE_FN(propose), ACCEPT_FN(accept), REWIND_FN(rewind))
    code = L.qlp_speculative_search_fn(cbs[0], None, 1, cbs[1], cbs[2], cbs[3], None, 6, 6, 8, C.byref(st),
                                       C.byref(idx))
    assert code == 0 and idx.value == 3
    assert log == [("p", i) for i in range(6)] + [("a", i) for i in range(4)] + [("r", 4)]
    assert (st.proposed, st.examined, st.accepted, st.discarded, st.batches) == (6, 4, 1, 2, 1)
    assert st.accept_rate == 0.25
    # none accepted within the limit: every candidate examined, no rewind
    log.clear()
    values[:] = [9.0] * 8
    st2 = qlp_search_state()
    code = L.qlp_speculative_search_fn(cbs[0], None, 1, cbs[1], cbs[2], cbs[3], None, 3, 3, 7, C.byref(st2),
                                       C.byref(idx))
    assert code == 0 and idx.value == -1
    assert [e for e in log if e[0] == "r"] == []
    assert st2.proposed == st2.examined == 7 and st2.batches == 3
    # a callback can stop the search
    stop = PROPOSE_FN(lambda _u, i, p, lam: 1)
    code = L.qlp_speculative_search_fn(cbs[0], None, 1, stop, cbs[2], cbs[3], None, 1, 4, 7, C.byref(st2),
                                       C.byref(idx))
    assert code == abi.QLP_ERR_ARG


def test_batch_size_follows_acceptance_rate():
    """K = the smallest batch that holds an acceptance with 90% chance."""
    L = load_library()
    _bind(L)
    sizes = []

    def ev(_u, params, lam, n, out):
        sizes.append(n)
        for k in range(n):
            out[k] = abi.qlp_result()
        return 0

    cbs = (BATCH_EVAL_FN(ev), PROPOSE_FN(lambda _u, i, p, lam: 0), ACCEPT_FN(lambda _u, i, r: 0),
           REWIND_FN(lambda _u, n: None))
    for rate, want in [(0.5, 4), (0.1, 22), (0.9, 1), (0.0, 64)]:
        sizes.clear()
        st = qlp_search_state(accept_rate=rate)
        idx = C.c_long()
        L.qlp_speculative_search_fn(cbs[0], None, 1, cbs[1], cbs[2], cbs[3], None, 1, 64, 100, C.byref(st),
                                    C.byref(idx))
        assert sizes[0] == want, (rate, sizes)
        assert sum(sizes) == 100                 # never past max_candidates
        assert sizes[1] == min(64, 100 - sizes[0])   # nothing accepted: the rate drops to 0


def test_prior_term_and_flat_likelihood_plateaus():
    """A non-flat prior term (QLens's LogPrior added to -log L) and a
    likelihood with exact ties: the batched run still equals the serial one,
    and every accepted replacement beats the point it replaced."""
    def lp(x):
        return 0.5 * float(np.sum((x / 3.0) ** 2))

    def stepped(X):
        return np.floor(4 * gauss_nll(X)) / 4           # ties between candidates

    runs = []
    for batch in [(1, 1), (2, 16)]:
        ns = NestedSampler(FunctionTarget(stepped, 2), [-5, -5], [5, 5], 40, seed=9, log_prior=lp, batch=batch)
        runs.append(ns.run(max_dead=400))
    a, b = runs
    assert a["count"] == b["count"] and a["tries"] == b["tries"] and a["lnZ"] == b["lnZ"]
    for (xa, la, pa), (xb, lb, pb) in zip(a["dead"], b["dead"]):
        assert np.array_equal(xa, xb) and la == lb and pa == pb
    L = [d[1] for d in a["dead"]]
    assert all(L[k + 1] <= L[k] for k in range(len(L) - 1))   # dead points in decreasing -log L order
