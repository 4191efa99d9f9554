"""Samplers that batch their candidates: the speculative first-accept search
(qlp_speculative_search) under QLens's nested sampler.

NestedSampler restates the control flow of QLens's own nested sampler,
UCMC::MonoSample (mcmchdr.cpp:2901-3400): N live points drawn uniformly in
the unit cube of the fit parameters (Convert: lower + u (upper - lower)); at
each step the worst live point (largest -log L + prior term) is recorded as
dead and replaced by the first new draw that beats it (mcmchdr.cpp:3063-3098);
the running inverse slope slope = w0 e^(1/N) + e^(1/N - L_last + L_old) slope
(mcmchdr.cpp:3133); a first stage that ends when the acceptance ratio
(count + 1) / tries falls to 1/2 (senfac = 2) and a second that ends when
slope e^(L_max - L_old) reaches 1/tol = 2 (mcmchdr.cpp:3274-3286); then
ln Z = ln(slope + sum_live e^(L_old - L_i) / N) - L_old - count / N and the
posterior weights w0 e^(-L_k - k/N - ln Z) of the dead points and
e^(-L_i - count/N - ln Z) / N of the live ones (mcmchdr.cpp:3319-3390).  The
reference's second stage draws its candidates from bounding ellipsoids
around the live points (the Points class); this sampler keeps drawing them
uniformly in the cube in both stages.

Each replacement is a rejection loop, so its candidates go through the
speculative search: K draws are proposed before any is evaluated, evaluated
in one batch, and examined in draw order; the draws after the accepted one
are discarded and the random generator is wound back to just after it.  The
run -- every dead point, every count, ln Z -- is then the one the
one-candidate-at-a-time loop gives (batch=1), which the tests check.
"""
import ctypes as C
import math

import numpy as np

from . import abi
from .pixlike import QLPixError, load_library

PROPOSE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_long, C.POINTER(C.c_double), C.POINTER(C.c_double))
ACCEPT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_long, C.POINTER(abi.qlp_result))
REWIND_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_long)
BATCH_EVAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                            C.POINTER(abi.qlp_result))


class qlp_search_state(C.Structure):
    _fields_ = [("accept_rate", C.c_double), ("proposed", C.c_long), ("evaluated", C.c_long),
                ("examined", C.c_long), ("accepted", C.c_long), ("discarded", C.c_long), ("batches", C.c_long)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _bind(L):
    if getattr(L, "_search_bound", False):
        return
    P = C.POINTER
    L.qlp_speculative_search.argtypes = [C.c_void_p, PROPOSE_FN, ACCEPT_FN, REWIND_FN, C.c_void_p, C.c_int, C.c_int,
                                         C.c_long, P(qlp_search_state), P(C.c_long)]
    L.qlp_speculative_search_fn.argtypes = [BATCH_EVAL_FN, C.c_void_p, C.c_int, PROPOSE_FN, ACCEPT_FN, REWIND_FN,
                                            C.c_void_p, C.c_int, C.c_int, C.c_long, P(qlp_search_state),
                                            P(C.c_long)]
    L._search_bound = True


class PixelTarget:
    """-log L of QLens's pixel-image fit for a set of free lens parameters:
    0.5 x (-2 log evidence) (QLens::fitmodel_loglike_extended_source,
    lens.cpp:10657-10748, without its penalty terms), through a
    PixelLikelihood.  free: indices into the flat lens-parameter vector; the
    others stay at `base`.  A failed evaluation counts as 1e30."""

    def __init__(self, pl, base, free):
        self.pl = pl
        self.base = np.array(base, dtype=np.float64)
        self.free = list(free)

    def full(self, x):
        p = self.base.copy()
        p[self.free] = x
        return p

    def neg_loglike(self, result):
        return 1e30 if result["status"] != 0 else 0.5 * result["m2logev"]


class FunctionTarget:
    """-log L from a Python function of a batch of parameter vectors (rows),
    run through the same search (qlp_speculative_search_fn)."""

    def __init__(self, f, dim):
        self.f = f
        self.dim = dim

    def full(self, x):
        return np.asarray(x, dtype=np.float64)

    def neg_loglike(self, result):
        return 0.5 * result["m2logev"]


class NestedSampler:
    """QLens's nested sampler (UCMC::MonoSample) over a box prior, with its
    replacement draws batched.  log_prior(x) is the prior term added to -log L
    (QLens's LogPrior; 0 for a flat prior).  batch: (k_min, k_max) of the
    speculative search; (1, 1) is the one-at-a-time loop."""

    W_SENFAC = 2.0           # mcmchdr.cpp:2936-2940: tol, enfac, senfac
    TOL = 0.5

    def __init__(self, target, lower, upper, n_live, seed=0, log_prior=None, batch=(1, 32)):
        self.t = target
        self.lo = np.asarray(lower, dtype=np.float64)
        self.hi = np.asarray(upper, dtype=np.float64)
        self.ma = len(self.lo)
        self.N = int(n_live)
        self.rng = np.random.default_rng(seed)
        self.log_prior = log_prior or (lambda x: 0.0)
        self.k_min, self.k_max = batch
        self.state = qlp_search_state()
        self.L = load_library()
        _bind(self.L)
        self._keep = None

    def _eval_batch(self, X):
        """-log L of the rows of X (no prior term)."""
        if isinstance(self.t, FunctionTarget):
            return np.asarray(self.t.f(X), dtype=np.float64)
        P = np.stack([self.t.full(x) for x in X])
        return np.array([self.t.neg_loglike(r) for r in self.t.pl.eval_batch(P)])

    # ---- one speculative search: the first candidate with -log L + prior < bound
    def _search(self, bound, max_candidates):
        cand, states = {}, {}
        rng = self.rng
        counts = {"tries": 0}

        def propose(_u, i, lens_params, regparam):
            states[i] = rng.bit_generator.state
            u = rng.random(self.ma)
            x = self.lo + u * (self.hi - self.lo)
            lp = float(self.log_prior(x))
            cand[i] = (u, x, lp)
            full = self.t.full(x)
            C.memmove(lens_params, full.ctypes.data, full.nbytes)
            regparam[0] = 0.0
            return 0

        def accept(_u, i, res):
            r = res.contents.as_dict()
            u, x, lp = cand[i]
            nll = self.t.neg_loglike(r) + lp
            counts["tries"] += 1
            if nll < bound:
                cand["accepted"] = (u, x, lp, nll, r)
                return 1
            return 0

        def rewind(_u, nxt):
            rng.bit_generator.state = states[nxt]

        keep = (PROPOSE_FN(propose), ACCEPT_FN(accept), REWIND_FN(rewind))
        idx = C.c_long(-1)
        if isinstance(self.t, FunctionTarget):
            def ev(_u, params, lam, n, out):
                X = np.ctypeslib.as_array(params, shape=(n, self.t.dim)).copy()
                vals = self.t.f(X)
                for k in range(n):
                    out[k] = abi.qlp_result()
                    out[k].m2logev = 2.0 * float(vals[k])
                    out[k].status = 0
                return 0
            evf = BATCH_EVAL_FN(ev)
            code = self.L.qlp_speculative_search_fn(evf, None, self.t.dim, *keep, None, self.k_min, self.k_max,
                                                    int(max_candidates), C.byref(self.state), C.byref(idx))
        else:
            code = self.L.qlp_speculative_search(self.t.pl.ctx, *keep, None, self.k_min, self.k_max,
                                                 int(max_candidates), C.byref(self.state), C.byref(idx))
        if code != abi.QLP_OK:
            raise QLPixError(code, self.L.qlp_last_error().decode())
        if idx.value < 0:
            return None, counts["tries"]
        return cand["accepted"], counts["tries"]

    def run(self, max_dead=100000, max_tries=10 ** 7):
        N, ma = self.N, self.ma
        w0 = (1.0 - math.exp(-2.0 / N)) * 0.5
        # live points: uniform draws, a non-finite value drawn again
        # (mcmchdr.cpp:2961-2993) -- point i is the i-th finite draw, so the
        # draws can be evaluated a batch at a time
        pts, logL, logP = np.empty((N, ma)), np.empty(N), np.empty(N)
        i = drawn = 0
        while i < N:
            k = (N - i) if self.k_max > 1 else 1
            U = self.rng.random((k, ma))
            X = self.lo + U * (self.hi - self.lo)
            nll = self._eval_batch(X)
            drawn += k
            for j in range(k):
                lp = float(self.log_prior(X[j]))
                v = nll[j] + lp
                if math.isfinite(v) and i < N:
                    pts[i], logP[i], logL[i] = X[j], lp, v
                    i += 1
            if drawn > max_tries:
                raise RuntimeError("no finite likelihood in the prior box")
        likeMax = likeMin = logL[0]
        imin = 0
        for i in range(N):                       # the reference's scan (mcmchdr.cpp:3013-3026)
            if likeMax > logL[i]:
                likeMax = logL[i]
            elif likeMin < logL[i]:
                likeMin = logL[i]
                imin = i
        likeLast = likeMin
        slope, count, trystot, iterations = 0.0, 0, 0, 0
        dead = []
        best = (1e30, None)
        stage, ratio, test = 1, 1.0, 0.0
        while True:
            dead.append((pts[imin].copy(), likeMin, logP[imin]))
            likeOld = likeMin
            a, tries = self._search(likeMin, max_tries)
            trystot += tries
            iterations += tries
            if a is None:
                break
            _, x, lp, nll, _ = a
            if nll < best[0]:
                best = (nll, x.copy())
            ratio = (count + 1.0) / trystot
            pts[imin], logP[imin], logL[imin] = x, lp, nll
            if likeMax > logL[imin]:
                likeMax = logL[imin]
            likeMin, imin = logL[0], 0
            for i in range(N):
                if likeMin < logL[i]:
                    likeMin, imin = logL[i], i
            slope = w0 * math.exp(1.0 / N) + math.exp(1.0 / N - likeLast + likeOld) * slope
            if stage == 2:
                test = slope * math.exp(likeMax - likeOld)
            likeLast = likeOld
            count += 1
            if stage == 1 and not ratio > 1.0 / self.W_SENFAC:
                stage = 2
            elif stage == 2 and not test < 1.0 / self.TOL:
                break
            if count >= max_dead:
                break
        Z = slope + sum(math.exp(-logL[i] + likeOld) / N for i in range(N))
        lnZ = math.log(Z) - likeOld - count / N
        w_dead = [w0 * math.exp(-L - k / N - lnZ) for k, (_, L, _) in enumerate(dead[:count])]
        w_live = [math.exp(-logL[i] - count / N - lnZ) / N for i in range(N)]
        return dict(lnZ=lnZ, count=count, tries=trystot, dead=dead[:count], live=(pts.copy(), logL.copy()),
                    w_dead=np.array(w_dead), w_live=np.array(w_live), best=best, search=self.state.as_dict())


class TWalk:
    """QLens's T-Walk MCMC (UCMC::TWalk, mcmchdr.cpp:820-1210; Christen & Fox
    2010) over a box prior, with its proposals batched.

    n_chains chains in the unit cube of the fit parameters (at least ma + 2
    and 5).  Every iteration picks a chain t and another tt, draws u and moves
    t by a walk (u < div/2; Z = (1/sqrt(alim) + U (sqrt(alim) - 1/sqrt(alim)))^2
    along (a_t - a_tt) projected on a fresh random `proj`-plane, log-ratio
    (proj - 1) log Z), a traverse (u < div; Z = -U^(1/(alimt+1)) or
    -U^(1/(1-alimt)), log-ratio (proj - 2) log(-Z)), or a multivariate jump of
    t (u < (1+div)/2) or of tt (otherwise) of size din x dist along the
    Cholesky factor of the chains' covariance (AdvanceDevs::MultiDev,
    random.h:493-522; RandomPlane::Mult / RandRot, random.h:779-840); a
    proposal inside the cube is accepted if ans = L_new - L_t - log-ratio <= 0
    or an exponential variate is >= ans (-log L throughout).  Every n_chains
    iterations the Gelman-Rubin R of every parameter is updated; the run ends
    by the reference's rule (mcmchdr.cpp:1131-1185: once every R < tol, with
    one reset of the statistics after the first unconverged check).  The
    defaults are QLens's call (lens.cpp:9316: div 0.9836, proj 4, din 2.4,
    alim 2.5, alimt 6).  Random numbers come from numpy, not from QLens's
    generator, and calcCov uses the actual number of points (the reference
    fixes it at its first call through a static).

    While a chain's proposal is rejected nothing but the bookkeeping changes,
    so candidates are proposed K at a time, each assuming the ones before it
    were rejected, evaluated in one batch and examined in order
    (qlp_speculative_search); the draws after the first accepted one (or the
    one after which the run ends) are discarded and the generator is wound
    back to the point the one-at-a-time run reaches.  The acceptance variate
    is drawn with the proposal; a candidate accepted with ans <= 0, whose
    variate the reference never draws, winds the generator back to just
    before it.  The run -- every chain state, -log L, count, R -- is the
    one-candidate-at-a-time run's (batch=(1, 1)), which the tests check."""

    def __init__(self, target, lower, upper, n_chains=0, seed=0, log_prior=None, batch=(1, 32),
                 div=0.9836, proj=4, din=2.4, alim=2.5, alimt=6.0, tol=1.01):
        self.t = target
        self.lo = np.asarray(lower, dtype=np.float64)
        self.hi = np.asarray(upper, dtype=np.float64)
        self.ma = len(self.lo)
        nt = max(int(n_chains), self.ma + 2, 5 + 1)
        if nt <= proj:
            nt = proj + 1
        self.NT = nt
        self.rng = np.random.default_rng(seed)
        self.log_prior = log_prior or (lambda x: 0.0)
        self.k_min, self.k_max = batch
        self.div, self.proj, self.din, self.alim, self.alimt, self.tol = div, min(proj, self.ma), din, alim, alimt, tol
        self.state = qlp_search_state()
        self.L = load_library()
        _bind(self.L)

    # ---- -log L (+ prior term) of points of the unit cube, in a batch
    def _x(self, u):
        return self.lo + np.asarray(u) * (self.hi - self.lo)

    def _eval_units(self, U):
        X = np.stack([self._x(u) for u in U])
        if isinstance(self.t, FunctionTarget):
            nll = np.asarray(self.t.f(X), dtype=np.float64)
        else:
            nll = np.array([self.t.neg_loglike(r) for r in self.t.pl.eval_batch(np.stack([self.t.full(x) for x in X]))])
        return nll + np.array([float(self.log_prior(x)) for x in X])

    # ---- the move generators (draw order as the reference's)
    def _plane(self, rng):
        """RandRot(0, proj): proj orthonormal vectors by Gram-Schmidt of Gaussian draws."""
        V = np.zeros((self.proj, self.ma))
        for i in range(self.proj):
            v = rng.standard_normal(self.ma)
            for j in range(i):
                v = v - np.dot(v, V[j]) * V[j]
            V[i] = v / math.sqrt(np.dot(v, v))
        return V

    def _mult(self, rng, a, a0, Z):
        V = self._plane(rng)
        z = np.array([np.sum((Z - 1.0) * (a - a0) * V[i]) for i in range(self.proj)])
        return a + z @ V

    @staticmethod
    def _cov(pts):
        P = np.asarray(pts)
        n = len(P)
        return (P.T @ P) / n - np.outer(P.sum(0), P.sum(0)) / n / n

    @staticmethod
    def _indent(pts):
        P = np.asarray(pts)
        hi = np.maximum(1.0, P.max(0))
        lo = np.minimum(0.0, P.min(0))
        return np.diag((hi - lo) ** 2 / 12.0)

    @staticmethod
    def _chol(C):
        n = len(C)
        L = np.zeros((n, n))
        for i in range(n):
            for j in range(i, n):
                s = C[i, j] - sum(L[i, k] * L[j, k] for k in range(i - 1, -1, -1))
                if i == j:
                    if s <= 0.0:
                        return None
                    L[i, i] = math.sqrt(s)
                else:
                    L[j, i] = s / L[i, i]
        return L

    def _multi(self, rng, a0, pts):
        L = self._chol(self._cov(pts))
        if L is None:
            L = self._chol(self._indent(pts))
        vec = rng.standard_normal(self.ma)
        norm = math.sqrt(np.dot(vec, vec))
        if rng.random() < 0.33:
            dist = rng.standard_exponential()
        else:
            d = 0.0
            for _ in range(2):
                g = rng.standard_normal()
                d += g * g
            dist = math.sqrt(d / 2.0)
        return self.din * dist * (L @ vec) / norm + a0

    def _propose(self, rng, A):
        """One iteration's draws: (t, proposal, log-ratio)."""
        NT = self.NT
        t = int(NT * rng.random())
        tt = int((NT - 1) * rng.random())
        if tt >= t:
            tt += 1
        ran = rng.random()
        b0, b1, b2 = self.div / 2.0, self.div, (1.0 + self.div) / 2.0
        if ran < b0:
            sa = math.sqrt(self.alim)
            Z = (1.0 / sa + rng.random() * (sa - 1.0 / sa)) ** 2
            return t, self._mult(rng, A[t], A[tt], Z), (self.proj - 1.0) * math.log(Z)
        if ran < b1:
            if rng.random() < (self.alimt - 1.0) / (2.0 * self.alimt):
                Z = -rng.random() ** (1.0 / (self.alimt + 1.0))
            else:
                Z = -rng.random() ** (1.0 / (1.0 - self.alimt))
            return t, self._mult(rng, A[t], A[tt], Z), (self.proj - 2.0) * math.log(-Z)
        others = [A[i] for i in range(NT) if i != tt]
        if ran < b2:
            return t, self._multi(rng, A[t], list(A) + others), 0.0
        return t, self._multi(rng, A[tt], others), 0.0

    @staticmethod
    def _outside(u):
        return bool(np.any((u < 0.0) | (u > 1.0)))

    def run(self, max_iter=100000):
        NT, ma = self.NT, self.ma
        rng = self.rng
        A = [rng.random(ma) for _ in range(NT)]
        ll = list(self._eval_units(A))
        mult, count = [1] * NT, [1] * NT
        total, ttotal, nlength = 1, 0, 1
        covT = np.zeros((NT, ma)); avgT = np.zeros((NT, ma))
        W = np.zeros(ma); avgTot = np.zeros(ma)
        best = (min(ll), A[int(np.argmin(ll))].copy())
        chain = []                                 # accepted points: (chain t, multiplicity, x, -log L)
        R_hist = []
        run = {"stop": False}

        def bookkeeping():
            """After each iteration: the multiplicities, the counter and, every
            NT iterations, the R statistics and the stopping rule."""
            nonlocal total, ttotal, nlength, covT, avgT, W, avgTot, best
            for i in range(NT):
                mult[i] += 1
            total += 1
            for i in range(NT):
                if ll[i] < best[0]:
                    best = (ll[i], A[i].copy())
            if total % NT != 0:
                return False
            for k in range(NT):
                for i in range(ma):
                    davg = (A[k][i] - avgT[k][i]) / (ttotal + 1.0)
                    dcov = ttotal * davg * davg - covT[k][i] / (ttotal + 1.0)
                    avgTot[i] += davg / NT
                    covT[k][i] += dcov
                    avgT[k][i] += davg
                    W[i] += dcov / NT
            ttotal += 1
            cont = False
            Rmax = -1e30
            for i in range(ma):
                Bn = sum((avgT[s][i] - avgTot[i]) ** 2 for s in range(NT)) / (NT - 1.0)
                R = 1.0 + (NT + 1.0) * Bn / W[i] / NT if W[i] != 0 else float("inf")
                Rmax = max(Rmax, R)
                if W[i] <= 0.0 or R >= self.tol or R <= 0.0:
                    if nlength == 0:
                        cont = True
                    else:
                        cont = False
                        nlength -= 1
                        covT = np.zeros((NT, ma)); avgT = np.zeros((NT, ma))
                        W = np.zeros(ma); avgTot = np.zeros(ma)
                        ttotal += 1
            R_hist.append(Rmax)
            return not cont

        it = 0
        while not run["stop"] and it < max_iter:
            cand, before, after = {}, {}, {}

            def propose(_u, i, lens_params, regparam):
                t, u, logZ = self._propose(rng, A)
                before[i] = rng.bit_generator.state
                inside = not self._outside(u)
                e = rng.standard_exponential() if inside else None     # the acceptance variate
                after[i] = rng.bit_generator.state
                cand[i] = (t, u, logZ, inside, e)
                x = self._x(u if inside else A[t])
                full = self.t.full(x)
                C.memmove(lens_params, full.ctypes.data, full.nbytes)
                regparam[0] = 0.0
                return 0

            def accept(_u, i, res):
                nonlocal it
                t, u, logZ, inside, e = cand[i]
                took = False
                used_e = False
                if inside:
                    r = res.contents.as_dict()
                    nll = self.t.neg_loglike(r) + float(self.log_prior(self._x(u)))
                    ans = nll - ll[t] - logZ
                    used_e = ans > 0.0
                    if ans <= 0.0 or e >= ans:
                        chain.append((t, mult[t], self._x(u), nll))
                        A[t] = u
                        ll[t] = nll
                        mult[t] = 0
                        count[t] += 1
                        took = True
                cand["used_e"] = used_e
                it += 1
                stop = bookkeeping() or it >= max_iter
                if stop:
                    run["stop"] = True
                cand["last"] = i
                return 1 if (took or stop) else 0

            def rewind(_u, nxt):
                rng.bit_generator.state = after[nxt - 1] if cand["used_e"] else before[nxt - 1]

            keep = (PROPOSE_FN(propose), ACCEPT_FN(accept), REWIND_FN(rewind))
            idx = C.c_long(-1)
            if isinstance(self.t, FunctionTarget):
                def ev(_u, params, lam, n, out):
                    X = np.ctypeslib.as_array(params, shape=(n, self.t.dim)).copy()
                    vals = self.t.f(X)
                    for k in range(n):
                        out[k] = abi.qlp_result()
                        out[k].m2logev = 2.0 * float(vals[k])
                        out[k].status = 0
                    return 0
                evf = BATCH_EVAL_FN(ev)
                code = self.L.qlp_speculative_search_fn(evf, None, self.t.dim, *keep, None, self.k_min, self.k_max,
                                                        max_iter + 1, C.byref(self.state), C.byref(idx))
            else:
                code = self.L.qlp_speculative_search(self.t.pl.ctx, *keep, None, self.k_min, self.k_max,
                                                     max_iter + 1, C.byref(self.state), C.byref(idx))
            if code != abi.QLP_OK:
                raise QLPixError(code, self.L.qlp_last_error().decode())
            if idx.value < 0:
                break
            # the generator where the one-at-a-time run has it (rewind is not
            # called when the accepted candidate was the last one proposed)
            rng.bit_generator.state = after[idx.value] if cand["used_e"] else before[idx.value]
        return dict(chains=[a.copy() for a in A], loglike=list(ll), count=list(count), mult=list(mult),
                    iterations=it, chain=chain, R=R_hist, best=best, search=self.state.as_dict(), n_chains=NT)
