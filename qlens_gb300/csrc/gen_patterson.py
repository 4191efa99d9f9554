"""Generate patterson_rule.h: the nested Gauss-Patterson quadrature rules on
[-1, 1] with 1, 3, 7, 15, 31, 63, 127, 255 and 511 points.

QLens integrates the NFW deflection with these rules (GaussPatterson,
gauss.cpp; LensIntegral::PattersonIntegrate, profile.cpp:3830-3876).  The
rules are published mathematics (T. N. L. Patterson, "The optimum addition
of points to quadrature formulae", Math. Comp. 22 (1968) 847-856); this
script recomputes them from that construction in 320-digit arithmetic (the Legendre-basis system for the 511-point level has a condition number near 1e100) and
rounds every node and weight to the nearest double:

* level 0 is the 1-point Gauss rule {0};
* level k+1 keeps the n = 2^(k+1) - 1 nodes X of level k and adds the
  m = n + 1 zeros of the degree-m polynomial F that is orthogonal to every
  polynomial of degree < m under the weight w(x) = prod_j (x - X_j).
  Equivalently S = F w (degree 2m - 1) has no Legendre component below
  degree m and vanishes on X, so S = sum_{n=m}^{2m-1} d_n P_n with
  S(X_j) = 0; S is odd, which leaves m/2 coefficients and m/2 - 1
  conditions (one free scale).  The zeros of F interlace with X, so each
  gap between consecutive non-negative nodes (and the last node and 1)
  holds exactly one new positive node;
* the weights of every level are those of the interpolatory rule on its
  nodes, w_j = integral of the Lagrange basis polynomial l_j, evaluated
  exactly with a Gauss-Legendre rule of sufficient degree.

Layout in the header (what PattersonIntegrate indexes):
  qlp_pat_points[511]  all 511 nodes in ascending order; level L uses
                       indices (j + 1) * 2^(8 - L) - 1, j = 0 .. 2^(L+1) - 2
  qlp_pat_weights[]    level L's weights in ascending node order, level
                       after level, starting at qlp_pat_offset[L]

Run:  python qlens_gb300/csrc/gen_patterson.py   (needs mpmath; ~1 min)
"""
import os
import sys

import mpmath as mp
from mpmath.calculus.quadrature import GaussLegendre

mp.mp.dps = 320
LEVELS = 9
HERE = os.path.dirname(os.path.abspath(__file__))


def legendre_all(x, nmax):
    """P_0(x) .. P_nmax(x) by the three-term recurrence."""
    p = [mp.mpf(1), x]
    for n in range(1, nmax):
        p.append(((2 * n + 1) * x * p[n] - n * p[n - 1]) / (n + 1))
    return p


def extend(nodes):
    """Positive new nodes added to the symmetric node set `nodes`."""
    n = len(nodes)
    m = n + 1
    pos = [x for x in nodes if x > 0]
    degs = list(range(m + 1, 2 * m, 2))          # odd degrees m+1 .. 2m-1
    k = len(degs)                                 # m/2 unknowns, k-1 conditions
    # d_{2m-1} = 1; solve the other k-1 coefficients from S(X_j) = 0
    A = mp.matrix(k - 1, k - 1)
    b = mp.matrix(k - 1, 1)
    for r, x in enumerate(pos):
        p = legendre_all(x, 2 * m - 1)
        for c in range(k - 1):
            A[r, c] = p[degs[c]]
        b[r] = -p[degs[k - 1]]
    d = list(mp.lu_solve(A, b)) if k > 1 else []
    d.append(mp.mpf(1))

    def S(x):
        p = legendre_all(x, 2 * m - 1)
        return mp.fsum(dc * p[dg] for dc, dg in zip(d, degs))

    def g(x):                                     # F = S / w
        w = mp.mpf(1)
        for xj in nodes:
            w *= (x - xj)
        return S(x) / w

    edges = [mp.mpf(0)] + pos + [mp.mpf(1)]
    new = []
    for a, bnd in zip(edges[:-1], edges[1:]):
        # the one sign change of F in (a, b), found on an interior sample
        # (F is smooth there; the endpoints are zeros of S and w)
        found = None
        for ns in (8, 32, 128):
            xs = [a + (bnd - a) * mp.mpf(i) / ns for i in range(1, ns)]
            gs = [g(x) for x in xs]
            ch = [i for i in range(len(xs) - 1) if mp.sign(gs[i]) != mp.sign(gs[i + 1])]
            if len(ch) == 1:
                found = ch[0]
                break
            if len(ch) > 1:
                raise RuntimeError("several sign changes in (%s, %s)" % (mp.nstr(a, 8), mp.nstr(bnd, 8)))
            if mp.sign(g(a + (bnd - a) / (4 * ns))) != mp.sign(gs[0]):
                xs, gs, found = [a + (bnd - a) / (4 * ns)] + xs, [g(a + (bnd - a) / (4 * ns))] + gs, 0
                break
            if mp.sign(g(bnd - (bnd - a) / (4 * ns))) != mp.sign(gs[-1]):
                xs, gs = xs + [bnd - (bnd - a) / (4 * ns)], gs + [g(bnd - (bnd - a) / (4 * ns))]
                found = len(xs) - 2
                break
        if found is None:
            raise RuntimeError("no sign change in (%s, %s)" % (mp.nstr(a, 8), mp.nstr(bnd, 8)))
        lo, hi, glo, ghi = xs[found], xs[found + 1], gs[found], gs[found + 1]
        # bisection to a few digits, then Illinois (regula falsi) inside the bracket
        for _ in range(20):
            mid = (lo + hi) / 2
            gm = g(mid)
            if mp.sign(gm) == mp.sign(glo):
                lo, glo = mid, gm
            else:
                hi, ghi = mid, gm
        side = 0
        for _ in range(2000):
            if hi - lo < mp.mpf(10) ** (20 - mp.mp.dps) * (abs(lo) + abs(hi)):   # nodes feed the next level's system
                break
            r = (lo * ghi - hi * glo) / (ghi - glo)
            if not (lo < r < hi):
                r = (lo + hi) / 2
            gr = g(r)
            if gr == 0:
                lo = hi = r
                break
            if mp.sign(gr) == mp.sign(glo):
                lo, glo = r, gr
                if side == -1:
                    ghi /= 2
                side = -1
            else:
                hi, ghi = r, gr
                if side == 1:
                    glo /= 2
                side = 1
        else:
            raise RuntimeError("root did not converge")
        new.append((lo + hi) / 2)
    return new


def weights(nodes, gl):
    """Interpolatory weights of the rule on `nodes` (exact via Gauss-Legendre `gl`)."""
    N = len(nodes)
    Pt = []
    for t, _ in gl:
        v = mp.mpf(1)
        for xk in nodes:
            v *= (t - xk)
        Pt.append(v)
    out = []
    for j in range(N):
        xj = nodes[j]
        if j > N // 2:                            # symmetric rule
            out.append(out[N - 1 - j])
            continue
        dp = mp.mpf(1)
        for k in range(N):
            if k != j:
                dp *= (xj - nodes[k])
        s = mp.fsum(wg * Pt[i] / (t - xj) for i, (t, wg) in enumerate(gl))
        out.append(s / dp)
    return out


def main(path):
    levels = [[mp.mpf(0)]]
    for L in range(1, LEVELS):
        prev = levels[-1]
        newpos = extend(prev)
        nodes = sorted(prev + newpos + [-x for x in newpos])
        levels.append(nodes)
        print("level %d: %d nodes" % (L, len(nodes)), file=sys.stderr)
    gl = GaussLegendre(mp.mp).calc_nodes(8, mp.mp.prec)   # 384 points: exact to degree 767
    allw = []
    for L, nodes in enumerate(levels):
        w = weights(nodes, gl)
        tot = mp.fsum(w)
        if abs(tot - 2) > mp.mpf(10) ** -45:
            raise RuntimeError("level %d weights sum to %s" % (L, tot))
        allw.append(w)
    full = levels[-1]
    # consistency: level L's nodes sit at the documented indices of the full set
    for L, nodes in enumerate(levels):
        step = 2 ** (8 - L)
        for j, x in enumerate(nodes):
            if full[(j + 1) * step - 1] != x:
                raise RuntimeError("node layout mismatch at level %d" % L)
    offs, o = [], 0
    for w in allw:
        offs.append(o)
        o += len(w)

    def lit(x):
        return repr(float(x))

    with open(path, "w") as f:
        f.write("// Generated by gen_patterson.py (Gauss-Patterson rules, Patterson 1968); do not edit.\n")
        f.write("// 511 nodes ascending on [-1,1]; level L uses indices (j+1)*2^(8-L)-1.\n")
        f.write("#pragma once\n\n")
        f.write("#define QLP_PAT_LEVELS 9\n#define QLP_PAT_N 511\n#define QLP_PAT_NW %d\n" % o)
        f.write("#define QLP_PAT_OFFSETS {%s}\n\n" % ", ".join(map(str, offs)))
        f.write("// nodes\n#define QLP_PAT_POINTS_INIT { \\\n")
        for i in range(0, len(full), 4):
            f.write("    " + ", ".join(lit(x) for x in full[i:i + 4]) + ", \\\n")
        f.write("}\n\n// weights, level after level\n#define QLP_PAT_WEIGHTS_INIT { \\\n")
        flat = [x for w in allw for x in w]
        for i in range(0, len(flat), 4):
            f.write("    " + ", ".join(lit(x) for x in flat[i:i + 4]) + ", \\\n")
        f.write("}\n\n")
        f.write("static const int qlp_pat_offset[QLP_PAT_LEVELS] = QLP_PAT_OFFSETS;\n")
        f.write("static const double qlp_pat_points_host[QLP_PAT_N] = QLP_PAT_POINTS_INIT;\n")
        f.write("static const double qlp_pat_weights_host[QLP_PAT_NW] = QLP_PAT_WEIGHTS_INIT;\n")
    print("wrote", path, file=sys.stderr)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "patterson_rule.h"))
