"""Python loader for the C oracle (oracle/qlpix_oracle.c, nfw_oracle.c,
mlp_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py as the checker.  The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from qlens_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libqlpix_oracle.so")
SOURCES = [os.path.join(HERE, "qlpix_oracle.c"), os.path.join(HERE, "nfw_oracle.c"),
           os.path.join(HERE, "mlp_oracle.c")]


def build(force=False):
    """Compile the oracle with gcc (OpenMP, no fused multiply-adds)."""
    deps = SOURCES + [os.path.join(HERE, "qlpix_oracle.h"),
                      os.path.join(os.path.dirname(HERE), "qlens_gb300", "csrc", "patterson_rule.h"),
                      os.path.join(os.path.dirname(HERE), "include", "qlpix.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-Wall", "-Wno-unknown-pragmas"] + SOURCES + ["-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


_lib = None
BRENT_FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.oracle_eval.restype = C.c_int
        _lib.oracle_eval.argtypes = [C.POINTER(abi.qlp_image), C.POINTER(abi.qlp_psf),
                                     C.POINTER(abi.qlp_srcgrid_opts), C.POINTER(abi.qlp_lens), C.c_int,
                                     C.POINTER(abi.qlp_planes), C.POINTER(C.c_double), C.c_double,
                                     C.POINTER(abi.qlp_result)]
        _lib.oracle_get.restype = C.c_long
        _lib.oracle_get.argtypes = [C.c_char_p, C.c_void_p, C.c_long]
        _lib.oracle_threads.restype = C.c_int
        _lib.oracle_set_regopt.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]
        _lib.oracle_set_noise_term.argtypes = [C.c_int]
        _lib.oracle_set_outside_sb.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_long]
        _lib.oracle_brent_min.restype = C.c_double
        _lib.oracle_brent_min.argtypes = [BRENT_FN, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int,
                                          C.POINTER(C.c_int)]
        _lib.oracle_mlp_n_params.restype = C.c_int
        _lib.oracle_mlp_loss_grad.restype = C.c_double
        _lib.oracle_mlp_loss_grad.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                              C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_double)]
    return _lib


_DT = {"srcpt": np.float64, "L_rowptr": np.int32, "L_index": np.int32, "L_value": np.float64,
       "active_index": np.int32, "Lpsf": np.float64, "D": np.float64, "s": np.float64,
       "model": np.float64, "F_diag": np.float64, "grid": np.float64, "osb_sb": np.float64, "osb_maps": np.uint8,
       "osb_penalty": np.float64}


def get(name):
    L = lib()
    n = L.oracle_get(name.encode(), None, 0)
    if n < 0:
        raise KeyError(name)
    out = np.empty(max(n, 0), dtype=_DT[name])
    if n > 0:
        L.oracle_get(name.encode(), out.ctypes.data_as(C.c_void_p), n)
    return out


def evaluate(image_bufs, psf_buf, opts, lens_spec, lens_params=None, regparam=0.0, planes=None, regopt=None,
             noise_term=False, outside_sb=None):
    """Run the oracle; returns the qlp_result as a dict.  regopt: None, or
    (minlog, maxlog, tol, max_iter) for QLens's 'optimize_regparam on';
    noise_term: QLens's 'include_noise_term_in_loglike on'; outside_sb: None,
    or dict(frac, noise_frac, emask_nsplit, emask) for 'outside_sb_prior on'
    (emask: uint8 [nx*ny] or None for every pixel)."""
    L = lib()
    L.oracle_set_noise_term(1 if noise_term else 0)
    if outside_sb is None:
        L.oracle_set_outside_sb(0, 0.3, -1e30, 1, None, 0)
    else:
        em = outside_sb.get("emask")
        em = None if em is None else np.ascontiguousarray(em, dtype=np.uint8)
        L.oracle_set_outside_sb(1, float(outside_sb.get("frac", 0.3)), float(outside_sb.get("noise_frac", -1e30)),
                                int(outside_sb.get("emask_nsplit", 1)), None if em is None else em.ctypes.data,
                                0 if em is None else em.size)
    if regopt is None:
        L.oracle_set_regopt(0, -3.0, 5.0, 0.01, 20)
    else:
        L.oracle_set_regopt(1, *map(float, regopt[:3]), int(regopt[3]))
    lenses = abi.make_lenses(lens_spec)
    pl = planes if planes is not None else abi.make_planes()
    res = abi.qlp_result()
    pp = None
    if lens_params is not None:
        arr = np.ascontiguousarray(lens_params, dtype=np.float64)
        pp = arr.ctypes.data_as(C.POINTER(C.c_double))
    L.oracle_eval(C.byref(image_bufs.image), C.byref(psf_buf.psf), C.byref(opts), lenses, len(lens_spec),
                  C.byref(pl), pp, float(regparam), C.byref(res))
    return res.as_dict()


def threads():
    return lib().oracle_threads()


def mlp_loss_grad(params, x, t):
    """Surrogate network in double precision (mlp_oracle.c): returns
    (loss, dloss/dparams, outputs) for params [n_params], x [n][3], t [n][2]."""
    L = lib()
    p = np.ascontiguousarray(params, dtype=np.float64)
    assert p.shape == (L.oracle_mlp_n_params(),)
    x = np.ascontiguousarray(x, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    g = np.empty_like(p)
    y = np.empty((x.shape[0], 2))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    loss = L.oracle_mlp_loss_grad(dp(p), x.shape[0], dp(x), dp(t), dp(g), dp(y))
    return loss, g, y


def brent_min(f, ax, bx, tol, maxit):
    """QLens's Brent minimiser (oracle_brent_min) on a Python function of one
    variable; returns (x_min, evaluations, list of the points evaluated)."""
    L = lib()
    pts = []

    def cb(x, _):
        pts.append(x)
        return float(f(x))

    fn = BRENT_FN(cb)
    n = C.c_int(0)
    x = L.oracle_brent_min(fn, None, ax, bx, tol, maxit, C.byref(n))
    return x, n.value, pts
