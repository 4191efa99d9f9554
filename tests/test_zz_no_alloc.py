"""The no-allocation SPD solve (qlp_spd_solve_logdet_noalloc) against qlp_eval.

The entry point is for callers that cannot call cudaMalloc (see
include/qlpix.h): it factors F in a static device scratch.  This test gives it
the F of the tiny_sie golden case (the reference's F, lambda R included) and
the D that qlp_eval computes, in device buffers owned by the test, and checks
log det F and s = F^-1 D against qlp_eval's own results with the 1e-6
relative tolerance of the plain path, on two calls in a row.  The file is
named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from goldens import Golden

pytestmark = pytest.mark.gpu

REL = 1e-6


def _dense_from_packed_upper(p, n):
    F = np.zeros((n, n))
    k = 0
    for i in range(n):
        F[i, i:] = p[k:k + n - i]
        k += n - i
    return F + np.triu(F, 1).T


def test_noalloc_matches_eval_twice():
    torch = pytest.importorskip("torch")
    from qlens_gb300 import PixelLikelihood, QLP_FP64
    g = Golden("tiny_sie")
    pl = PixelLikelihood.from_opts(g.image, g.psf, g.opts, precision=QLP_FP64)
    pl.set_lens_model(g.lenses)
    r = pl.invert_image_surface_brightness_map()
    assert r["status"] == 0
    n = r["n_active_src"]
    d = pl.dump(g.n_sub, r)
    F = _dense_from_packed_upper(g.arr["F_packed_upper"], n)
    dev = torch.device("cuda:0")
    Fd = torch.tensor(F, dtype=torch.float64, device=dev).contiguous()
    Dd = torch.tensor(d["D"], dtype=torch.float64, device=dev)
    lib = pl.lib
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for _ in range(2):
        sd = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        ld = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.qlp_spd_solve_logdet_noalloc(C.c_void_p(Fd.data_ptr()), n, n, C.c_void_p(Dd.data_ptr()),
                                              C.c_void_p(sd.data_ptr()), C.c_void_p(ld.data_ptr()),
                                              C.c_void_p(stream))
        assert rc == 0, lib.qlp_last_error().decode()
        outs.append((sd.cpu().numpy(), float(ld.cpu().item())))
    for s_out, logdet in outs:
        assert abs(logdet - r["logdet_F"]) / abs(r["logdet_F"]) < REL
        assert np.allclose(s_out, d["s"], rtol=REL, atol=REL * np.abs(d["s"]).max())
    # the second call starts from the first call's leftovers and still agrees
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1] == outs[1][1]
    pl.close()


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    from qlens_gb300 import load_library, abi
    lib = load_library()
    dev = torch.device("cuda:0")
    buf = torch.zeros(4, dtype=torch.float64, device=dev)
    p = C.c_void_p(buf.data_ptr())
    rc = lib.qlp_spd_solve_logdet_noalloc(p, 513, 513, p, p, p, None)
    assert rc == abi.QLP_ERR_ARG
    assert b"512" in lib.qlp_last_error()


def _call(lib, F, n, ld, D, stream=None):
    """One call through the C ABI on caller-owned device buffers."""
    import torch
    s = torch.full((n,), float("nan"), dtype=torch.float64, device=F.device)
    lg = torch.full((1,), float("nan"), dtype=torch.float64, device=F.device)
    rc = lib.qlp_spd_solve_logdet_noalloc(C.c_void_p(F.data_ptr()), n, ld, C.c_void_p(D.data_ptr()),
                                          C.c_void_p(s.data_ptr()), C.c_void_p(lg.data_ptr()),
                                          C.c_void_p(stream) if stream else None)
    return rc, s, lg


def test_noalloc_largest_size_with_padded_rows():
    """n = 512 (the scratch's limit) with a leading dimension above n: only the
    lower triangle of the n x n block is read; log det and F^-1 D against
    numpy in FP64, on two calls in a row."""
    torch = pytest.importorskip("torch")
    from qlens_gb300 import load_library
    lib = load_library()
    n, ld = 512, 520
    rng = np.random.default_rng(5)
    A = rng.normal(size=(n, n))
    F = A @ A.T / n + np.eye(n)
    D = rng.normal(size=n)
    Fp = np.full((n, ld), np.nan)
    Fp[:, :n] = np.tril(F) + np.triu(np.full((n, n), np.nan), 1)   # upper triangle never read
    dev = torch.device("cuda:0")
    Fd = torch.tensor(Fp, dtype=torch.float64, device=dev).contiguous()
    Dd = torch.tensor(D, dtype=torch.float64, device=dev)
    ref_logdet = np.linalg.slogdet(F)[1]
    ref_s = np.linalg.solve(F, D)
    for _ in range(2):
        rc, s, lg = _call(lib, Fd, n, ld, Dd, torch.cuda.current_stream().cuda_stream)
        assert rc == 0, lib.qlp_last_error().decode()
        assert abs(float(lg.item()) - ref_logdet) <= REL * abs(ref_logdet)
        assert np.allclose(s.cpu().numpy(), ref_s, rtol=REL, atol=REL * np.abs(ref_s).max())


def test_noalloc_not_positive_definite():
    """An indefinite matrix: QLP_ERR_NOT_SPD with the first non-positive
    pivot's index in qlp_last_error; a following SPD call succeeds (the status
    word starts from zero on every call)."""
    torch = pytest.importorskip("torch")
    from qlens_gb300 import load_library, abi
    lib = load_library()
    n = 5
    F = np.diag([2.0, 1.0, -3.0, 4.0, 5.0]) + 0.01 * (np.ones((n, n)) - np.eye(n))
    dev = torch.device("cuda:0")
    Fd = torch.tensor(F, dtype=torch.float64, device=dev).contiguous()
    Dd = torch.ones(n, dtype=torch.float64, device=dev)
    rc, _s, _lg = _call(lib, Fd, n, n, Dd)
    assert rc == abi.QLP_ERR_NOT_SPD
    assert b"pivot 2" in lib.qlp_last_error()
    G = F.copy()
    G[2, 2] = 3.0
    Gd = torch.tensor(G, dtype=torch.float64, device=dev).contiguous()
    rc, s, lg = _call(lib, Gd, n, n, Dd)
    assert rc == 0, lib.qlp_last_error().decode()
    assert abs(float(lg.item()) - np.linalg.slogdet(G)[1]) <= REL * abs(np.linalg.slogdet(G)[1])
    assert np.allclose(s.cpu().numpy(), np.linalg.solve(G, np.ones(n)), rtol=REL)
