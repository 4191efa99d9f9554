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
    d = pl.dump(g.arr["srcpt_x"].size, r)
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
