"""CPU-only checks of the C ABI library and the host-side set-up.

* libqlpix.so loads and exports every function include/qlpix.h declares
  (no compute call is made without a GPU);
* without a GPU the library refuses to create a context (no CPU fallback);
* the host helpers that rebuild QLens's inputs -- the Gaussian PSF of
  QLens::generate_PSF_matrix, the pixel corners of ImagePixelGrid and the
  annulus mask of ImagePixelData::set_mask_annulus -- equal what the compiled
  reference produced for the golden cases.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from goldens import Golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "qlpix.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qlp_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from qlens_gb300 import pixlike
    return pixlike.load_library(build_if_missing=True)


def test_every_declared_symbol_is_exported(lib):
    names = _declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_gpu_means_no_context(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from qlens_gb300 import abi
    g = Golden("tiny_sie")
    st = C.c_int(-1)
    ctx = lib.qlp_create(C.byref(g.image.image), C.byref(g.psf.psf), C.byref(g.opts), 0, C.byref(st))
    assert not ctx
    assert st.value == abi.QLP_ERR_NO_DEVICE
    assert lib.qlp_last_error()


def test_srcgrid_defaults_match_python(lib):
    from qlens_gb300 import abi
    o = abi.qlp_srcgrid_opts()
    lib.qlp_srcgrid_defaults(C.byref(o))
    p = abi.srcgrid_defaults()
    for name, _ in abi.qlp_srcgrid_opts._fields_:
        if name in ("npixels_x", "npixels_y"):
            continue
        assert getattr(o, name) == getattr(p, name), name


@pytest.mark.parametrize("name,sigma", [("cfg1", 0.04247), ("powerlaw", 0.05), ("tiny_sie", 0.06)])
def test_gaussian_psf_matches_reference(name, sigma):
    from qlens_gb300 import gaussian_psf
    g = Golden(name)
    xv = g.arr["xvals"]
    px = (xv[-1] - xv[0]) / (len(xv) - 1)
    psf = gaussian_psf(sigma, sigma, px, px)
    ref = g.psf.arr
    assert psf.shape == ref.shape
    assert np.allclose(psf, ref, rtol=1e-14, atol=0)


@pytest.mark.parametrize("name", ["cfg1", "powerlaw", "tiny_sie", "fixed_grid"])
def test_pixel_corners_and_masks_match_reference(name):
    from qlens_gb300 import pixel_corners, synthetic
    g = Golden(name)
    xv, yv = g.arr["xvals"], g.arr["yvals"]
    assert np.array_equal(pixel_corners(len(xv) - 1, xv[0], xv[-1]), xv)
    assert np.array_equal(pixel_corners(len(yv) - 1, yv[0], yv[-1]), yv)
    for line in g.meta["script"].splitlines():
        w = line.split()
        if len(w) >= 6 and w[0] == "sbmap" and w[1] == "set_data_annulus":
            xc, yc, rmin, rmax = map(float, w[2:6])
            m = synthetic.annulus_mask(xv, yv, rmin, rmax, xc, yc)
            assert np.array_equal(m.ravel(), g.arr["mask"])


def test_lens_param_packing():
    from qlens_gb300 import abi
    spec = [dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0]),
            dict(type="shear", params=[0.05, 10.0, 0.0, 0.0])]
    arr = abi.make_lenses(spec)
    assert arr[0].type == abi.QLP_LENS_SPLE and arr[1].type == abi.QLP_LENS_SHEAR
    assert abi.n_params(spec) == 11
    assert abi.flat_params(spec)[7] == 0.05
