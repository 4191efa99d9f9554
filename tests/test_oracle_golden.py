"""Pin the CPU oracle against golden vectors dumped from the compiled reference.

The fixtures come from oracle/ref_harness.cpp driving QLens's own
invert_image_surface_brightness_map (lens.cpp:12293) and its Cartesian-branch
steps; tests/golden/make_golden.py regenerates them.  The oracle restates the
reference in the same floating-point order, so everything is compared for
exact equality.
"""
import numpy as np
import pytest

from goldens import CASES, Golden
from oracle import oracle as O


@pytest.fixture(scope="module", params=CASES)
def case(request):
    g = Golden(request.param)
    r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    return g, r


def test_status_and_sizes(case):
    g, r = case
    assert r["status"] == 0
    assert r["n_active_pixels"] == int(g.sc["n_active_pixels"])
    assert r["n_active_src"] == int(g.sc["n_active_src"])
    assert r["L_nnz"] == int(g.sc["L_nnz"])


def test_source_points_bitexact(case):
    g, _ = case
    sp = O.get("srcpt")
    assert g.exact("srcpt_x", sp[0::2]) and g.exact("srcpt_y", sp[1::2])


def test_source_grid_bounds(case):
    g, _ = case
    grid = O.get("grid")
    assert grid[0] == g.sc["src_xmin"] and grid[1] == g.sc["src_xmax"]
    assert grid[2] == g.sc["src_ymin"] and grid[3] == g.sc["src_ymax"]


def test_lensing_matrix_bitexact(case):
    g, _ = case
    assert np.array_equal(O.get("active_index"), g.arr["active_index"])
    assert np.array_equal(O.get("L_rowptr"), g.arr["L_rowptr"])
    assert np.array_equal(O.get("L_index"), g.arr["L_index"])
    assert g.exact("L_value", O.get("L_value"))


def test_psf_convolved_rows_bitexact(case):
    g, r = case
    M = r["n_active_src"]
    rows = g.arr["Lpsf_rows"].reshape(-1, M)
    Lp = O.get("Lpsf").reshape(r["n_active_pixels"], M)
    assert np.array_equal(Lp[:rows.shape[0]], rows)
    assert np.allclose(Lp.sum(0), g.arr["Lpsf_colsum"], rtol=1e-12, atol=1e-15)


def test_vectors_exact(case):
    g, _ = case
    for k in ("D", "s", "model", "F_diag"):
        assert np.array_equal(O.get(k), g.arr[k]), k


def test_scalars_exact(case):
    g, r = case
    assert r["m2logev"] == g.sc["m2logev"]
    assert r["chisq0"] == g.sc["chisq0"]
    assert r["logdet_F"] == g.sc["logdetF"]
    assert r["logdet_R"] == g.sc["logdetR"]
    assert r["regterms"] == g.sc["regterms"]


def test_missing_data_sentinel():
    g = Golden("tiny_sie")
    img = g.image.image
    saved = img.surface_brightness
    img.surface_brightness = None
    try:
        r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    finally:
        img.surface_brightness = saved
    assert r["m2logev"] == -1e30


def test_grid_too_small_sentinel():
    g = Golden("tiny_sie")
    g.opts.npixels_x = 1
    r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    assert r["m2logev"] == 2e30


def test_no_source_pixels_sentinel():
    g = Golden("fixed_grid")
    g.opts.xmin, g.opts.xmax, g.opts.ymin, g.opts.ymax = 50.0, 51.0, 50.0, 51.0
    r = O.evaluate(g.image, g.psf, g.opts, g.lenses, planes=g.planes())
    assert r["m2logev"] == 2e30 and r["n_active_src"] == 0
