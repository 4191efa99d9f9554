"""FITS input (the reference's 'sbmap loadimg / loadmask / loadpsf', which it
reads through CFITSIO: pixelgrid.cpp:6016-6870), through the library's own
reader.  No device is needed.

* the reader against the generator's own values for every pixel type
  (tests/golden/fits/formats.fits, written by make_fits.py): BITPIX 8, 16
  through BZERO 32768, 32 with BSCALE/BZERO, 64, -32 with NaN and -0.0, a
  3-axis cube (first plane), primary and IMAGE-extension HDUs;
* the loaders against the reference's own loaders run on the same files
  (golden fits_synth: the harness compiled with a CFITSIO stand-in): pixel
  edges from the PXSIZE card, the image in HDU 2, a smaller mask centred on
  the image, the PSF's threshold crop and normalisation -- all bit-exact;
* the error paths: a missing file, a truncated file, an HDU past the end, a
  mask larger than the image, a PSF whose above-threshold part reaches past
  the symmetric box.
"""
import os
import sys

import numpy as np
import pytest

from goldens import Golden

HERE = os.path.dirname(os.path.abspath(__file__))
FITS = os.path.join(HERE, "golden", "fits")
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_fits  # noqa: E402


def _pl():
    from qlens_gb300 import pixlike
    return pixlike


@pytest.mark.parametrize("k", range(6))
def test_reader_pixel_types(k):
    bitpix, stored, bscale, bzero = make_fits.formats_hdus()[k]
    img, info = _pl().fits_read_image(os.path.join(FITS, "formats.fits"), hdu=k + 1)
    want = stored.astype(np.float64)
    if bscale is not None:
        want = bzero + bscale * want
    if want.ndim == 3:
        want = want[:, :, 0]
    assert info["bitpix"] == bitpix
    assert img.shape == want.shape
    assert np.array_equal(img, want, equal_nan=True)
    assert np.array_equal(np.signbit(img), np.signbit(want))     # -0.0 kept


def test_loaders_match_reference_loaders():
    pl = _pl()
    g = Golden("fits_synth")
    xv, yv, data, info = pl.load_data_fits(os.path.join(FITS, "image.fits"), hdu=2)
    assert info["has_pxsize"] and info["pxsize"] == 0.1
    assert info["has_pxnoise"] and info["pxnoise"] == 0.03
    assert np.array_equal(xv, g.arr["xvals"]) and np.array_equal(yv, g.arr["yvals"])
    assert np.array_equal(data.ravel(), g.arr["data"])
    # 'sbmap loadimg' leaves every pixel in the mask; the 20x20 file is centred
    mask = pl.load_mask_fits(os.path.join(FITS, "mask.fits"), np.ones(data.shape, np.uint8))
    assert np.array_equal(mask.ravel(), g.arr["mask"])
    psf = pl.load_psf_fits(os.path.join(FITS, "psf.fits"), 1e-2)
    assert psf.shape == (int(g.sc["psf_nx"]), int(g.sc["psf_ny"])) == (5, 3)
    assert np.array_equal(psf.ravel(), g.arr["psf"])


def test_data_grid_without_pxsize():
    pl = _pl()
    # the formats file's primary HDU has no PXSIZE: the caller's pixel size,
    # then the caller's bounds, with edges accumulated from the low edge
    p = os.path.join(FITS, "formats.fits")
    xv, yv, d, info = pl.load_data_fits(p, 1, pixel_size=0.05)
    assert not info["has_pxsize"] and d.shape == (5, 3)
    x = -0.5 * 5 * 0.05
    for i in range(6):
        assert xv[i] == x
        x += 0.05
    xv, yv, d, _ = pl.load_data_fits(p, 1, bounds=(-1.0, 2.0, 0.0, 0.3))
    step, y = (0.3 - 0.0) / 3, 0.0
    for j in range(4):
        assert yv[j] == y
        y += step
    assert xv[0] == -1.0 and abs(xv[-1] - 2.0) < 1e-15


def test_mask_add_and_noise_map(tmp_path):
    pl = _pl()
    base = np.zeros((24, 24), np.uint8)
    base[0, 0] = 1
    m = pl.load_mask_fits(os.path.join(FITS, "mask.fits"), base, add=True)
    assert m[0, 0] == 1                                   # outside the file: kept
    m2 = pl.load_mask_fits(os.path.join(FITS, "mask.fits"), np.ones((24, 24), np.uint8), add=True)
    assert m2.all()                                       # adding never unsets
    sig = np.full((4, 3), 0.02)
    sig[1, 2] = 0.01
    f = tmp_path / "noise.fits"
    f.write_bytes(make_fits.hdu_bytes(sig, -64, True))
    cov, mn = pl.load_noise_map_fits(str(f), (4, 3))
    assert mn == 0.01
    assert np.array_equal(cov, 1.0 / (sig * sig))


def test_errors(tmp_path):
    from qlens_gb300.pixlike import QLPixError
    pl = _pl()
    with pytest.raises(QLPixError):
        pl.fits_read_image(str(tmp_path / "missing.fits"))
    raw = open(os.path.join(FITS, "psf.fits"), "rb").read()
    (tmp_path / "trunc.fits").write_bytes(raw[:2880 + 100])
    with pytest.raises(QLPixError):
        pl.fits_read_image(str(tmp_path / "trunc.fits"))
    with pytest.raises(QLPixError):
        pl.fits_read_image(os.path.join(FITS, "formats.fits"), hdu=7)
    with pytest.raises(QLPixError):                       # HDU 1 of image.fits holds no image
        pl.fits_read_image(os.path.join(FITS, "image.fits"), hdu=1)
    with pytest.raises(QLPixError):                       # a 20x20 mask on a 10x10 image
        pl.load_mask_fits(os.path.join(FITS, "mask.fits"), np.ones((10, 10), np.uint8))
    p = np.zeros((6, 6))
    p[3, 3], p[0, 3], p[5, 3] = 1.0, 0.5, 0.5             # even size, signal on both edge rows
    (tmp_path / "edge.fits").write_bytes(make_fits.hdu_bytes(p, -64, True))
    with pytest.raises(QLPixError):
        pl.load_psf_fits(str(tmp_path / "edge.fits"), 1e-2)


def test_header_keyword_rules(tmp_path):
    """QLens's scan of a data image's header (pixelgrid.cpp:6059-6116): a card
    holding 'ql: ' opens a run of COMMENT cards that the scan reads as text,
    and the first card after the run that is not a COMMENT ends the scan --
    keywords after it are not read; keywords before it are."""
    pl = _pl()
    img = np.arange(12, dtype=np.float64).reshape(4, 3)
    extra = [make_fits.card("PXNOISE", 0.5), make_fits.card("ZLENS", 0.3),
             make_fits.comment_card("ql: model description"), make_fits.comment_card("second line"),
             make_fits.card("PXSIZE", 0.07), make_fits.card("ZSRC", 2.0)]
    f = tmp_path / "hdr.fits"
    f.write_bytes(make_fits.hdu_bytes(img, -64, True, extra=extra))
    data, info = pl.fits_read_image(str(f))
    assert np.array_equal(data, img)
    assert info["has_pxnoise"] and info["pxnoise"] == 0.5
    assert info["has_zlens"] and info["zlens"] == 0.3
    assert not info["has_pxsize"] and not info["has_zsrc"]
    # without the comment run every keyword is read, and PXSIZE sets the grid
    f2 = tmp_path / "hdr2.fits"
    f2.write_bytes(make_fits.hdu_bytes(img, -64, True, extra=[make_fits.card("PXSIZE", 0.07),
                                                              make_fits.card("ZSRC", 2.0)]))
    xv, yv, d, info = pl.load_data_fits(str(f2), pixel_size=0.5)
    assert info["has_pxsize"] and info["pxsize"] == 0.07 and info["zsrc"] == 2.0
    assert xv[0] == -0.5 * 4 * 0.07 and yv[0] == -0.5 * 3 * 0.07      # the file's PXSIZE wins
