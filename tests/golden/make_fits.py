"""Write the small FITS fixtures under tests/golden/fits/ (test infrastructure).

* image.fits, mask.fits, psf.fits: a lensing data set for the reference's own
  FITS loaders (the golden case fits_synth in make_golden.py): the tiny_sie
  golden's mock image as 32-bit floats in an IMAGE extension (HDU 2, empty
  primary) with PXSIZE and PXNOISE cards; a 20x20 16-bit annular mask smaller
  than the 24x24 image (the loader centres it); and a 9x9 64-bit PSF with
  faint wings and one off-centre pixel above the threshold, so the
  reference's crop keeps a 5x3 box.
* formats.fits: one HDU per pixel type (BITPIX 8, 16 with BZERO 32768, 32 with
  BSCALE/BZERO, 64, -32 holding NaN and -0.0, and a 3-axis cube) for the
  reader's own tests.

The writer follows the FITS standard (4.0): 80-character cards in 2880-byte
blocks, big-endian pixels, data padded with zeros to a whole block.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "fits")


def card(key, value=None, comment=None):
    if value is None:
        s = key.ljust(8)
    else:
        if isinstance(value, bool):
            v = "T" if value else "F"
        elif isinstance(value, str):
            v = ("'" + value.ljust(8) + "'").ljust(20)
        elif isinstance(value, (int, np.integer)):
            v = str(int(value))
        else:
            v = repr(float(value)).upper()
        s = key.ljust(8) + "= " + v.rjust(20)
        if comment:
            s += " / " + comment
    assert len(s) <= 80, s
    return s.ljust(80)


def comment_card(text):
    return ("COMMENT   " + text).ljust(80)


def hdu_bytes(arr_xy, bitpix, primary, extra=(), bscale=None, bzero=None):
    """Stored values arr_xy[i, j] -> FITS pixel (i+1, j+1) (axis 1 fastest)."""
    shape = arr_xy.shape
    cards = [card("SIMPLE", True)] if primary else [card("XTENSION", "IMAGE")]
    cards += [card("BITPIX", bitpix), card("NAXIS", len(shape))]
    for a, n in enumerate(shape):
        cards.append(card("NAXIS%d" % (a + 1), n))
    if primary:
        cards.append(card("EXTEND", True))
    else:
        cards += [card("PCOUNT", 0), card("GCOUNT", 1)]
    if bscale is not None:
        cards.append(card("BSCALE", bscale))
    if bzero is not None:
        cards.append(card("BZERO", bzero))
    cards += list(extra)
    cards.append(card("END"))
    hdr = "".join(cards)
    hdr = hdr.ljust((len(hdr) + 2879) // 2880 * 2880).encode("ascii")
    if len(shape) == 0 or 0 in shape:
        return hdr
    dt = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}[bitpix]
    data = np.asarray(arr_xy).astype(dt).transpose(tuple(range(len(shape)))[::-1]).tobytes()  # axis 1 fastest
    data = data + b"\0" * ((-len(data)) % 2880)
    return hdr + data


def empty_primary():
    hdr = "".join([card("SIMPLE", True), card("BITPIX", 8), card("NAXIS", 0), card("EXTEND", True), card("END")])
    return hdr.ljust(2880).encode("ascii")


def lensing_set():
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from goldens import Golden
    g = Golden("tiny_sie")
    data = g.arr["data"].reshape(g.nx, g.ny)
    img = empty_primary() + hdu_bytes(data.astype(np.float32), -32, False, extra=[
        card("PXSIZE", 0.1, "length of square pixels (in arcsec)"),
        card("PXNOISE", 0.03, "pixel surface brightness noise"),
        comment_card("mock image of a small SIE + shear lens")])
    # 20x20 annulus 0.2" < r < 1.0" on the image's pixel centres (offset 2, 2)
    c = (np.arange(20) + 2 - 12 + 0.5) * 0.1
    r = np.hypot(c[:, None], c[None, :])
    m = ((r > 0.2) & (r < 1.0)).astype(np.int16)
    mask = hdu_bytes(m, 16, True)
    # PSF: tiny_sie's 5x5 kernel scaled, inside 1e-5 wings, with one
    # above-threshold pixel at (1, 4) that widens the crop along x
    k = g.arr["psf"].reshape(5, 5) * 3.7
    p = np.full((9, 9), 1e-5 * k.max())
    p[2:7, 2:7] = k
    p[1, 4] = 0.05 * k.max()
    psf = hdu_bytes(p, -64, True)
    return img, mask, psf


def formats_hdus():
    """(bitpix, stored array, bscale, bzero) per HDU of formats.fits; the
    physical value is bzero + bscale * stored."""
    rng = np.random.default_rng(5)
    u8 = rng.integers(0, 256, (5, 3))
    u16 = rng.integers(0, 65536, (4, 6)) - 32768               # unsigned 16-bit through BZERO 32768
    i32 = rng.integers(-2 ** 31, 2 ** 31, (3, 3))
    i64 = rng.integers(-2 ** 62, 2 ** 62, (2, 4))
    f32 = rng.normal(0, 1, (4, 4)).astype(np.float32)
    f32[0, 0], f32[1, 2] = np.nan, -0.0
    cube = rng.normal(0, 1, (3, 2, 2))
    return [(8, u8, None, None), (16, u16, 1.0, 32768.0), (32, i32, 0.5, -3.0), (64, i64, None, None),
            (-32, f32, None, None), (-64, cube, None, None)]


def formats():
    out = []
    for k, (bitpix, a, bscale, bzero) in enumerate(formats_hdus()):
        out.append(hdu_bytes(a, bitpix, k == 0, bscale=bscale, bzero=bzero))
    return b"".join(out)


def main():
    os.makedirs(OUT, exist_ok=True)
    img, mask, psf = lensing_set()
    for name, b in (("image.fits", img), ("mask.fits", mask), ("psf.fits", psf), ("formats.fits", formats())):
        with open(os.path.join(OUT, name), "wb") as f:
            f.write(b)
        print(name, len(b))


if __name__ == "__main__":
    main()
