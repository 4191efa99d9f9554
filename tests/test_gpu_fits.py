"""FITS files to likelihood on the device: the fits_synth fixtures read by the
library's own loaders (data in HDU 2 with its PXSIZE grid, the 20x20 mask
centred on the 24x24 image, the 9x9 PSF cropped at 1e-2 of its peak), the
uniform noise map of the PXNOISE card, then one evaluation -- against the
reference's -2 log(evidence) for the same files (golden fits_synth), plain
FP64 within 1e-6 relative and mixed precision within the stated bound."""
import os

import numpy as np
import pytest

from goldens import Golden

pytestmark = pytest.mark.gpu

FITS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fits")


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_fits_files_to_likelihood(precision):
    from qlens_gb300 import PixelLikelihood, pixlike
    g = Golden("fits_synth")
    xv, yv, data, info = pixlike.load_data_fits(os.path.join(FITS, "image.fits"), hdu=2)
    mask = pixlike.load_mask_fits(os.path.join(FITS, "mask.fits"), np.ones(data.shape, np.uint8))
    psf = pixlike.load_psf_fits(os.path.join(FITS, "psf.fits"), 1e-2)
    sigma = info["pxnoise"]
    covinv = np.full(data.shape, 1.0 / (sigma * sigma))      # 'sbmap generate_uniform_noisemap'
    pl = PixelLikelihood(xv, yv, data, mask.astype(bool), psf, covinv=covinv, bg_noise=sigma, nsplit=3,
                         src_npixels=(8, 8), regparam=5.0, precision=precision)
    pl.set_lens_model(g.lenses)
    r = pl.invert_image_surface_brightness_map()
    assert r["status"] == 0
    assert r["n_active_pixels"] == int(g.sc["n_active_pixels"]) and r["n_active_src"] == int(g.sc["n_active_src"])
    tol = 1e-6 * abs(g.sc["m2logev"]) if precision == 0 else 0.2
    assert abs(r["m2logev"] - g.sc["m2logev"]) <= tol, (r["m2logev"], g.sc["m2logev"])
    pl.close()
