"""Seeded synthetic workloads with the shapes of the reference's benchmark configurations.

No dataset is involved: every image is a mock made here (an elliptical Sersic
source lensed by an SIE + external shear, convolved with the PSF, plus seeded
Gaussian noise), and every lens-parameter vector is drawn from the stated
prior boxes.  The numbers that matter for the likelihood's cost -- image size,
mask, split factor, PSF size, source-grid size -- follow the configurations:

  cfg1  80x80 @ 0.05", r < 2.5" mask, 2x2 split, 7x7 Gaussian PSF, 30x30 source, SIE+shear
  cfg2  200x200 @ 0.04", annulus 0.5"-2.5", 4x4 split, 21x21 Airy-like PSF, 64x64 source,
        power law alpha in [0.9,1.2], b in [1,1.5], q in [0.6,0.95], shear in [0,0.1], sigma 0.01
  cfg3  100x100 @ 0.05", per-instance circle r in [1.5,3.0]", 2x2 split, 11x11 Gaussian PSF,
        source side in [20,64], SIE+shear (b,q,phi,x0,y0,gamma,phi_gamma) + log lambda
  cfg4  200x200 @ 0.04", r < 4.5" (the whole frame), 4x4 split (~640k rays), 21x21 Airy-like PSF,
        48x48 source, SIE host + elliptical NFW ks in [0.05,0.5], rs in [2,20]", q in [0.5,1]
  cfg5  300x300 @ 0.03", annulus 0.3"-3.5", 4x4 split, 31x31 Airy-like PSF, 48x48 source; two lens
        planes: SIE + shear at z=0.5, NFW subhalo (ks in [0.05,0.3], rs in [0.05,0.3]") at z=0.8,
        source at z=2 (plane factors: the reference's own for those redshifts)
"""
import math

import numpy as np

from .pixlike import gaussian_psf, pixel_corners


def annulus_mask(xvals, yvals, rmin, rmax, xc=0.0, yc=0.0):
    """ImagePixelData::set_mask_annulus (pixelgrid.cpp:7447-7500), full circle."""
    x = 0.5 * (xvals[:-1] + xvals[1:])
    y = 0.5 * (yvals[:-1] + yvals[1:])
    X, Y = np.meshgrid(x, y, indexing="ij")
    rsq = (X - xc) ** 2 + (Y - yc) ** 2
    return ((rsq > rmin * rmin) & (rsq < rmax * rmax)).astype(np.uint8)


def airy_psf(n, pixel, fwhm):
    """Airy-like kernel, (2 J1(x)/x)^2 sampled at pixel centres, normalised to 1."""
    try:
        from scipy.special import j1
    except Exception:  # pragma: no cover - scipy is in the image
        j1 = None
    h = n // 2
    c = (np.arange(n) - h) * pixel
    X, Y = np.meshgrid(c, c, indexing="ij")
    r = np.sqrt(X * X + Y * Y)
    # first zero of J1 at 3.8317; FWHM of the Airy core ~ 1.029 lambda/D -> scale
    k = 1.6163 * 2 / fwhm
    x = k * r
    if j1 is not None:
        with np.errstate(invalid="ignore", divide="ignore"):
            v = np.where(x > 1e-12, (2 * j1(x) / np.where(x > 1e-12, x, 1.0)) ** 2, 1.0)
    else:
        v = np.exp(-0.5 * (r / (fwhm / 2.3548)) ** 2)
    return v / v.sum()


def _sie_shear_sourcepts(x, y, b, q, theta_deg, shear, shear_deg, xc=0.0, yc=0.0):
    """Vectorised SIE + shear lens equation in QLens's conventions (emode 1,
    major axis north), for making mock images only."""
    th = math.radians(theta_deg)
    cs, sn = -math.sin(th), math.cos(th)
    dx, dy = x - xc, y - yc
    xr = dx * cs + dy * sn
    yr = -dx * sn + dy * cs
    bp = b / math.sqrt(q)
    qsq = q * q
    psi = np.sqrt(qsq * xr * xr + yr * yr)
    u = math.sqrt(1 - qsq)
    ax = (bp * q / u) * np.arctan(u * xr / psi)
    ay = (bp * q / u) * np.arctanh(u * yr / psi)
    axr = ax * cs - ay * sn
    ayr = ax * sn + ay * cs
    te = math.radians(shear_deg) + math.pi / 2
    g1, g2 = shear * math.cos(2 * te), shear * math.sin(2 * te)
    sx = dx * g1 + dy * g2
    sy = -dy * g1 + dx * g2
    return x - (axr + sx), y - (ayr + sy)


def _sersic(bx, by, s0, reff, n, q, theta_deg, xc, yc):
    th = math.radians(theta_deg)
    dx, dy = bx - xc, by - yc
    xr = dx * math.cos(th) + dy * math.sin(th)
    yr = -dx * math.sin(th) + dy * math.cos(th)
    r = np.sqrt(q * xr * xr + yr * yr / q)
    bn = 2 * n - 1.0 / 3 + 4.0 / (405 * n)
    return s0 * np.exp(-bn * ((r / reff) ** (1.0 / n) - 1))


def mock_image(xvals, yvals, psf, noise, seed, lens=(1.2, 0.8, 30.0, 0.05, 10.0), nsplit=2,
               source=(1.0, 0.15, 1.5, 0.8, 20.0, 0.05, 0.0)):
    """Lensed, PSF-convolved, noisy Sersic image [i*ny + j layout as (nx, ny)]."""
    nx, ny = len(xvals) - 1, len(yvals) - 1
    img = np.zeros((nx, ny))
    for ii in range(nsplit):
        for jj in range(nsplit):
            u0 = (1 + 2 * ii) / (2 * nsplit)
            w0 = (1 + 2 * jj) / (2 * nsplit)
            x = (1 - u0) * xvals[:-1] + u0 * xvals[1:]
            y = (1 - w0) * yvals[:-1] + w0 * yvals[1:]
            X, Y = np.meshgrid(x, y, indexing="ij")
            bx, by = _sie_shear_sourcepts(X, Y, *lens)
            img += _sersic(bx, by, *source)
    img /= nsplit * nsplit
    # direct convolution (same orientation convention as the PSF taps)
    pnx, pny = psf.shape
    out = np.zeros_like(img)
    hx, hy = pnx // 2, pny // 2
    pad = np.pad(img, ((hx, hx), (hy, hy)))
    for k in range(pnx):
        for l in range(pny):
            out += psf[k, l] * pad[2 * hx - k:2 * hx - k + nx, 2 * hy - l:2 * hy - l + ny]
    rng = np.random.default_rng(seed)
    return out + noise * rng.standard_normal(out.shape)


class Workload:
    """Everything needed to construct a PixelLikelihood and draw parameters."""

    def __init__(self, name, xvals, yvals, data, mask, psf, noise, nsplit, src_npixels, lenses, regparam,
                 draw, instance_masks=None, instance_src=None, zfac=None, beta=None):
        self.name = name
        self.xvals, self.yvals, self.data, self.mask, self.psf = xvals, yvals, data, mask, psf
        self.noise = noise
        self.nsplit = nsplit
        self.src_npixels = src_npixels
        self.lenses = lenses
        self.regparam = regparam
        self.draw = draw
        self.instance_masks = instance_masks
        self.instance_src = instance_src
        self.zfac, self.beta = zfac, beta
        self.draw_instances = None     # (rng, n) -> (mask ids, source sizes, lambdas) for uneven batches

    @property
    def n_mask(self):
        return int(self.mask.sum())

    def describe(self):
        return dict(workload=self.name, image="%dx%d" % (len(self.xvals) - 1, len(self.yvals) - 1),
                    masked_pixels=self.n_mask, nsplit=self.nsplit, psf="%dx%d" % self.psf.shape,
                    source_grid="%dx%d" % tuple(self.src_npixels))


def cfg1(seed=10):
    xv = pixel_corners(80, -2.0, 2.0)
    yv = pixel_corners(80, -2.0, 2.0)
    psf = gaussian_psf(0.04247, 0.04247, 0.05, 0.05)
    data = mock_image(xv, yv, psf, 0.02, seed)
    mask = annulus_mask(xv, yv, 0.0, 2.5)
    lenses = [dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0]),
              dict(type="shear", params=[0.05, 10.0, 0.0, 0.0])]

    def draw(rng, n):
        p = np.tile(np.array([1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0, 0.05, 10.0, 0.0, 0.0]), (n, 1))
        p[:, 0] = rng.uniform(1.1, 1.3, n)
        p[:, 3] = rng.uniform(0.7, 0.9, n)
        p[:, 4] = rng.uniform(20, 40, n)
        return p

    return Workload("cfg1: 80x80, r<2.5\", 2x2 split, 7x7 PSF, 30x30 source, SIE+shear", xv, yv, data, mask, psf,
                    0.02, 2, (30, 30), lenses, 10.0, draw)


def cfg2(seed=2):
    xv = pixel_corners(200, -4.0, 4.0)
    yv = pixel_corners(200, -4.0, 4.0)
    psf = airy_psf(21, 0.04, 0.1)
    data = mock_image(xv, yv, psf, 0.01, seed, lens=(1.25, 0.78, 25.0, 0.05, 15.0), nsplit=2,
                      source=(1.0, 0.2, 1.5, 0.75, 20.0, 0.04, -0.02))
    mask = annulus_mask(xv, yv, 0.5, 2.5)
    lenses = [dict(type="sple", params=[1.25, 1.05, 0.0, 0.78, 25.0, 0.0, 0.0]),
              dict(type="shear", params=[0.05, 15.0, 0.0, 0.0])]

    def draw(rng, n):
        p = np.zeros((n, 11))
        p[:, 0] = rng.uniform(1.0, 1.5, n)      # b
        p[:, 1] = rng.uniform(0.9, 1.2, n)      # alpha (slope)
        p[:, 2] = 0.0                           # s (core-free)
        p[:, 3] = rng.uniform(0.6, 0.95, n)     # q
        p[:, 4] = rng.uniform(0.0, 180.0, n)    # theta
        p[:, 7] = rng.uniform(0.0, 0.1, n)      # shear
        p[:, 8] = rng.uniform(0.0, 180.0, n)    # shear angle
        return p

    return Workload("cfg2: 200x200 @0.04\", annulus 0.5-2.5\", 4x4 split, 21x21 Airy PSF, 64x64 source, power law",
                    xv, yv, data, mask, psf, 0.01, 4, (64, 64), lenses, 10.0, draw)


def cfg3(seed=3, n_instances=64):
    xv = pixel_corners(100, -2.5, 2.5)
    yv = pixel_corners(100, -2.5, 2.5)
    psf = gaussian_psf(0.082, 0.082, 0.05, 0.05)   # half-width round(3.035*0.082/0.05) = 5 -> 11x11
    data = mock_image(xv, yv, psf, 0.02, seed)
    mask = annulus_mask(xv, yv, 0.0, 3.0)
    rng = np.random.default_rng(seed)
    radii = rng.uniform(1.5, 3.0, n_instances)
    masks = np.stack([annulus_mask(xv, yv, 0.0, r).ravel() for r in radii])
    sides = rng.integers(20, 65, n_instances)
    lenses = [dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0]),
              dict(type="shear", params=[0.05, 10.0, 0.0, 0.0])]

    def draw(rng, n):
        p = np.zeros((n, 11))
        b = rng.uniform(1.0, 1.4, n)
        x0 = rng.uniform(-0.1, 0.1, n)
        y0 = rng.uniform(-0.1, 0.1, n)
        p[:, 0] = b
        p[:, 1] = 1.0
        p[:, 3] = rng.uniform(0.6, 0.95, n)
        p[:, 4] = rng.uniform(0, 180, n)
        p[:, 5], p[:, 6] = x0, y0
        p[:, 7] = rng.uniform(0.0, 0.1, n)
        p[:, 8] = rng.uniform(0, 180, n)
        p[:, 9], p[:, 10] = x0, y0
        return p

    wl = Workload("cfg3: 100x100 @0.05\", per-instance r in [1.5,3]\", 2x2 split, 11x11 PSF, source side 20-64",
                  xv, yv, data, mask, psf, 0.02, 2, (64, 64), lenses, 10.0, draw,
                  instance_masks=masks, instance_src=np.stack([sides, sides], 1))

    def draw_instances(rng, n):
        """Per vector: one of the instance masks, its own source-grid side
        (uniform 20-64) and regularisation parameter (log10 lambda uniform 0-2)."""
        ids = rng.integers(0, n_instances, n)
        side = rng.integers(20, 65, n)
        lam = 10.0 ** rng.uniform(0.0, 2.0, n)
        return ids, np.stack([side, side], 1), lam

    wl.draw_instances = draw_instances
    return wl


def cfg4(seed=4):
    xv = pixel_corners(200, -4.0, 4.0)
    yv = pixel_corners(200, -4.0, 4.0)
    psf = airy_psf(21, 0.04, 0.1)
    data = mock_image(xv, yv, psf, 0.01, seed, lens=(1.2, 0.8, 30.0, 0.0, 0.0), nsplit=2,
                      source=(1.0, 0.2, 1.5, 0.75, 20.0, 0.04, -0.02))
    mask = annulus_mask(xv, yv, 0.0, 4.5)
    lenses = [dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0]),
              dict(type="nfw", params=[0.2, 8.0, 0.7, 40.0, 0.3, -0.2])]

    def draw(rng, n):
        p = np.zeros((n, 13))
        p[:, 0] = rng.uniform(1.0, 1.4, n)      # SIE b
        p[:, 1] = 1.0
        p[:, 3] = rng.uniform(0.6, 0.95, n)     # SIE q
        p[:, 4] = rng.uniform(0.0, 180.0, n)
        p[:, 7] = rng.uniform(0.05, 0.5, n)     # NFW ks
        p[:, 8] = rng.uniform(2.0, 20.0, n)     # NFW rs
        p[:, 9] = rng.uniform(0.5, 1.0, n)      # NFW q
        p[:, 10] = rng.uniform(0.0, 180.0, n)   # NFW theta
        p[:, 11] = 0.3 + rng.uniform(-0.5, 0.5, n)
        p[:, 12] = -0.2 + rng.uniform(-0.5, 0.5, n)
        return p

    return Workload("cfg4: 200x200 @0.04\", r<4.5\", 4x4 split, 21x21 Airy PSF, 48x48 source, SIE + elliptical NFW",
                    xv, yv, data, mask, psf, 0.01, 4, (48, 48), lenses, 10.0, draw)


# QLens's own plane factors for lens planes at z = 0.5 and 0.8 and a source at
# z = 2 (default cosmology; the twoplane golden case records the same numbers)
CFG5_ZFAC = [1.0, 1.0]
CFG5_BETA = [[0.50757349]]


def cfg5(seed=5):
    xv = pixel_corners(300, -4.5, 4.5)
    yv = pixel_corners(300, -4.5, 4.5)
    psf = airy_psf(31, 0.03, 0.08)
    data = mock_image(xv, yv, psf, 0.01, seed, lens=(1.2, 0.8, 30.0, 0.05, 10.0), nsplit=2,
                      source=(1.0, 0.2, 1.5, 0.75, 20.0, 0.04, -0.02))
    mask = annulus_mask(xv, yv, 0.3, 3.5)
    lenses = [dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0], plane=0),
              dict(type="shear", params=[0.05, 10.0, 0.0, 0.0], plane=0),
              dict(type="nfw", params=[0.1, 0.1, 0.8, 0.0, 0.9, 0.6], plane=1)]

    def draw(rng, n):
        p = np.zeros((n, 17))
        p[:, 0] = rng.uniform(1.0, 1.4, n)
        p[:, 1] = 1.0
        p[:, 3] = rng.uniform(0.6, 0.95, n)
        p[:, 4] = rng.uniform(0.0, 180.0, n)
        p[:, 7] = rng.uniform(0.0, 0.1, n)
        p[:, 8] = rng.uniform(0.0, 180.0, n)
        p[:, 11] = rng.uniform(0.05, 0.3, n)    # subhalo ks
        p[:, 12] = rng.uniform(0.05, 0.3, n)    # subhalo rs
        p[:, 13] = rng.uniform(0.5, 1.0, n)
        p[:, 14] = rng.uniform(0.0, 180.0, n)
        ang = rng.uniform(0, 2 * math.pi, n)
        p[:, 15] = 1.2 * np.cos(ang)            # on the Einstein ring
        p[:, 16] = 1.2 * np.sin(ang)
        return p

    return Workload("cfg5: 300x300 @0.03\", annulus 0.3-3.5\", 4x4 split, 31x31 Airy PSF, 48x48 source, "
                    "two planes (SIE+shear z=0.5, NFW subhalo z=0.8)",
                    xv, yv, data, mask, psf, 0.01, 4, (48, 48), lenses, 10.0, draw, zfac=CFG5_ZFAC, beta=CFG5_BETA)


CONFIGS = {"cfg1": cfg1, "cfg2": cfg2, "cfg3": cfg3, "cfg4": cfg4, "cfg5": cfg5}
