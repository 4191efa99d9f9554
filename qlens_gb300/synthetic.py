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
  cfg5  300x300 @ 0.03", annulus 0.3"-3.5", 4x4 split, 31x31 Airy-like PSF; two lens planes: SIE +
        shear at z=0.5, elliptical NFW subhalo at z=0.8 given by its mass (m200 log-uniform in
        1e8-1e10 M_sun, c200 uniform in 5-20; QLens 'pmode=1'), source at z=2 (plane factors and
        the subhalo's cosmology: the reference's own for those redshifts); per vector its own
        source grid, side uniform in 32-64; batches of 1024 vectors
  cfg5_fixed  the same two-plane workload with one 48x48 source grid for every vector and the
        subhalo given by ks, rs (both uniform in 0.05-0.3)
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
    ax, ay = _sie_shear_deflection(x, y, b, q, theta_deg, shear, shear_deg, xc, yc)
    return x - ax, y - ay


def _nfw_kappa(ks, rs, rsq):
    """NFW convergence kappa(r^2) (QLens NFW::kappa_rsq), vectorised."""
    xsq = rsq / (rs * rs)
    out = np.empty_like(xsq)
    lo = xsq < 1.0 - 1e-5
    hi = xsq > 1.0 + 1e-5
    mid = ~(lo | hi)
    s = np.sqrt(1.0 - xsq[lo])
    out[lo] = 2 * ks * (1 - np.arctanh(s) / s) / (xsq[lo] - 1)
    s = np.sqrt(xsq[hi] - 1.0)
    out[hi] = 2 * ks * (1 - np.arctan(s) / s) / (xsq[hi] - 1)
    out[mid] = 2 * ks * (1.0 / 3 - (xsq[mid] - 1) / 5.0)
    return out


def _nfw_deflection(x, y, ks, rs, q, theta_deg, xc, yc, nodes=64):
    """Elliptical NFW deflection (QLens's LensProfile::deflection_numerical
    integrals, emode 1, major axis north) by fixed Gauss-Legendre quadrature,
    vectorised -- for making mock images only."""
    th = math.radians(theta_deg)
    cs, sn = -math.sin(th), math.cos(th)
    dx, dy = x - xc, y - yc
    xr = dx * cs + dy * sn
    yr = -dx * sn + dy * cs
    t, wt = np.polynomial.legendre.leggauss(nodes)
    eps = 1.0 - q * q
    I0 = np.zeros_like(xr)
    I1 = np.zeros_like(xr)
    xsq, ysq = xr * xr, yr * yr
    for tk, wk in zip(t, wt):
        w = 0.5 + 0.5 * tk
        u = w * w
        qfac = 1.0 - eps * u
        f = 2 * w * _nfw_kappa(ks, rs, u * (xsq + ysq / qfac) * q)
        I0 += 0.5 * wk * f / math.sqrt(qfac)
        I1 += 0.5 * wk * f / (qfac * math.sqrt(qfac))
    bx, by = xr * (q * I0), yr * (q * I1)
    return bx * cs - by * sn, bx * sn + by * cs


def nfw_ks_rs_from_m200_c200(m200, c200, cosmo):
    """QLens's NFW::set_ks_rs_from_m200_c200 (models.cpp:968-976) for the
    lens cosmology (sigma_cr, kpc_to_arcsec, critical_density)."""
    sigma_cr, kpc_to_arcsec, rho_crit = cosmo
    rvir_kpc = (m200 / (200.0 * 12.5663706144 / 3.0 * 1e-9 * rho_crit)) ** 0.333333333333
    rs = rvir_kpc / c200 * kpc_to_arcsec
    ks = m200 / (12.5663706144 * rs * rs * sigma_cr * (math.log(1 + c200) - c200 / (1 + c200)))
    return ks, rs


def _sie_shear_deflection(x, y, b, q, theta_deg, shear, shear_deg, xc=0.0, yc=0.0):
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
    return axr + sx, ayr + sy


def _sersic(bx, by, s0, reff, n, q, theta_deg, xc, yc):
    th = math.radians(theta_deg)
    dx, dy = bx - xc, by - yc
    xr = dx * math.cos(th) + dy * math.sin(th)
    yr = -dx * math.sin(th) + dy * math.cos(th)
    r = np.sqrt(q * xr * xr + yr * yr / q)
    bn = 2 * n - 1.0 / 3 + 4.0 / (405 * n)
    return s0 * np.exp(-bn * ((r / reff) ** (1.0 / n) - 1))


def mock_image(xvals, yvals, psf, noise, seed, lens=(1.2, 0.8, 30.0, 0.05, 10.0), nsplit=2,
               source=(1.0, 0.15, 1.5, 0.8, 20.0, 0.05, 0.0), subhalo=None):
    """Lensed, PSF-convolved, noisy Sersic image [i*ny + j layout as (nx, ny)].
    subhalo: None, or (ks, rs, q, theta_deg, xc, yc, beta) -- an elliptical NFW
    on a second lens plane whose rays are deflected by the first plane's
    deflection times beta (QLens's two-plane recursion with unit plane factors)."""
    nx, ny = len(xvals) - 1, len(yvals) - 1
    img = np.zeros((nx, ny))
    for ii in range(nsplit):
        for jj in range(nsplit):
            u0 = (1 + 2 * ii) / (2 * nsplit)
            w0 = (1 + 2 * jj) / (2 * nsplit)
            x = (1 - u0) * xvals[:-1] + u0 * xvals[1:]
            y = (1 - w0) * yvals[:-1] + w0 * yvals[1:]
            X, Y = np.meshgrid(x, y, indexing="ij")
            ax, ay = _sie_shear_deflection(X, Y, *lens)
            bx, by = X - ax, Y - ay
            if subhalo is not None:
                ks, rs, sq, sth, sxc, syc, beta = subhalo
                a2x, a2y = _nfw_deflection(X - beta * ax, Y - beta * ay, ks, rs, sq, sth, sxc, syc)
                bx, by = bx - a2x, by - a2y
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
        self.batch = None              # the workload's batch per step (None: the bench's default)
        self.uneven_note = None
        self.draw_prior = None         # (rng, n) -> vectors from the whole prior box, where draw() is narrower
        self.draws_note = None

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
    wl.batch = 4096
    wl.uneven_note = ("per vector: one of %d masks (r 1.5-3.0\"), source side 20-64, log10 lambda 0-2"
                      % n_instances)
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
# The cosmology QLens's lens object holds for an NFW lens at z = 0.8 with the
# source at z = 2 (default cosmology): sigma_cr (M_sun/arcsec^2),
# kpc_to_arcsec, critical_density(0.8) (M_sun/Mpc^3) -- the cfg5_m200 golden
# case records the same numbers from the reference.
CFG5_SUBHALO_COSMO = [131218470966.34126, 0.13318529787886016, 333084360000.0]


# The cfg5 mock's subhalo: m200 = 1e9 M_sun, c200 = 10, q = 0.8 at (0.9", 0.6")
# on the Einstein ring, on the z = 0.8 plane.
CFG5_SUBHALO_TRUTH = (1e9, 10.0, 0.8, 0.0, 0.9, 0.6)
# The cfg5 mock's pixel noise: a peak signal-to-noise of ~75 (the lensed
# source peaks near 7.6).
CFG5_NOISE = 0.1
# Widths of the cfg5 posterior at the mock's parameters, per entry of the
# lens-parameter vector (b, q, theta, shear, shear angle; subhalo m200, c200,
# q, theta, x, y): the curvature of -2 log(evidence) along each parameter,
# sigma = sqrt(2 / (d^2(-2 log ev)/dp^2)), measured with the library's plain
# FP64 path by central differences.
CFG5_SIGMA = {0: 2e-5, 3: 6e-5, 4: 2e-3, 7: 4e-5, 8: 1e-2, 11: 5e6, 12: 0.12, 13: 5e-3, 14: 2.0, 15: 2e-3,
              16: 1e-3}


def cfg5(seed=5, batch_sides=(32, 64), widths=1.0):
    """Two-plane subhalo workload: the subhalo by its mass and concentration,
    uneven source grids (side uniform in batch_sides per vector).

    The mock image is made with the subhalo in it (numpy ray tracing through
    both planes).  draw() gives the batch of the posterior region, where a
    sampler's late live points and its proposals concentrate: every
    parameter uniform within +-3 posterior widths (CFG5_SIGMA, times
    `widths`) of the mock's values.  draw_prior() gives vectors from the whole
    prior box instead (the subhalo's m200 log-uniform over 1e8-1e10 M_sun),
    where the model fits the data badly."""
    xv = pixel_corners(300, -4.5, 4.5)
    yv = pixel_corners(300, -4.5, 4.5)
    psf = airy_psf(31, 0.03, 0.08)
    m, c, sq, sth, sxc, syc = CFG5_SUBHALO_TRUTH
    ks, rs = nfw_ks_rs_from_m200_c200(m, c, CFG5_SUBHALO_COSMO)
    data = mock_image(xv, yv, psf, CFG5_NOISE, seed, lens=(1.2, 0.8, 30.0, 0.05, 10.0), nsplit=2,
                      source=(1.0, 0.2, 1.5, 0.75, 20.0, 0.04, -0.02),
                      subhalo=(ks, rs, sq, sth, sxc, syc, CFG5_BETA[0][0]))
    mask = annulus_mask(xv, yv, 0.3, 3.5)
    lenses = [dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0], plane=0),
              dict(type="shear", params=[0.05, 10.0, 0.0, 0.0], plane=0),
              dict(type="nfw_m200_c", params=list(CFG5_SUBHALO_TRUTH), plane=1, cosmo=CFG5_SUBHALO_COSMO)]

    def subhalo(rng, p):
        n = len(p)
        p[:, 11] = 10.0 ** rng.uniform(8.0, 10.0, n)   # m200 (M_sun)
        p[:, 12] = rng.uniform(5.0, 20.0, n)          # c200
        p[:, 13] = rng.uniform(0.5, 1.0, n)           # q
        p[:, 14] = rng.uniform(0.0, 180.0, n)         # theta
        p[:, 15] = sxc + rng.uniform(-0.1, 0.1, n)
        p[:, 16] = syc + rng.uniform(-0.1, 0.1, n)

    truth = np.zeros(17)
    truth[[0, 1, 3, 4, 7, 8]] = [1.2, 1.0, 0.8, 30.0, 0.05, 10.0]
    truth[11:17] = CFG5_SUBHALO_TRUTH

    def draw(rng, n):
        p = np.tile(truth, (n, 1))
        for i, sg in CFG5_SIGMA.items():
            p[:, i] += widths * 3.0 * sg * rng.uniform(-1.0, 1.0, n)
        p[:, 13] = np.minimum(p[:, 13], 0.999)
        return p

    def draw_prior(rng, n):
        p = np.zeros((n, 17))
        p[:, 0] = rng.uniform(1.0, 1.4, n)
        p[:, 1] = 1.0
        p[:, 3] = rng.uniform(0.6, 0.95, n)
        p[:, 4] = rng.uniform(0.0, 180.0, n)
        p[:, 7] = rng.uniform(0.0, 0.1, n)
        p[:, 8] = rng.uniform(0.0, 180.0, n)
        subhalo(rng, p)
        return p

    def draw_instances(rng, n):
        """Per vector its own source-grid side (uniform in 32-64); the
        image's mask and the context's lambda."""
        side = rng.integers(batch_sides[0], batch_sides[1] + 1, n)
        return None, np.stack([side, side], 1), None

    wl = Workload("cfg5: 300x300 @0.03\", annulus 0.3-3.5\", 4x4 split, 31x31 Airy PSF, two planes (SIE+shear "
                  "z=0.5, NFW subhalo m200 1e8-1e10 Msun z=0.8), source grids 32x32-64x64 per vector",
                  xv, yv, data, mask, psf, CFG5_NOISE, 4, (batch_sides[1], batch_sides[1]), lenses, 10.0, draw,
                  zfac=CFG5_ZFAC, beta=CFG5_BETA)
    wl.draw_prior = draw_prior
    wl.draw_instances = draw_instances
    wl.batch = 1024
    wl.uneven_note = "per vector: source grid side uniform in %d-%d" % batch_sides
    wl.draws_note = ("posterior region: every parameter uniform within +-%.3g posterior widths of the mock's "
                     "(subhalo m200 = 1e9 M_sun, c200 = 10); prior box: m200 log-uniform 1e8-1e10 M_sun, c200 5-20, "
                     "b 1.0-1.4, q 0.6-0.95, any angles, shear 0-0.1" % (3.0 * widths))
    return wl


def cfg5_fixed(seed=5):
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

    return Workload("cfg5_fixed: 300x300 @0.03\", annulus 0.3-3.5\", 4x4 split, 31x31 Airy PSF, 48x48 source, "
                    "two planes (SIE+shear z=0.5, NFW subhalo ks/rs z=0.8)",
                    xv, yv, data, mask, psf, 0.01, 4, (48, 48), lenses, 10.0, draw, zfac=CFG5_ZFAC, beta=CFG5_BETA)


CONFIGS = {"cfg1": cfg1, "cfg2": cfg2, "cfg3": cfg3, "cfg4": cfg4, "cfg5": cfg5, "cfg5_fixed": cfg5_fixed}
