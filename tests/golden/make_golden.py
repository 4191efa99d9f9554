"""Generate the committed golden fixtures from the compiled QLens reference.

Run in a container that has the reference sources (read-only) and g++:

    make -f oracle/Makefile.ref -j8          # REF=<reference sources> to override
    python tests/golden/make_golden.py

For every case below this writes a QLens script, runs oracle/_ref/qlens_harness
on it (the reference's own mock-data generator, lens models and pixel
likelihood, see oracle/ref_harness.cpp) and packs what the harness dumped into
tests/golden/<case>.npz.  The .npz holds:

* inputs the product needs: pixel corner coordinates, data, inverse-variance
  map, mask, PSF matrix and the lens/source-grid configuration;
* reference intermediates: sub-pixel source points, pre-PSF L in CSR form,
  active source cells, R, D, diag(F) (full packed F for small grids), s, the
  model image, and a few rows plus row/column sums of the PSF-convolved L;
* reference scalars: chi^2_0, log det F, log det R, regularisation terms and
  -2 log(evidence) as returned by QLens::invert_image_surface_brightness_map.

The lens configuration is stored in the library's own parameter convention
(SPLE: b, alpha, s, q, theta_deg, xc, yc; SHEAR: shear, theta_deg, xc, yc;
NFW: ks, rs, q, theta_deg, xc, yc), which is the same convention the QLens
'lens' command uses, with each lens's redshift plane; the plane factors the
reference ray-traced with are stored as zfactors / betafactors.
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(REPO, "oracle", "_ref", "qlens_harness")

# Each case: QLens script lines (everything up to, but not including, the
# inversion) and the lens model in library convention.
CASES = {
    # 80x80 SIE + shear, the configuration of the reference's headline
    # single-likelihood run (r < 2.5" mask, 2x2 split, 30x30 source, lambda=10).
    "cfg1": dict(
        script="""random_seed 10
grid -2 2 -2 2
img_npixels 80 80
emode 1
lens sple 1.2 1 0 0.8 30 0 0 shear=0.05 10
source sersic 1 0.15 1.5 0.8 20 0.05 0
psf_width 0.04247
bg_pixel_noise 0.02
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0 2.5
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 30 30
fit regularization curvature
regparam 10
imgpixel_nsplit 2
split_imgpixels on
inversion_method dense
""",
        lenses=[dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0]),
                dict(type="shear", params=[0.05, 10.0, 0.0, 0.0])],
        dense_rows=48,
        full_F=False,
    ),
    # small SIE + shear off the origin, 3x3 split, annular mask, 8x8 source
    "tiny_sie": dict(
        script="""random_seed 3
grid -1.2 1.2 -1.2 1.2
img_npixels 24 24
emode 1
lens sple 0.7 1 0 0.7 40 0.05 -0.03 shear=0.03 -20
source sersic 2 0.12 1.2 0.85 10 0.02 0.03
psf_width 0.06
bg_pixel_noise 0.03
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0.2 1.2
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 8 8
fit regularization curvature
regparam 5
imgpixel_nsplit 3
split_imgpixels on
inversion_method dense
""",
        lenses=[dict(type="sple", params=[0.7, 1.0, 0.0, 0.7, 40.0, 0.05, -0.03]),
                dict(type="shear", params=[0.03, -20.0, 0.05, -0.03])],
        dense_rows=-1,
        full_F=True,
    ),
    # power-law slope alpha != 1 (Tessore et al. series), 4x4 split, annulus
    "powerlaw": dict(
        script="""random_seed 7
grid -2 2 -2 2
img_npixels 40 40
emode 1
lens sple 1.1 1.15 0 0.75 -35 0.02 0.01 shear=0.06 25
source sersic 1.5 0.2 1 0.7 -15 0.04 -0.02
psf_width 0.05
bg_pixel_noise 0.01
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0.5 1.9
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 14 14
fit regularization curvature
regparam 20
imgpixel_nsplit 4
split_imgpixels on
inversion_method dense
""",
        lenses=[dict(type="sple", params=[1.1, 1.15, 0.0, 0.75, -35.0, 0.02, 0.01]),
                dict(type="shear", params=[0.06, 25.0, 0.02, 0.01])],
        dense_rows=-1,
        full_F=True,
    ),
    # fixed source grid smaller than the lensed source: some sub-pixels and
    # some whole image pixels map outside the grid, some source cells stay
    # inactive (unmapped pixels then add data^2 to chi^2)
    "fixed_grid": dict(
        script="""random_seed 5
grid -1.5 1.5 -1.5 1.5
img_npixels 30 30
emode 1
lens sple 0.9 1 0 0.8 10 0 0 shear=0.04 60
source sersic 2 0.1 1.5 0.9 0 0.03 0.02
psf_width 0.05
bg_pixel_noise 0.02
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0 1.5
fit source_mode cartesian
srcgrid -0.12 0.18 -0.15 0.09
auto_src_npixels off
src_npixels 10 9
fit regularization curvature
regparam 3
imgpixel_nsplit 2
split_imgpixels on
inversion_method dense
""",
        lenses=[dict(type="sple", params=[0.9, 1.0, 0.0, 0.8, 10.0, 0.0, 0.0]),
                dict(type="shear", params=[0.04, 60.0, 0.0, 0.0])],
        dense_rows=-1,
        full_F=True,
    ),
    # elliptical NFW perturber (numerical deflection: adaptive Gauss-Patterson
    # quadrature, profile.cpp:2359-2375) beside an SIE host and shear
    "nfw": dict(
        script="""random_seed 11
grid -1.5 1.5 -1.5 1.5
img_npixels 30 30
emode 1
lens sple 0.9 1 0 0.8 15 0 0 shear=0.04 -30
lens nfw 0.35 1.8 0.65 40 0.45 -0.3
source sersic 2 0.12 1.3 0.85 5 0.03 0.02
psf_width 0.05
bg_pixel_noise 0.02
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0.2 1.5
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 12 12
fit regularization curvature
regparam 8
imgpixel_nsplit 3
split_imgpixels on
inversion_method dense
""",
        lenses=[dict(type="sple", params=[0.9, 1.0, 0.0, 0.8, 15.0, 0.0, 0.0]),
                dict(type="shear", params=[0.04, -30.0, 0.0, 0.0]),
                dict(type="nfw", params=[0.35, 1.8, 0.65, 40.0, 0.45, -0.3])],
        dense_rows=-1,
        full_F=True,
    ),
    # two lens planes: SIE + shear at z=0.5, elliptical NFW at z=0.8, source
    # at z=2 (multi-plane recursion, lenscalc.cpp:81-113)
    "twoplane": dict(
        script="""random_seed 13
zsrc 2
zlens 0.5
grid -1.5 1.5 -1.5 1.5
img_npixels 30 30
emode 1
lens sple 0.85 1 0 0.75 -20 0 0 shear=0.05 35
lens nfw 0.5 1.2 0.7 -50 -0.35 0.25 z=0.8
source sersic 2 0.12 1.3 0.85 5 0.03 0.02
psf_width 0.05
bg_pixel_noise 0.02
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0.2 1.5
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 12 12
fit regularization curvature
regparam 8
imgpixel_nsplit 3
split_imgpixels on
inversion_method dense
""",
        lenses=[dict(type="sple", params=[0.85, 1.0, 0.0, 0.75, -20.0, 0.0, 0.0], plane=0),
                dict(type="shear", params=[0.05, 35.0, 0.0, 0.0], plane=0),
                dict(type="nfw", params=[0.5, 1.2, 0.7, -50.0, -0.35, 0.25], plane=1)],
        dense_rows=-1,
        full_F=True,
    ),
}

# 'optimize_regparam on': the entry point chooses lambda by Brent's method over
# log10(lambda) in [-3, 5] (QLens::optimize_regularization_parameter,
# pixelgrid.cpp:15865); the scalars then hold the chosen lambda ('regparam')
# and the intermediates are those of the plain inversion at that lambda.
for _base in ("tiny_sie", "powerlaw"):
    CASES["regopt_" + _base] = dict(CASES[_base], script=CASES[_base]["script"].replace(
        "inversion_method dense\n", "inversion_method dense\noptimize_regparam on\n"))
assert all("optimize_regparam on" in CASES[k]["script"] for k in ("regopt_tiny_sie", "regopt_powerlaw"))
# 'include_noise_term_in_loglike on': -2 log(evidence) gains the pixel noise
# normalisation (lens.cpp:13033-13043).  Uniform noise without a noise map:
# with a noise map the reference reads imgpixel_covinv_vector after
# clear_pixel_matrices has freed it (pixelgrid.cpp:13107-13119) and crashes.
# Without one its dense D loop reads an OpenMP-private covinv that is never
# initialised (pixelgrid.cpp:15637-15653), so D, s and the model come out zero;
# tests/test_noise_term.py pins the noise term from its scalars regardless.
CASES["noise_tiny_sie"] = dict(CASES["tiny_sie"], script=CASES["tiny_sie"]["script"].replace(
    "inversion_method dense\n", "inversion_method dense\ninclude_noise_term_in_loglike on\n").replace(
    "sbmap generate_uniform_noisemap\n", ""))
assert "include_noise_term_in_loglike on" in CASES["noise_tiny_sie"]["script"]

# 'outside_sb_prior on': after the inversion the model is re-made over the
# extended mask (every pixel by default; pixels outside the mask split
# emask_nsplit = 1 ways), PSF-convolved, and a penalty added where it exceeds
# a fraction of the in-mask peak outside the mask (lens.cpp:13063-13158).
# The thresholds are set so that one case pays a penalty and one does not.
# The extended mask: 'sbmap unset_all_pixels' empties it and
# 'set_data_annulus' does not touch it, so 'emask_n_neighbors n' grows it from
# the mask by n rings of pixels.
CASES["osb_tiny_sie"] = dict(CASES["tiny_sie"], script=CASES["tiny_sie"]["script"].replace(
    "fit source_mode cartesian\n", "emask_n_neighbors 3\nfit source_mode cartesian\n").replace(
    "inversion_method dense\n", "inversion_method dense\noutside_sb_prior on\noutside_sb_frac_threshold 0.15\n"))
CASES["osb_powerlaw"] = dict(CASES["powerlaw"], script=CASES["powerlaw"]["script"].replace(
    "fit source_mode cartesian\n", "emask_n_neighbors 2\nfit source_mode cartesian\n").replace(
    "inversion_method dense\n", "inversion_method dense\noutside_sb_prior on\n"))
assert all("emask_n_neighbors" in CASES[k]["script"] for k in ("osb_tiny_sie", "osb_powerlaw"))

# FITS input through the reference's own loaders (ImagePixelData::load_data_fits,
# load_mask_fits, QLens::load_psf_fits), run by the harness built against the
# CFITSIO stand-in (oracle/fitsio_shim).  fits_synth: this repository's
# fixtures (tests/golden/fits, written by make_fits.py: a 32-bit float image in
# HDU 2 with PXSIZE/PXNOISE cards, a smaller 16-bit mask, a 9x9 PSF cropped at
# the threshold).  hst_fits: the FITS files the reference ships with its pixel
# fitting demo (81x81 at 0.049", 37x37 PSF, mask), in Cartesian mode.
FITS_FIXTURES = os.path.join(HERE, "fits")
# where oracle/Makefile.ref reads the reference sources (its REF)
REF_DIR = subprocess.run(["make", "-s", "-f", os.path.join(REPO, "oracle", "Makefile.ref"), "ref-dir"],
                         capture_output=True, text=True).stdout.strip()
CASES["fits_synth"] = dict(
    script="""emode 1
sbmap loadimg image.fits -hdu=2
sbmap generate_uniform_noisemap
psf_threshold 1e-2
sbmap loadpsf psf.fits
sbmap loadmask mask.fits
lens sple 0.7 1 0 0.7 40 0.05 -0.03 shear=0.03 -20
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 8 8
fit regularization curvature
regparam 5
imgpixel_nsplit 3
split_imgpixels on
inversion_method dense
""",
    lenses=[dict(type="sple", params=[0.7, 1.0, 0.0, 0.7, 40.0, 0.05, -0.03]),
            dict(type="shear", params=[0.03, -20.0, 0.05, -0.03])],
    dense_rows=-1, full_F=True, harness="fits",
    files=[os.path.join(FITS_FIXTURES, f) for f in ("image.fits", "mask.fits", "psf.fits")])
CASES["hst_fits"] = dict(
    script="""emode 1
data_pixel_size 0.049
sbmap loadimg sim_hst_image.fits
bg_pixel_noise 0.00941285
sbmap generate_uniform_noisemap
psf_threshold 1e-2
sbmap loadpsf hst_psf.fits
sbmap loadmask mask.fits
lens sple 1.3634 1.17163 0 0.963867 81.9 0.0102892 0.00358392 shear=0.0866 -20.8
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 40 40
fit regularization curvature
regparam 20
imgpixel_nsplit 2
split_imgpixels on
inversion_method dense
""",
    lenses=[dict(type="sple", params=[1.3634, 1.17163, 0.0, 0.963867, 81.9, 0.0102892, 0.00358392]),
            dict(type="shear", params=[0.0866, -20.8, 0.0102892, 0.00358392])],
    dense_rows=64, full_F=True, harness="fits",
    files=[os.path.join(REF_DIR, f) for f in ("sim_hst_image.fits", "mask.fits", "hst_psf.fits")])

# Cases at the sizes of the benchmarked workloads.  Their PSFs are Airy-like
# kernels (the workloads' own), given to the reference as FITS files through
# its loader ('sbmap loadpsf', run by the FITS harness) with a threshold low
# enough to keep the whole kernel.  Their largest arrays are slimmed before
# packing (see SLIM below).
#
# cfg2_draw: one draw from the 200x200 power-law workload's prior box (0.04"
# pixels, annulus 0.5"-2.5", 4x4 split, 21x21 Airy-like PSF, 64x64 source,
# sigma 0.01, lambda 10).
CASES["cfg2_draw"] = dict(
    script="""random_seed 21
grid -4 4 -4 4
img_npixels 200 200
emode 1
psf_threshold 1e-9
sbmap loadpsf psf.fits
lens sple 1.31 1.08 0 0.72 47 0 0 shear=0.06 112
source sersic 1 0.2 1.5 0.75 20 0.04 -0.02
bg_pixel_noise 0.01
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0.5 2.5
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 64 64
fit regularization curvature
regparam 10
imgpixel_nsplit 4
split_imgpixels on
inversion_method dense
""",
    lenses=[dict(type="sple", params=[1.31, 1.08, 0.0, 0.72, 47.0, 0.0, 0.0]),
            dict(type="shear", params=[0.06, 112.0, 0.0, 0.0])],
    dense_rows=16, full_F=False, harness="fits", psf_airy=(21, 0.04, 0.1), slim=True)
# cfg5_m200: the two-plane workload at its sampling (0.03" pixels, 4x4 split,
# 31x31 Airy-like PSF) on a smaller 160x160 image (annulus 0.3"-2.3"), with the
# z = 0.8 subhalo given by its mass and concentration (QLens 'pmode=1':
# NFW::set_ks_rs_from_m200_c200, models.cpp:968-976) -- the library's
# QLP_LENS_NFW_M200_C with the cosmology the reference used for that lens.
CASES["cfg5_m200"] = dict(
    script="""random_seed 23
zsrc 2
zlens 0.5
grid -2.4 2.4 -2.4 2.4
img_npixels 160 160
emode 1
psf_threshold 1e-9
sbmap loadpsf psf.fits
lens sple 1.2 1 0 0.8 30 0 0 shear=0.05 10
lens nfw 5e9 12 0.7 -50 0.85 0.8 z=0.8 pmode=1
source sersic 1 0.2 1.5 0.75 20 0.04 -0.02
bg_pixel_noise 0.01
sbmap plotimg -pnoise -mkdata -nocc
source clear
sbmap generate_uniform_noisemap
sbmap unset_all_pixels
sbmap set_data_annulus 0 0 0.3 2.3
fit source_mode cartesian
auto_srcgrid on
auto_src_npixels off
src_npixels 40 40
fit regularization curvature
regparam 10
imgpixel_nsplit 4
split_imgpixels on
inversion_method dense
""",
    lenses=[dict(type="sple", params=[1.2, 1.0, 0.0, 0.8, 30.0, 0.0, 0.0], plane=0),
            dict(type="shear", params=[0.05, 10.0, 0.0, 0.0], plane=0),
            dict(type="nfw_m200_c", params=[5e9, 12.0, 0.7, -50.0, 0.85, 0.8], plane=1)],
    dense_rows=16, full_F=False, harness="fits", psf_airy=(31, 0.03, 0.08), slim=True)

# Slimmed cases keep every input, the active set, the CSR row pointers, the L
# column indices (as int16: M <= 4096), the source-grid corners and the
# M- and N-sized vectors in full.  The sub-pixel source points and the L values
# (about 3 and 5 MB at cfg2's size) are replaced by their SHA-256 digests (exact
# comparisons) plus every SLIM_STRIDE-th element (tolerance comparisons).
SLIM_STRIDE = 61
SLIM_HASHED = ["srcpt_x", "srcpt_y", "L_value"]

ARRAYS_F64 = ["lens_cosmo", "zfactors", "betafactors", "xvals", "yvals", "data", "covinv", "psf", "srcpt_x", "srcpt_y", "src_corner_x",
              "src_corner_y", "L_value", "R_value", "Lpsf_rows", "Lpsf_colsum", "Lpsf_rowsum", "D",
              "F_diag", "F_packed_upper", "s", "model", "osb_sb"]
ARRAYS_I32 = ["lens_plane", "masked_pixels", "active_index", "active_pixels", "L_rowptr", "L_index", "R_index"]
ARRAYS_U8 = ["mask", "emask", "osb_maps"]


def write_airy_psf(path, n, pixel, fwhm):
    """The workloads' Airy-like PSF (qlens_gb300.synthetic.airy_psf) as a
    64-bit FITS image, for the reference's own PSF loader."""
    sys.path.insert(0, REPO)
    sys.path.insert(0, HERE)
    from make_fits import hdu_bytes
    from qlens_gb300.synthetic import airy_psf
    with open(path, "wb") as f:
        f.write(hdu_bytes(airy_psf(n, pixel, fwhm), -64, True))


def run_case(name, case, outdir):
    tmp = tempfile.mkdtemp(prefix="golden_" + name + "_")
    try:
        script = os.path.join(tmp, name + ".in")
        with open(script, "w") as f:
            f.write(case["script"])
        for src in case.get("files", []):
            shutil.copy(src, os.path.join(tmp, os.path.basename(src)))
        if case.get("psf_airy"):
            write_airy_psf(os.path.join(tmp, "psf.fits"), *case["psf_airy"])
        dump = os.path.join(tmp, "dump")
        os.makedirs(dump)
        env = dict(os.environ, OMP_NUM_THREADS="4")
        harness = HARNESS + "_fits" if case.get("harness") == "fits" else HARNESS
        r = subprocess.run([harness, script, dump, str(case["dense_rows"])], cwd=tmp, env=env,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("harness failed on %s:\n%s\n%s" % (name, r.stdout[-2000:], r.stderr[-2000:]))
        out = {}
        for key, dt, ext in ([(k, np.float64, "f64") for k in ARRAYS_F64] +
                             [(k, np.int32, "i32") for k in ARRAYS_I32] +
                             [(k, np.uint8, "u8") for k in ARRAYS_U8]):
            p = os.path.join(dump, key + "." + ext)
            if os.path.exists(p):
                out[key] = np.fromfile(p, dtype=dt)
        scalars = {}
        with open(os.path.join(dump, "scalars.txt")) as f:
            for line in f:
                k, v = line.split()
                scalars[k] = float(v)
        lenses = [dict(l) for l in case["lenses"]]
        if "lens_cosmo" in out:
            lc = out["lens_cosmo"].reshape(len(lenses), 5)
            for k, l in enumerate(lenses):
                if l["type"] in ("nfw_m200_c", "nfw_m200_rs"):
                    l["cosmo"] = [float(v) for v in lc[k, :3]]
        meta = dict(name=name, lenses=lenses, script=case["script"], scalars=scalars)
        if case.get("slim"):
            import hashlib
            slim = {"stride": SLIM_STRIDE, "sha256": {}}
            for k in SLIM_HASHED:
                a = np.ascontiguousarray(out.pop(k))
                slim["sha256"][k] = hashlib.sha256(a.tobytes()).hexdigest()
                out[k + "_sub"] = a[::SLIM_STRIDE].copy()
            out.pop("F_packed_upper", None)
            assert int(out["L_index"].max()) < 32768
            out["L_index"] = out["L_index"].astype(np.int16)
            meta["slim"] = slim
        out["meta_json"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **out)
        print("%-10s -2logev=%.10f chi2=%.6f logdetF=%.6f logdetR=%.6f npix=%d nsrc=%d" % (
            name, scalars["m2logev"], scalars["chisq0"], scalars["logdetF"], scalars["logdetR"],
            scalars["n_active_pixels"], scalars["n_active_src"]))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main(argv):
    if not os.path.exists(HARNESS):
        sys.exit("build the harness first: make -f oracle/Makefile.ref -j8")
    names = argv[1:] or list(CASES)
    for n in names:
        run_case(n, CASES[n], HERE)


if __name__ == "__main__":
    main(sys.argv)
