"""ctypes mirror of include/qlpix.h (structs, constants, library loading)."""
import ctypes as C
import os

QLP_OK = 0
QLP_ERR_ARG = 1
QLP_ERR_CUDA = 2
QLP_ERR_NOT_SPD = 3
QLP_ERR_NO_SOURCE_PIXELS = 4
QLP_ERR_GRID_TOO_SMALL = 5
QLP_ERR_NO_DATA = 6
QLP_ERR_NOMEM = 7
QLP_ERR_TIMEOUT = 8
QLP_ERR_NO_DEVICE = 9

QLP_LENS_SPLE = 0
QLP_LENS_SHEAR = 1
QLP_LENS_NFW = 2
QLP_LENS_NFW_M200_C = 3
QLP_LENS_NFW_M200_RS = 4
QLP_MAX_LENSES = 8
QLP_MAX_PLANES = 4
QLP_MAX_PARAMS = 8

QLP_FP64 = 0
QLP_MIXED = 1

QLP_NFW_QUADRATURE = 0
QLP_NFW_SURROGATE = 1

LENS_TYPES = {"sple": QLP_LENS_SPLE, "shear": QLP_LENS_SHEAR, "nfw": QLP_LENS_NFW,
              "nfw_m200_c": QLP_LENS_NFW_M200_C, "nfw_m200_rs": QLP_LENS_NFW_M200_RS}
N_PARAMS = {QLP_LENS_SPLE: 7, QLP_LENS_SHEAR: 4, QLP_LENS_NFW: 6, QLP_LENS_NFW_M200_C: 6, QLP_LENS_NFW_M200_RS: 6}
NFW_TYPES = ("nfw", "nfw_m200_c", "nfw_m200_rs")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_ubyte)


class qlp_lens(C.Structure):
    _fields_ = [("type", C.c_int), ("plane", C.c_int), ("p", C.c_double * QLP_MAX_PARAMS),
                ("sigma_cr", C.c_double), ("kpc_to_arcsec", C.c_double), ("critical_density", C.c_double)]


class qlp_planes(C.Structure):
    _fields_ = [("n_planes", C.c_int), ("zfac", C.c_double * QLP_MAX_PLANES),
                ("beta", (C.c_double * QLP_MAX_PLANES) * QLP_MAX_PLANES)]


class qlp_image(C.Structure):
    _fields_ = [("npixels_x", C.c_int), ("npixels_y", C.c_int), ("xvals", _dp), ("yvals", _dp),
                ("surface_brightness", _dp), ("covinv_map", _dp),
                ("background_pixel_noise", C.c_double), ("in_mask", _up)]


class qlp_psf(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("matrix", _dp)]


class qlp_srcgrid_opts(C.Structure):
    _fields_ = [("nsplit", C.c_int), ("npixels_x", C.c_int), ("npixels_y", C.c_int),
                ("auto_sourcegrid", C.c_int),
                ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
                ("limit_xmin", C.c_double), ("limit_xmax", C.c_double), ("limit_ymin", C.c_double),
                ("limit_ymax", C.c_double), ("noise_threshold", C.c_double), ("size_scale", C.c_double),
                ("regularization", C.c_int), ("regparam", C.c_double)]


class qlp_result(C.Structure):
    _fields_ = [("m2logev", C.c_double), ("chisq0", C.c_double), ("logdet_F", C.c_double),
                ("logdet_R", C.c_double), ("Es_times_two", C.c_double), ("regterms", C.c_double),
                ("n_active_pixels", C.c_int), ("n_active_src", C.c_int), ("L_nnz", C.c_longlong),
                ("status", C.c_int), ("refine_iters", C.c_int), ("nfw_fallbacks", C.c_int),
                ("regparam", C.c_double), ("regopt_evals", C.c_int), ("outside_sb_penalty", C.c_double),
                ("nfw_exact_rays", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class qlp_schedule(C.Structure):
    _fields_ = [("slots", C.c_int), ("ray_threads", C.c_int), ("psfx_threads", C.c_int), ("psfx_split", C.c_int),
                ("psfx_mode", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


QLP_TUNE_MAX_TRIALS = 32


class qlp_tune_report(C.Structure):
    _fields_ = [("best", qlp_schedule), ("best_ms", C.c_double), ("start_ms", C.c_double), ("n_trials", C.c_int),
                ("trial", qlp_schedule * QLP_TUNE_MAX_TRIALS), ("trial_ms", C.c_double * QLP_TUNE_MAX_TRIALS)]

    def as_dict(self):
        n = self.n_trials
        return {"best": self.best.as_dict(), "best_ms": self.best_ms, "start_ms": self.start_ms, "n_trials": n,
                "trials": [dict(self.trial[i].as_dict(), ms=self.trial_ms[i]) for i in range(n)]}


class qlp_fits_info(C.Structure):
    _fields_ = [("bitpix", C.c_int), ("naxis", C.c_int), ("has_pxsize", C.c_int), ("has_pxnoise", C.c_int),
                ("has_psfsig", C.c_int), ("has_zsrc", C.c_int), ("has_zlens", C.c_int), ("pxsize", C.c_double),
                ("pxnoise", C.c_double), ("psfsig", C.c_double), ("zsrc", C.c_double), ("zlens", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class qlp_surrogate_opts(C.Structure):
    _fields_ = [("n_train", C.c_int), ("batch", C.c_int), ("steps", C.c_int), ("lr", C.c_double),
                ("seed", C.c_ulonglong)]


class qlp_surrogate_report(C.Structure):
    _fields_ = [("final_loss", C.c_double), ("val_max_rel", C.c_double), ("val_mean_rel", C.c_double),
                ("cells_below_1e5", C.c_double), ("train_ms", C.c_double), ("n_params", C.c_int),
                ("n_train", C.c_int), ("steps", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


QLP_TRANSFORM_NONE = 0
QLP_TRANSFORM_LOG = 1
QLP_TRANSFORM_LINEAR = 2
QLP_TRANSFORM_RATIO = 3
QLP_PRIOR_UNIFORM = 0
QLP_PRIOR_LOG = 1
QLP_PRIOR_GAUSS = 2
QLP_FIT_REGPARAM = -1


class qlp_fit_param(C.Structure):
    _fields_ = [("target", C.c_int), ("transform", C.c_int), ("a", C.c_double), ("b", C.c_double),
                ("ratio_param", C.c_int), ("include_jacobian", C.c_int), ("prior", C.c_int),
                ("prior_pos", C.c_double), ("prior_sig", C.c_double), ("prior_norm", C.c_double),
                ("use_penalty_limits", C.c_int), ("penalty_lo", C.c_double), ("penalty_hi", C.c_double)]


def make_fit_params(spec):
    """spec: list of dicts with the qlp_fit_param fields (missing fields: 0,
    prior_norm 1)."""
    arr = (qlp_fit_param * len(spec))()
    for k, d in enumerate(spec):
        arr[k].prior_norm = 1.0
        for key, v in d.items():
            setattr(arr[k], key, v)
    return arr


class qlp_instance(C.Structure):
    _fields_ = [("mask_id", C.c_int), ("src_npixels_x", C.c_int), ("src_npixels_y", C.c_int)]


def srcgrid_defaults():
    """QLens constructor defaults (lens.cpp:185-560) for the Cartesian path."""
    o = qlp_srcgrid_opts()
    o.nsplit = 2
    o.npixels_x = o.npixels_y = 20
    o.auto_sourcegrid = 1
    o.xmin, o.xmax, o.ymin, o.ymax = -1.0, 1.0, -1.0, 1.0
    o.limit_xmin, o.limit_xmax, o.limit_ymin, o.limit_ymax = -1e30, 1e30, -1e30, 1e30
    o.noise_threshold = 0.0
    o.size_scale = 0.0
    o.regularization = 1
    o.regparam = 100.0
    return o


def make_lenses(spec):
    """spec: list of dict(type='sple'|'shear'|'nfw'|'nfw_m200_c'|'nfw_m200_rs', params=[...],
    plane=0, cosmo=(sigma_cr, kpc_to_arcsec, critical_density) for the mass parameterisations)."""
    arr = (qlp_lens * len(spec))()
    for k, l in enumerate(spec):
        t = LENS_TYPES[l["type"]] if isinstance(l["type"], str) else int(l["type"])
        arr[k].type = t
        arr[k].plane = int(l.get("plane", 0))
        for i, v in enumerate(l["params"]):
            arr[k].p[i] = float(v)
        cosmo = l.get("cosmo")
        if cosmo is not None:
            arr[k].sigma_cr, arr[k].kpc_to_arcsec, arr[k].critical_density = (float(v) for v in cosmo)
    return arr


def make_planes(zfac=None, beta=None):
    pl = qlp_planes()
    if zfac is None:
        pl.n_planes = 1
        pl.zfac[0] = 1.0
        return pl
    pl.n_planes = len(zfac)
    for i, z in enumerate(zfac):
        pl.zfac[i] = z
    if beta is not None:
        for i, row in enumerate(beta):
            for j, v in enumerate(row):
                pl.beta[i][j] = v
    return pl


def n_params(spec):
    return sum(N_PARAMS[LENS_TYPES[l["type"]] if isinstance(l["type"], str) else l["type"]] for l in spec)


def flat_params(spec):
    out = []
    for l in spec:
        out.extend(float(v) for v in l["params"])
    return out


class ImageBuffers:
    """Keeps the numpy arrays referenced by a qlp_image alive."""

    def __init__(self, xvals, yvals, data, mask, covinv=None, bg_noise=0.0):
        import numpy as np
        self.xvals = np.ascontiguousarray(xvals, dtype=np.float64)
        self.yvals = np.ascontiguousarray(yvals, dtype=np.float64)
        self.data = np.ascontiguousarray(data, dtype=np.float64).ravel()
        self.mask = np.ascontiguousarray(mask, dtype=np.uint8).ravel()
        self.covinv = None if covinv is None else np.ascontiguousarray(covinv, dtype=np.float64).ravel()
        im = qlp_image()
        im.npixels_x = len(self.xvals) - 1
        im.npixels_y = len(self.yvals) - 1
        assert self.data.size == im.npixels_x * im.npixels_y
        im.xvals = self.xvals.ctypes.data_as(_dp)
        im.yvals = self.yvals.ctypes.data_as(_dp)
        im.surface_brightness = self.data.ctypes.data_as(_dp)
        im.covinv_map = self.covinv.ctypes.data_as(_dp) if self.covinv is not None else None
        im.background_pixel_noise = float(bg_noise)
        im.in_mask = self.mask.ctypes.data_as(_up)
        self.image = im


class PSFBuffer:
    def __init__(self, psf):
        import numpy as np
        self.arr = np.ascontiguousarray(psf, dtype=np.float64)
        p = qlp_psf()
        p.nx, p.ny = self.arr.shape
        p.matrix = self.arr.ctypes.data_as(_dp)
        self.psf = p


def package_dir():
    return os.path.dirname(os.path.abspath(__file__))
