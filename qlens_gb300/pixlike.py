"""Host-side mirror of QLens's pixel-likelihood interface over libqlpix.so.

``PixelLikelihood`` plays the role of the QLens object for the Cartesian
pixel inversion: it holds the image data (ImagePixelData), the source-grid
settings, the PSF and the lens list, and ``invert_image_surface_brightness_map``
returns -2 log(evidence) and chi^2_0 like
QLens::invert_image_surface_brightness_map (lens.cpp:12293).  Every evaluation
runs on the GPU through the C ABI in include/qlpix.h; there is no CPU path, and
a missing or unloadable library raises instead of falling back.
"""
import ctypes as C
import math
import os

import numpy as np

from . import abi

_lib = None
BRENT_FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


class LibraryUnavailable(RuntimeError):
    pass


def library_path():
    return os.path.join(abi.package_dir(), "_lib", "libqlpix.so")


def load_library(build_if_missing=False):
    """Load libqlpix.so (built by qlens_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path) and build_if_missing:
        from . import build
        build.build()
    if not os.path.exists(path):
        raise LibraryUnavailable("libqlpix.so not built: run python -c 'import __graft_entry__ as g; g.build()'")
    L = C.CDLL(path)
    P = C.POINTER
    L.qlp_srcgrid_defaults.argtypes = [P(abi.qlp_srcgrid_opts)]
    L.qlp_create.restype = C.c_void_p
    L.qlp_create.argtypes = [P(abi.qlp_image), P(abi.qlp_psf), P(abi.qlp_srcgrid_opts), C.c_int, P(C.c_int)]
    L.qlp_set_lens_model.argtypes = [C.c_void_p, P(abi.qlp_lens), C.c_int, P(abi.qlp_planes)]
    L.qlp_set_precision.argtypes = [C.c_void_p, C.c_int]
    L.qlp_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.qlp_eval.argtypes = [C.c_void_p, P(C.c_double), C.c_double, P(abi.qlp_result)]
    L.qlp_n_params.argtypes = [C.c_void_p]
    L.qlp_set_batch_slots.argtypes = [C.c_void_p, C.c_int]
    L.qlp_set_instance_masks.argtypes = [C.c_void_p, P(C.c_ubyte), C.c_int]
    L.qlp_eval_batch.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), P(abi.qlp_instance), C.c_int,
                                 P(abi.qlp_result)]
    L.qlp_dump.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int), P(C.c_int), P(C.c_double), P(C.c_int),
                           P(C.c_double), P(C.c_double), P(C.c_double)]
    L.qlp_dump_Lpsf.argtypes = [C.c_void_p, C.c_int, P(C.c_double)]
    L.qlp_stage_times.argtypes = [C.c_void_p, P(C.c_float), C.c_int]
    L.qlp_last_device_time.argtypes = [C.c_void_p, P(C.c_float)]
    L.qlp_last_launch_count.restype = C.c_longlong
    L.qlp_last_launch_count.argtypes = [C.c_void_p]
    L.qlp_set_graphs.argtypes = [C.c_void_p, C.c_int]
    L.qlp_set_refinement.argtypes = [C.c_void_p, C.c_int]
    L.qlp_set_noise_term.argtypes = [C.c_void_p, C.c_int]
    L.qlp_set_outside_sb_prior.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_int]
    L.qlp_set_regparam_optimization.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]
    L.qlp_brent_min.argtypes = [BRENT_FN, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, P(C.c_double),
                                P(C.c_int)]
    L.qlp_get_schedule.argtypes = [C.c_void_p, P(abi.qlp_schedule)]
    L.qlp_set_schedule.argtypes = [C.c_void_p, P(abi.qlp_schedule)]
    L.qlp_autotune.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), P(abi.qlp_instance), C.c_int, C.c_int,
                               P(abi.qlp_tune_report)]
    L.qlp_last_transfer_bytes.argtypes = [C.c_void_p, P(C.c_longlong), P(C.c_longlong)]
    L.qlp_spd_solve_logdet_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p]
    L.qlp_surrogate_defaults.argtypes = [P(abi.qlp_surrogate_opts)]
    L.qlp_nfw_surrogate_train.argtypes = [C.c_int, P(abi.qlp_surrogate_opts), P(abi.qlp_surrogate_report)]
    L.qlp_set_nfw_mode.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.qlp_set_nfw_tolerance.argtypes = [C.c_void_p, C.c_double]
    L.qlp_surrogate_grad_check.argtypes = [C.c_int, P(C.c_float), P(C.c_float), P(C.c_float), C.c_int,
                                           P(C.c_double), P(C.c_float)]
    L.qlp_surrogate_eval.argtypes = [C.c_int, P(C.c_double), C.c_int, P(C.c_double), P(C.c_double),
                                     P(C.c_double), P(C.c_double)]
    L.qlp_fits_read_image.argtypes = [C.c_char_p, C.c_int, P(C.c_double), C.c_long, P(C.c_int), P(C.c_int),
                                      P(abi.qlp_fits_info)]
    L.qlp_load_data_fits.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                     P(C.c_double), P(C.c_double), P(C.c_double), C.c_long, P(C.c_int), P(C.c_int),
                                     P(abi.qlp_fits_info)]
    L.qlp_load_mask_fits.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, P(C.c_ubyte), P(C.c_int)]
    L.qlp_load_noise_map_fits.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, P(C.c_double), P(C.c_double)]
    L.qlp_load_psf_fits.argtypes = [C.c_char_p, C.c_double, P(C.c_double), C.c_long, P(C.c_int), P(C.c_int)]
    L.qlp_set_fit_params.argtypes = [C.c_void_p, P(abi.qlp_fit_param), C.c_int]
    L.qlp_fit_loglike_batch.argtypes = [C.c_void_p, P(C.c_double), C.c_int, P(C.c_double), P(abi.qlp_result)]
    L.qlp_fit_terms.argtypes = [P(abi.qlp_fit_param), C.c_int, P(C.c_double), P(C.c_double), P(C.c_int),
                                P(C.c_double)]
    L.qlp_last_error.restype = C.c_char_p
    L.qlp_destroy.argtypes = [C.c_void_p]
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class QLPixError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("qlpix status %d: %s" % (code, msg))
        self.code = code


def gaussian_psf(sigma_x, sigma_y, pixel_x, pixel_y, psf_threshold=0.01):
    """QLens::generate_PSF_matrix (pixelgrid.cpp:14601-14668), no supersampling."""
    sigma_fraction = math.sqrt(-2 * math.log(psf_threshold))
    nxh_dec = sigma_fraction * sigma_x / pixel_x
    nyh_dec = sigma_fraction * sigma_y / pixel_y
    nxh, nyh = int(nxh_dec), int(nyh_dec)
    if nxh_dec - nxh > 0.5:
        nxh += 1
    if nyh_dec - nyh > 0.5:
        nyh += 1
    nx, ny = 2 * nxh + 1, 2 * nyh + 1
    xmax_sup = ((2 * nxh + 1) * pixel_x - pixel_x) / 2
    ymax_sup = ((2 * nyh + 1) * pixel_y - pixel_y) / 2
    psf = np.empty((nx, ny))
    norm = 0.0
    x = -xmax_sup
    for i in range(nx):
        y = -ymax_sup
        for j in range(ny):
            psf[i, j] = math.exp(-0.5 * ((x / sigma_x) ** 2 + (y / sigma_y) ** 2))
            norm += psf[i, j]
            y += pixel_y
        x += pixel_x
    return psf / norm


def pixel_corners(nx, xmin, xmax):
    """ImagePixelGrid corner coordinates: xmin + i*pixel_xlength (pixelgrid.cpp:9581-9590)."""
    step = (xmax - xmin) / nx
    return np.array([xmin + i * step for i in range(nx + 1)])


class PixelLikelihood:
    """One GPU context: image data, mask, PSF, source-grid settings and lens list."""

    def __init__(self, xvals, yvals, data, mask, psf, covinv=None, bg_noise=0.0, nsplit=2,
                 src_npixels=(20, 20), auto_sourcegrid=True, sourcegrid=(-1, 1, -1, 1),
                 regularization=True, regparam=100.0, device=0, precision=abi.QLP_FP64):
        self.lib = load_library()
        self._img = abi.ImageBuffers(xvals, yvals, data, mask, covinv, bg_noise)
        self._psf = abi.PSFBuffer(psf)
        o = abi.srcgrid_defaults()
        o.nsplit = int(nsplit)
        o.npixels_x, o.npixels_y = int(src_npixels[0]), int(src_npixels[1])
        o.auto_sourcegrid = 1 if auto_sourcegrid else 0
        o.xmin, o.xmax, o.ymin, o.ymax = map(float, sourcegrid)
        o.regularization = 1 if regularization else 0
        o.regparam = float(regparam)
        self.opts = o
        self._create(device)
        self.set_precision(precision)
        self.lens_spec = None

    @classmethod
    def from_opts(cls, image_bufs, psf_buf, opts, device=0, precision=abi.QLP_FP64):
        self = cls.__new__(cls)
        self.lib = load_library()
        self._img, self._psf, self.opts = image_bufs, psf_buf, opts
        self._create(device)
        self.set_precision(precision)
        self.lens_spec = None
        return self

    def _create(self, device):
        st = C.c_int(0)
        self.ctx = self.lib.qlp_create(C.byref(self._img.image), C.byref(self._psf.psf), C.byref(self.opts),
                                       int(device), C.byref(st))
        if not self.ctx:
            raise QLPixError(st.value, self.lib.qlp_last_error().decode())

    def _check(self, code):
        if code not in (abi.QLP_OK,):
            raise QLPixError(code, self.lib.qlp_last_error().decode())

    def set_precision(self, mode):
        self._check(self.lib.qlp_set_precision(self.ctx, int(mode)))

    def set_stream(self, stream_ptr):
        self._check(self.lib.qlp_set_stream(self.ctx, C.c_void_p(stream_ptr) if stream_ptr else None))

    def set_batch_slots(self, n):
        self._check(self.lib.qlp_set_batch_slots(self.ctx, int(n)))

    def set_graphs(self, on):
        """Replay captured CUDA graphs in eval_batch (default) or launch kernel by kernel."""
        self._check(self.lib.qlp_set_graphs(self.ctx, 1 if on else 0))

    def set_nfw_mode(self, mode, threshold_arcsec=0.0):
        """abi.QLP_NFW_QUADRATURE or abi.QLP_NFW_SURROGATE (after train_nfw_surrogate);
        threshold_arcsec <= 0 keeps the default gate (2e-5 arcsec)."""
        self._check(self.lib.qlp_set_nfw_mode(self.ctx, int(mode), float(threshold_arcsec)))

    def set_nfw_tolerance(self, tol):
        """QLens's 'integral_tolerance' for the NFW quadrature (default 1e-3)."""
        self._check(self.lib.qlp_set_nfw_tolerance(self.ctx, float(tol)))

    def schedule(self):
        s = abi.qlp_schedule()
        self._check(self.lib.qlp_get_schedule(self.ctx, C.byref(s)))
        return s.as_dict()

    def set_schedule(self, **kw):
        s = abi.qlp_schedule()
        self._check(self.lib.qlp_get_schedule(self.ctx, C.byref(s)))
        for k, v in kw.items():
            setattr(s, k, int(v))
        self._check(self.lib.qlp_set_schedule(self.ctx, C.byref(s)))

    def autotune(self, params, regparams=None, mask_ids=None, src_sizes=None, reps=2):
        """Time the sample batch under candidate launch schedules and keep the
        fastest (qlp_autotune); returns the report as a dict."""
        params = np.ascontiguousarray(params, dtype=np.float64)
        n = params.shape[0]
        rp = None
        if regparams is not None:
            rpa = np.ascontiguousarray(regparams, dtype=np.float64)
            rp = _dp(rpa)
        inst = self._instances(n, mask_ids, src_sizes)
        rep = abi.qlp_tune_report()
        self._check(self.lib.qlp_autotune(self.ctx, _dp(params), rp, inst, n, int(reps), C.byref(rep)))
        return rep.as_dict()

    def _instances(self, n, mask_ids, src_sizes):
        if mask_ids is None and src_sizes is None:
            return None
        inst = (abi.qlp_instance * n)()
        for i in range(n):
            inst[i].mask_id = -1 if mask_ids is None else int(mask_ids[i])
            if src_sizes is None:
                inst[i].src_npixels_x = inst[i].src_npixels_y = 0
            else:
                inst[i].src_npixels_x, inst[i].src_npixels_y = map(int, src_sizes[i])
        return inst

    def set_regparam_optimization(self, on=True, minlog=-3.0, maxlog=5.0, tol=0.01, max_iter=20):
        """QLens's 'optimize_regparam on': choose lambda per evaluation by
        Brent's method over log10(lambda) (defaults: QLens's)."""
        self._check(self.lib.qlp_set_regparam_optimization(self.ctx, 1 if on else 0, float(minlog), float(maxlog),
                                                           float(tol), int(max_iter)))

    def set_refinement(self, sweeps):
        """FP64 refinement sweeps of the mixed path (0..4, default 1)."""
        self._check(self.lib.qlp_set_refinement(self.ctx, int(sweeps)))

    def set_noise_term(self, on):
        """QLens's 'include_noise_term_in_loglike': add the pixel-noise
        normalisation to -2 log(evidence)."""
        self._check(self.lib.qlp_set_noise_term(self.ctx, 1 if on else 0))

    def set_outside_sb_prior(self, on, frac_threshold=0.3, noise_frac=-1e30, emask=None, emask_nsplit=1):
        """QLens's 'outside_sb_prior': penalise model surface brightness
        outside the mask (over the extended mask `emask`, uint8 [nx, ny] or
        None for every pixel)."""
        em = None if emask is None else np.ascontiguousarray(emask, dtype=np.uint8).ravel()
        self._keep_emask = em
        self._check(self.lib.qlp_set_outside_sb_prior(self.ctx, 1 if on else 0, float(frac_threshold),
                                                      float(noise_frac), None if em is None else em.ctypes.data,
                                                      int(emask_nsplit)))

    def last_transfer_bytes(self):
        """(host->device, device->host) bytes moved by the last call."""
        h, d = C.c_longlong(), C.c_longlong()
        self._check(self.lib.qlp_last_transfer_bytes(self.ctx, C.byref(h), C.byref(d)))
        return h.value, d.value

    def set_lens_model(self, spec, zfac=None, beta=None):
        self.lens_spec = spec
        lenses = abi.make_lenses(spec)
        planes = abi.make_planes(zfac, beta)
        self._planes = planes
        self._check(self.lib.qlp_set_lens_model(self.ctx, lenses, len(spec), C.byref(planes)))

    @property
    def n_params(self):
        return self.lib.qlp_n_params(self.ctx)

    def invert_image_surface_brightness_map(self, params=None, regparam=0.0):
        """Returns the qlp_result as a dict (m2logev = -2 log evidence, chisq0, ...)."""
        res = abi.qlp_result()
        pp = None
        if params is not None:
            arr = np.ascontiguousarray(params, dtype=np.float64)
            pp = _dp(arr)
        self.lib.qlp_eval(self.ctx, pp, float(regparam), C.byref(res))
        return res.as_dict()

    def set_instance_masks(self, masks):
        m = np.ascontiguousarray(masks, dtype=np.uint8)
        self._masks = m
        self._check(self.lib.qlp_set_instance_masks(self.ctx, m.ctypes.data_as(C.POINTER(C.c_ubyte)), m.shape[0]))

    def eval_batch(self, params, regparams=None, mask_ids=None, src_sizes=None):
        params = np.ascontiguousarray(params, dtype=np.float64)
        n = params.shape[0]
        out = (abi.qlp_result * n)()
        rp = None
        if regparams is not None:
            self._rp = np.ascontiguousarray(regparams, dtype=np.float64)
            rp = _dp(self._rp)
        inst = self._instances(n, mask_ids, src_sizes)
        code = self.lib.qlp_eval_batch(self.ctx, _dp(params), rp, inst, n, out)
        if code not in (abi.QLP_OK, abi.QLP_ERR_NOT_SPD, abi.QLP_ERR_NO_SOURCE_PIXELS, abi.QLP_ERR_GRID_TOO_SMALL):
            self._check(code)
        return [out[i].as_dict() for i in range(n)]

    def set_fit_params(self, spec):
        """QLens's fit parameters over the lens parameters (qlp_set_fit_params):
        spec is a list of dicts of qlp_fit_param fields."""
        self._fit = abi.make_fit_params(spec)
        self._nfit = len(spec)
        self._check(self.lib.qlp_set_fit_params(self.ctx, self._fit, len(spec)))

    def fit_loglike_batch(self, fit_params):
        """-log L of each fit vector (QLens::fitmodel_loglike_extended_source)
        and its evaluation's result dict."""
        x = np.ascontiguousarray(fit_params, dtype=np.float64).reshape(-1, self._nfit)
        n = x.shape[0]
        ll = np.zeros(n)
        out = (abi.qlp_result * n)()
        self._check(self.lib.qlp_fit_loglike_batch(self.ctx, _dp(x), n, _dp(ll), out))
        return ll, [out[i].as_dict() for i in range(n)]

    def dump(self, n_sub, res):
        """Intermediates of the last single evaluation (parity hooks)."""
        N, M, nnz = res["n_active_pixels"], res["n_active_src"], res["L_nnz"]
        sp = np.empty(2 * n_sub)
        rp = np.empty(N + 1, dtype=np.int32)
        li = np.empty(max(nnz, 1), dtype=np.int32)
        lv = np.empty(max(nnz, 1))
        ai = np.empty(self.opts.npixels_x * self.opts.npixels_y, dtype=np.int32)
        D = np.empty(max(M, 1))
        s = np.empty(max(M, 1))
        model = np.empty(max(N, 1))
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        self._check(self.lib.qlp_dump(self.ctx, _dp(sp), ip(rp), ip(li), _dp(lv), ip(ai), _dp(D), _dp(s), _dp(model)))
        return dict(srcpt=sp, L_rowptr=rp, L_index=li[:nnz], L_value=lv[:nnz], active_index=ai, D=D[:M], s=s[:M],
                    model=model[:N])

    def dump_Lpsf(self, rows, M):
        out = np.empty((rows, M))
        self._check(self.lib.qlp_dump_Lpsf(self.ctx, rows, _dp(out)))
        return out

    def stage_times(self):
        ms = (C.c_float * 6)()
        self._check(self.lib.qlp_stage_times(self.ctx, ms, 6))
        return list(ms)

    def last_device_ms(self):
        ms = C.c_float(0)
        self._check(self.lib.qlp_last_device_time(self.ctx, C.byref(ms)))
        return ms.value

    def last_launch_count(self):
        return self.lib.qlp_last_launch_count(self.ctx)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.qlp_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- learned NFW deflection -------------------------------------------------
SURROGATE_NP = 50306        # 3 -> 4 x 128 tanh -> 2


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def train_nfw_surrogate(device=0, **kw):
    """Train the NFW deflection surrogate on `device` (qlp_nfw_surrogate_train);
    keyword arguments override qlp_surrogate_opts fields.  Returns the report."""
    L = load_library()
    o = abi.qlp_surrogate_opts()
    L.qlp_surrogate_defaults(C.byref(o))
    for k, v in kw.items():
        if k not in dict(abi.qlp_surrogate_opts._fields_):
            raise TypeError("unknown surrogate option %r" % k)
        setattr(o, k, v)
    rep = abi.qlp_surrogate_report()
    code = L.qlp_nfw_surrogate_train(int(device), C.byref(o), C.byref(rep))
    if code != abi.QLP_OK:
        raise QLPixError(code, L.qlp_last_error().decode())
    return rep.as_dict()


def surrogate_grad_check(params, x, t, device=0):
    """One forward + backward pass of the training kernels (unweighted mean
    squared error): returns (loss, grad) for params [50306], x [n][3], t [n][2]."""
    L = load_library()
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    assert params.shape == (SURROGATE_NP,) and x.shape[1] == 3 and t.shape == (x.shape[0], 2)
    grad = np.empty(SURROGATE_NP, dtype=np.float32)
    loss = C.c_double(0)
    code = L.qlp_surrogate_grad_check(int(device), _fp(params), _fp(x), _fp(t), x.shape[0], C.byref(loss),
                                      _fp(grad))
    if code != abi.QLP_OK:
        raise QLPixError(code, L.qlp_last_error().decode())
    return loss.value, grad


def surrogate_eval(rho_phi_q, device=0):
    """The trained network through the tensor-core inference path at points
    (log R, phi, q): returns (t [n][2] = log(G/B), quadrature G [n][2],
    baseline B [n], cell bound [n])."""
    L = load_library()
    p = np.ascontiguousarray(rho_phi_q, dtype=np.float64)
    n = p.shape[0]
    t = np.empty((n, 2))
    G = np.empty((n, 2))
    B = np.empty(n)
    bound = np.empty(n)
    code = L.qlp_surrogate_eval(int(device), _dp(p), n, _dp(t), _dp(G), _dp(B), _dp(bound))
    if code != abi.QLP_OK:
        raise QLPixError(code, L.qlp_last_error().decode())
    return t, G, B, bound


def fit_terms(spec, fit_params):
    """Host side of one fit vector (qlp_fit_terms): (transformed values,
    penalised, prior + Jacobian terms).  No device needed."""
    L = load_library()
    fp = abi.make_fit_params(spec)
    x = np.ascontiguousarray(fit_params, dtype=np.float64)
    t = np.zeros(len(spec))
    pen = C.c_int()
    terms = C.c_double()
    code = L.qlp_fit_terms(fp, len(spec), _dp(x), _dp(t), C.byref(pen), C.byref(terms))
    if code != abi.QLP_OK:
        raise QLPixError(code, L.qlp_last_error().decode())
    return t, bool(pen.value), terms.value


def brent_min(f, ax, bx, tol, max_iter):
    """The library's Brent minimiser (qlp_brent_min) on a Python function:
    returns (x_min, evaluations, list of the points evaluated)."""
    L = load_library()
    pts = []

    def cb(x, _):
        pts.append(x)
        return float(f(x))

    fn = BRENT_FN(cb)
    x = C.c_double(0)
    n = C.c_int(0)
    code = L.qlp_brent_min(fn, None, float(ax), float(bx), float(tol), int(max_iter), C.byref(x), C.byref(n))
    if code != abi.QLP_OK:
        raise QLPixError(code, L.qlp_last_error().decode())
    return x.value, n.value, pts


# ---- FITS input: the reference's 'sbmap loadimg / loadmask / loadnoisemap /
# loadpsf' (pixelgrid.cpp:6016-6870), through the library's own reader.
# Arrays are indexed [i, j] with i along FITS axis 1 (x) and j along axis 2.

def _fits_call(L, code):
    if code != abi.QLP_OK:
        raise QLPixError(code, L.qlp_last_error().decode())


def fits_read_image(path, hdu=1):
    """The 2-D image of HDU `hdu` (1 = primary) as an (nx, ny) array, and the
    header keywords QLens reads (PXSIZE, PXNOISE, PSFSIG, ZSRC, ZLENS)."""
    L = load_library()
    nx, ny, info = C.c_int(), C.c_int(), abi.qlp_fits_info()
    _fits_call(L, L.qlp_fits_read_image(os.fsencode(path), int(hdu), None, 0, C.byref(nx), C.byref(ny),
                                        C.byref(info)))
    out = np.empty((nx.value, ny.value))
    _fits_call(L, L.qlp_fits_read_image(os.fsencode(path), int(hdu), _dp(out), out.size, C.byref(nx), C.byref(ny),
                                        None))
    return out, info.as_dict()


def load_data_fits(path, hdu=1, pixel_size=0.0, bounds=None):
    """'sbmap loadimg <file.fits>' (ImagePixelData::load_data_fits): returns
    (xvals, yvals, data[nx, ny], keywords).  Square pixels of the file's
    PXSIZE, else of pixel_size (> 0, QLens 'data_pixel_size'), centred on the
    origin; otherwise bounds = (xmin, xmax, ymin, ymax), QLens's 'grid'."""
    L = load_library()
    b = bounds if bounds is not None else (0.0, 0.0, 0.0, 0.0)
    nx, ny, info = C.c_int(), C.c_int(), abi.qlp_fits_info()
    args = (os.fsencode(path), int(hdu), float(pixel_size), float(b[0]), float(b[1]), float(b[2]), float(b[3]))
    _fits_call(L, L.qlp_load_data_fits(*args, None, None, None, 0, C.byref(nx), C.byref(ny), C.byref(info)))
    xv, yv = np.empty(nx.value + 1), np.empty(ny.value + 1)
    data = np.empty((nx.value, ny.value))
    _fits_call(L, L.qlp_load_data_fits(*args, _dp(xv), _dp(yv), _dp(data), data.size, C.byref(nx), C.byref(ny),
                                       None))
    return xv, yv, data, info.as_dict()


def load_mask_fits(path, mask, add=False):
    """'sbmap loadmask <file.fits> [-add]' applied to `mask` (bool or uint8
    array [nx, ny]); returns the new mask as uint8."""
    L = load_library()
    m = np.ascontiguousarray(mask, dtype=np.uint8).copy()
    n = C.c_int()
    _fits_call(L, L.qlp_load_mask_fits(os.fsencode(path), m.shape[0], m.shape[1], 1 if add else 0,
                                       m.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(n)))
    return m


def load_noise_map_fits(path, shape, hdu=1):
    """'sbmap loadnoisemap <file.fits>': returns (covinv[nx, ny], smallest sigma)."""
    L = load_library()
    cov = np.empty(shape)
    mn = C.c_double()
    _fits_call(L, L.qlp_load_noise_map_fits(os.fsencode(path), int(hdu), shape[0], shape[1], _dp(cov), C.byref(mn)))
    return cov, mn.value


def load_psf_fits(path, psf_threshold=0.01):
    """'sbmap loadpsf <file.fits>' (QLens::load_psf_fits): the thresholded,
    symmetric, unit-sum PSF matrix [pnx, pny]."""
    L = load_library()
    pnx, pny = C.c_int(), C.c_int()
    _fits_call(L, L.qlp_load_psf_fits(os.fsencode(path), float(psf_threshold), None, 0, C.byref(pnx), C.byref(pny)))
    psf = np.empty((pnx.value, pny.value))
    _fits_call(L, L.qlp_load_psf_fits(os.fsencode(path), float(psf_threshold), _dp(psf), psf.size, C.byref(pnx),
                                      C.byref(pny)))
    return psf
