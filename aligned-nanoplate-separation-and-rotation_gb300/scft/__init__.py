"""ctypes binding of libscft (include/scft.h).

The library is the product: CUDA kernels for sm_103a behind a C ABI.  This
module only loads it and converts numpy arrays; it has no compute path of its
own, and every call fails with ScftError if the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "build", "libscft.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NAN, ERR_QNONPOS, ERR_UNSUPPORTED, ERR_NOMEM, ERR_COMPLEX = -1, -2, -3, -4, -5, -6, -7
PREC_FP64, PREC_MIXED = 0, 1
PLATE_REFERENCE, PLATE_CUBOID = 0, 1
UPDATE_1S, UPDATE_EULER = 0, 1
FIELD_NAMES = ("wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm")

# Every extern "C" symbol declared in include/scft.h.
EXPORTS = ("scft_last_error", "scft_version", "scft_create", "scft_destroy", "scft_get_info",
           "scft_set_fields", "scft_get_fields", "scft_calc_poly_density", "scft_update_1s",
           "scft_calc_H", "scft_grad_geom", "scft_get_density", "scft_get_plate_density", "scft_get_smeared", "scft_diblock_density",
           "scft_homopolymer_density", "scft_fft3d", "scft_sync", "scft_get_stream", "scft_launch_count",
           "scft_profile_step", "scft_diblock_density_noalloc", "scft_set_sweep_groups", "scft_autotune",
           "scft_set_fields_all", "scft_set_wait_limit", "scft_fp64_fma_rate",
           "scft_set_persistent", "scft_get_schedule", "scft_profile_sweep",
           "scft_get_fft_plan", "scft_step_fields", "scft_set_plane_form", "scft_get_plane_form",
           "scft_iterate_fields")


class ScftError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"scft error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [
        ("Nda", ctypes.c_int), ("Ndb", ctypes.c_int),
        ("a_smear", ctypes.c_double), ("rho0", ctypes.c_double),
        ("chi_ab", ctypes.c_double), ("chi_bc", ctypes.c_double), ("chi_ac", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("Nx", ctypes.c_int * 3), ("L", ctypes.c_double * 3),
        ("lam_pl", ctypes.c_double), ("lam_mi", ctypes.c_double),
        ("n_exp_nr", ctypes.c_int), ("np_chem", ctypes.c_int),
        ("sigma", ctypes.c_double), ("Ng", ctypes.c_int),
        ("L_nr", ctypes.c_double), ("R_nr", ctypes.c_double), ("xi_nr", ctypes.c_double),
        ("center", (ctypes.c_double * 3) * 2), ("orient", (ctypes.c_double * 3) * 2),
        ("precision", ctypes.c_int), ("plate_shape", ctypes.c_int),
        ("shell_lambda", ctypes.c_double), ("shell_width", ctypes.c_double), ("update_scheme", ctypes.c_int),
        ("do_cl", ctypes.c_int), ("cl_seed", ctypes.c_longlong),
    ]


class Info(ctypes.Structure):
    _fields_ = [
        ("M", ctypes.c_long), ("V", ctypes.c_double), ("Vf", ctypes.c_double), ("nD", ctypes.c_double),
        ("phiD", ctypes.c_double), ("phiG", ctypes.c_double), ("np_frac", ctypes.c_double),
        ("nP", ctypes.c_double), ("ng_per_np", ctypes.c_double), ("N", ctypes.c_int),
        ("dx", ctypes.c_double * 3),
    ]


_lib = None


def library_path() -> str:
    return LIB_PATH


def load(path: str | None = None):
    """Loads libscft.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ScftError(ERR_UNSUPPORTED, f"{p} not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(p)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    lib.scft_last_error.restype = ctypes.c_char_p
    lib.scft_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(vp)]
    lib.scft_destroy.argtypes = [vp]
    lib.scft_destroy.restype = None
    lib.scft_get_info.argtypes = [vp, ctypes.c_int, ctypes.POINTER(Info)]
    lib.scft_set_fields.argtypes = [vp, ctypes.c_int, dp]
    lib.scft_get_fields.argtypes = [vp, ctypes.c_int, dp]
    lib.scft_calc_poly_density.argtypes = [vp]
    lib.scft_update_1s.argtypes = [vp, ctypes.c_int]
    lib.scft_calc_H.argtypes = [vp, dp]
    lib.scft_get_density.argtypes = [vp, ctypes.c_int, dp, dp, dp]
    lib.scft_get_smeared.argtypes = [vp, ctypes.c_int, dp, dp, dp]
    lib.scft_get_plate_density.argtypes = [vp, ctypes.c_int, dp]
    lib.scft_grad_geom.argtypes = [vp, dp]
    lib.scft_diblock_density.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp, dp]
    lib.scft_homopolymer_density.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, dp, dp]
    lib.scft_fft3d.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int]
    lib.scft_sync.argtypes = [vp]
    lib.scft_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    lib.scft_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    lib.scft_profile_step.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
    lib.scft_set_sweep_groups.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.scft_set_wait_limit.argtypes = [vp, ctypes.c_int]
    lib.scft_fp64_fma_rate.argtypes = [ctypes.c_int, dp]
    lib.scft_set_persistent.argtypes = [vp, ctypes.c_int]
    lib.scft_set_plane_form.argtypes = [vp, ctypes.c_int]
    lib.scft_get_plane_form.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    lib.scft_profile_sweep.argtypes = [vp, ctypes.c_int, dp, dp]
    lib.scft_step_fields.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_void_p]
    lib.scft_iterate_fields.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                        ctypes.c_void_p]
    lib.scft_get_fft_plan.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int)]
    lib.scft_get_schedule.argtypes = [vp] + [ctypes.POINTER(ctypes.c_int)] * 4
    lib.scft_set_fields_all.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p)]
    ip = ctypes.POINTER(ctypes.c_int)
    lib.scft_autotune.argtypes = [vp, ctypes.c_int, ip, ip, ip, dp]
    lib.scft_diblock_density_noalloc.argtypes = [ctypes.POINTER(ctypes.c_int), dp, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_double, vp, vp, vp, vp, vp, vp]
    _lib = lib
    return lib


def _check(code):
    if code != OK:
        raise ScftError(code, load().scft_last_error().decode(errors="replace"))


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(**kw) -> Params:
    """Params with the reference defaults for anything not given."""
    p = Params()
    defaults = dict(Nda=4, Ndb=4, a_smear=0.2, rho0=5.0, chi_ab=0.5, chi_bc=0.0, chi_ac=0.0, kappa=50.0,
                    Nx=(8, 8, 8), L=(4.0, 4.0, 4.0), lam_pl=0.005, lam_mi=0.005, n_exp_nr=0, np_chem=0,
                    sigma=0.0, Ng=0, L_nr=1.0, R_nr=1.0, xi_nr=0.2,
                    center=((0.5, 0.5, 0.5), (0.5, 0.5, 0.5)), orient=((1.0, 0.0, 0.0), (1.0, 0.0, 0.0)),
                    precision=PREC_FP64, plate_shape=PLATE_REFERENCE, shell_lambda=0.0, shell_width=0.0,
                    update_scheme=UPDATE_1S, do_cl=0, cl_seed=1)
    defaults.update(kw)
    for k, v in defaults.items():
        if k in ("Nx", "L"):
            arr = getattr(p, k)
            for i in range(3):
                arr[i] = v[i]
        elif k in ("center", "orient"):
            arr = getattr(p, k)
            for j in range(2):
                for i in range(3):
                    arr[j][i] = v[j][i]
        else:
            setattr(p, k, v)
    return p


def params_from_case(c, **extra) -> Params:
    """Params from an oracle Case (bcp.input semantics)."""
    return make_params(Nda=c.Nda, Ndb=c.Ndb, a_smear=c.a_smear, rho0=c.rho0, chi_ab=c.chi_ab, chi_bc=c.chi_bc,
                       chi_ac=c.chi_ac, kappa=c.kappa, Nx=c.Nx, L=c.L, lam_pl=c.lam_pl, lam_mi=c.lam_mi,
                       n_exp_nr=c.n_exp_nr, np_chem=c.np_chem, sigma=c.sigma, Ng=c.Ng, L_nr=c.L_nr,
                       R_nr=c.R_nr, xi_nr=c.xi_nr, center=c.centers, orient=c.orients, **extra)


class Context:
    """One scft_ctx: a batch of SCFT instances on the current GPU."""

    def __init__(self, params):
        lib = load()
        if isinstance(params, Params):
            params = [params]
        arr = (Params * len(params))(*params)
        h = ctypes.c_void_p()
        _check(lib.scft_create(arr, len(params), ctypes.byref(h)))
        self._h = h
        self.n = len(params)
        self.shapes = [(p.Nx[2], p.Nx[1], p.Nx[0]) for p in params]

    def close(self):
        if getattr(self, "_h", None):
            load().scft_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self, inst=0) -> dict:
        i = Info()
        _check(load().scft_get_info(self._h, inst, ctypes.byref(i)))
        return {f: (tuple(getattr(i, f)) if f == "dx" else getattr(i, f)) for f, _ in Info._fields_}

    def _shape(self, inst):
        return self.shapes[inst]

    def set_fields(self, inst, fields: dict):
        sh = self._shape(inst)
        buf = np.zeros((7,) + sh, np.complex128)
        for k, name in enumerate(FIELD_NAMES):
            if name in fields:
                buf[k] = np.asarray(fields[name], np.complex128).reshape(sh)
        _check(load().scft_set_fields(self._h, inst, _ptr(buf.view(np.float64))))

    def get_fields(self, inst) -> dict:
        sh = self._shape(inst)
        buf = np.zeros((7,) + sh, np.complex128)
        _check(load().scft_get_fields(self._h, inst, _ptr(buf.view(np.float64))))
        return {name: buf[k] for k, name in enumerate(FIELD_NAMES)}

    def calc_poly_density(self):
        _check(load().scft_calc_poly_density(self._h))

    def update_1s(self, n_iter=1):
        _check(load().scft_update_1s(self._h, n_iter))

    def calc_H(self) -> np.ndarray:
        out = np.zeros((self.n, 5), np.float64)
        code = load().scft_calc_H(self._h, _ptr(out))
        if code not in (OK, ERR_NAN):
            _check(code)
        self.last_status = code
        return out

    def grad_geom(self) -> np.ndarray:
        """dH/d(theta_z, c_x, c_y, c_z) per instance and plate: shape (n, 2, 4)."""
        out = np.zeros((self.n, 2, 4), np.float64)
        _check(load().scft_grad_geom(self._h, _ptr(out)))
        return out

    def density(self, inst):
        sh = self._shape(inst)
        a = np.zeros(sh, np.complex128)
        b = np.zeros(sh, np.complex128)
        g = np.zeros(sh, np.complex128)
        _check(load().scft_get_density(self._h, inst, _ptr(a.view(np.float64)), _ptr(b.view(np.float64)),
                                       _ptr(g.view(np.float64))))
        return a, b, g

    def plate_density(self, inst) -> np.ndarray:
        """The explicit plates' core density rho_exp_nr of one instance (real)."""
        out = np.zeros(self._shape(inst), np.float64)
        _check(load().scft_get_plate_density(self._h, inst, _ptr(out)))
        return out

    def smeared(self, inst):
        sh = self._shape(inst)
        a, b, g = (np.zeros(sh, np.complex128) for _ in range(3))
        _check(load().scft_get_smeared(self._h, inst, _ptr(a.view(np.float64)), _ptr(b.view(np.float64)),
                                       _ptr(g.view(np.float64))))
        return a, b, g

    def diblock_density(self, inst, smwa, smwb):
        sh = self._shape(inst)
        wa = np.ascontiguousarray(smwa, np.complex128).reshape(sh)
        wb = np.ascontiguousarray(smwb, np.complex128).reshape(sh)
        ra, rb = np.zeros(sh, np.complex128), np.zeros(sh, np.complex128)
        Q = np.zeros(2, np.float64)
        _check(load().scft_diblock_density(self._h, inst, _ptr(wa.view(np.float64)), _ptr(wb.view(np.float64)),
                                           _ptr(ra.view(np.float64)), _ptr(rb.view(np.float64)), _ptr(Q)))
        return ra, rb, complex(Q[0], Q[1])

    def homopolymer_density(self, inst, W, N, nK):
        sh = self._shape(inst)
        w = np.ascontiguousarray(W, np.complex128).reshape(sh)
        r = np.zeros(sh, np.complex128)
        Q = np.zeros(2, np.float64)
        _check(load().scft_homopolymer_density(self._h, inst, _ptr(w.view(np.float64)), int(N), float(nK),
                                               _ptr(r.view(np.float64)), _ptr(Q)))
        return r, complex(Q[0], Q[1])

    def set_sweep_groups(self, groups: int, phases: int = 1):
        _check(load().scft_set_sweep_groups(self._h, groups, phases))

    def set_wait_limit(self, polls: int):
        _check(load().scft_set_wait_limit(self._h, int(polls)))

    def set_persistent(self, on: bool):
        _check(load().scft_set_persistent(self._h, int(bool(on))))

    def set_plane_form(self, form: int):
        _check(load().scft_set_plane_form(self._h, int(form)))

    def schedule(self) -> dict:
        v = [ctypes.c_int() for _ in range(4)]
        _check(load().scft_get_schedule(self._h, *[ctypes.byref(x) for x in v]))
        f = ctypes.c_int()
        _check(load().scft_get_plane_form(self._h, ctypes.byref(f)))
        return {"groups": v[0].value, "phases": v[1].value, "col_tile": v[2].value, "persistent": bool(v[3].value),
                "plane_form": f.value}

    def autotune(self, reps=3) -> dict:
        g, ph, t, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(load().scft_autotune(self._h, reps, ctypes.byref(g), ctypes.byref(ph), ctypes.byref(t),
                                    ctypes.byref(ms)))
        return dict(self.schedule(), ms_per_sweep=ms.value)

    def stream(self) -> int:
        h = ctypes.c_void_p()
        _check(load().scft_get_stream(self._h, ctypes.byref(h)))
        return h.value or 0

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        _check(load().scft_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def profile_step(self, reps=20) -> dict:
        v = [ctypes.c_double() for _ in range(4)]
        _check(load().scft_profile_step(self._h, int(reps), *[ctypes.byref(x) for x in v]))
        return {"ms_plane": v[0].value, "bytes_plane": v[1].value, "ms_col": v[2].value, "bytes_col": v[3].value}

    def fft_plan(self, inst: int, axis: int) -> list:
        """Radices of the generic FFT stages along one axis, in order."""
        r = (ctypes.c_int * 8)()
        n = ctypes.c_int()
        _check(load().scft_get_fft_plan(self._h, int(inst), int(axis), r, ctypes.byref(n)))
        return list(r[: n.value])

    def profile_sweep(self, reps=5) -> dict:
        ms, by = ctypes.c_double(), ctypes.c_double()
        _check(load().scft_profile_sweep(self._h, int(reps), ctypes.byref(ms), ctypes.byref(by)))
        return {"ms_sweep": ms.value, "bytes_sweep": by.value}

    def step_fields_raw(self, ptrs, n_iter: int, out_ptr: int) -> int:
        """scft_step_fields from host pointers (one per instance, 7 x M complex
        each) into a host buffer of 5 doubles per instance; returns the status
        (OK or ERR_NAN), raises on other errors."""
        arr = (ctypes.c_void_p * self.n)(*ptrs)
        code = load().scft_step_fields(self._h, arr, int(n_iter), ctypes.c_void_p(out_ptr))
        if code not in (OK, ERR_NAN):
            _check(code)
        return code

    def step_fields(self, fields: list, n_iter: int = 1) -> np.ndarray:
        """step_fields_raw from a list of field dicts (as set_fields takes)."""
        bufs = []
        for k, f in enumerate(fields):
            b = np.zeros((7,) + self._shape(k), np.complex128)
            for q, name in enumerate(FIELD_NAMES):
                if name in f:
                    b[q] = np.asarray(f[name], np.complex128).reshape(self._shape(k))
            bufs.append(b)
        out = np.zeros((self.n, 5), np.float64)
        self.last_status = self.step_fields_raw([b.ctypes.data for b in bufs], n_iter, out.ctypes.data)
        return out

    def iterate_fields_raw(self, ptrs, out_ptrs, h_ptr: int) -> int:
        """scft_iterate_fields from host pointers (one per instance, 7 x M
        complex each) into out_ptrs (None: no download; may equal ptrs) and a
        host buffer of 5 doubles per instance; returns the status (OK or
        ERR_NAN), raises on other errors."""
        arr = (ctypes.c_void_p * self.n)(*ptrs)
        oarr = (ctypes.c_void_p * self.n)(*out_ptrs) if out_ptrs is not None else None
        code = load().scft_iterate_fields(self._h, arr, oarr, ctypes.c_void_p(h_ptr))
        if code not in (OK, ERR_NAN):
            _check(code)
        return code

    def iterate_fields(self, bufs: list, download: bool = True) -> np.ndarray:
        """iterate_fields_raw on complex128 arrays of shape (7,) + grid, one
        per instance, updated in place when `download`; returns H (n x 5) of
        the fields passed in."""
        for k, b in enumerate(bufs):
            if b.dtype != np.complex128 or b.shape != (7,) + self._shape(k) or not b.flags.c_contiguous:
                raise ValueError("instance %d: need a C-contiguous complex128 array of shape %s"
                                 % (k, (7,) + self._shape(k)))
        out = np.zeros((self.n, 5), np.float64)
        ptrs = [b.ctypes.data for b in bufs]
        self.last_status = self.iterate_fields_raw(ptrs, ptrs if download else None, out.ctypes.data)
        return out

    def set_fields_all_raw(self, ptrs):
        """scft_set_fields_all from device-visible host pointers (one per instance)."""
        arr = (ctypes.c_void_p * self.n)(*ptrs)
        _check(load().scft_set_fields_all(self._h, arr))

    def set_fields_raw(self, inst, ptr: int):
        """set_fields from a host buffer given by address (7*M complex, e.g. pinned memory)."""
        _check(load().scft_set_fields(self._h, inst, ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double))))

    def calc_H_raw(self, ptr: int):
        """calc_H into a host buffer given by address (5 doubles per instance)."""
        code = load().scft_calc_H(self._h, ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double)))
        if code not in (OK, ERR_NAN):
            _check(code)
        return code

    def fft3d(self, inst, data, sign):
        sh = self._shape(inst)
        a = np.ascontiguousarray(data, np.complex128).copy()
        count = a.size // int(np.prod(sh))
        _check(load().scft_fft3d(self._h, inst, _ptr(a.view(np.float64)), count, int(sign)))
        return a


def fp64_fma_rate(reps: int = 5) -> float:
    """Measured FP64 FMA throughput of the current GPU, GFLOP/s."""
    v = ctypes.c_double()
    _check(load().scft_fp64_fma_rate(int(reps), ctypes.byref(v)))
    return v.value


def mixed_available() -> bool:
    """True when the library was built with the FP32-propagator (mixed) path."""
    try:
        return bool(load().scft_version() >= 2)
    except ScftError:
        return False
