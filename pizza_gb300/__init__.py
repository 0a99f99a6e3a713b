"""GB300 (sm_103a) time step of pizza: Python binding over the C ABI.

The library in ``_lib/libpizza_gb300.so`` (declared in ``include/pizza_gpu.h``)
advances one or many independent annulus instances of pizza's rotating
quasi-geostrophic convection problem with the reference's collocation method.
This module is a thin ctypes layer: configurations mirror pizza's input.nml
(src/namelists.f90:162-189), spectral arrays use the reference's
m-distributed layout ``f(n_m, n_r)`` (numpy shape ``(n_m_max, n_r_max)``,
complex128), and time series rows mirror pizza's e_kin / e_kin_3D / heat files
(src/outputs.f90:677-793).

There is no CPU fallback: if the library is missing or no GPU is present,
every call raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpizza_gb300.so")

SCHEMES = {"CNAB2": 0, "SBDF2": 1, "BDF2AB2": 1, "SBDF3": 2, "BDF3AB3": 2, "SBDF4": 3,
           "BDF4AB4": 3, "CNLF": 4, "MODCNAB": 5, "TVB33": 6,
           # DIRK IMEX Runge-Kutta (src/dirk_schemes.f90)
           "ARS222": 10, "ARS232": 11, "ARS233": 12, "SSP222": 13, "LSDIRK222": 14, "LZ232": 15,
           "CK232": 16, "ARS443": 17, "BPR353": 18, "PC2": 19, "ARS343": 20, "MARS343": 21,
           "SSP322": 22, "SSP332": 23, "SSP433": 24, "DP1-242": 25, "DP2-242": 26, "LZ453": 27,
           "KC343": 28, "KC564": 29, "KC785": 30, "DBM453": 31}
KERNEL_KINDS = 10
SOLVE_INFLUENCE, SOLVE_DIRECT = 0, 1
CHEB_COLL, CHEB_INTEG = 0, 1
TS_VISC, TS_ROT = 0, 1
SERIES_COLS = 22
SERIES_NAMES = ("time", "us2_2D", "up2_2D", "up2_axi_2D", "us2_3D", "up2_3D", "uz2_3D",
                "up2_axi_3D", "NuTop", "NuBot", "Nu_vol", "Nu_int", "tTop", "tBot", "beta_t", "dt",
                "ShTop", "ShBot", "Sh_vol", "xiTop", "xiBot", "beta_xi")

PZ_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "singular matrix",
             -4: "time step too small", -5: "non-finite state", -6: "unsupported option",
             -7: "out of device memory"}


class PizzaError(RuntimeError):
    """Error returned by the library (code < 0)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{PZ_ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class _CConfig(ctypes.Structure):
    _fields_ = [("n_r_max", ctypes.c_int), ("n_cheb_max", ctypes.c_int), ("m_max", ctypes.c_int),
                ("minc", ctypes.c_int), ("ra", ctypes.c_double), ("ek", ctypes.c_double),
                ("pr", ctypes.c_double), ("radratio", ctypes.c_double), ("g0", ctypes.c_double),
                ("g1", ctypes.c_double), ("g2", ctypes.c_double), ("ktopt", ctypes.c_int),
                ("kbott", ctypes.c_int), ("ktopv", ctypes.c_int), ("kbotv", ctypes.c_int),
                ("l_ek_pump", ctypes.c_int), ("l_non_rot", ctypes.c_int), ("l_temp_advz", ctypes.c_int),
                ("time_scheme", ctypes.c_int), ("matrix_solve", ctypes.c_int), ("corio_imp", ctypes.c_int),
                ("buo_imp", ctypes.c_int), ("dtMax", ctypes.c_double), ("courfac", ctypes.c_double),
                ("alpha", ctypes.c_double), ("dt_fac", ctypes.c_double), ("cheb_method", ctypes.c_int),
                ("time_scale", ctypes.c_int), ("l_rerror_fix", ctypes.c_int), ("rerror_fac", ctypes.c_double),
                ("raxi", ctypes.c_double), ("sc", ctypes.c_double), ("ktopxi", ctypes.c_int),
                ("kbotxi", ctypes.c_int), ("xicond_fac", ctypes.c_double)]


@dataclasses.dataclass
class Config:
    """One instance's namelist values (defaults: src/namelists.f90:530-672).
    matrix_solve 'DIRECT' is pizza's coupled smat solve, 'INFLUENCE' the dmat
    influence-matrix solve (the one the adjoint covers).  cheb_method 'COLL'
    is the collocation method, 'INTEG' the sparse Chebyshev integration
    method with tau boundary rows.  raxi /= 0 adds the composition equation
    (Schmidt number sc)."""
    n_r_max: int = 32
    n_cheb_max: int | None = None
    m_max: int = 32
    minc: int = 1
    ra: float = 1.0e5
    ek: float = 1.0e-3
    pr: float = 1.0
    radratio: float = 0.35
    g0: float = 0.0
    g1: float = 1.0
    g2: float = 0.0
    ktopt: int = 1
    kbott: int = 1
    ktopv: int = 2
    kbotv: int = 2
    l_ek_pump: bool = False
    l_non_rot: bool = False
    l_temp_advz: bool = False
    time_scheme: str = "CNAB2"
    matrix_solve: str = "DIRECT"
    corio_term: str = "IMPLICIT"
    buo_term: str = "IMPLICIT"
    dtMax: float = 1.0e-5
    courfac: float = 1.0e3
    alpha: float = 0.5
    dt_fac: float = 2.0
    cheb_method: str = "COLL"
    time_scale: str = "VISC"
    l_rerror_fix: bool = False
    rerror_fac: float = 500.0
    raxi: float = 0.0
    sc: float = 0.0
    ktopxi: int = 1
    kbotxi: int = 1
    xicond_fac: float = 1.0

    def to_c(self) -> _CConfig:
        c = _CConfig()
        for f in ("n_r_max", "m_max", "minc", "ra", "ek", "pr", "radratio", "g0", "g1", "g2",
                  "ktopt", "kbott", "ktopv", "kbotv", "dtMax", "courfac", "alpha", "dt_fac",
                  "raxi", "sc", "ktopxi", "kbotxi", "xicond_fac"):
            setattr(c, f, getattr(self, f))
        c.n_cheb_max = self.n_r_max if self.n_cheb_max is None else self.n_cheb_max
        c.l_ek_pump = int(bool(self.l_ek_pump))
        c.l_non_rot = int(bool(self.l_non_rot))
        c.l_temp_advz = int(bool(self.l_temp_advz))
        ts = self.time_scheme.upper()
        if ts not in SCHEMES:
            raise ValueError(f"time integrator {self.time_scheme} not found")
        c.time_scheme = SCHEMES[ts]
        c.matrix_solve = SOLVE_DIRECT if "DIRECT" in self.matrix_solve.upper() else SOLVE_INFLUENCE
        c.corio_imp = int("IMP" in self.corio_term.upper())
        c.buo_imp = int("IMP" in self.buo_term.upper())
        c.cheb_method = CHEB_COLL if "COLL" in self.cheb_method.upper() else CHEB_INTEG
        c.time_scale = TS_ROT if "ROT" in self.time_scale.upper() else TS_VISC
        c.l_rerror_fix = int(bool(self.l_rerror_fix))
        c.rerror_fac = float(self.rerror_fac)
        return c

    @property
    def n_m_max(self) -> int:
        return self.m_max // self.minc + 1

    @property
    def n_phi_max(self) -> int:
        return 3 * self.m_max // self.minc


_lib = None


def load_library(path: str | None = None):
    """Load the CUDA library (raises if it is absent: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"pizza_gb300 CUDA library not built: {p} (run `python -m pizza_gb300.build`)")
    lib = ctypes.CDLL(p)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.pz_config_default.argtypes = [ctypes.POINTER(_CConfig)]
    lib.pz_config_default.restype = None
    lib.pz_create.argtypes = [ctypes.POINTER(_CConfig), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    lib.pz_set_state.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp]
    lib.pz_set_state_all.argtypes = [ctypes.c_void_p, dp, dp, dp]
    lib.pz_set_state_xi.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, dp]
    lib.pz_get_state_xi.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp]
    lib.pz_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.pz_sync.argtypes = [ctypes.c_void_p]
    lib.pz_get_state.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp]
    lib.pz_get_series.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.POINTER(ctypes.c_int)]
    lib.pz_get_dims.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 3
    lib.pz_launches_per_step.argtypes = [ctypes.c_void_p]
    lib.pz_latest_rows.argtypes = [ctypes.c_void_p, dp]
    lib.pz_stream.argtypes = [ctypes.c_void_p]
    lib.pz_stream.restype = ctypes.c_void_p
    lib.pz_step_profile.argtypes = [ctypes.c_void_p, ctypes.c_int, dp]
    lib.pz_kernel_name.argtypes = [ctypes.c_int]
    lib.pz_kernel_name.restype = ctypes.c_char_p
    vp = ctypes.c_void_p
    lib.pz_explicit_terms.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.pz_explicit_terms_noalloc.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.pz_adjoint_forward.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp]
    lib.pz_adjoint_backward.argtypes = [vp, dp, dp]
    lib.pz_set_ra.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    lib.pz_adjoint_grid_snapshots.argtypes = [vp, ctypes.c_int]
    lib.pz_get_history.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    lib.pz_set_history.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    lib.pz_get_step_state.argtypes = [vp, ctypes.c_int, dp, dp, ctypes.POINTER(ctypes.c_int)]
    lib.pz_set_step_state.argtypes = [vp, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int]
    lib.pz_set_restart_ab1.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.pz_get_spectra.argtypes = [vp, ctypes.c_int, dp]
    lib.pz_get_spectra_2d.argtypes = [vp, ctypes.c_int, dp]
    lib.pz_balance_step.argtypes = [vp, ctypes.c_int, dp, dp]
    lib.pz_integ_operator.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, ctypes.POINTER(ctypes.c_int)]
    lib.pz_fast_path.argtypes = [ctypes.c_int]
    lib.pz_integ_banded.argtypes = [ctypes.c_int]
    lib.pz_probe_peaks.argtypes = [dp, dp]
    lib.pz_tune_set.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.pz_fast_eigen.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp]
    lib.pz_destroy.argtypes = [ctypes.c_void_p]
    lib.pz_last_error.argtypes = [ctypes.c_void_p]
    lib.pz_last_error.restype = ctypes.c_char_p
    for f in ("pz_create", "pz_set_state", "pz_set_state_all", "pz_set_state_xi", "pz_get_state_xi", "pz_step",
              "pz_sync", "pz_get_state",
              "pz_get_series", "pz_get_dims", "pz_launches_per_step", "pz_latest_rows",
              "pz_step_profile", "pz_explicit_terms", "pz_explicit_terms_noalloc", "pz_adjoint_forward",
              "pz_adjoint_backward", "pz_adjoint_grid_snapshots", "pz_set_ra", "pz_get_history", "pz_set_history", "pz_get_step_state",
              "pz_set_step_state", "pz_set_restart_ab1", "pz_get_spectra", "pz_get_spectra_2d", "pz_balance_step", "pz_integ_operator",
              "pz_fast_path", "pz_integ_banded", "pz_fast_eigen", "pz_probe_peaks", "pz_tune_set", "pz_destroy"):
        getattr(lib, f).restype = ctypes.c_int
    _lib = lib
    return lib


INTEG_OPERATORS = ("I2R1", "I2R2", "I2", "LT0", "ULAP", "I4R3", "I4R4", "Q0", "Q1", "S0", "S1", "S2", "P0", "P1",
                   "N0", "N1", "L0", "L1", "L2")


def integ_operator(n_r_max: int, radratio: float, name: str):
    """One banded operator of the integration method as the library derives
    it (host code, no GPU needed): (n_r_max, n_r_max) array and bandwidth."""
    lib = load_library()
    out = np.zeros(n_r_max * n_r_max)
    bw = ctypes.c_int(0)
    rc = lib.pz_integ_operator(n_r_max, float(radratio), INTEG_OPERATORS.index(name), _dptr(out), ctypes.byref(bw))
    if rc != 0:
        raise RuntimeError(lib.pz_last_error(None).decode())
    return out.reshape(n_r_max, n_r_max, order="F"), bw.value


def integ_banded(enable=None) -> bool:
    """Bordered banded factors (True) or dense per-m inverses (False, the
    default) for the integration method's solves, for handles created
    afterwards (pz_integ_banded); None only queries.  Returns the previous
    setting."""
    lib = load_library()
    return bool(lib.pz_integ_banded(-1 if enable is None else int(bool(enable))))


def fast_path(enable=None) -> bool:
    """The tensor-core stage for handles created afterwards (pz_fast_path):
    ``enable`` True/False sets it, None only queries; returns the previous
    setting."""
    lib = load_library()
    return bool(lib.pz_fast_path(-1 if enable is None else int(bool(enable))))


TUNE_FAST_G, TUNE_RLOOP_RG, TUNE_LANES = 0, 1, 2


def tune_set(what: int, key: int, value: int):
    """Process-wide launch-shape table for handles created afterwards
    (pz_tune_set): TUNE_FAST_G (instances per tensor-core block),
    TUNE_RLOOP_RG (radii per transform block for n_phi_max = key) or
    TUNE_LANES (parallel lanes of an all-tensor-core step); value <= 0
    restores the default."""
    lib = load_library()
    rc = lib.pz_tune_set(int(what), int(key), int(value))
    if rc != 0:
        raise PizzaError(rc, lib.pz_last_error(None).decode())


def probe_peaks():
    """(DFMA, bf16 mma.sync) peak issue rates of the current GPU in TFLOP/s,
    measured by the library's probe kernels (pz_probe_peaks)."""
    lib = load_library()
    a, b = np.zeros(1), np.zeros(1)
    rc = lib.pz_probe_peaks(_dptr(a), _dptr(b))
    if rc != 0:
        raise PizzaError(rc, "pz_probe_peaks failed")
    return float(a[0]), float(b[0])


def fast_eigen(n_r_max: int, radratio: float, m: int):
    """The eigen-decomposition the tensor-core stage uses for mode m (host
    code, no GPU needed): lam (n,) and U (n, n), n = n_r_max - 2, with
    (D2 + D/r - m^2/r^2) on the interior points = U diag(lam) U^-1."""
    lib = load_library()
    n = n_r_max - 2
    lam = np.zeros(n)
    U = np.zeros(n * n)
    rc = lib.pz_fast_eigen(n_r_max, float(radratio), int(m), _dptr(lam), _dptr(U))
    if rc != 0:
        raise PizzaError(rc, lib.pz_last_error(None).decode())
    return lam, U.reshape(n, n)


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _carr(a, shape):
    """(n_m, n_r) complex array -> C-contiguous complex128 in Fortran (n_m fastest) order."""
    if a is None:
        return None
    a = np.asarray(a, dtype=np.complex128)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    # (n_m, n_r) with n_m fastest == row-major (n_r, n_m)
    return np.ascontiguousarray(a.T)


class Ensemble:
    """A batch of independent pizza instances advanced together on one GPU."""

    def __init__(self, configs):
        if isinstance(configs, Config):
            configs = [configs]
        self.configs = list(configs)
        self.lib = load_library()
        arr = (_CConfig * len(self.configs))(*[c.to_c() for c in self.configs])
        h = ctypes.c_void_p()
        rc = self.lib.pz_create(arr, len(self.configs), ctypes.byref(h))
        if rc != 0:
            raise PizzaError(rc, self.lib.pz_last_error(None).decode())
        self._h = h
        self.dims = []
        for i in range(len(self.configs)):
            a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            self._check(self.lib.pz_get_dims(self._h, i, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
            self.dims.append((a.value, b.value, c.value))

    def _check(self, rc):
        if rc != 0:
            raise PizzaError(rc, self.lib.pz_last_error(self._h).decode())

    def __len__(self):
        return len(self.configs)

    def shape(self, i):
        n, m, _ = self.dims[i]
        return (m, n)

    def set_state(self, i, us=None, up=None, temp=None, xi=None):
        """pizza's start fields (src/init_fields.f90:54-258) from physical
        fields; ``xi`` is the composition perturbation (raxi /= 0)."""
        shp = self.shape(i)
        a, b, c = _carr(us, shp), _carr(up, shp), _carr(temp, shp)
        if xi is None:
            self._check(self.lib.pz_set_state(self._h, i, _dptr(a), _dptr(b), _dptr(c)))
        else:
            x = _carr(xi, shp)
            self._check(self.lib.pz_set_state_xi(self._h, i, _dptr(a), _dptr(b), _dptr(c), _dptr(x)))

    def set_state_all(self, temps, us=None, up=None):
        """Start fields of every instance; ``temps`` is a list of (n_m, n_r) arrays."""
        def cat(lst):
            if lst is None:
                return None
            return np.concatenate([_carr(x, self.shape(i)).ravel() for i, x in enumerate(lst)])
        a, b, c = cat(us), cat(up), cat(temps)
        self._check(self.lib.pz_set_state_all(self._h, _dptr(a), _dptr(b), _dptr(c)))

    def step(self, n_steps=1, sync=True):
        self._check(self.lib.pz_step(self._h, int(n_steps)))
        if sync:
            self.sync()

    def sync(self):
        self._check(self.lib.pz_sync(self._h))

    def get_state(self, i):
        """Physical fields of instance i as (n_m, n_r) complex arrays, plus time and dt."""
        n, m, _ = self.dims[i]
        bufs = {k: np.zeros((n, m), np.complex128) for k in ("us", "up", "om", "psi", "temp", "dtemp")}
        t, dt = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.pz_get_state(self._h, i, *[_dptr(bufs[k]) for k in ("us", "up", "om", "psi", "temp", "dtemp")],
                                          ctypes.byref(t), ctypes.byref(dt)))
        out = {k: v.T.copy() for k, v in bufs.items()}
        out["time"] = t.value
        out["dt"] = dt.value
        if self.configs[i].raxi != 0.0:
            xi, dxi = np.zeros((n, m), np.complex128), np.zeros((n, m), np.complex128)
            self._check(self.lib.pz_get_state_xi(self._h, i, _dptr(xi), _dptr(dxi)))
            out["xi"], out["dxi"] = xi.T.copy(), dxi.T.copy()
        return out

    def series(self, i, max_rows=1024):
        """Time series rows of instance i (columns: SERIES_NAMES)."""
        rows = np.zeros((max_rows, SERIES_COLS))
        n = ctypes.c_int(max_rows)
        self._check(self.lib.pz_get_series(self._h, i, _dptr(rows), ctypes.byref(n)))
        return rows[: n.value].copy()

    def explicit_terms(self, i, us, up, om, temp, out=None, noalloc=False):
        """Explicit terms of instance i from device tensors (anything with
        ``data_ptr()``, e.g. torch complex128 CUDA tensors of shape
        (n_r_max, n_m_max) row-major, i.e. the reference's (n_m, n_r) layout
        with n_m fastest).  Returns (dTdt_expl, dpsidt_expl, dtr, dth) in the
        given or newly created torch tensors; ordered on the handle's stream.
        ``noalloc=True`` calls pz_explicit_terms_noalloc, which takes no device
        memory (its intermediates live in a static device array shared by all
        calls on the device; overlapping calls race)."""
        import torch
        n, m, _ = self.dims[i]
        dev = us.device
        if out is None:
            out = (torch.empty((n, m), dtype=torch.complex128, device=dev),
                   torch.empty((n, m), dtype=torch.complex128, device=dev),
                   torch.empty(n, dtype=torch.float64, device=dev),
                   torch.empty(n, dtype=torch.float64, device=dev))
        for t in (us, up, om, temp) + tuple(out[:2]):
            if tuple(t.shape) != (n, m) or t.dtype != torch.complex128 or not t.is_contiguous():
                raise ValueError(f"expected contiguous complex128 tensors of shape {(n, m)}")
        fn = self.lib.pz_explicit_terms_noalloc if noalloc else self.lib.pz_explicit_terms
        self._check(fn(self._h, i, us.data_ptr(), up.data_ptr(), om.data_ptr(), temp.data_ptr(),
                       out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr()))
        return out

    def launches_per_step(self):
        return self.lib.pz_launches_per_step(self._h)

    # -- history and step state (checkpoints) ------------------------------
    def get_history(self, i, field, kind, slot):
        """History slot (1-based) of the time arrays: field 0 temperature, 1
        vorticity, 2 composition; kind 0 old, 1 impl, 2 expl.  (n_m, n_r)
        complex."""
        n, m, _ = self.dims[i]
        buf = np.zeros((n, m), np.complex128)
        self._check(self.lib.pz_get_history(self._h, i, int(field), int(kind), int(slot), _dptr(buf.view(np.float64))))
        return buf.T.copy()

    def set_history(self, i, field, kind, slot, arr):
        a = _carr(arr, self.shape(i))
        self._check(self.lib.pz_set_history(self._h, i, int(field), int(kind), int(slot), _dptr(a.view(np.float64))))

    def get_step_state(self, i):
        """(time, dt history, n_step) of instance i."""
        t = ctypes.c_double()
        dt = np.zeros(4)
        ns = ctypes.c_int()
        self._check(self.lib.pz_get_step_state(self._h, i, ctypes.byref(t), _dptr(dt), ctypes.byref(ns)))
        return t.value, dt, ns.value

    def set_step_state(self, i, time, dt, n_step):
        d = np.zeros(4)
        dt = np.atleast_1d(np.asarray(dt, np.float64))
        d[:len(dt)] = dt
        self._check(self.lib.pz_set_step_state(self._h, i, float(time), _dptr(d), int(n_step)))

    def spectra(self, i):
        """Snapshot spectra of instance i on the device: (n_m_max, 5) array of
        the r-integrated us^2, up^2, enstrophy, T^2 and xi^2 per m
        (spectra.f90)."""
        out = np.zeros(5 * self.dims[i][1])
        self._check(self.lib.pz_get_spectra(self._h, i, _dptr(out)))
        return out.reshape(-1, 5)

    def spectra_2d(self, i):
        """(r, m) spectra of instance i on the device: (3, n_r_max, n_m_max)
        array of pi cc2real(f) r height for f = us, up, om (the integrands of
        spectra, before the r-integration)."""
        N, M = self.dims[i][0], self.dims[i][1]
        out = np.zeros(3 * N * M)
        self._check(self.lib.pz_get_spectra_2d(self._h, i, _dptr(out)))
        return out.reshape(3, N, M)

    BALANCE_TERMS = ("buo", "cor", "adv", "dwdt", "visc", "pump")
    VP_TERMS = ("rey_stress", "dvpdt", "visc", "pump")

    def balance_step(self, i):
        """One step of the handle (every instance) that also returns the force
        balances of instance i over it (pz_balance_step): {"vort": {term:
        (n_m_max, n_r_max) complex}, "vp": {term: (n_r_max,) real}}."""
        N, M = self.dims[i][0], self.dims[i][1]
        vort = np.zeros(12 * N * M)
        vpo = np.zeros(4 * N)
        self._check(self.lib.pz_balance_step(self._h, i, _dptr(vort), _dptr(vpo)))
        z = vort.view(np.complex128).reshape(6, N, M)
        return {"vort": {t: z[k].T.copy() for k, t in enumerate(self.BALANCE_TERMS)},
                "vp": {t: vpo[k * N:(k + 1) * N].copy() for k, t in enumerate(self.VP_TERMS)}}

    def set_restart_ab1(self, i, on=True):
        """First step after a restart with first-order explicit weights (pizza's l_AB1)."""
        self._check(self.lib.pz_set_restart_ab1(self._h, i, int(bool(on))))

    # -- discrete adjoint -------------------------------------------------
    def set_ra(self, i, ra):
        """Change Ra of instance i (BuoFac = Ra/Pr)."""
        self._check(self.lib.pz_set_ra(self._h, i, float(ra)))
        self.configs[i] = dataclasses.replace(self.configs[i], ra=float(ra))

    def adjoint_forward(self, n_steps, n_window, checkpoint_every=0, dt_sched=None, objective="ekin3d"):
        """Forward sweep of the objective ('ekin3d': us2_3D+up2_3D+uz2_3D, or
        'nutop': NuTop) averaged over the last n_window states, from the start
        state of every instance (pz_adjoint_forward).  ``dt_sched``
        (n_instances, n_steps) prescribes the time steps; None lets the
        Courant controller choose.  Returns (J, dt_used) as numpy arrays."""
        obj = {"ekin3d": 0, "nutop": 1}[objective]
        nI = len(self)
        J = np.zeros(nI)
        dt_used = np.zeros((nI, int(n_steps)))
        sched = None
        if dt_sched is not None:
            sched = np.ascontiguousarray(np.broadcast_to(np.asarray(dt_sched, np.float64), (nI, int(n_steps))))
        self._check(self.lib.pz_adjoint_forward(self._h, obj, int(n_steps), int(n_window), int(checkpoint_every),
                                                _dptr(sched), _dptr(J), _dptr(dt_used)))
        return J, dt_used

    def adjoint_grid_snapshots(self, enable=True):
        """Keep (default) or drop the phi-grids of the stored stage states
        (32 n_r_max n_phi_max bytes each); kept, the backward sweep skips
        their inverse transforms (pz_adjoint_grid_snapshots)."""
        self._check(self.lib.pz_adjoint_grid_snapshots(self._h, int(bool(enable))))

    def adjoint_backward(self):
        """Gradient of the last forward sweep's objective: a list of
        (n_m, n_r) complex arrays dJ/dtemp (dJ = Re sum conj(g) dtemp) and an
        array dJ/dRa."""
        sizes = [m * n for (n, m, _) in self.dims]
        g = np.zeros(sum(sizes), np.complex128)
        dra = np.zeros(len(self))
        self._check(self.lib.pz_adjoint_backward(self._h, _dptr(g.view(np.float64)), _dptr(dra)))
        out, o = [], 0
        for i, (n, m, _) in enumerate(self.dims):
            out.append(g[o:o + m * n].reshape(n, m).T.copy())
            o += m * n
        return out, dra

    def latest_rows(self, out=None):
        """Latest time-series row of every instance, shape (n_instances, SERIES_COLS)."""
        if out is None:
            out = np.zeros((len(self), SERIES_COLS))
        self._check(self.lib.pz_latest_rows(self._h, _dptr(out)))
        return out

    @property
    def stream_ptr(self) -> int:
        """cudaStream_t of the handle (for torch.cuda.ExternalStream)."""
        return int(self.lib.pz_stream(self._h) or 0)

    def profile_steps(self, n_steps):
        """Mean device ms per step of each kernel, launched one by one."""
        ms = np.zeros(KERNEL_KINDS)
        self._check(self.lib.pz_step_profile(self._h, int(n_steps), _dptr(ms)))
        return {self.lib.pz_kernel_name(k).decode(): float(ms[k]) for k in range(KERNEL_KINDS)}

    def close(self):
        if getattr(self, "_h", None):
            self.lib.pz_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
