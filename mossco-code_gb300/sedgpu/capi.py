"""ctypes binding of the C ABI in include/mossco_sed.h.

This is the same binding a Python caller of the library would write; the
Fortran host binds the same symbols through ISO_C_BINDING.  The library is
the only compute path: if it cannot be loaded, or no GPU is present,
:class:`Solver` raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import Optional

import numpy as np

from . import build as _build
from .model import BGC_NAMES, NTR, ColumnSet

SED_OK, SED_E_ARG, SED_E_NAN, SED_E_SUBSTEP_CAP = 0, -1, -2, -3
SED_E_CUDA, SED_E_STATE, SED_E_NOMEM, SED_E_NODEVICE = -4, -5, -6, -7
SED_E_TOO_LARGE = -9
SED_FP32, SED_FP64 = 0, 1
SED_CUT_PER_COLUMN, SED_CUT_GLOBAL = 0, 1
SED_KMAX_LIMIT = 127
SED_HIST_BINS = 16


class SedError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (code {code})")
        self.code = code


class SedParams(ctypes.Structure):
    _fields_ = ([("diffusivity", ctypes.c_double),
                 ("bioturbation", ctypes.c_double),
                 ("bcup_dissolved", ctypes.c_int),
                 ("bcup_particulate", ctypes.c_int),
                 ("mol_diff_mode", ctypes.c_int),
                 ("mol_diff_d0", ctypes.c_double),
                 ("dt_min", ctypes.c_double),
                 ("relative_change_min", ctypes.c_double),
                 ("atol", ctypes.c_double),
                 ("max_attempts", ctypes.c_int),
                 ("cut_scope", ctypes.c_int)]
                + [(n, ctypes.c_double) for n in BGC_NAMES]
                + [("epilogue", ctypes.c_int),
                   ("minimum", ctypes.c_double * NTR),
                   ("precision", ctypes.c_int),
                   ("budgets", ctypes.c_int),
                   ("device", ctypes.c_int),
                   ("bioturbation_profile", ctypes.c_int),
                   ("bioturb_k_l", ctypes.c_double),
                   ("bioturb_L1", ctypes.c_double),
                   ("bioturb_L2", ctypes.c_double),
                   ("bioturb_beta", ctypes.c_double),
                   ("bioturb_b", ctypes.c_double),
                   ("bioturb_dry_density", ctypes.c_double),
                   ("temp_activation", ctypes.c_double),
                   ("adaptive_solver_diagnostics", ctypes.c_int)])


class SedStats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_longlong),
                ("accepted", ctypes.c_longlong),
                ("column_steps", ctypes.c_longlong),
                ("max_col_attempts", ctypes.c_int),
                ("capped_columns", ctypes.c_int),
                ("nan_cells", ctypes.c_int),
                ("gpu_launches", ctypes.c_int),
                ("min_dt", ctypes.c_double),
                ("device_ms", ctypes.c_double),
                ("surrogate_columns", ctypes.c_longlong)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class SedTuning(ctypes.Structure):
    _fields_ = [("tile_columns", ctypes.c_int * 2),
                ("threads", ctypes.c_int * 2),
                ("blocks_per_sm", ctypes.c_int * 2),
                ("pipeline_chunks", ctypes.c_int),
                ("segments", ctypes.c_int),
                ("max_attempts", ctypes.c_int),
                ("step_ms", ctypes.c_float),
                ("ode_solver_ms", ctypes.c_float),
                ("trials", ctypes.c_int)]

    def as_dict(self):
        d = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            d[n] = list(v) if isinstance(v, ctypes.Array) else v
        return d


SED_SPINUP_COLUMN, SED_SPINUP_ALL = 0, 1
SED_TUNE_PIPELINE = 1
SED_TUNE_CAP = 2

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_H = ctypes.c_void_p

# name -> (restype, argtypes); must list every function of mossco_sed.h
SIGNATURES = {
    "sed_default_params": (ctypes.c_int, [ctypes.POINTER(SedParams)]),
    "sed_set_column_bgc": (ctypes.c_int, [_H, _dp]),
    "sed_create": (ctypes.c_int, [ctypes.POINTER(SedParams), ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(_H)]),
    "sed_set_grid": (ctypes.c_int, [_H, _dp, _dp, _dp, _dp, _dp, _dp, _ip,
                                    _ip]),
    "sed_set_forcing": (ctypes.c_int, [_H, _dp, _dp]),
    "sed_set_boundary": (ctypes.c_int, [_H, _dp, _dp, _dp, _ip]),
    "sed_get_boundary": (ctypes.c_int, [_H, _dp, _dp]),
    "sed_spinup": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_longlong, ctypes.POINTER(SedStats)]),
    "sed_set_state": (ctypes.c_int, [_H, _dp]),
    "sed_get_state": (ctypes.c_int, [_H, _dp]),
    "sed_step": (ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int,
                                ctypes.c_int, ctypes.POINTER(SedStats)]),
    "sed_ode_solver": (ctypes.c_int, [_H, _dp, _dp, _dp, ctypes.c_double,
                                      ctypes.c_int,
                                      ctypes.POINTER(SedStats)]),
    "sed_get_rhs": (ctypes.c_int, [_H, _dp, _dp, _dp]),
    "sed_get_fluxes": (ctypes.c_int, [_H, _dp]),
    "sed_get_attempts": (ctypes.c_int, [_H, _ip]),
    "sed_get_budgets": (ctypes.c_int, [_H, _dp]),
    "sed_get_min_dt": (ctypes.c_int, [_H, _dp]),
    "sed_get_min_dt_grid_cell": (ctypes.c_int, [_H, _dp, ctypes.POINTER(ctypes.c_int)]),
    "sed_set_stream": (ctypes.c_int, [_H, _vp]),
    "sed_host_register": (ctypes.c_int, [_vp, ctypes.c_size_t]),
    "sed_host_unregister": (ctypes.c_int, [_vp]),
    "sed_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "sed_get_attempt_histogram": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.c_longlong)]),
    "sed_host_free": (ctypes.c_int, [_vp]),
    "sed_get_tuning": (ctypes.c_int, [_H, ctypes.POINTER(SedTuning)]),
    "sed_set_tuning": (ctypes.c_int, [_H, ctypes.POINTER(SedTuning)]),
    "sed_autotune": (ctypes.c_int, [_H, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(SedTuning)]),
    "sed_ode_solver_noalloc": (ctypes.c_int, [
        ctypes.POINTER(SedParams), ctypes.c_int, ctypes.c_int, ctypes.c_int,
        _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp, ctypes.c_double,
        ctypes.c_int, ctypes.POINTER(SedStats)]),
    "sed_sur_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int,
                                      ctypes.c_ulonglong, ctypes.c_int,
                                      ctypes.POINTER(_H)]),
    "sed_sur_num_params": (ctypes.c_int, [_H]),
    "sed_sur_set_weights": (ctypes.c_int, [_H, _fp]),
    "sed_sur_get_weights": (ctypes.c_int, [_H, _fp]),
    "sed_sur_state_size": (ctypes.c_int, [_H]),
    "sed_sur_get_state": (ctypes.c_int, [_H, _fp, ctypes.POINTER(ctypes.c_longlong)]),
    "sed_sur_set_state": (ctypes.c_int, [_H, _fp, ctypes.c_longlong]),
    "sed_sur_forward": (ctypes.c_int, [_H, _fp, _fp, ctypes.c_int]),
    "sed_sur_forward_device": (ctypes.c_int, [_H, _vp, _vp, ctypes.c_int]),
    "sed_sur_train_step": (ctypes.c_int, [_H, _vp, _vp, ctypes.c_int,
                                          ctypes.c_float, _fp]),
    "sed_sur_grads": (ctypes.c_int, [_H, _fp, _fp, ctypes.c_int, _fp, _fp]),
    "sed_sur_last_error": (ctypes.c_char_p, [_H]),
    "sed_sur_set_tensor_cores": (ctypes.c_int, [_H, ctypes.c_int]),
    "sed_sur_set_stream": (ctypes.c_int, [_H, _vp]),
    "sed_sur_destroy": (None, [_H]),
    "sed_sur_set_norm": (ctypes.c_int, [_H, _fp, ctypes.c_int]),
    "sed_step_surrogate": (ctypes.c_int, [_H, _H, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double,
                                          ctypes.POINTER(SedStats)]),
    "sed_ode_solver_surrogate": (ctypes.c_int, [_H, _H, _dp, _dp, _dp, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_double,
                                                ctypes.POINTER(SedStats)]),
    "sed_sur_collect": (ctypes.c_int, [_H, _fp, ctypes.c_double, _vp, _vp, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_longlong,
                                       ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(SedStats)]),
    "sed_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "sed_last_error": (ctypes.c_char_p, [_H]),
    "sed_tracer_name": (ctypes.c_char_p, [ctypes.c_int]),
    "sed_tracer_is_particulate": (ctypes.c_int, [ctypes.c_int]),
    "sed_destroy": (None, [_H]),
}

_lib = None


def header_functions() -> list:
    """Function names declared in include/mossco_sed.h."""
    path = os.path.join(_build.INCLUDE, "mossco_sed.h")
    text = open(path).read()
    return sorted(set(re.findall(r"\b(sed_[a-z_0-9]+)\s*\(", text)))


def load(build: bool = True):
    """Load libsedgpu.so (building it first when sources changed)."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB_PATH
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray], ptype=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(ptype)


def default_params() -> SedParams:
    p = SedParams()
    rc = load().sed_default_params(ctypes.byref(p))
    if rc != SED_OK:
        raise SedError(rc, "sed_default_params")
    return p


def params_from(cs: ColumnSet, precision: int = SED_FP32, budgets: bool = False,
                cut_scope: int = SED_CUT_PER_COLUMN, epilogue: bool = True,
                device: int = 0) -> SedParams:
    """sed_params for a ColumnSet (driver + OMEXDIA+P parameters)."""
    p = default_params()
    d = cs.driver
    p.diffusivity = d.diffusivity
    p.bioturbation = d.bioturbation
    p.bcup_dissolved = d.bcup_dissolved
    p.bcup_particulate = d.bcup_particulate
    p.mol_diff_mode = d.mol_diff_mode
    p.mol_diff_d0 = d.mol_diff_d0
    p.dt_min = d.dt_min
    p.relative_change_min = d.relative_change_min
    p.atol = d.atol
    p.max_attempts = int(d.max_attempts)
    p.cut_scope = cut_scope
    for n in BGC_NAMES:
        setattr(p, n, float(cs.bgc[n]))
    p.epilogue = int(epilogue)
    mins = d.minimum_array()
    for i in range(NTR):
        p.minimum[i] = float(mins[i])
    p.precision = precision
    p.budgets = int(budgets)
    p.device = device
    p.bioturbation_profile = int(d.bioturbation_profile)
    for n in ("bioturb_k_l", "bioturb_L1", "bioturb_L2", "bioturb_beta", "bioturb_b",
              "bioturb_dry_density"):
        setattr(p, n, float(getattr(d, n)))
    p.temp_activation = float(getattr(d, "temp_activation", 0.0))
    p.adaptive_solver_diagnostics = int(bool(getattr(d, "adaptive_solver_diagnostics", False)))
    return p


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Solver:
    """One library handle over a ColumnSet's grid."""

    def __init__(self, cs: ColumnSet, precision: int = SED_FP32,
                 budgets: bool = False, cut_scope: int = SED_CUT_PER_COLUMN,
                 epilogue: bool = True, params: Optional[SedParams] = None):
        self.lib = load()
        self.cs = cs
        self.params = params or params_from(cs, precision, budgets, cut_scope,
                                            epilogue)
        h = _H()
        rc = self.lib.sed_create(ctypes.byref(self.params), cs.inum, cs.jnum,
                                 cs.kmax, NTR, ctypes.byref(h))
        if rc != SED_OK:
            raise SedError(rc, "sed_create: " +
                           self.lib.sed_error_string(rc).decode())
        self.h = h
        self._keep = {}
        self._check(self.lib.sed_set_grid(
            h, _p(_f64(cs.dz)), _p(_f64(cs.dzc)), _p(_f64(cs.phi)),
            _p(_f64(cs.phi_i)), _p(_f64(cs.biofac)),
            _p(_f64(cs.flux_cap)),
            _p(np.ascontiguousarray(cs.kact, dtype=np.int32), _ip), None),
            "sed_set_grid")
        if cs.bgc_col is not None:
            self.set_column_bgc(cs.bgc_col)

    def set_column_bgc(self, params: Optional[np.ndarray]):
        """An OMEXDIA+P parameter set per column, [SED_NBGC][ncol] in
        BGC_NAMES order (per-day units), or None for the handle's set."""
        a = None if params is None else _f64(params)
        if a is not None and a.shape != (len(BGC_NAMES), self.cs.ncol):
            raise ValueError(f"params must be [{len(BGC_NAMES)}][{self.cs.ncol}]")
        self._check(self.lib.sed_set_column_bgc(self.h, _p(a)), "sed_set_column_bgc")

    def _check(self, rc: int, what: str):
        if rc != SED_OK:
            msg = self.lib.sed_last_error(self.h).decode()
            raise SedError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.sed_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state / forcing -------------------------------------------------
    def set_forcing(self, bdys=None, fluxes=None):
        cs = self.cs
        b = _f64(cs.bdys if bdys is None else bdys)
        f = _f64(cs.fluxes if fluxes is None else fluxes)
        self._check(self.lib.sed_set_forcing(self.h, _p(b), _p(f)),
                    "sed_set_forcing")

    def set_boundary(self, temperature, surface, velocity=None, present=None):
        """get_boundary_conditions on the device from pelagic surface fields."""
        pr = None if present is None else np.ascontiguousarray(present, dtype=np.int32)
        self._check(self.lib.sed_set_boundary(
            self.h, _p(_f64(temperature)), _p(_f64(surface)),
            None if velocity is None else _p(_f64(velocity)),
            None if pr is None else _p(pr, _ip)), "sed_set_boundary")

    def boundary(self):
        cs = self.cs
        bd = np.zeros((NTR + 1, cs.ncol))
        fl = np.zeros((NTR, cs.ncol))
        self._check(self.lib.sed_get_boundary(self.h, _p(bd), _p(fl)), "sed_get_boundary")
        return bd, fl

    def set_state(self, conc):
        c = _f64(conc)
        self._check(self.lib.sed_set_state(self.h, _p(c)), "sed_set_state")

    def get_state(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        cs = self.cs
        if out is None:
            out = np.array(cs.conc, dtype=np.float64, copy=True)
        self._check(self.lib.sed_get_state(self.h, _p(out)), "sed_get_state")
        return out

    # -- stepping ------------------------------------------------------------
    def step(self, nsteps: int = 1, dt: Optional[float] = None,
             method: int = 2, raise_on_error: bool = True):
        st = SedStats()
        dt = self.cs.dt if dt is None else dt
        rc = self.lib.sed_step(self.h, float(dt), int(method), int(nsteps),
                               ctypes.byref(st))
        if raise_on_error:
            self._check(rc, "sed_step")
            return st.as_dict()
        return rc, st.as_dict()

    def spinup(self, nsteps: int, mode: int = SED_SPINUP_COLUMN, column: int = -1,
               bdys1=None, fluxes1=None, dt: Optional[float] = None, method: int = 2) -> dict:
        """sed_spinup: nsteps coupling steps of the 1-column model (then its
        profile copied into every column) or of every column."""
        st = SedStats()
        dt = self.cs.dt if dt is None else dt
        b1 = None if bdys1 is None else _f64(bdys1)
        f1 = None if fluxes1 is None else _f64(fluxes1)
        self._check(self.lib.sed_spinup(self.h, int(mode), int(column),
                                        None if b1 is None else _p(b1),
                                        None if f1 is None else _p(f1), float(dt),
                                        int(method), int(nsteps), ctypes.byref(st)),
                    "sed_spinup")
        return st.as_dict()

    def ode_solver(self, conc: np.ndarray, bdys: np.ndarray,
                   fluxes: np.ndarray, dt: float, method: int = 2,
                   raise_on_error: bool = True):
        """Drop-in for `call ode_solver(sed, dt, method)` + epilogue on host
        arrays (conc and fluxes updated in place)."""
        assert conc.dtype == np.float64 and conc.flags.c_contiguous
        assert fluxes.dtype == np.float64 and fluxes.flags.c_contiguous
        b = _f64(bdys)
        st = SedStats()
        rc = self.lib.sed_ode_solver(self.h, _p(conc), _p(b), _p(fluxes),
                                     float(dt), int(method), ctypes.byref(st))
        if raise_on_error:
            self._check(rc, "sed_ode_solver")
            return st.as_dict()
        return rc, st.as_dict()

    def get_rhs(self, conc: np.ndarray, fluxes: Optional[np.ndarray] = None):
        cs = self.cs
        c = _f64(conc)
        rhs = np.zeros_like(c)
        fl = np.array(cs.fluxes if fluxes is None else fluxes,
                      dtype=np.float64, copy=True)
        self._check(self.lib.sed_get_rhs(self.h, _p(c), _p(rhs), _p(fl)),
                    "sed_get_rhs")
        return rhs, fl

    def set_stream(self, stream_handle: int) -> None:
        """Use a caller's CUDA stream (e.g. torch.cuda.Stream().cuda_stream)."""
        self._check(self.lib.sed_set_stream(self.h, ctypes.c_void_p(stream_handle)),
                    "sed_set_stream")

    # -- launch tuning ----------------------------------------------------
    def tuning(self) -> SedTuning:
        t = SedTuning()
        self._check(self.lib.sed_get_tuning(self.h, ctypes.byref(t)), "sed_get_tuning")
        return t

    def set_tuning(self, t: SedTuning = None, **fields) -> None:
        """Apply a tuning; keyword fields (tile_columns=(32, 16), ...) edit
        the current one."""
        t = t if t is not None else self.tuning()
        for k, v in fields.items():
            if isinstance(getattr(t, k), ctypes.Array):
                getattr(t, k)[:] = list(v)
            else:
                setattr(t, k, v)
        self._check(self.lib.sed_set_tuning(self.h, ctypes.byref(t)), "sed_set_tuning")

    def autotune(self, dt: Optional[float] = None, method: int = 2,
                 flags: int = 0) -> dict:
        t = SedTuning()
        dt = self.cs.dt if dt is None else dt
        self._check(self.lib.sed_autotune(self.h, float(dt), int(method), int(flags),
                                          ctypes.byref(t)), "sed_autotune")
        return t.as_dict()

    def fluxes(self) -> np.ndarray:
        out = np.array(self.cs.fluxes, dtype=np.float64, copy=True)
        self._check(self.lib.sed_get_fluxes(self.h, _p(out)), "sed_get_fluxes")
        return out

    def attempts(self) -> np.ndarray:
        out = np.zeros(self.cs.ncol, dtype=np.int32)
        self._check(self.lib.sed_get_attempts(self.h, _p(out, _ip)),
                    "sed_get_attempts")
        return out

    def attempt_histogram(self) -> np.ndarray:
        """Substep histogram of the last step (sed_get_attempt_histogram):
        [SED_HIST_BINS] column counts, bin 0 without an attempt, bin b the
        columns with 2^(b-1) <= attempts < 2^b, the last bin all above."""
        out = np.zeros(SED_HIST_BINS, dtype=np.int64)
        self._check(self.lib.sed_get_attempt_histogram(
            self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))),
            "sed_get_attempt_histogram")
        return out

    def min_dt(self) -> np.ndarray:
        """Smallest accepted substep of every column in the last step (s)."""
        out = np.zeros(self.cs.ncol)
        self._check(self.lib.sed_get_min_dt(self.h, _p(out)), "sed_get_min_dt")
        return out

    def min_dt_grid_cell(self):
        """type_rhs_driver's last_min_dt and last_min_dt_grid_cell (i, j, k, n),
        1-based, of the grid-wide cut with adaptive_solver_diagnostics."""
        v = ctypes.c_double(0.0)
        cell = (ctypes.c_int * 4)()
        self._check(self.lib.sed_get_min_dt_grid_cell(self.h, ctypes.byref(v), cell),
                    "sed_get_min_dt_grid_cell")
        return v.value, tuple(cell)

    def budgets(self) -> np.ndarray:
        out = np.zeros((4, self.cs.ncol))
        self._check(self.lib.sed_get_budgets(self.h, _p(out)),
                    "sed_get_budgets")
        return out


def host_register(a: np.ndarray) -> None:
    rc = load().sed_host_register(a.ctypes.data, a.nbytes)
    if rc != SED_OK:
        raise SedError(rc, "sed_host_register")


def host_unregister(a: np.ndarray) -> None:
    load().sed_host_unregister(a.ctypes.data)


def host_empty(shape, dtype=np.float64) -> np.ndarray:
    """An uninitialised numpy array in pinned host memory (sed_host_alloc),
    freed with sed_host_free when the array and its views are gone."""
    import weakref
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    lib = load()
    p = _vp()
    rc = lib.sed_host_alloc(max(n, 1), ctypes.byref(p))
    if rc != SED_OK:
        raise SedError(rc, "sed_host_alloc")
    buf = (ctypes.c_char * max(n, 1)).from_address(p.value)
    a = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)
    weakref.finalize(buf, lib.sed_host_free, ctypes.c_void_p(p.value))
    return a
