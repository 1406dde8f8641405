"""ctypes front end of the FP64 CPU oracle of the pelagic path (pel_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
compare against and by bench.py's CPU-baseline leg of the pelagic line.  The
product (the CUDA library under mossco-code_gb300/) never imports it.

Parity status: the stepper, light, Run loop and clip follow the reference
source (src/utilities/solver_library.F90:80-189,
src/drivers/fabm_pelagic_driver.F90:380-417,774-814,910-927,
src/components/fabm_pelagic_component.F90:1931,2061-2240); the gotm_npzd
rates restate the published GOTM NPZD model and are UNPINNED (FABM is not
in the reference tree).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpeloracle.so")
SRC = os.path.join(HERE, "pel_oracle.c")
SRCS = [SRC, os.path.join(HERE, "cpl_oracle.c")]

_PKG = os.path.join(os.path.dirname(HERE), "mossco-code_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
from sedgpu.pelagic import NPZD_NAMES, PelColumnSet  # noqa: E402

# pelagic_soil_connector's namelist and looked-up fields (cpl_oracle.h)
CPL_PARAM_NAMES = ("sinking_factor", "sinking_factor_min", "NC_ldet", "NC_sdet", "convertN",
                   "convertP", "half_sedimentation_depth", "half_sedimentation_tke",
                   "critical_detritus")
CPL_FIELD_NAMES = ("detN", "detC", "detP", "din", "nitrate", "ammonium", "oxygen", "odu")

CFLAGS = ["-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
          "-ffp-contract=off", "-fno-math-errno"]


def build(force: bool = False) -> str:
    """Compile the pelagic and connector oracles with gcc into oracle/_build."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = SRCS + [os.path.join(HERE, h) for h in ("pel_oracle.h", "cpl_oracle.h")]
    if (not force and os.path.exists(LIB_PATH)
            and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *CFLAGS, *SRCS, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_dp = ctypes.POINTER(ctypes.c_double)


class Npzd(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in NPZD_NAMES]


class Pel(ctypes.Structure):
    _fields_ = [("ncol", ctypes.c_int), ("knum", ctypes.c_int),
                ("layer_height", _dp), ("mask", ctypes.POINTER(ctypes.c_ubyte)),
                ("I_0", _dp), ("albedo", _dp), ("bottom_flux", _dp),
                ("surface_flux", _dp), ("soil_flux", _dp), ("minimum", _dp),
                ("background_extinction", ctypes.c_double),
                ("dt_min", ctypes.c_double), ("relative_change_min", ctypes.c_double),
                ("atol", ctypes.c_double), ("max_attempts", ctypes.c_long),
                ("cut_scope", ctypes.c_int), ("bgc", Npzd),
                ("open_boundary", ctypes.POINTER(ctypes.c_ubyte)), ("boundary_value", _dp),
                ("has_boundary_value", ctypes.POINTER(ctypes.c_int))]


class PelStats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_long), ("accepted", ctypes.c_long),
                ("max_cell_attempts", ctypes.c_long), ("min_dt", ctypes.c_double),
                ("capped", ctypes.c_int), ("nan_cells", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class OrcCpl(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in CPL_PARAM_NAMES] + [("as_named", ctypes.c_int)]


class OrcCplFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in CPL_FIELD_NAMES]


CPL_SOIL_PARAM_NAMES = ("dinflux_const", "dipflux_const", "NC_ldet", "NC_sdet", "convertN",
                        "convertP")
CPL_SOIL_FIELD_NAMES = ("nitrate", "ammonium", "din", "dip", "oxygen", "odu", "detN", "detC",
                        "detP")


class OrcCplSoil(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in CPL_SOIL_PARAM_NAMES]


class OrcCplSoilFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in CPL_SOIL_FIELD_NAMES]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P = ctypes.POINTER
        L.orc_pel_exp.argtypes = [ctypes.c_double]
        L.orc_pel_exp.restype = ctypes.c_double
        L.orc_npzd_rates.argtypes = [P(Npzd), _dp, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_pel_light.argtypes = [P(Pel), _dp, _dp]
        L.orc_pel_get_rhs.argtypes = [P(Pel), _dp, _dp, _dp]
        L.orc_pel_ode_solver.argtypes = [P(Pel), _dp, _dp, ctypes.c_double, ctypes.c_int,
                                         P(PelStats)]
        L.orc_pel_ode_solver.restype = ctypes.c_int
        L.orc_pel_run.argtypes = [P(Pel), _dp, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, P(PelStats), _dp, ctypes.c_int]
        L.orc_pel_run.restype = ctypes.c_int
        L.orc_cpl_defaults.argtypes = [P(OrcCpl)]
        L.orc_cpl_defaults.restype = None
        L.orc_cpl_run.argtypes = [P(OrcCpl), P(OrcCplFields), _dp, ctypes.c_int, ctypes.c_int,
                                  _dp, _dp, _dp, _dp, P(ctypes.c_int)]
        L.orc_cpl_run.restype = ctypes.c_int
        L.orc_cpl_soil_defaults.argtypes = [P(OrcCplSoil)]
        L.orc_cpl_soil_defaults.restype = None
        L.orc_cpl_soil_run.argtypes = [P(OrcCplSoil), P(OrcCplSoilFields), _dp, ctypes.c_int,
                                       ctypes.c_int, _dp, P(ctypes.c_int)]
        L.orc_cpl_soil_run.restype = None
        _lib = L
    return _lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_dp)


def npzd_struct(npzd: dict) -> Npzd:
    """Parameters with the per-day rates divided by 86400."""
    day = 86400.0
    b = Npzd()
    for n in NPZD_NAMES:
        v = float(npzd[n])
        if n in ("rmax", "gmax", "rpn", "rzn", "rdn", "rpdu", "rpdl", "rzd"):
            v = v / day
        setattr(b, n, v)
    # the device squares Iv once; the oracle squares it in the rate (same bits)
    return b


def pel_exp(x: float) -> float:
    return lib().orc_pel_exp(float(x))


class PelOracle:
    """Keeps the numpy arrays behind an orc_pel alive."""

    def __init__(self, pcs: PelColumnSet, cut_scope: int = 0, open_boundary=None,
                 boundary_value=None):
        """open_boundary [ncol] (nonzero: an open-boundary column) and
        boundary_value [ntr][ncol] with NaN rows for tracers without a
        <name>_boundary_value_hz field (fabm_pelagic_component.F90
        :2115-2155); None: no open boundary."""
        self.pcs = pcs
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        self._keep = dict(
            h=f(pcs.layer_height), I0=f(pcs.I_0), alb=f(pcs.albedo),
            bfl=f(pcs.bottom_flux), sfl=f(pcs.surface_flux), soil=f(pcs.soil_flux),
            minimum=f(pcs.minimum),
            mask=None if pcs.mask is None else np.ascontiguousarray(pcs.mask > 0, dtype=np.uint8))
        k = self._keep
        m = Pel()
        m.ncol, m.knum = pcs.ncol, pcs.knum
        m.layer_height = _ptr(k["h"])
        m.mask = None if k["mask"] is None else k["mask"].ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))
        m.I_0, m.albedo = _ptr(k["I0"]), _ptr(k["alb"])
        m.bottom_flux, m.surface_flux, m.soil_flux = _ptr(k["bfl"]), _ptr(k["sfl"]), _ptr(k["soil"])
        m.minimum = _ptr(k["minimum"])
        m.background_extinction = pcs.background_extinction
        m.dt_min, m.relative_change_min, m.atol = pcs.dt_min, pcs.relative_change_min, pcs.atol
        m.max_attempts = int(pcs.max_attempts)
        m.cut_scope = cut_scope
        m.bgc = npzd_struct(pcs.npzd)
        if open_boundary is not None:
            bv = np.ascontiguousarray(boundary_value, dtype=np.float64)
            has = np.ascontiguousarray(~np.isnan(bv).all(axis=1), dtype=np.int32)
            ob = np.ascontiguousarray(np.asarray(open_boundary) != 0, dtype=np.uint8)
            k.update(ob=ob, bv=np.nan_to_num(bv), has=has)
            m.open_boundary = k["ob"].ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))
            m.boundary_value = _ptr(k["bv"])
            m.has_boundary_value = k["has"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self.m = m

    def light(self, conc: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(conc, dtype=np.float64)
        par = np.empty((self.pcs.knum, self.pcs.ncol))
        lib().orc_pel_light(ctypes.byref(self.m), _ptr(c), _ptr(par))
        return par

    def get_rhs(self, conc: np.ndarray, par: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(conc, dtype=np.float64)
        rhs = np.empty_like(c)
        lib().orc_pel_get_rhs(ctypes.byref(self.m), _ptr(c), _ptr(np.ascontiguousarray(par)),
                              _ptr(rhs))
        return rhs

    def ode_solver(self, conc: np.ndarray, par: np.ndarray, dt: float, method: int):
        """In place on conc; returns (status, stats)."""
        assert conc.dtype == np.float64 and conc.flags.c_contiguous
        st = PelStats()
        st.min_dt = np.inf
        rc = lib().orc_pel_ode_solver(ctypes.byref(self.m), _ptr(conc),
                                      _ptr(np.ascontiguousarray(par)), dt, method,
                                      ctypes.byref(st))
        return rc, st.as_dict()

    def run(self, conc: np.ndarray, t_couple: Optional[float] = None,
            dt: Optional[float] = None, method: Optional[int] = None,
            nthreads: int = 0, nruns: int = 1):
        """nruns Runs in place on conc; returns (status, statistics over the
        Runs, PAR of the last Run)."""
        assert conc.dtype == np.float64 and conc.flags.c_contiguous
        pcs = self.pcs
        par = np.empty((pcs.knum, pcs.ncol))
        tot = None
        rc = 0
        for _ in range(nruns):
            st = PelStats()
            rc = lib().orc_pel_run(ctypes.byref(self.m), _ptr(conc),
                                   pcs.t_couple if t_couple is None else t_couple,
                                   pcs.dt if dt is None else dt,
                                   pcs.method if method is None else method,
                                   ctypes.byref(st), _ptr(par), nthreads)
            d = st.as_dict()
            if tot is None:
                tot = d
            else:
                for k in ("attempts", "accepted", "nan_cells"):
                    tot[k] += d[k]
                tot["max_cell_attempts"] = max(tot["max_cell_attempts"], d["max_cell_attempts"])
                tot["min_dt"] = min(tot["min_dt"], d["min_dt"])
                tot["capped"] = max(tot["capped"], d["capped"])
            if rc:
                break
        return rc, tot, par


def cpl_defaults() -> dict:
    p = OrcCpl()
    lib().orc_cpl_defaults(ctypes.byref(p))
    return {n: getattr(p, n) for n in CPL_PARAM_NAMES}


def cpl_run(conc: np.ndarray, fields: dict, params: Optional[dict] = None,
            as_named: bool = False, depth=None, tke=None, velocity_in=None):
    """One pelagic_soil_connector Run on the pelagic state conc [ntr][knum][ncol].

    Returns (rc, surface [11][ncol], velocity [11][ncol], present [11]); the
    soil fields start at zero (velocity at velocity_in's particulate rows)."""
    conc = np.ascontiguousarray(conc, dtype=np.float64)
    ntr, knum, ncol = conc.shape
    p = OrcCpl()
    lib().orc_cpl_defaults(ctypes.byref(p))
    for k, v in (params or {}).items():
        setattr(p, k, float(v))
    p.as_named = int(bool(as_named))
    f = OrcCplFields(*[int(fields.get(n, -1)) for n in CPL_FIELD_NAMES])
    surface = np.zeros((11, ncol))
    velocity = np.zeros((11, ncol))
    if velocity_in is not None:
        velocity[:6] = np.asarray(velocity_in, dtype=np.float64)[:6]
    present = np.zeros(11, dtype=np.int32)
    f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    d, t = f64(depth), f64(tke)
    rc = lib().orc_cpl_run(ctypes.byref(p), ctypes.byref(f), _ptr(conc), ncol, knum, _ptr(d),
                           _ptr(t), _ptr(surface), _ptr(velocity),
                           present.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return rc, surface, velocity, present


def cpl_soil_defaults() -> dict:
    p = OrcCplSoil()
    lib().orc_cpl_soil_defaults(ctypes.byref(p))
    return {n: getattr(p, n) for n in CPL_SOIL_PARAM_NAMES}


def cpl_soil_run(fluxes: np.ndarray, fields: dict, params: Optional[dict] = None,
                 bfl_in: Optional[np.ndarray] = None, ntr: int = 4):
    """One soil_pelagic_connector Run on the sediment fluxes [11][ncol]
    (downward positive).  Returns (bfl [ntr][ncol], present [ntr]); rows the
    Run does not write keep bfl_in (zeros by default)."""
    fl = np.ascontiguousarray(fluxes, dtype=np.float64)
    ncol = fl.shape[1]
    p = OrcCplSoil()
    lib().orc_cpl_soil_defaults(ctypes.byref(p))
    for k, v in (params or {}).items():
        setattr(p, k, float(v))
    f = OrcCplSoilFields(*[int(fields.get(n, -1)) for n in CPL_SOIL_FIELD_NAMES])
    bfl = np.zeros((ntr, ncol)) if bfl_in is None else np.array(bfl_in, dtype=np.float64)
    present = np.zeros(ntr, dtype=np.int32)
    lib().orc_cpl_soil_run(ctypes.byref(p), ctypes.byref(f), _ptr(fl), ncol, ntr, _ptr(bfl),
                           present.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return bfl, present
