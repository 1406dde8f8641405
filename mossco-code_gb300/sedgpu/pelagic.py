"""The pelagic driver path: ctypes binding of include/mossco_pel.h, the
seeded synthetic water-column workloads, and a host-side mirror of the
reference's fabm_pelagic driver names.

MOSSCO's fabm_pelagic driver (src/drivers/fabm_pelagic_driver.F90) computes
light once per Run of its component (:774-814, called at
src/components/fabm_pelagic_component.F90:1931) and a purely local
right-hand side (:380-417) that solver_library's ode_solver integrates
over the component's internal steps (:2061-2081), each followed by the
soil-surface fluxes, the external flux fields and clip_below_minimum.  The
FABM model is gotm_npzd, the one the reference's pelagic set-ups select
(examples/fabmsed_fabm0d/fabm.nml:8).

The library is the only compute path: :class:`PelagicSolver` raises if it
cannot be loaded or no GPU is present.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Dict, Optional

import numpy as np

from . import capi
from .capi import SED_FP32, SED_OK, SedError
from .model import ADAPTIVE_EULER, EULER, RUNGE_KUTTA_4, RUNGE_KUTTA_4_38
from .synth import normal, uniform

PEL_NTR = 4
PEL_TRACERS = ("nutrient", "phytoplankton", "zooplankton", "detritus")
PEL_CUT_PER_CELL, PEL_CUT_GLOBAL = 0, 1
PEL_KMAX_LIMIT = 4096

NPZD_NAMES = ("p0", "z0", "kc", "I_min", "rmax", "gmax", "Iv", "alpha", "rpn",
              "rzn", "rdn", "rpdu", "rpdl", "rzd")
# &gotm_npzd of examples/fabmsed_fabm0d/fabm.nml:57-79 (rates per day)
NPZD_DEFAULTS = dict(p0=0.0225, z0=0.0225, kc=0.03, I_min=25.0, rmax=1.0,
                     gmax=0.2, Iv=1.1, alpha=1.35, rpn=0.01, rzn=0.01, rdn=0.01,
                     rpdu=0.02, rpdl=0.1, rzd=0.02)
# n_initial, p_initial, z_initial, d_initial of the same namelist
NPZD_INITIAL = (4.5, 1.0e-15, 1.0e-15, 4.5)

__all__ = ["PEL_NTR", "PEL_TRACERS", "PEL_CUT_PER_CELL", "PEL_CUT_GLOBAL",
           "NPZD_DEFAULTS", "PelColumnSet", "PelagicSolver",
           "make_pelagic_workload", "TypePelagic", "EULER", "RUNGE_KUTTA_4",
           "ADAPTIVE_EULER", "RUNGE_KUTTA_4_38"]


class PelParams(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_double) for n in NPZD_NAMES] +
                [("dt_min", ctypes.c_double),
                 ("relative_change_min", ctypes.c_double),
                 ("background_extinction", ctypes.c_double),
                 ("atol", ctypes.c_double),
                 ("max_attempts", ctypes.c_int), ("cut_scope", ctypes.c_int),
                 ("minimum", ctypes.c_double * PEL_NTR),
                 ("precision", ctypes.c_int), ("device", ctypes.c_int)])


class PelStats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_longlong), ("accepted", ctypes.c_longlong),
                ("column_steps", ctypes.c_longlong),
                ("max_cell_attempts", ctypes.c_int), ("capped_cells", ctypes.c_int),
                ("nan_cells", ctypes.c_int), ("gpu_launches", ctypes.c_int),
                ("min_dt", ctypes.c_double), ("device_ms", ctypes.c_double)]

    def as_dict(self) -> Dict[str, float]:
        return {n: getattr(self, n) for n, _ in self._fields_}


_H = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_d = ctypes.c_double
_i = ctypes.c_int

PEL_SIGNATURES = {
    "pel_default_params": (_i, [ctypes.POINTER(PelParams)]),
    "pel_create": (_i, [ctypes.POINTER(PelParams), _i, _i, _i, _i,
                        ctypes.POINTER(_H)]),
    "pel_destroy": (None, [_H]),
    "pel_last_error": (ctypes.c_char_p, [_H]),
    "pel_set_grid": (_i, [_H, _dp, _ip]),
    "pel_set_forcing": (_i, [_H, _dp, _dp, _dp, _dp, _dp]),
    "pel_set_open_boundary": (_i, [_H, _ip, _dp, _ip]),
    "pel_set_state": (_i, [_H, _dp]),
    "pel_get_state": (_i, [_H, _dp]),
    "pel_light": (_i, [_H, _dp, _dp]),
    "pel_get_rhs": (_i, [_H, _dp, _dp]),
    "pel_ode_solver": (_i, [_H, _dp, _d, _i, ctypes.POINTER(PelStats)]),
    "pel_run": (_i, [_H, _dp, _d, _d, _i, ctypes.POINTER(PelStats)]),
    "pel_step": (_i, [_H, _d, _d, _i, _i, ctypes.POINTER(PelStats)]),
}

_registered = False


def load(build: bool = True):
    """libsedgpu.so with the pelagic entry points typed."""
    global _registered
    L = capi.load(build)
    if not _registered:
        for name, (res, args) in PEL_SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _registered = True
    return L


def _p(a: Optional[np.ndarray], ptype=_dp):
    return None if a is None else a.ctypes.data_as(ptype)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def default_params() -> PelParams:
    p = PelParams()
    if load().pel_default_params(ctypes.byref(p)) != SED_OK:
        raise SedError(-1, "pel_default_params")
    return p


@dataclasses.dataclass
class PelColumnSet:
    """A grid of water columns with the pelagic state and forcing.

    Shapes (C order, the reference's Fortran order read backwards):
      layer_height, mask [knum][ncol]    k = 0 bottom, knum-1 surface
      I_0, albedo        [ncol]
      bottom_flux, surface_flux, soil_flux  [4][ncol]  (mmol/m2/s)
      conc               [4][knum][ncol] (mmol N/m3: n, p, z, d)
    """
    inum: int
    jnum: int
    knum: int
    layer_height: np.ndarray
    conc: np.ndarray
    I_0: np.ndarray
    mask: Optional[np.ndarray] = None
    albedo: Optional[np.ndarray] = None
    bottom_flux: Optional[np.ndarray] = None
    surface_flux: Optional[np.ndarray] = None
    soil_flux: Optional[np.ndarray] = None
    npzd: Dict[str, float] = dataclasses.field(default_factory=lambda: dict(NPZD_DEFAULTS))
    dt_min: float = 1.0e-8
    relative_change_min: float = -0.9
    background_extinction: float = 1.0 / 7.9
    atol: float = 0.0
    max_attempts: int = 4096
    minimum: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(PEL_NTR))
    t_couple: float = 3600.0
    dt: float = 360.0
    method: int = RUNGE_KUTTA_4
    nruns: int = 24
    seed: int = 0

    @property
    def ncol(self) -> int:
        return self.inum * self.jnum

    def water(self) -> np.ndarray:
        """[knum][ncol] True for water (unmasked) cells."""
        if self.mask is None:
            return np.ones((self.knum, self.ncol), dtype=bool)
        return self.mask <= 0

    def water_columns(self) -> int:
        return int(self.water().any(axis=0).sum())

    def copy(self) -> "PelColumnSet":
        out = dataclasses.replace(self)
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, np.ndarray):
                setattr(out, f.name, v.copy())
            elif isinstance(v, dict):
                setattr(out, f.name, dict(v))
        return out

    def subset(self, cols) -> "PelColumnSet":
        """The columns ``cols`` as a 1 x len(cols) grid (copies)."""
        cols = np.asarray(cols, dtype=np.int64)
        out = self.copy()
        out.inum, out.jnum = len(cols), 1
        for name in ("layer_height", "mask"):
            v = getattr(self, name)
            if v is not None:
                setattr(out, name, np.ascontiguousarray(v[:, cols]))
        for name in ("I_0", "albedo"):
            v = getattr(self, name)
            if v is not None:
                setattr(out, name, np.ascontiguousarray(v[cols]))
        for name in ("bottom_flux", "surface_flux", "soil_flux"):
            v = getattr(self, name)
            if v is not None:
                setattr(out, name, np.ascontiguousarray(v[:, cols]))
        out.conc = np.ascontiguousarray(self.conc[:, :, cols])
        return out

    def params(self, precision: int = SED_FP32,
               cut_scope: int = PEL_CUT_PER_CELL) -> PelParams:
        p = default_params()
        for n in NPZD_NAMES:
            setattr(p, n, float(self.npzd[n]))
        p.dt_min = self.dt_min
        p.relative_change_min = self.relative_change_min
        p.background_extinction = self.background_extinction
        p.atol = self.atol
        p.max_attempts = int(self.max_attempts)
        p.cut_scope = cut_scope
        for n in range(PEL_NTR):
            p.minimum[n] = float(self.minimum[n])
        p.precision = precision
        return p

    def inventory(self, conc: Optional[np.ndarray] = None) -> np.ndarray:
        """Total nitrogen per column, sum over water cells of h * (n+p+z+d)."""
        c = self.conc if conc is None else conc
        w = self.water()
        return (np.where(w, self.layer_height, 0.0)[None] * np.where(w[None], c, 0.0)).sum(axis=(0, 1))


class PelagicSolver:
    """One pel_handle: grid, forcing and (optionally) device-resident state."""

    def __init__(self, pcs: PelColumnSet, precision: int = SED_FP32,
                 cut_scope: int = PEL_CUT_PER_CELL, params: Optional[PelParams] = None):
        self.lib = load()
        self.pcs = pcs
        self.params = params or pcs.params(precision, cut_scope)
        h = _H()
        rc = self.lib.pel_create(ctypes.byref(self.params), pcs.inum, pcs.jnum,
                                 pcs.knum, PEL_NTR, ctypes.byref(h))
        if rc != SED_OK:
            raise SedError(rc, "pel_create")
        self.h = h
        mask = None if pcs.mask is None else np.ascontiguousarray(pcs.mask, dtype=np.int32)
        self._check(self.lib.pel_set_grid(self.h, _p(_f64(pcs.layer_height)),
                                          _p(mask, _ip)), "pel_set_grid")
        self.set_forcing()

    def _check(self, rc: int, what: str):
        if rc != SED_OK:
            msg = self.lib.pel_last_error(self.h)
            raise SedError(rc, f"{what}: {msg.decode() if msg else ''}")

    def set_forcing(self, I_0=None, albedo=None, bottom_flux=None, surface_flux=None,
                    soil_flux=None):
        pcs = self.pcs
        arrs = [pcs.I_0 if I_0 is None else I_0,
                pcs.albedo if albedo is None else albedo,
                pcs.bottom_flux if bottom_flux is None else bottom_flux,
                pcs.surface_flux if surface_flux is None else surface_flux,
                pcs.soil_flux if soil_flux is None else soil_flux]
        arrs = [None if a is None else _f64(a) for a in arrs]
        self._check(self.lib.pel_set_forcing(self.h, *[_p(a) for a in arrs]),
                    "pel_set_forcing")

    def set_open_boundary(self, open_boundary=None, boundary_value=None, has_value=None):
        """Open-boundary values (fabm_pelagic_component.F90:2115-2155):
        open_boundary [ncol] (nonzero: open; None: none), boundary_value
        [ntr][ncol]; has_value [ntr] defaults to the tracers whose values
        are finite in every open column."""
        if open_boundary is None:
            self._check(self.lib.pel_set_open_boundary(self.h, None, None, None),
                        "pel_set_open_boundary")
            return
        ob = np.ascontiguousarray(np.asarray(open_boundary) != 0, dtype=np.int32)
        bv = _f64(boundary_value)
        if has_value is None:
            has_value = [bool(np.isfinite(bv[n, ob != 0]).all()) for n in range(PEL_NTR)]
        hv = np.ascontiguousarray(np.asarray(has_value) != 0, dtype=np.int32)
        bv = np.where(np.isfinite(bv), bv, 0.0)   # rows without a value are not read
        self._check(self.lib.pel_set_open_boundary(self.h, _p(ob, _ip), _p(_f64(bv)),
                                                   _p(hv, _ip)), "pel_set_open_boundary")

    def set_state(self, conc):
        self._check(self.lib.pel_set_state(self.h, _p(_f64(conc))), "pel_set_state")

    def get_state(self) -> np.ndarray:
        out = np.empty((PEL_NTR, self.pcs.knum, self.pcs.ncol))
        self._check(self.lib.pel_get_state(self.h, _p(out)), "pel_get_state")
        return out

    def light(self, conc=None) -> np.ndarray:
        par = np.empty((self.pcs.knum, self.pcs.ncol))
        c = None if conc is None else _f64(conc)
        self._check(self.lib.pel_light(self.h, _p(c), _p(par)), "pel_light")
        return par

    def get_rhs(self, conc) -> np.ndarray:
        c = _f64(conc)
        rhs = np.empty_like(c)
        self._check(self.lib.pel_get_rhs(self.h, _p(c), _p(rhs)), "pel_get_rhs")
        return rhs

    def ode_solver(self, conc: np.ndarray, dt: float, method: int) -> Dict[str, float]:
        """Drop-in `call ode_solver(pel, dt, method)` on a host array, in place."""
        assert conc.dtype == np.float64 and conc.flags.c_contiguous
        st = PelStats()
        self._check(self.lib.pel_ode_solver(self.h, _p(conc), dt, method, ctypes.byref(st)),
                    "pel_ode_solver")
        return st.as_dict()

    def run(self, conc: Optional[np.ndarray] = None, t_couple: Optional[float] = None,
            dt: Optional[float] = None, method: Optional[int] = None,
            raise_on_error: bool = True):
        """One Run on a host array (in place) or on the device state (None)."""
        pcs = self.pcs
        if conc is not None:
            assert conc.dtype == np.float64 and conc.flags.c_contiguous
        st = PelStats()
        rc = self.lib.pel_run(self.h, _p(conc), pcs.t_couple if t_couple is None else t_couple,
                              pcs.dt if dt is None else dt,
                              pcs.method if method is None else method, ctypes.byref(st))
        if raise_on_error:
            self._check(rc, "pel_run")
            return st.as_dict()
        return rc, st.as_dict()

    def step(self, nruns: int, t_couple: Optional[float] = None, dt: Optional[float] = None,
             method: Optional[int] = None) -> Dict[str, float]:
        pcs = self.pcs
        st = PelStats()
        self._check(self.lib.pel_step(self.h, pcs.t_couple if t_couple is None else t_couple,
                                      pcs.dt if dt is None else dt,
                                      pcs.method if method is None else method, nruns,
                                      ctypes.byref(st)), "pel_step")
        return st.as_dict()

    def close(self):
        if getattr(self, "h", None):
            self.lib.pel_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Seeded synthetic workloads (no data set is published for this path).

F_PLAND, F_DEPTH, F_I0, F_ALB, F_N, F_P, F_Z, F_D = 101, 102, 103, 104, 105, 106, 107, 108
F_BN, F_BD, F_SN, F_NOISE = 109, 110, 111, 112

PEL_WORKLOADS = {
    "pelagic_cpu_16x16": dict(inum=16, jnum=16, knum=20, land=0.2, nruns=24),
    "pelagic_1024x1024": dict(inum=1024, jnum=1024, knum=30, land=0.3, nruns=24),
}


def make_pelagic_workload(name: str, cols=None, seed: int = 0) -> PelColumnSet:
    """A GETM-like grid of water columns: land columns masked, water depth
    log-uniform 5..100 m split into knum equal sigma layers, surface PAR
    U[0,250] W/m2 (day and night), albedo U[0.05,0.1]; nutrient U[2,10],
    phytoplankton U[0.05,2] decaying with a 15 m depth scale below the
    surface, zooplankton U[0.02,0.5], detritus U[0.5,3.5] mmol N/m3, each
    with 1 % noise per cell; soil-surface upward fluxes of nutrient
    U[0,3] mmol/m2/d and of detritus -U[0,2] (deposition); atmospheric
    nutrient deposition U[0,0.2] mmol/m2/d at the surface.  The Run is the
    component's: 3600 s coupling, 360 s internal steps, RUNGE_KUTTA_4 (the
    component's default ode_method, fabm_pelagic_component.F90:50)."""
    w = PEL_WORKLOADS[name]
    inum, jnum, K = w["inum"], w["jnum"], w["knum"]
    n_all = inum * jnum
    gid = np.arange(n_all, dtype=np.int64) if cols is None else np.asarray(cols, dtype=np.int64)
    n = gid.size
    land = uniform(seed, F_PLAND, gid) < w["land"]
    H = np.exp(np.log(5.0) + uniform(seed, F_DEPTH, gid) * (np.log(100.0) - np.log(5.0)))
    h = np.repeat((H / K)[None, :], K, axis=0)
    mask = np.repeat(land[None, :].astype(np.int32), K, axis=0)
    I0 = 250.0 * uniform(seed, F_I0, gid)
    alb = 0.05 + 0.05 * uniform(seed, F_ALB, gid)
    zc = (np.arange(K)[:, None] + 0.5) * h          # height above the bottom
    depth = H[None, :] - zc                          # below the surface
    cell = gid[None, :] * K + np.arange(K)[:, None]
    noise = lambda f: 1.0 + 0.01 * normal(seed, F_NOISE + f, cell)  # noqa: E731
    conc = np.empty((PEL_NTR, K, n))
    conc[0] = (2.0 + 8.0 * uniform(seed, F_N, gid))[None, :] * noise(0)
    conc[1] = (0.05 + 1.95 * uniform(seed, F_P, gid))[None, :] * np.exp(-depth / 15.0) * noise(1)
    conc[2] = (0.02 + 0.48 * uniform(seed, F_Z, gid))[None, :] * noise(2)
    conc[3] = (0.5 + 3.0 * uniform(seed, F_D, gid))[None, :] * noise(3)
    conc[:, mask > 0] = 0.0
    day = 86400.0
    bfl = np.zeros((PEL_NTR, n))
    bfl[0] = 3.0 * uniform(seed, F_BN, gid) / day
    bfl[3] = -2.0 * uniform(seed, F_BD, gid) / day
    sfl = np.zeros((PEL_NTR, n))
    sfl[0] = 0.2 * uniform(seed, F_SN, gid) / day
    return PelColumnSet(inum=n if cols is not None else inum,
                        jnum=1 if cols is not None else jnum, knum=K,
                        layer_height=np.ascontiguousarray(h), conc=np.ascontiguousarray(conc),
                        I_0=I0, mask=np.ascontiguousarray(mask), albedo=alb,
                        bottom_flux=bfl, surface_flux=sfl, nruns=w["nruns"], seed=seed)


# ---------------------------------------------------------------------------
# Host-side mirror of type_mossco_fabm_pelagic (fabm_pelagic_driver.F90).

class TypePelagic:
    """The driver names a caller of the reference knows, on the GPU library:

        pf = TypePelagic(inum, jnum, knum)                 # mossco_create_fabm_pelagic
        pf.initialize_domain(zi, mask)                     # :215-293, update_grid :362-378
        pf.initialize_concentrations()                     # :295-304
        pf.light()                                         # :774-814
        rhs = pf.get_rhs()                                 # :380-417
        pf.ode_solver(dt, method)                          # solver_library ode_solver
        pf.clip_below_minimum()                            # :910-927

    conc is conc(i,j,k,n) as [n][k][col]; I_0, albedo and the flux fields
    are set as attributes before light() / a Run."""

    def __init__(self, inum: int, jnum: int, knum: int, precision: int = SED_FP32,
                 cut_scope: int = PEL_CUT_PER_CELL, npzd: Optional[dict] = None):
        self.inum, self.jnum, self.knum = inum, jnum, knum
        self.nvar = PEL_NTR
        self.npzd = dict(NPZD_DEFAULTS, **(npzd or {}))
        self.precision, self.cut_scope = precision, cut_scope
        self.dt_min, self.relative_change_min = 1.0e-8, -0.9
        self.background_extinction = 1.0 / 7.9
        self.minimum = np.zeros(PEL_NTR)
        self.layer_height = None
        self.mask = None
        self.conc = None
        self.par = None
        self.I_0 = np.zeros(inum * jnum)
        self.albedo = np.zeros(inum * jnum)
        self.bottom_flux = self.surface_flux = self.soil_flux = None
        self._solver: Optional[PelagicSolver] = None

    @property
    def ncol(self) -> int:
        return self.inum * self.jnum

    def initialize_domain(self, zi: np.ndarray, mask: Optional[np.ndarray] = None):
        """zi [knum+1][ncol] interface heights; layer_height(k) = zi(k+1) - zi(k)
        for water cells (update_grid :362-378)."""
        zi = np.asarray(zi, dtype=np.float64)
        self.mask = None if mask is None else np.asarray(mask, dtype=np.int32)
        lh = zi[1:] - zi[:-1]
        if self.mask is not None:
            lh = np.where(self.mask > 0, 0.0, lh)
        self.layer_height = np.ascontiguousarray(lh)
        self._solver = None

    def initialize_concentrations(self, initial=NPZD_INITIAL):
        """conc(:,:,:,n) = the model's initial value (:295-304)."""
        iv = np.asarray(initial, dtype=np.float64)
        self.conc = np.ascontiguousarray(np.broadcast_to(
            iv[:, None, None], (PEL_NTR, self.knum, self.ncol)).copy())

    def _pcs(self) -> PelColumnSet:
        return PelColumnSet(inum=self.inum, jnum=self.jnum, knum=self.knum,
                            layer_height=np.where(self.layer_height > 0, self.layer_height, 1.0),
                            conc=self.conc, I_0=self.I_0, mask=self.mask,
                            albedo=self.albedo, bottom_flux=self.bottom_flux,
                            surface_flux=self.surface_flux, soil_flux=self.soil_flux,
                            npzd=dict(self.npzd), dt_min=self.dt_min,
                            relative_change_min=self.relative_change_min,
                            background_extinction=self.background_extinction,
                            minimum=self.minimum)

    def solver(self) -> PelagicSolver:
        if self._solver is None:
            self._solver = PelagicSolver(self._pcs(), precision=self.precision,
                                         cut_scope=self.cut_scope)
        return self._solver

    def _refresh_forcing(self) -> PelagicSolver:
        """The current I_0, albedo and flux fields into the handle (this
        invalidates the handle's PAR)."""
        s = self.solver()
        s.pcs = self._pcs()
        s.set_forcing()
        return s

    def light(self) -> np.ndarray:
        self.par = self._refresh_forcing().light(self.conc)
        return self.par

    def get_rhs(self) -> np.ndarray:
        s = self.solver()
        if self.par is None:
            self.light()
        return s.get_rhs(self.conc)

    def ode_solver(self, dt: float, method: int) -> Dict[str, float]:
        s = self.solver()
        if self.par is None:
            self.light()
        return s.ode_solver(self.conc, dt, method)

    def run(self, t_couple: float, dt: float, method: int = RUNGE_KUTTA_4) -> Dict[str, float]:
        """The component's Run on conc: light, internal steps, epilogues."""
        st = self._refresh_forcing().run(self.conc, t_couple, dt, method)
        self.par = None
        return st

    def clip_below_minimum(self):
        """conc below the tracer's minimum set to it, water cells only
        (:910-927); a Run does this on the device after every step."""
        clipped = np.maximum(self.conc, self.minimum[:, None, None])
        if self.mask is not None:
            clipped = np.where((self.mask > 0)[None], self.conc, clipped)
        self.conc[...] = clipped
