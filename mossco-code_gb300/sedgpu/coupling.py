"""ctypes binding of include/mossco_cpl.h: the pelagic -> soil coupling.

MOSSCO couples its pelagic and soil components through the
pelagic_soil_connector (src/mediators/pelagic_soil_connector.F90), whose Run
maps the pelagic fields' bottom layer to the soil's "_at_soil_surface"
fields; the sediment component then turns these into bdys / fluxes
(get_boundary_conditions, src/components/fabm_sediment_component.F90
:1865-2030).  ``pelagic_soil`` does both on the device, from a
PelagicSolver's state into a Solver's boundary, with the mapping's
namelist as ``CplParams`` and the field lookup as ``CplFields``.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import Optional, Tuple

import numpy as np

from . import build as _build
from .capi import NTR, SED_OK, SedError, Solver, load as _load_sed
from .pelagic import PelagicSolver

CPL_AS_RUN = 0
CPL_AS_NAMED = 1

PARAM_NAMES = ("sinking_factor", "sinking_factor_min", "NC_ldet", "NC_sdet", "convertN",
               "convertP", "half_sedimentation_depth", "half_sedimentation_tke",
               "critical_detritus")
FIELD_NAMES = ("detN", "detC", "detP", "din", "nitrate", "ammonium", "oxygen", "odu", "dip")
SOIL_PARAM_NAMES = ("dinflux_const", "dipflux_const", "NC_ldet", "NC_sdet", "convertN",
                    "convertP")


class CplParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in PARAM_NAMES] + [("mode", ctypes.c_int)]


class CplFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in FIELD_NAMES]


class CplSoilParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in SOIL_PARAM_NAMES]


class CplStats(ctypes.Structure):
    _fields_ = [("gpu_launches", ctypes.c_int), ("columns", ctypes.c_longlong),
                ("kernel_ms", ctypes.c_double), ("device_ms", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_H = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

CPL_SIGNATURES = {
    "cpl_default_params": (ctypes.c_int, [ctypes.POINTER(CplParams)]),
    "cpl_npzd_fields": (ctypes.c_int, [ctypes.POINTER(CplFields)]),
    "cpl_pelagic_soil": (ctypes.c_int, [_H, _H, ctypes.POINTER(CplParams),
                                        ctypes.POINTER(CplFields), _dp, _dp, _dp, _dp, _dp,
                                        _dp, _ip, ctypes.POINTER(CplStats)]),
    "cpl_soil_default_params": (ctypes.c_int, [ctypes.POINTER(CplSoilParams)]),
    "cpl_soil_pelagic": (ctypes.c_int, [_H, _H, ctypes.POINTER(CplSoilParams),
                                        ctypes.POINTER(CplFields), _dp, _ip,
                                        ctypes.POINTER(CplStats)]),
}

_registered = False


def load(build: bool = True):
    """libsedgpu.so with the coupling entry points typed."""
    global _registered
    L = _load_sed(build)
    if not _registered:
        for name, (res, args) in CPL_SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _registered = True
    return L


def header_functions() -> list:
    """Function names declared in include/mossco_cpl.h."""
    text = open(os.path.join(_build.INCLUDE, "mossco_cpl.h")).read()
    return sorted(set(re.findall(r"\b(cpl_[a-z_0-9]+)\s*\(", text)))


def default_params(**overrides) -> CplParams:
    p = CplParams()
    if load().cpl_default_params(ctypes.byref(p)) != SED_OK:
        raise SedError(-1, "cpl_default_params")
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def npzd_fields(**overrides) -> CplFields:
    f = CplFields()
    if load().cpl_npzd_fields(ctypes.byref(f)) != SED_OK:
        raise SedError(-1, "cpl_npzd_fields")
    for k, v in overrides.items():
        setattr(f, k, v)
    return f


def soil_default_params(**overrides) -> CplSoilParams:
    p = CplSoilParams()
    if load().cpl_soil_default_params(ctypes.byref(p)) != SED_OK:
        raise SedError(-1, "cpl_soil_default_params")
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def pelagic_soil(pel: PelagicSolver, sed: Solver, temperature, water_depth=None, tke=None,
                 velocity_in=None, params: Optional[CplParams] = None,
                 fields: Optional[CplFields] = None, stats: Optional[CplStats] = None,
                 read_back: bool = True
                 ) -> Tuple[Optional[np.ndarray], Optional[np.ndarray], np.ndarray]:
    """One connector Run from ``pel``'s device state into ``sed``'s boundary.

    Returns the soil fields it wrote (host copies, None without
    ``read_back``): surface [NTR][ncol], velocity [NTR][ncol], and present
    [NTR] (1 where a concentration field was written).  ``stats``, when
    given, receives the call's launches and device times."""
    L = load()
    ncol = sed.cs.ncol
    p = params or default_params()
    f = fields or npzd_fields()
    t, d, k = _f64(temperature), _f64(water_depth), _f64(tke)
    v = _f64(velocity_in)
    for name, a in (("temperature", t), ("water_depth", d), ("tke", k)):
        if a is not None and a.size != ncol:
            raise ValueError(f"{name} must have {ncol} values")
    if v is not None and v.size < 6 * ncol:
        raise ValueError("velocity_in must hold the particulate rows [6][ncol]")
    surface = np.zeros((NTR, ncol)) if read_back else None
    velocity = np.zeros((NTR, ncol)) if read_back else None
    present = np.zeros(NTR, dtype=np.int32)
    rc = L.cpl_pelagic_soil(pel.h, sed.h, ctypes.byref(p), ctypes.byref(f), _p(t), _p(d), _p(k),
                            _p(v), _p(surface), _p(velocity), _p(present, _ip),
                            None if stats is None else ctypes.byref(stats))
    if rc != SED_OK:
        raise SedError(rc, "cpl_pelagic_soil: " + L.sed_last_error(sed.h).decode())
    return surface, velocity, present


def soil_pelagic(sed: Solver, pel: PelagicSolver, params: Optional[CplSoilParams] = None,
                 fields: Optional[CplFields] = None, stats: Optional[CplStats] = None,
                 read_back: bool = True) -> Tuple[Optional[np.ndarray], np.ndarray]:
    """One soil_pelagic_connector Run from ``sed``'s fluxes after its last
    step into ``pel``'s bottom-flux rows, on the device.  Returns the
    pelagic bottom fluxes [PEL_NTR][ncol] (host copy, None without
    ``read_back``) and present [PEL_NTR] (1 for the rows written)."""
    from .pelagic import PEL_NTR
    L = load()
    p = params or soil_default_params()
    f = fields or npzd_fields()
    out = np.zeros((PEL_NTR, sed.cs.ncol)) if read_back else None
    present = np.zeros(PEL_NTR, dtype=np.int32)
    rc = L.cpl_soil_pelagic(sed.h, pel.h, ctypes.byref(p), ctypes.byref(f), _p(out),
                            _p(present, _ip), None if stats is None else ctypes.byref(stats))
    if rc != SED_OK:
        raise SedError(rc, "cpl_soil_pelagic: " + L.sed_last_error(sed.h).decode())
    return out, present
