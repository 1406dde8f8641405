"""ctypes front end of the FP64 CPU oracle (sed_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
compare against and by bench.py's CPU-baseline leg.  The product (the CUDA
library under mossco-code_gb300/) never imports it.

Parity status: stepper and transport follow the reference source
(src/utilities/solver_library.F90:80-189,
src/drivers/fabm_sediment_driver.F90:575-825) and are pinned by known-answer
tests; the OMEXDIA+P rates restate the published model and are UNPINNED
(the reference's rates live in the external FABM library).
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
LIB_PATH = os.path.join(BUILD_DIR, "libsedoracle.so")
SRC = os.path.join(HERE, "sed_oracle.c")

_PKG = os.path.join(os.path.dirname(HERE), "mossco-code_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
from sedgpu.model import BGC_NAMES, NTR, PARTICULATE, ColumnSet  # noqa: E402

CFLAGS = ["-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
          "-ffp-contract=off", "-fno-math-errno"]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc into oracle/_build (same flags on x86 and
    aarch64; FMA contraction off so both give the same bits)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(
                os.path.join(HERE, "sed_oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *CFLAGS, SRC, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Bgc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in BGC_NAMES]


_dp = ctypes.POINTER(ctypes.c_double)


class Model(ctypes.Structure):
    _fields_ = [
        ("ncol", ctypes.c_int), ("kmax", ctypes.c_int), ("ntr", ctypes.c_int),
        ("kact", ctypes.POINTER(ctypes.c_int)),
        ("dz", _dp), ("dzc", _dp), ("phi", _dp), ("phi_i", _dp),
        ("biofac", _dp), ("flux_cap", _dp),
        ("particulate", ctypes.POINTER(ctypes.c_ubyte)),
        ("minimum", _dp),
        ("diffusivity", ctypes.c_double), ("bioturbation", ctypes.c_double),
        ("bcup_dissolved", ctypes.c_int), ("bcup_particulate", ctypes.c_int),
        ("mol_diff_mode", ctypes.c_int), ("mol_diff_d0", ctypes.c_double),
        ("dt_min", ctypes.c_double), ("relative_change_min", ctypes.c_double),
        ("atol", ctypes.c_double),
        ("max_attempts", ctypes.c_long),
        ("bgc", Bgc),
        ("bioturbation_profile", ctypes.c_int),
        ("bioturb_k_l", ctypes.c_double), ("bioturb_L1", ctypes.c_double),
        ("bioturb_L2", ctypes.c_double), ("bioturb_beta", ctypes.c_double),
        ("bioturb_b", ctypes.c_double), ("bioturb_dry_density", ctypes.c_double),
        ("bgc_col", ctypes.POINTER(Bgc)),
        ("temp_activation", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [("attempts", ctypes.c_long), ("accepted", ctypes.c_long),
                ("rejected", ctypes.c_long),
                ("max_col_attempts", ctypes.c_long),
                ("min_dt", ctypes.c_double), ("capped", ctypes.c_int),
                ("nan_cells", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


class Diag(ctypes.Structure):
    """orc_diag: type_rhs_driver's last_min_dt and last_min_dt_grid_cell."""
    _fields_ = [("last_min_dt", ctypes.c_double),
                ("last_min_dt_grid_cell", ctypes.c_int * 4), ("inum", ctypes.c_int)]

    def cell(self):
        return tuple(self.last_min_dt_grid_cell)


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.orc_get_rhs.argtypes = [P(Model), _dp, _dp, _dp, _dp, _dp]
        L.orc_ode_solver.argtypes = [P(Model), _dp, _dp, _dp, ctypes.c_double,
                                     ctypes.c_int, P(Stats)]
        L.orc_ode_solver.restype = ctypes.c_int
        L.orc_run.argtypes = [P(Model), _dp, _dp, _dp, ctypes.c_double,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, P(Stats)]
        L.orc_run.restype = ctypes.c_int
        L.orc_epilogue.argtypes = [P(Model), _dp]
        L.orc_diag_init.argtypes = [P(Diag), ctypes.c_int]
        L.orc_diag_init.restype = None
        L.orc_ode_solver_diag.argtypes = [P(Model), _dp, _dp, _dp, ctypes.c_double, P(Diag),
                                          P(Stats)]
        L.orc_ode_solver_diag.restype = ctypes.c_int
        L.orc_epilogue.restype = ctypes.c_int
        L.orc_omexdia_p.argtypes = [P(Bgc), ctypes.c_double, _dp, _dp, _dp]
        L.orc_diff3d.argtypes = [ctypes.c_int, _dp, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                 _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_init_grid_linear.argtypes = [ctypes.c_int, ctypes.c_double,
                                           _dp, _dp, _dp, _dp]
        L.orc_init_profiles.argtypes = [
            ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, _dp, _dp, _dp, _dp]
        L.orc_bc_flux_estimate.argtypes = [P(Model), _dp, _dp, _dp]
        L.orc_assemble_bc.argtypes = [P(Model), _dp, _dp, _dp, _dp,
                                      P(ctypes.c_int), _dp, _dp]
        L.orc_inventory.argtypes = [P(Model), _dp, _dp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class OracleModel:
    """Keeps the numpy arrays behind an orc_model alive."""

    def __init__(self, cs: ColumnSet):
        self.cs = cs
        d = cs.driver
        self._keep = dict(
            kact=np.ascontiguousarray(cs.kact, dtype=np.int32),
            dz=np.ascontiguousarray(cs.dz, dtype=np.float64),
            dzc=np.ascontiguousarray(cs.dzc, dtype=np.float64),
            phi=np.ascontiguousarray(cs.phi, dtype=np.float64),
            phi_i=np.ascontiguousarray(cs.phi_i, dtype=np.float64),
            biofac=np.ascontiguousarray(cs.biofac, dtype=np.float64),
            flux_cap=np.ascontiguousarray(cs.flux_cap, dtype=np.float64),
            particulate=np.ascontiguousarray(PARTICULATE, dtype=np.uint8),
            minimum=d.minimum_array(),
        )
        k = self._keep
        m = Model()
        m.ncol, m.kmax, m.ntr = cs.ncol, cs.kmax, NTR
        m.kact = k["kact"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        for name in ("dz", "dzc", "phi", "phi_i", "biofac", "flux_cap",
                     "minimum"):
            setattr(m, name, _ptr(k[name]))
        m.particulate = k["particulate"].ctypes.data_as(
            ctypes.POINTER(ctypes.c_ubyte))
        m.diffusivity = d.diffusivity
        m.bioturbation = d.bioturbation
        m.bcup_dissolved = d.bcup_dissolved
        m.bcup_particulate = d.bcup_particulate
        m.mol_diff_mode = d.mol_diff_mode
        m.mol_diff_d0 = d.mol_diff_d0
        m.dt_min = d.dt_min
        m.relative_change_min = d.relative_change_min
        m.atol = d.atol
        m.max_attempts = d.max_attempts
        for n in BGC_NAMES:
            setattr(m.bgc, n, float(cs.bgc[n]))
        m.bioturbation_profile = int(d.bioturbation_profile)
        for n in ("bioturb_k_l", "bioturb_L1", "bioturb_L2", "bioturb_beta",
                  "bioturb_b", "bioturb_dry_density"):
            setattr(m, n, float(getattr(d, n)))
        m.temp_activation = float(d.temp_activation)
        if cs.bgc_col is not None:
            # [ncol] structs: the transpose of the [param][col] table
            tab = np.ascontiguousarray(np.asarray(cs.bgc_col, dtype=np.float64).T)
            self._keep["bgc_col"] = tab
            m.bgc_col = tab.ctypes.data_as(ctypes.POINTER(Bgc))
        self.m = m

    def get_rhs(self, conc: np.ndarray, fluxes: Optional[np.ndarray] = None):
        cs = self.cs
        conc = np.ascontiguousarray(conc, dtype=np.float64)
        fl = np.array(cs.fluxes if fluxes is None else fluxes,
                      dtype=np.float64, copy=True)
        bd = np.ascontiguousarray(cs.bdys, dtype=np.float64)
        rhs = np.zeros_like(conc)
        denit = np.zeros((cs.kmax, cs.ncol))
        lib().orc_get_rhs(ctypes.byref(self.m), _ptr(conc), _ptr(bd),
                          _ptr(fl), _ptr(rhs), _ptr(denit))
        return rhs, fl, denit

    def run(self, conc: np.ndarray, nsteps: int, dt: float = None,
            method: int = 2, percol: bool = True, nthreads: int = 0,
            fluxes: Optional[np.ndarray] = None):
        """nsteps coupling steps (ode_solver + clamp) in place on ``conc``.
        Returns (status, stats dict, fluxes after the run)."""
        cs = self.cs
        assert conc.dtype == np.float64 and conc.flags.c_contiguous
        dt = cs.dt if dt is None else dt
        fl = np.array(cs.fluxes if fluxes is None else fluxes,
                      dtype=np.float64, copy=True)
        bd = np.ascontiguousarray(cs.bdys, dtype=np.float64)
        st = Stats()
        rc = lib().orc_run(ctypes.byref(self.m), _ptr(conc), _ptr(bd),
                           _ptr(fl), float(dt), int(method), int(percol),
                           int(nsteps), int(nthreads), ctypes.byref(st))
        return rc, st.as_dict(), fl

    def new_diag(self) -> Diag:
        """Diagnostics as a fresh driver holds them (last_min_dt 1e20, cell -99)."""
        d = Diag()
        lib().orc_diag_init(ctypes.byref(d), self.cs.inum)
        return d

    def ode_solver_diag(self, conc: np.ndarray, diag: Diag, dt: float = None,
                        fluxes: Optional[np.ndarray] = None):
        """One grid-wide ADAPTIVE_EULER call with adaptive_solver_diagnostics,
        in place on ``conc``; ``diag`` carries across calls.  Returns
        (status, stats dict, fluxes)."""
        cs = self.cs
        assert conc.dtype == np.float64 and conc.flags.c_contiguous
        fl = np.array(cs.fluxes if fluxes is None else fluxes, dtype=np.float64, copy=True)
        bd = np.ascontiguousarray(cs.bdys, dtype=np.float64)
        st = Stats()
        rc = lib().orc_ode_solver_diag(ctypes.byref(self.m), _ptr(conc), _ptr(bd), _ptr(fl),
                                       float(cs.dt if dt is None else dt), ctypes.byref(diag),
                                       ctypes.byref(st))
        return rc, st.as_dict(), fl

    def assemble_bc(self, conc, temperature, surface, velocity, present=None,
                    bdys=None, fluxes=None):
        """get_boundary_conditions on host arrays; returns (bdys, fluxes)."""
        cs = self.cs
        bd = np.array(cs.bdys if bdys is None else bdys, dtype=np.float64, copy=True)
        fl = np.array(cs.fluxes if fluxes is None else fluxes, dtype=np.float64, copy=True)
        pr = None if present is None else np.ascontiguousarray(present, dtype=np.int32)
        lib().orc_assemble_bc(
            ctypes.byref(self.m), _ptr(np.ascontiguousarray(conc, dtype=np.float64)),
            _ptr(np.ascontiguousarray(temperature, dtype=np.float64)),
            _ptr(np.ascontiguousarray(surface, dtype=np.float64)),
            _ptr(np.ascontiguousarray(velocity, dtype=np.float64)),
            None if pr is None else pr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
            _ptr(bd), _ptr(fl))
        return bd, fl

    def inventory(self, conc: np.ndarray) -> np.ndarray:
        cs = self.cs
        conc = np.ascontiguousarray(conc, dtype=np.float64)
        inv = np.zeros((NTR, cs.ncol))
        lib().orc_inventory(ctypes.byref(self.m), _ptr(conc), _ptr(inv))
        return inv


def omexdia_rates(bgc: dict, cell: np.ndarray, fr: float = 1.0):
    """Local rates of one cell; fr multiplies the microbial rate constants."""
    b = Bgc(*[float(bgc[n]) for n in BGC_NAMES])
    c = np.ascontiguousarray(cell, dtype=np.float64)
    r = np.zeros(NTR)
    dn = np.zeros(1)
    lib().orc_omexdia_p(ctypes.byref(b), float(fr), _ptr(c), _ptr(r), _ptr(dn))
    return r, float(dn[0])


def diff3d(C, Cup, fluxup, bcup, D, VF, dz, dzc, flux_cap=None, Cdown=0.0,
           fluxdown=0.0, bcdown=3):
    C = np.ascontiguousarray(C, dtype=np.float64)
    K = len(C)
    D = np.ascontiguousarray(D, dtype=np.float64)
    VF = np.ascontiguousarray(VF, dtype=np.float64)
    dz = np.ascontiguousarray(dz, dtype=np.float64)
    dzc = np.ascontiguousarray(np.concatenate([dzc, [1.0]]), dtype=np.float64)
    cap = np.ascontiguousarray(np.zeros(K) if flux_cap is None else flux_cap,
                               dtype=np.float64)
    flux = np.zeros(K + 1)
    dC = np.zeros(K)
    lib().orc_diff3d(K, _ptr(C), float(Cup), float(Cdown), float(fluxup),
                     float(fluxdown), int(bcup), int(bcdown), _ptr(D),
                     _ptr(VF), _ptr(dz), _ptr(dzc), _ptr(cap), _ptr(flux),
                     _ptr(dC))
    return flux, dC


def init_grid_linear(kmax: int, dzmin: float):
    dz, zc, zi, dzc = (np.zeros(kmax), np.zeros(kmax), np.zeros(kmax + 1),
                       np.zeros(max(kmax - 1, 1)))
    lib().orc_init_grid_linear(kmax, dzmin, _ptr(dz), _ptr(zc), _ptr(zi),
                               _ptr(dzc))
    return dz, zc, zi, dzc[:kmax - 1]
