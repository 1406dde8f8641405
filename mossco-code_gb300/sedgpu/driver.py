"""Host-side mirror of the reference's driver / solver interface.

A caller that knows MOSSCO's ``fabm_sediment_driver`` finds the same names
here, with the same argument meaning and in-place behaviour:

    sed = TypeSed(inum, jnum, knum)          # type_sed
    init_grid(sed.grid, dzmin)               # fabm_sed_grid%init_grid
    initialize(sed, sed_nml)                 # type_sed%initialize
    init_concentrations(sed, initial_values) # type_sed%init_concentrations
    ode_solver(sed, dt, ADAPTIVE_EULER)      # solver_library ode_solver
    rhs = get_rhs(sed)                       # type_sed%get_rhs

``ode_solver`` and ``get_rhs`` run on the GPU through the C ABI
(sed_ode_solver / sed_get_rhs); the set-up routines are host code, as in the
reference.  Arrays are C-ordered views of the Fortran arrays:
``conc[n, k, col]`` is ``conc(i, j, k, n)`` with ``col = i + inum*j``.
"""
from __future__ import annotations

import dataclasses
from typing import Dict, Optional

import numpy as np

from .capi import SED_CUT_GLOBAL, SED_CUT_PER_COLUMN, SED_FP32, Solver
from .model import (ADAPTIVE_EULER, BGC_DEFAULTS, EULER, NTR, RUNGE_KUTTA_4,
                    RUNGE_KUTTA_4_38, ColumnSet, DriverParams)

__all__ = ["TypeSed", "SedGrid", "init_grid", "initialize",
           "init_concentrations", "update_porosity", "ode_solver", "get_rhs", "update_min_dt",
           "EULER", "RUNGE_KUTTA_4", "ADAPTIVE_EULER", "RUNGE_KUTTA_4_38",
           "SED_CUT_GLOBAL", "SED_CUT_PER_COLUMN"]


@dataclasses.dataclass
class SedGrid:
    """fabm_sed_grid (src/drivers/fabm_sediment_driver.F90:41-56)."""
    inum: int
    jnum: int
    knum: int
    dzmin: float = 0.005
    dz: Optional[np.ndarray] = None
    zc: Optional[np.ndarray] = None
    zi: Optional[np.ndarray] = None
    dzc: Optional[np.ndarray] = None


class TypeSed:
    """type_sed / type_rhs_driver fields that the hot path reads or writes
    (fabm_sediment_driver.F90:69-113, solver_library.F90:37-49)."""

    def __init__(self, inum: int, jnum: int, knum: int):
        self.grid = SedGrid(inum, jnum, knum)
        self.inum, self.jnum, self.knum = inum, jnum, knum
        self.nvar = NTR
        self.dt_min = 1.0e-9
        self.relative_change_min = -0.9
        # absolute floor of the adaptive positivity test; 0 is the
        # reference's purely relative test (solver_library.F90:121)
        self.atol = 0.0
        self.bioturbation = 0.9
        self.diffusivity = 0.9
        self.bioturbation_profile = 1
        # sed_nml bioturb_* (:226-231): Zhang & Wirtz profile 3 constants
        self.bioturb_k_l = 0.11
        self.bioturb_L1 = 0.2
        self.bioturb_L2 = 0.6
        self.bioturb_beta = 0.22
        self.bioturb_b = 1.334
        self.bioturb_dry_density = 1000.0
        self.porosity_fac = 0.9
        self.pom_flux_max = 2.0e4
        self.missing_value = 1.0e20
        self.bcup_dissolved_variables = 2
        self.bcup_particulate_variables = 1
        self.mol_diff_mode = 0
        self.mol_diff_d0 = 1.0e-9
        self.k_par = 2.0e-3
        self.bgc: Dict[str, float] = dict(BGC_DEFAULTS)
        self.minimum = np.zeros(NTR)
        self.mask = np.zeros((knum, inum * jnum), dtype=np.int32)
        self.porosity = None
        self.intf_porosity = None
        self.bioturbation_factor = None
        self.flux_cap = None
        self.conc: Optional[np.ndarray] = None
        self.bdys = np.zeros((NTR + 1, inum * jnum))
        self.fluxes = np.zeros((NTR, inum * jnum))
        self.cut_scope = SED_CUT_PER_COLUMN
        self.precision = SED_FP32
        # type_rhs_driver's diagnostics (solver_library.F90:43-45): kept
        # across ode_solver calls while adaptive_solver_diagnostics is set
        self.adaptive_solver_diagnostics = False
        self.last_min_dt = float(np.float32(1.0e20))
        self.last_min_dt_grid_cell = [-99, -99, -99, -99]
        self._solver: Optional[Solver] = None
        self._solver_key = None

    @property
    def ncol(self) -> int:
        return self.inum * self.jnum

    def kact(self) -> np.ndarray:
        """Active layers per column from the 3-D mask (masked tail only)."""
        unmasked = self.mask <= 0
        return np.where(unmasked[0], np.cumprod(unmasked, axis=0).sum(axis=0),
                        0).astype(np.int32)

    def to_columns(self) -> ColumnSet:
        g = self.grid
        drv = DriverParams(diffusivity=self.diffusivity,
                           bioturbation=self.bioturbation,
                           bcup_dissolved=self.bcup_dissolved_variables,
                           bcup_particulate=self.bcup_particulate_variables,
                           mol_diff_mode=self.mol_diff_mode,
                           mol_diff_d0=self.mol_diff_d0, dt_min=self.dt_min,
                           relative_change_min=self.relative_change_min,
                           atol=self.atol, minimum=self.minimum,
                           bioturbation_profile=self.bioturbation_profile,
                           bioturb_k_l=self.bioturb_k_l,
                           bioturb_L1=self.bioturb_L1,
                           bioturb_L2=self.bioturb_L2,
                           bioturb_beta=self.bioturb_beta,
                           bioturb_b=self.bioturb_b,
                           bioturb_dry_density=self.bioturb_dry_density)
        return ColumnSet(inum=self.inum, jnum=self.jnum, kmax=self.knum,
                         kact=self.kact(), dz=g.dz, dzc=g.dzc, zc=g.zc,
                         zi=g.zi, phi=self.porosity,
                         phi_i=self.intf_porosity,
                         biofac=self.bioturbation_factor,
                         flux_cap=self.flux_cap, bdys=self.bdys,
                         fluxes=self.fluxes, conc=self.conc, driver=drv,
                         bgc=dict(self.bgc))

    def solver(self) -> Solver:
        key = (self.cut_scope, self.precision, self.dt_min,
               self.relative_change_min, self.atol, self.bcup_dissolved_variables,
               self.bcup_particulate_variables, tuple(sorted(self.bgc.items())),
               self.diffusivity, self.bioturbation, self.mol_diff_mode,
               self.bioturbation_profile, self.bioturb_k_l, self.bioturb_L1,
               self.bioturb_L2, self.bioturb_beta, self.bioturb_b,
               self.bioturb_dry_density,
               id(self.porosity), id(self.grid.dz), id(self.mask))
        if self._solver is None or self._solver_key != key:
            if self._solver is not None:
                self._solver.close()
            self._solver = Solver(self.to_columns(), precision=self.precision,
                                  cut_scope=self.cut_scope)
            self._solver_key = key
        return self._solver


def init_grid(grid: SedGrid, dzmin: Optional[float] = None) -> None:
    """Linear layer growth to 0.18 m (fabm_sediment_driver.F90:127-177)."""
    if dzmin is not None:
        grid.dzmin = dzmin
    K, n = grid.knum, grid.inum * grid.jnum
    fac = 0.18 / ((K + 1) / 2.0 * grid.dzmin) - 1.0
    k = np.arange(1, K + 1, dtype=np.float64)
    dz1 = (1.0 + (fac - 1.0) * (k - 1) / max(K - 1, 1)) * grid.dzmin
    zi1 = np.concatenate([[0.0], np.cumsum(dz1)])
    zc1 = zi1[:-1] + 0.5 * dz1
    grid.dz = np.repeat(dz1[:, None], n, axis=1)
    grid.zi = np.repeat(zi1[:, None], n, axis=1)
    grid.zc = np.repeat(zc1[:, None], n, axis=1)
    grid.dzc = np.ascontiguousarray(grid.zc[1:] - grid.zc[:-1])


def update_porosity(sed: TypeSed, from_surface: bool = False,
                    reinitialize_concentrations: bool = False) -> None:
    """type_sed%update_porosity (fabm_sediment_driver.F90:393-442).

    from_surface: porosity below the top layer from the top layer's value,
    phi(k) = phi(1) * (1 - porosity_fac * (zc(k) - zc(1))), and the POM flux
    cap recomputed with its downward-monotone limit (:408-428).  Then, always:
    masked cells get porosity 1 (:431) and the interface porosity is
    phi_i(1) = phi(1), phi_i(k) = (phi(k-1) + phi(k)) / 2 (:434-435).
    reinitialize_concentrations: init_concentrations again from the initial
    values last given to it, if concentrations exist (:438-440)."""
    g = sed.grid
    phi = np.array(sed.porosity, dtype=np.float64)
    if from_surface:
        for k in range(1, g.knum):
            phi[k] = phi[0] * (1.0 - sed.porosity_fac * (g.zc[k] - g.zc[0]))
        sed.flux_cap = _flux_cap(sed.pom_flux_max, phi, g.dz)
    phi = np.where(sed.mask > 0, 1.0, phi)
    phi_i = np.empty_like(phi)
    phi_i[0] = phi[0]
    phi_i[1:] = 0.5 * (phi[:-1] + phi[1:])
    sed.porosity = phi
    sed.intf_porosity = phi_i
    if reinitialize_concentrations and sed.conc is not None:
        init_concentrations(sed, getattr(sed, "initial_values", None))


def _flux_cap(pom_flux_max: float, phi: np.ndarray, dz: np.ndarray) -> np.ndarray:
    """POM flux cap per layer, each layer from the third down capped by the
    one above (fabm_sediment_driver.F90:284-291, :419-426)."""
    cap = pom_flux_max / 86400.0 * (1.0 - phi) * dz
    for k in range(2, cap.shape[0]):
        cap[k] = np.minimum(cap[k], cap[k - 1])
    return cap


def initialize(sed: TypeSed, sed_nml: Optional[dict] = None) -> None:
    """Porosity, flux cap and bioturbation profile from the sed_nml values
    (fabm_sediment_driver.F90:211-304; defaults :217-231).  Profile 1 is a
    linear decrease to bioturbation_min at bioturbation_depth, 2 an
    exponential decrease, any other value a factor of 1 (:294-303)."""
    nml = dict(diffusivity=0.9, bioturbation=0.9, bioturbation_profile=1,
               bioturbation_depth=5.0, bioturbation_min=0.2, porosity_max=0.7,
               porosity_fac=0.9, k_par=2.0e-3, pom_flux_max=2.0e4,
               distributed_pom_flux=False, bioturb_k_l=0.11, bioturb_L1=0.2,
               bioturb_L2=0.6, bioturb_beta=0.22, bioturb_b=1.334,
               bioturb_dry_density=1000.0)
    unknown = set(sed_nml or {}) - set(nml)
    if unknown:
        raise ValueError(f"unknown sed_nml entries: {sorted(unknown)}")
    nml.update(sed_nml or {})
    if sed.grid.dz is None:
        init_grid(sed.grid)
    g = sed.grid
    sed.diffusivity = nml["diffusivity"]
    sed.bioturbation = nml["bioturbation"]
    sed.bioturbation_profile = nml["bioturbation_profile"]
    sed.k_par = nml["k_par"]
    sed.porosity_fac = nml["porosity_fac"]
    sed.pom_flux_max = nml["pom_flux_max"]
    for name in ("bioturb_k_l", "bioturb_L1", "bioturb_L2", "bioturb_beta",
                 "bioturb_b", "bioturb_dry_density"):
        setattr(sed, name, nml[name])
    sed.bcup_particulate_variables = 4 if nml["distributed_pom_flux"] else 1
    phi = nml["porosity_max"] * (1.0 - nml["porosity_fac"] * g.zc)
    prof = nml["bioturbation_profile"]
    if prof == 1:
        lin = np.maximum(nml["bioturbation_depth"] - 100.0 * g.zi[:g.knum], 0.0)
        bf = np.maximum(nml["bioturbation_min"] / nml["bioturbation"],
                        lin / nml["bioturbation_depth"])
    elif prof == 2:
        bf = np.exp(-100.0 * g.zi[:g.knum] / nml["bioturbation_depth"])
    else:
        bf = np.ones_like(phi)
    sed.porosity = phi
    sed.flux_cap = _flux_cap(nml["pom_flux_max"], phi, g.dz)
    sed.bioturbation_factor = bf
    update_porosity(sed, from_surface=False)


def init_concentrations(sed: TypeSed, initial_values=None) -> None:
    """type_sed%init_concentrations (fabm_sediment_driver.F90:449-467):
    conc = initial_value / porosity, the namelist values being per total
    cell volume; masked cells at sed.missing_value (1e20, :85).  initial_values has one
    entry per tracer; None reuses the last values given."""
    if initial_values is None:
        initial_values = getattr(sed, "initial_values", None)
        if initial_values is None:
            raise ValueError("init_concentrations: no initial values")
    iv = np.asarray(initial_values, dtype=np.float64)
    if iv.shape != (sed.nvar,):
        raise ValueError(f"initial_values must have {sed.nvar} entries, got {iv.shape}")
    sed.initial_values = iv.copy()
    conc = iv[:, None, None] / sed.porosity[None, :, :]
    conc = np.where((sed.mask > 0)[None], sed.missing_value, conc)
    sed.conc = np.ascontiguousarray(conc)


def update_min_dt(rhs_driver: TypeSed, min_dt: np.ndarray) -> None:
    """last_min_dt / last_min_dt_grid_cell (solver_library.F90:129-136) from
    the smallest accepted substep of every column in the last call ([ncol],
    0 where a column accepted none).  The substep is the grid's smallest;
    its cell is (i, j) of the first column in Fortran order that took it,
    with the layer and tracer not recorded by the device (-99)."""
    md = np.asarray(min_dt, dtype=np.float64)
    pos = np.where(md > 0.0, md, np.inf)
    if not np.isfinite(pos).any():
        return
    col = int(np.argmin(pos))
    if pos[col] < rhs_driver.last_min_dt:
        rhs_driver.last_min_dt = float(pos[col])
        rhs_driver.last_min_dt_grid_cell = [col % rhs_driver.inum + 1,
                                            col // rhs_driver.inum + 1, -99, -99]


def ode_solver(rhs_driver: TypeSed, dt: float, method: int) -> None:
    """solver_library ode_solver (src/utilities/solver_library.F90:80-189):
    advances rhs_driver.conc in place by dt with the given method, followed
    by the component's NaN check and clamp.  Raises SedError on NaN, on the
    substep cap or on a CUDA error.  With adaptive_solver_diagnostics and
    ADAPTIVE_EULER it updates last_min_dt and last_min_dt_grid_cell."""
    s = rhs_driver.solver()
    s.ode_solver(rhs_driver.conc, rhs_driver.bdys, rhs_driver.fluxes, dt, method)
    if rhs_driver.adaptive_solver_diagnostics and method == ADAPTIVE_EULER:
        update_min_dt(rhs_driver, s.min_dt())


def get_rhs(rhs_driver: TypeSed) -> np.ndarray:
    """type_sed%get_rhs (fabm_sediment_driver.F90:575-717): tendencies of
    rhs_driver.conc; the dissolved rows of rhs_driver.fluxes receive the
    surface fluxes."""
    s = rhs_driver.solver()
    s.set_forcing(rhs_driver.bdys, rhs_driver.fluxes)
    rhs, fl = s.get_rhs(rhs_driver.conc, rhs_driver.fluxes)
    rhs_driver.fluxes[...] = fl
    return rhs
