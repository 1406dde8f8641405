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
           "init_concentrations", "update_porosity", "ode_solver", "get_rhs",
           "EULER", "RUNGE_KUTTA_4", "ADAPTIVE_EULER", "RUNGE_KUTTA_4_38"]


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
        self.bioturbation = 0.9
        self.diffusivity = 0.9
        self.bioturbation_profile = 1
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
                           minimum=self.minimum)
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
               self.relative_change_min, self.bcup_dissolved_variables,
               self.bcup_particulate_variables, tuple(sorted(self.bgc.items())),
               self.diffusivity, self.bioturbation, self.mol_diff_mode,
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


def update_porosity(sed: TypeSed) -> None:
    """Masked cells to porosity 1 and the interface porosity
    (fabm_sediment_driver.F90:430-435)."""
    sed.porosity = np.where(sed.mask > 0, 1.0, sed.porosity)
    phi_i = np.empty_like(sed.porosity)
    phi_i[0] = sed.porosity[0]
    phi_i[1:] = 0.5 * (sed.porosity[:-1] + sed.porosity[1:])
    sed.intf_porosity = phi_i


def initialize(sed: TypeSed, sed_nml: Optional[dict] = None) -> None:
    """Porosity, flux cap and bioturbation profile from the sed_nml values
    (fabm_sediment_driver.F90:211-304; defaults :217-231)."""
    nml = dict(diffusivity=0.9, bioturbation=0.9, bioturbation_profile=1,
               bioturbation_depth=5.0, bioturbation_min=0.2, porosity_max=0.7,
               porosity_fac=0.9, k_par=2.0e-3, pom_flux_max=2.0e4,
               distributed_pom_flux=False)
    nml.update(sed_nml or {})
    if sed.grid.dz is None:
        init_grid(sed.grid)
    g = sed.grid
    sed.diffusivity = nml["diffusivity"]
    sed.bioturbation = nml["bioturbation"]
    sed.bioturbation_profile = nml["bioturbation_profile"]
    sed.k_par = nml["k_par"]
    sed.bcup_particulate_variables = 4 if nml["distributed_pom_flux"] else 1
    phi = nml["porosity_max"] * (1.0 - nml["porosity_fac"] * g.zc)
    cap = nml["pom_flux_max"] / 86400.0 * (1.0 - phi) * g.dz
    for k in range(2, g.knum):
        cap[k] = np.minimum(cap[k], cap[k - 1])
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
    sed.flux_cap = cap
    sed.bioturbation_factor = bf
    update_porosity(sed)


def init_concentrations(sed: TypeSed, initial_values) -> None:
    """conc = initial_value / porosity, masked cells at the missing value
    1e20 (fabm_sediment_driver.F90:449-468)."""
    iv = np.asarray(initial_values, dtype=np.float64)
    conc = iv[:, None, None] / sed.porosity[None, :, :]
    conc = np.where((sed.mask > 0)[None], 1.0e20, conc)
    sed.conc = np.ascontiguousarray(conc)


def ode_solver(rhs_driver: TypeSed, dt: float, method: int) -> None:
    """solver_library ode_solver (src/utilities/solver_library.F90:80-189):
    advances rhs_driver.conc in place by dt with the given method, followed
    by the component's NaN check and clamp.  Raises SedError on NaN, on the
    substep cap or on a CUDA error."""
    s = rhs_driver.solver()
    s.ode_solver(rhs_driver.conc, rhs_driver.bdys, rhs_driver.fluxes, dt, method)


def get_rhs(rhs_driver: TypeSed) -> np.ndarray:
    """type_sed%get_rhs (fabm_sediment_driver.F90:575-717): tendencies of
    rhs_driver.conc; the dissolved rows of rhs_driver.fluxes receive the
    surface fluxes."""
    s = rhs_driver.solver()
    s.set_forcing(rhs_driver.bdys, rhs_driver.fluxes)
    rhs, fl = s.get_rhs(rhs_driver.conc, rhs_driver.fluxes)
    rhs_driver.fluxes[...] = fl
    return rhs
