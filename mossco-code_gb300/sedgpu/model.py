"""Tracer set, parameters and the column-set container of the sediment path.

The tracer set is the 11-tracer OMEXDIA+P layout used throughout the
package.  It follows the reference's C/N/P detritus pools (the five
``pflux_*`` deposition fluxes of examples/standalone/omexdia_p/main.F90:28-29,
97-101: labile C, N, P and semilabile C, N), adds an explicit adsorbed-P pool
and the five dissolved species.  Order is fixed; the kernels and the C-ABI
use the same indices.

All concentrations are per unit pore-water volume for every tracer, as the
reference driver stores them (src/drivers/fabm_sediment_driver.F90:15-16,456).
Arrays use the reference's Fortran ``conc(i,j,k,n)`` order: element
``(n, k, col)`` of a C-contiguous ``[n][k][col]`` array, ``col = i + inum*j``.
"""
from __future__ import annotations

import dataclasses
from typing import Dict, Optional

import numpy as np

TRACERS = (
    "detritus_labile_carbon",        # 0 fdetC
    "detritus_semilabile_carbon",    # 1 sdetC
    "detritus_labile_nitrogen",      # 2 fdetN
    "detritus_semilabile_nitrogen",  # 3 sdetN
    "detritus_labile_phosphorus",    # 4 fdetP
    "adsorbed_phosphorus",           # 5 adsP
    "dissolved_oxygen",              # 6 O2
    "dissolved_nitrate",             # 7 NO3
    "dissolved_ammonium",            # 8 NH4
    "dissolved_reduced_substances",  # 9 ODU
    "dissolved_phosphate",           # 10 PO4
)
SHORT = ("fdetC", "sdetC", "fdetN", "sdetN", "fdetP", "adsP",
         "O2", "NO3", "NH4", "ODU", "PO4")
NTR = len(TRACERS)
PARTICULATE = np.array([1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0], dtype=np.uint8)

# Tracers whose sum is conserved by the reaction model (P) and the ones whose
# sum changes only by denitrification (N, loss 0.8 mol N per mol C).
P_TRACERS = (4, 5, 10)
N_TRACERS = (2, 3, 7, 8)

# ode_solver methods, src/utilities/solver_library.F90:32-35
EULER, RUNGE_KUTTA_4, ADAPTIVE_EULER, RUNGE_KUTTA_4_38 = 0, 1, 2, 3

# OMEXDIA+P parameters in per-day units:
# examples/standalone/omexdia_p/fabm_sed.nml:51-77 (&hzg_omexdia_p).
BGC_NAMES = ("rLabile", "rSemilabile", "NCrLdet", "NCrSdet", "PAds",
             "PAdsODU", "NH3Ads", "CprodMax", "rnit", "ksO2nitri", "rODUox",
             "ksO2oduox", "ksO2oxic", "ksNO3denit", "kinO2denit",
             "kinNO3anox", "kinO2anox")
BGC_DEFAULTS: Dict[str, float] = dict(
    rLabile=0.043, rSemilabile=0.001, NCrLdet=0.22, NCrSdet=0.005,
    PAds=0.01, PAdsODU=70.0, NH3Ads=0.0, CprodMax=9600.0, rnit=200.0,
    ksO2nitri=20.0, rODUox=20.0, ksO2oduox=1.0, ksO2oxic=3.0,
    ksNO3denit=1.0, kinO2denit=70.0, kinNO3anox=1.0, kinO2anox=1.0)


@dataclasses.dataclass
class DriverParams:
    """Scalars of type_sed / type_rhs_driver that the hot path reads.

    Defaults are the reference's: sed_nml defaults
    (src/drivers/fabm_sediment_driver.F90:217-231), BcUp choices (:79-80),
    solver limits (src/utilities/solver_library.F90:40-41).
    """
    diffusivity: float = 0.9            # cm2/d
    bioturbation: float = 0.9           # cm2/d
    bcup_dissolved: int = 2             # 1 flux, 2 concentration, 3 none
    bcup_particulate: int = 1           # 1 flux, 4 capped cascade
    mol_diff_mode: int = 0              # 0 reference, 1 tortuosity
    mol_diff_d0: float = 1.0e-9         # m2/s (mode 1)
    dt_min: float = 1.0e-9              # s
    relative_change_min: float = -0.9
    atol: float = 0.0                   # absolute floor of the positivity test
    max_attempts: int = 8192            # adaptive loop guard per step
    minimum: Optional[np.ndarray] = None  # clamp per tracer (default 0)
    # 3: bioturbation factor of Zhang & Wirtz (2017) recomputed from the TOC
    # profile at every right-hand side (get_rhs :618-645); any other value:
    # the static biofac profile.  Constants: sed_nml bioturb_* (:226-231).
    bioturbation_profile: int = 1
    bioturb_k_l: float = 0.11
    bioturb_L1: float = 0.2
    bioturb_L2: float = 0.6
    bioturb_beta: float = 0.22
    bioturb_b: float = 1.334
    bioturb_dry_density: float = 1000.0
    # > 0: the microbial rates (rLabile, rSemilabile, CprodMax, rnit, rODUox)
    # times exp(-temp_activation (1/(T+273) - 1/288)) in each column, the
    # Arrhenius form of the driver's bioturbation factor f_T (:648); 0: none
    temp_activation: float = 0.0
    # type_rhs_driver's adaptive_solver_diagnostics (solver_library.F90:43):
    # last_min_dt and last_min_dt_grid_cell of the grid-wide cut
    adaptive_solver_diagnostics: bool = False

    def minimum_array(self) -> np.ndarray:
        if self.minimum is None:
            return np.zeros(NTR, dtype=np.float64)
        return np.ascontiguousarray(self.minimum, dtype=np.float64)


@dataclasses.dataclass
class ColumnSet:
    """A grid of sediment columns with its state and forcing.

    Shapes (C order, reference Fortran order read backwards):
      kact      [ncol]            active layers (0 = land column)
      dz, phi, phi_i, biofac, flux_cap  [kmax][ncol]
      dzc       [kmax-1][ncol]
      zc, zi    [kmax][ncol], [kmax+1][ncol]   (set-up and PAR only)
      bdys      [ntr+1][ncol]     temperature then bottom-water values
      fluxes    [ntr][ncol]       downward flux at the surface (/s)
      conc      [ntr][kmax][ncol]
    """
    inum: int
    jnum: int
    kmax: int
    kact: np.ndarray
    dz: np.ndarray
    dzc: np.ndarray
    zc: np.ndarray
    zi: np.ndarray
    phi: np.ndarray
    phi_i: np.ndarray
    biofac: np.ndarray
    flux_cap: np.ndarray
    bdys: np.ndarray
    fluxes: np.ndarray
    conc: np.ndarray
    driver: DriverParams = dataclasses.field(default_factory=DriverParams)
    bgc: Dict[str, float] = dataclasses.field(
        default_factory=lambda: dict(BGC_DEFAULTS))
    dt: float = 3600.0
    nsteps: int = 1
    name: str = ""
    seed: int = 0
    # per-column OMEXDIA+P parameter sets [len(BGC_NAMES)][ncol] (an
    # ensemble), or None for the one set ``bgc``
    bgc_col: Optional[np.ndarray] = None

    @property
    def ncol(self) -> int:
        return self.inum * self.jnum

    def bgc_columns(self) -> np.ndarray:
        """[len(BGC_NAMES)][ncol]: bgc_col, or ``bgc`` repeated."""
        if self.bgc_col is not None:
            return np.ascontiguousarray(self.bgc_col, dtype=np.float64)
        v = np.array([self.bgc[n] for n in BGC_NAMES], dtype=np.float64)
        return np.ascontiguousarray(np.repeat(v[:, None], self.ncol, axis=1))

    @property
    def n_active(self) -> int:
        return int(np.count_nonzero(self.kact))

    def copy(self) -> "ColumnSet":
        out = dataclasses.replace(self)
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, np.ndarray):
                setattr(out, f.name, v.copy())
        out.driver = dataclasses.replace(self.driver)
        out.bgc = dict(self.bgc)
        return out

    def subset(self, cols: np.ndarray) -> "ColumnSet":
        """The columns ``cols`` as a 1 x len(cols) grid (copies)."""
        cols = np.asarray(cols, dtype=np.int64)
        out = self.copy()
        out.inum, out.jnum = len(cols), 1
        out.kact = self.kact[cols].copy()
        for name in ("dz", "dzc", "zc", "zi", "phi", "phi_i", "biofac",
                     "flux_cap", "bdys", "fluxes"):
            setattr(out, name, np.ascontiguousarray(getattr(self, name)[:, cols]))
        out.conc = np.ascontiguousarray(self.conc[:, :, cols])
        if self.bgc_col is not None:
            out.bgc_col = np.ascontiguousarray(self.bgc_col[:, cols])
        return out
