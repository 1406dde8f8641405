"""Seeded synthetic sediment-column workloads.

The reference publishes no benchmark data set for this path; these are the
synthetic column sets the package is measured and tested on.  Every random
number is a counter-based draw ``u(seed, field, index)`` (splitmix64 of a
key built from the three), so any column can be regenerated alone and the
CPU and GPU paths see bit-identical inputs.

Workloads (``make_workload``):

``plain_cpu_10x10``      10 x 10 columns, 20 layers, geometric grid from 1 mm
                        to 0.18 m, 10 days at 3600 s, FP64.
``plain_gpu_256x256``    256 x 256 columns, 30 layers to 0.20 m, 30 days.
``uneven_1024x1024``     1024 x 1024 columns, 30 % land, 10..60 layers,
                        log-uniform POC flux, 10 days.
``surrogate_200k``       200 000 columns of 30 layers from the uneven
                        distributions (training data generator).
``surrogate_2048x2048``  2048 x 2048 columns, 30 % land, 30 layers, 60 days.

Profiles (all workloads): porosity 0.7 + 0.2 exp(-z/0.02 m); molecular
diffusivity 1e-9 m2/s / (1 - 2 ln phi) (tortuosity mode of the driver);
bioturbation 1e-11 m2/s exp(-z/0.05 m), i.e. the reference's exponential
bioturbation profile (src/drivers/fabm_sediment_driver.F90:299-301) with a
5 cm depth scale and bioturbation = 1e-11 m2/s in cm2/d; bottom water O2
U[150,300], NO3 U[5,30], NH4 U[1,10], PO4 U[0.2,2] mmol/m3, ODU 0,
temperature U[5,15] degC; positivity-test floor atol = 1e-6 mmol/m3 (the
reference's test is recovered with atol = 0); surface POC flux split evenly
between the labile and semilabile classes, N and P by Redfield 106:16:1 (all
detrital P to the labile P pool, no adsorbed-P deposition).  Initial profiles: bottom-water
values times exp(-z/z_e) (z_e = 5 mm for O2, 2 cm otherwise) times
(1 + 0.01 N(0,1)); particulate pools start from the fabm_sed.nml initial
values (per total volume, divided by porosity as init_concentrations does,
:456) decaying with a 5 cm scale, with the same 1 % noise.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from .model import (ColumnSet, DriverParams, NTR, BGC_DEFAULTS)

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)

# field ids of the counter-based generator
F_LAND, F_KACT, F_POC, F_TEMP, F_BW0 = 1, 2, 3, 4, 10
F_NOISE_A, F_NOISE_B = 40, 41


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, field: int, index) -> np.ndarray:
    """Counter-based U[0,1) doubles (53 random bits) for integer ``index``."""
    with np.errstate(over="ignore"):
        idx = np.asarray(index, dtype=np.uint64)
        key = _splitmix64(np.uint64(seed) * np.uint64(0x100000001B3)
                          + np.uint64(field))
        r = _splitmix64(key ^ _splitmix64(idx))
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, field: int, index) -> np.ndarray:
    """Counter-based standard normals (Box-Muller on two uniform streams)."""
    u1 = uniform(seed, field, index)
    u2 = uniform(seed, field + 1000, index)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


def geometric_grid(K: int, dz1: float, total: float
                   ) -> Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Layers growing geometrically from ``dz1`` to a ``total`` depth.

    Returns dz[K], zc[K], zi[K+1], dzc[K-1] with the reference's definitions
    (src/drivers/fabm_sediment_driver.F90:150-168).
    """
    if K == 1:
        r = 1.0
    else:
        lo, hi = 1.0 + 1e-12, 10.0
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            s = dz1 * (mid ** K - 1.0) / (mid - 1.0)
            if s > total:
                hi = mid
            else:
                lo = mid
        r = 0.5 * (lo + hi)
    dz = dz1 * r ** np.arange(K, dtype=np.float64)
    zi = np.concatenate([[0.0], np.cumsum(dz)])
    zc = zi[:-1] + 0.5 * dz
    dzc = zc[1:] - zc[:-1]
    return dz, zc, zi, dzc


def interface_porosity(phi: np.ndarray) -> np.ndarray:
    """update_porosity (fabm_sediment_driver.F90:434-435) along axis 0."""
    out = np.empty_like(phi)
    out[0] = phi[0]
    out[1:] = 0.5 * (phi[:-1] + phi[1:])
    return out


# (name, surface value per total volume) of the particulate pools; the
# values are the &hzg_omexdia_cnp initial values of
# examples/standalone/omexdia_p/fabm_sed.nml:36-41, adsorbed P from po4_init.
_PART_INIT = (4.0e3, 4.0e3, 0.92e3, 0.04e3, 4.0e1, 10.0)
_BW_RANGE = {6: (150.0, 300.0), 7: (5.0, 30.0), 8: (1.0, 10.0), 10: (0.2, 2.0)}
FAST_FRACTION = 0.5
# Absolute tolerance of the positivity test in the workloads (mmol/m3).
# The reference's test is purely relative, so concentrations decaying
# towards zero keep forcing substep cuts at any magnitude; FP32 state cannot
# represent them below ~1e-38 and cannot resolve them next to neighbours ~1e8
# times larger, so an FP32 solver can only follow an FP64 one with a floor
# well above that range.  1 nmol/m3 is negligible for every tracer.  0
# restores the reference's test.
ATOL = 1.0e-6
REDFIELD_NC = 16.0 / 106.0
REDFIELD_PC = 1.0 / 106.0

WORKLOADS = {
    "plain_cpu_10x10": dict(inum=10, jnum=10, kmin=20, kmax=20, total=0.18,
                            land=0.0, poc="uniform", days=10),
    "plain_gpu_256x256": dict(inum=256, jnum=256, kmin=30, kmax=30,
                              total=0.20, land=0.0, poc="uniform", days=30),
    "uneven_1024x1024": dict(inum=1024, jnum=1024, kmin=10, kmax=60,
                             total=0.20, land=0.3, poc="loguniform", days=10),
    "surrogate_200k": dict(inum=200000, jnum=1, kmin=30, kmax=30, total=0.20,
                           land=0.0, poc="loguniform", days=30),
    "surrogate_2048x2048": dict(inum=2048, jnum=2048, kmin=30, kmax=30,
                                total=0.20, land=0.3, poc="loguniform",
                                days=60),
    # the soil under pelagic_1024x1024 for the coupling measurement: the
    # 15 layers of examples/standalone/omexdia_p/run_sed.nml:34
    "soil_1024x1024": dict(inum=1024, jnum=1024, kmin=15, kmax=15, total=0.18,
                           land=0.3, poc="loguniform", days=1),
}


def make_columns(inum: int, jnum: int, kmin: int, kmax: int, total: float,
                 land: float, poc: str, days: int, seed: int = 1234,
                 cols: Optional[np.ndarray] = None, name: str = "",
                 dt: float = 3600.0) -> ColumnSet:
    """Build a ColumnSet; ``cols`` selects a subset of global column ids
    (the generator is counter based, so a subset equals the same columns of
    the full grid)."""
    ncol_full = inum * jnum
    if cols is None:
        gid = np.arange(ncol_full, dtype=np.int64)
        oi, oj = inum, jnum
    else:
        gid = np.asarray(cols, dtype=np.int64)
        oi, oj = len(gid), 1
    n = len(gid)

    if land > 0:
        is_land = uniform(seed, F_LAND, gid) < land
    else:
        is_land = np.zeros(n, dtype=bool)
    if kmin == kmax:
        kact = np.full(n, kmax, dtype=np.int32)
    else:
        u = uniform(seed, F_KACT, gid)
        kact = (kmin + np.floor(u * (kmax - kmin + 1))).astype(np.int32)
        kact = np.minimum(kact, kmax)
    kact[is_land] = 0

    dz = np.zeros((kmax, n))
    zc = np.zeros((kmax, n))
    zi = np.zeros((kmax + 1, n))
    dzc = np.zeros((max(kmax - 1, 1), n))
    for K in np.unique(np.where(kact > 0, kact, kmax)):
        sel = np.where((kact == K) | ((kact == 0) & (K == kmax)))[0]
        g_dz, g_zc, g_zi, g_dzc = geometric_grid(int(K), 1.0e-3, total)
        # layers below the active depth continue the last spacing (unused)
        ext = int(kmax - K)
        if ext > 0:
            last = g_dz[-1]
            g_dz = np.concatenate([g_dz, np.full(ext, last)])
            g_zi = np.concatenate([[0.0], np.cumsum(g_dz)])
            g_zc = g_zi[:-1] + 0.5 * g_dz
            g_dzc = g_zc[1:] - g_zc[:-1]
        dz[:, sel] = g_dz[:, None]
        zc[:, sel] = g_zc[:, None]
        zi[:, sel] = g_zi[:, None]
        if kmax > 1:
            dzc[:, sel] = g_dzc[:, None]

    phi = 0.7 + 0.2 * np.exp(-zc / 0.02)
    phi_i = interface_porosity(phi)
    biofac = np.exp(-zi[:kmax] / 0.05)   # profile 2 with 5 cm depth scale
    pom_flux_max = 2.0e4                 # sed_nml default (:225), cap only
    flux_cap = pom_flux_max / 86400.0 * (1.0 - phi) * dz
    for k in range(2, kmax):
        flux_cap[k] = np.minimum(flux_cap[k], flux_cap[k - 1])

    # forcing
    bdys = np.zeros((NTR + 1, n))
    bdys[0] = 5.0 + 10.0 * uniform(seed, F_TEMP, gid)
    for tr, (lo, hi) in _BW_RANGE.items():
        bdys[tr + 1] = lo + (hi - lo) * uniform(seed, F_BW0 + tr, gid)
    bdys[9 + 1] = 0.0  # ODU in bottom water
    u = uniform(seed, F_POC, gid)
    if poc == "uniform":
        pocf = 5.0 + 45.0 * u
    else:
        pocf = np.exp(np.log(1.0) + u * (np.log(100.0) - np.log(1.0)))
    fluxes = np.zeros((NTR, n))
    fast = FAST_FRACTION * pocf
    slow = (1.0 - FAST_FRACTION) * pocf
    fluxes[0] = fast / 86400.0
    fluxes[1] = slow / 86400.0
    fluxes[2] = fast * REDFIELD_NC / 86400.0
    fluxes[3] = slow * REDFIELD_NC / 86400.0
    fluxes[4] = pocf * REDFIELD_PC / 86400.0
    fluxes[5] = 0.0

    # initial state
    conc = np.zeros((NTR, kmax, n))
    kidx = np.arange(kmax, dtype=np.int64)
    for tr in range(NTR):
        noise_idx = (gid[None, :] * kmax + kidx[:, None]) * NTR + tr
        noise = 1.0 + 0.01 * normal(seed, F_NOISE_A, noise_idx)
        if tr < 6:
            prof = _PART_INIT[tr] * np.exp(-zc / 0.05) / phi
        else:
            ze = 0.005 if tr == 6 else 0.02
            prof = bdys[tr + 1][None, :] * np.exp(-zc / ze)
        conc[tr] = prof * noise
    # land columns hold the reference's missing value
    conc[:, :, kact == 0] = 1.0e20
    conc[:, :, :] = np.where(kidx[None, :, None] < np.maximum(kact, 0)[None, None, :],
                             conc, np.where(kact[None, None, :] == 0, 1.0e20, 0.0))

    drv = DriverParams(bioturbation=1.0e-11 * 1.0e4 * 86400.0,
                       mol_diff_mode=1, mol_diff_d0=1.0e-9, dt_min=1.0,
                       atol=ATOL)
    cs = ColumnSet(inum=oi, jnum=oj, kmax=kmax, kact=kact,
                   dz=np.ascontiguousarray(dz), dzc=np.ascontiguousarray(dzc),
                   zc=np.ascontiguousarray(zc), zi=np.ascontiguousarray(zi),
                   phi=np.ascontiguousarray(phi),
                   phi_i=np.ascontiguousarray(phi_i),
                   biofac=np.ascontiguousarray(biofac),
                   flux_cap=np.ascontiguousarray(flux_cap),
                   bdys=np.ascontiguousarray(bdys),
                   fluxes=np.ascontiguousarray(fluxes),
                   conc=np.ascontiguousarray(conc), driver=drv,
                   bgc=dict(BGC_DEFAULTS), dt=dt,
                   nsteps=int(round(days * 86400.0 / dt)), name=name,
                   seed=seed)
    return cs


def active_columns(name: str, seed: int = 1234) -> np.ndarray:
    """Global ids of the active (non-land) columns of a named workload,
    without building its arrays (the land mask is one counter-based draw per
    column, as in make_columns)."""
    spec = WORKLOADS[name]
    gid = np.arange(spec["inum"] * spec["jnum"], dtype=np.int64)
    if spec["land"] <= 0:
        return gid
    return gid[~(uniform(seed, F_LAND, gid) < spec["land"])]


# per-column arrays of a ColumnSet: the column is the last axis
_COLUMN_FIELDS = ("kact", "dz", "dzc", "zc", "zi", "phi", "phi_i", "biofac", "flux_cap",
                  "bdys", "fluxes", "conc")
CHUNK_COLUMNS = 1 << 17


def make_workload(name: str, seed: int = 1234,
                  cols: Optional[np.ndarray] = None, threads: Optional[int] = None,
                  **over) -> ColumnSet:
    """One of the named workloads (``WORKLOADS``), optionally a column
    subset; keyword overrides replace entries of the workload table.

    Grids of more than CHUNK_COLUMNS columns are built in column chunks on a
    thread pool (numpy releases the interpreter lock inside its array
    operations); every value is a function of its column id alone, so the
    result is the same as one pass over all columns."""
    spec = dict(WORKLOADS[name])
    spec.update(over)
    n = spec["inum"] * spec["jnum"] if cols is None else len(cols)
    if n <= CHUNK_COLUMNS:
        return make_columns(seed=seed, cols=cols, name=name, **spec)
    import os
    from concurrent.futures import ThreadPoolExecutor
    gid = np.arange(n, dtype=np.int64) if cols is None else np.asarray(cols, dtype=np.int64)
    parts = [gid[i:i + CHUNK_COLUMNS] for i in range(0, n, CHUNK_COLUMNS)]
    workers = threads or min(len(parts), os.cpu_count() or 1)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        sets = list(ex.map(lambda c: make_columns(seed=seed, cols=c, name=name, **spec),
                           parts))
    out = sets[0]
    for f in _COLUMN_FIELDS:
        setattr(out, f, np.ascontiguousarray(
            np.concatenate([getattr(cs, f) for cs in sets], axis=-1)))
    if cols is None:
        out.inum, out.jnum = spec["inum"], spec["jnum"]
    else:
        out.inum, out.jnum = n, 1
    return out
