"""Shared column-set builders for the tests (small seeded cases and the
degenerate parameter sets of the known-answer tests)."""
import numpy as np

from sedgpu import synth
from sedgpu.model import BGC_DEFAULTS

ZERO_RATES = dict(rLabile=0.0, rSemilabile=0.0, rnit=0.0, rODUox=0.0,
                  PAds=0.0)


def small(ncol=16, K=12, seed=7, land=0.0, kmin=None, poc="uniform",
          total=0.18, days=1):
    kmin = K if kmin is None else kmin
    return synth.make_columns(inum=ncol, jnum=1, kmin=kmin, kmax=K,
                              total=total, land=land, poc=poc, days=days,
                              seed=seed, name=f"small{ncol}x{K}")


def no_transport(cs):
    """Switch off every diffusive transport term (rates stay)."""
    cs.driver.bioturbation = 0.0
    cs.driver.mol_diff_mode = 1
    cs.driver.mol_diff_d0 = 0.0
    return cs


def no_reactions(cs):
    cs.bgc = dict(BGC_DEFAULTS)
    cs.bgc.update(ZERO_RATES)
    return cs


def constant_rhs_case(ncol=6, K=5):
    """Reactions and diffusion off: only the particulate surface fluxes act,
    so the right-hand side is the constant fluxup/(phi dz) in the top layer
    and zero elsewhere -- the constant-rhs construction of the reference's
    solver test (src/test/test_Solver.F90:36-43), which every method must
    integrate exactly."""
    cs = no_reactions(no_transport(small(ncol, K, seed=3)))
    i = np.arange(ncol)
    for n in range(6):
        cs.fluxes[n] = (i + 1 + n) * 1.0e-6
    return cs


def decay_case(ncol=4, K=3, lam_dt=8.0, dt=3600.0):
    """Only labile detritus decays, at rate lam with lam*dt = lam_dt; O2 and
    NO3 are zero so the carbon goes to the anoxic pathway.  With the
    reference's rule (reject if c1 < 0.1 c, cut by 4) the cut sequence is
    fixed by lam_dt alone."""
    cs = no_transport(small(ncol, K, seed=5))
    cs.bgc = dict(BGC_DEFAULTS)
    cs.bgc.update(ZERO_RATES)
    cs.bgc["rLabile"] = lam_dt / dt * 86400.0
    cs.bgc["CprodMax"] = 1.0e30   # no mineralisation cap
    cs.fluxes[:] = 0.0
    cs.conc[6] = 0.0   # O2
    cs.conc[7] = 0.0   # NO3
    cs.dt = dt
    return cs


def zhang_wirtz_factor(cs, conc):
    """Bioturbation factor of profile 3 (fabm_sediment_driver.F90:624-644),
    written from the reference's formula in numpy: weighted TOC from the two
    carbon detritus pools, its dz-weighted column sum over cumdepth (depth of
    the last layer's upper interface), biomass and beta biomass^b / TOC."""
    d = cs.driver
    f1 = 1.0 / 1.2 * 12.01 / d.bioturb_dry_density / 1000.0
    f2 = 1.0 / 6.0 * 12.01 / d.bioturb_dry_density / 1000.0
    fac = np.ones((cs.kmax, cs.ncol))
    for col in range(cs.ncol):
        K = int(cs.kact[col])
        if K == 0:
            continue
        dz = cs.dz[:K, col]
        phi = cs.phi[:K, col]
        wt = f1 * phi / (1 - phi) * conc[0, :K, col] + f2 * phi / (1 - phi) * conc[1, :K, col]
        avg = np.sum(dz * wt) / np.sum(dz[:K - 1])
        zc = np.concatenate([[0.0], np.cumsum(dz)])[:K] + 0.5 * dz
        biomass = (wt * np.exp(zc * 100 * d.bioturb_k_l) * avg /
                   (d.bioturb_L1 + d.bioturb_L2 * np.exp(zc * 200 * d.bioturb_k_l)))
        fac[:K, col] = d.bioturb_beta * biomass ** d.bioturb_b / wt
    return fac


def pelagic_fields(cs, seed=5):
    """Synthetic soil-surface fields of a coupled pelagic model: temperature,
    concentration of every tracer, settling velocity of the particulates."""
    rng = np.random.default_rng(seed)
    T = cs.bdys[0] + rng.uniform(-1, 1, cs.ncol)
    surface = np.empty((11, cs.ncol))
    surface[6:] = cs.bdys[7:] * rng.uniform(0.8, 1.2, (5, cs.ncol))
    surface[:6] = rng.uniform(10, 500, (6, cs.ncol))
    velocity = -rng.uniform(1e-6, 1e-4, (11, cs.ncol))
    return T, surface, velocity
