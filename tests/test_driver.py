"""The driver-facing interface of ``sedgpu.driver``.

CPU: the set-up routines (init_grid, initialize, update_porosity,
init_concentrations) against the reference's formulas, restated below as the
Fortran loops of src/drivers/fabm_sediment_driver.F90 in the reference's
operation order, so the comparisons are exact.

GPU: a caller's sequence -- TypeSed, initialize, init_concentrations,
ode_solver, get_rhs -- against the oracle on the same columns.
"""
import math

import numpy as np
import pytest

from sedgpu import capi, driver, synth
from sedgpu.model import ADAPTIVE_EULER, NTR, RUNGE_KUTTA_4


def _grid_loops(K, dzmin):
    """init_grid (fabm_sediment_driver.F90:146-168), element by element."""
    fac = 0.18 / ((K + 1) / 2.0 * dzmin) - 1.0
    dz, zc, zi = [0.0] * K, [0.0] * K, [0.0] * (K + 1)
    for k in range(1, K + 1):
        dz[k - 1] = (1.0 + (fac - 1.0) * (k - 1) / (K - 1)) * dzmin
        zc[k - 1] = zi[k - 1] + 0.5 * dz[k - 1]
        zi[k] = zi[k - 1] + dz[k - 1]
    dzc = [zc[k] - zc[k - 1] for k in range(1, K)]
    return [np.array(a) for a in (dz, zc, zi, dzc)]


def _initialize_loops(zc, zi, dz, nml):
    """Porosity, flux cap and bioturbation factor of one column
    (fabm_sediment_driver.F90:279-304)."""
    K = len(zc)
    phi, cap, bf = [0.0] * K, [0.0] * K, [1.0] * K
    for k in range(1, K + 1):
        phi[k - 1] = nml["porosity_max"] * (1.0 - nml["porosity_fac"] * zc[k - 1])
        cap[k - 1] = nml["pom_flux_max"] / 86400.0 * (1.0 - phi[k - 1]) * dz[k - 1]
        if k > 2 and cap[k - 1] > cap[k - 2]:
            cap[k - 1] = cap[k - 2]
        if nml["bioturbation_profile"] == 1:
            bf[k - 1] = max(nml["bioturbation_min"] / nml["bioturbation"],
                            max(nml["bioturbation_depth"] - 100.0 * zi[k - 1], 0.0)
                            / nml["bioturbation_depth"])
        elif nml["bioturbation_profile"] == 2:
            bf[k - 1] = math.exp(-100.0 * zi[k - 1] / nml["bioturbation_depth"])
    return np.array(phi), np.array(cap), np.array(bf)


NML = dict(diffusivity=0.9, bioturbation=0.9, bioturbation_depth=5.0,
           bioturbation_min=0.2, porosity_max=0.7, porosity_fac=0.9,
           pom_flux_max=2.0e4)


def _sed(inum=3, jnum=2, knum=12, dzmin=0.004, nml=None, masked=None):
    sed = driver.TypeSed(inum, jnum, knum)
    driver.init_grid(sed.grid, dzmin)
    if masked is not None:
        sed.mask[...] = masked
    driver.initialize(sed, nml)
    return sed


@pytest.mark.parametrize("K,dzmin", [(2, 0.005), (12, 0.004), (30, 0.005), (60, 0.001)])
def test_init_grid_matches_reference_loop(oracle_mod, K, dzmin):
    g = driver.SedGrid(3, 2, K)
    driver.init_grid(g, dzmin)
    dz, zc, zi, dzc = _grid_loops(K, dzmin)
    for got, ref in ((g.dz, dz), (g.zc, zc), (g.zi, zi), (g.dzc, dzc)):
        assert got.shape == (ref.size, 6)
        for c in range(6):
            np.testing.assert_array_equal(got[:, c], ref)
    # the oracle's C restatement of the same grid
    odz, ozc, ozi, odzc = oracle_mod.init_grid_linear(K, dzmin)
    np.testing.assert_array_equal(g.dz[:, 0], odz)
    np.testing.assert_array_equal(g.zi[:, 0], ozi)
    np.testing.assert_array_equal(g.dzc[:, 0], odzc)
    # the grid reaches 0.18 K / (K + 1) m and grows linearly to fac * dzmin
    assert g.zi[-1, 0] == pytest.approx(0.18 * K / (K + 1), rel=1e-12)
    fac = 0.18 / ((K + 1) / 2.0 * dzmin) - 1.0
    assert g.dz[-1, 0] == pytest.approx(fac * dzmin, rel=1e-12)


@pytest.mark.parametrize("profile", [1, 2, 3])
def test_initialize_matches_reference_loop(profile):
    nml = dict(NML, bioturbation_profile=profile)
    sed = _sed(nml=nml)
    g = sed.grid
    phi, cap, bf = _initialize_loops(g.zc[:, 0], g.zi[:, 0], g.dz[:, 0], nml)
    for c in range(sed.ncol):
        np.testing.assert_array_equal(sed.porosity[:, c], phi)
        np.testing.assert_array_equal(sed.flux_cap[:, c], cap)
        np.testing.assert_array_equal(sed.bioturbation_factor[:, c], bf)
        np.testing.assert_array_equal(sed.intf_porosity[:, c],
                                      synth.interface_porosity(phi))
    assert sed.bioturbation_profile == profile
    # the cap never grows downwards from the second layer on
    assert np.all(np.diff(sed.flux_cap[1:], axis=0) <= 0.0)


def test_initialize_namelist_entries():
    sed = _sed(nml=dict(distributed_pom_flux=True, bioturb_k_l=0.2, bioturb_b=2.0,
                        bioturbation_profile=3, diffusivity=1.5))
    assert sed.bcup_particulate_variables == 4
    assert sed.diffusivity == 1.5
    drv = sed.to_columns().driver
    assert drv.bioturbation_profile == 3
    assert drv.bioturb_k_l == 0.2 and drv.bioturb_b == 2.0
    assert drv.bioturb_L1 == 0.2 and drv.bioturb_dry_density == 1000.0
    assert drv.bcup_particulate == 4 and drv.diffusivity == 1.5
    assert _sed().bcup_particulate_variables == 1
    with pytest.raises(ValueError, match="unknown sed_nml"):
        _sed(nml=dict(porosity_maximum=0.8))


def _tail_mask(knum, kact):
    """Mask of a masked tail per column: layers at and below kact[c]."""
    return (np.arange(knum)[:, None] >= np.asarray(kact)[None, :]).astype(np.int32)


def test_update_porosity_mask_and_interface():
    K = 12
    kact = [12, 7, 0, 12, 1, 5]
    sed = _sed(knum=K, masked=_tail_mask(K, kact))
    phi0, _, _ = _initialize_loops(sed.grid.zc[:, 0], sed.grid.zi[:, 0],
                                   sed.grid.dz[:, 0], dict(NML, bioturbation_profile=1))
    np.testing.assert_array_equal(sed.kact(), kact)
    for c, ka in enumerate(kact):
        want = np.where(np.arange(K) >= ka, 1.0, phi0)
        np.testing.assert_array_equal(sed.porosity[:, c], want)
        wi = [want[0]] + [0.5 * (want[k - 1] + want[k]) for k in range(1, K)]
        np.testing.assert_array_equal(sed.intf_porosity[:, c], wi)


def test_update_porosity_from_surface():
    K = 10
    sed = _sed(knum=K, masked=_tail_mask(K, [10, 10, 6, 10, 10, 10]))
    g = sed.grid
    sed.porosity = sed.porosity.copy()
    sed.porosity[0] = np.array([0.55, 0.6, 0.65, 0.7, 0.75, 0.8])
    sed.porosity_fac = 1.3
    sed.pom_flux_max = 1.5e4
    driver.update_porosity(sed, from_surface=True)
    for c in range(sed.ncol):
        phi = [sed.porosity[0, c]] + [0.0] * (K - 1)
        for k in range(2, K + 1):   # :409-413
            phi[k - 1] = phi[0] * (1.0 - 1.3 * (g.zc[k - 1, c] - g.zc[0, c]))
        cap = [0.0] * K
        for k in range(1, K + 1):   # :415-427, before the mask
            cap[k - 1] = 1.5e4 / 86400.0 * (1.0 - phi[k - 1]) * g.dz[k - 1, c]
            if k > 2 and cap[k - 1] > cap[k - 2]:
                cap[k - 1] = cap[k - 2]
        phi = [1.0 if sed.mask[k, c] > 0 else phi[k] for k in range(K)]
        np.testing.assert_array_equal(sed.porosity[:, c], phi)
        np.testing.assert_array_equal(sed.flux_cap[:, c], cap)
        np.testing.assert_array_equal(sed.intf_porosity[:, c], synth.interface_porosity(np.array(phi)))
    # without from_surface the profile below the top stays as it was
    before = sed.porosity.copy()
    sed.porosity[0] += 0.01
    driver.update_porosity(sed)
    np.testing.assert_array_equal(sed.porosity[1:], before[1:])


def _initial_values():
    return np.array([4.0e3, 4.0e3, 0.92e3, 0.04e3, 4.0e1, 10.0,
                     250.0, 20.0, 5.0, 0.0, 1.0])


def test_init_concentrations():
    K = 8
    kact = [8, 3, 0, 8, 1, 6]
    sed = _sed(knum=K, masked=_tail_mask(K, kact))
    iv = _initial_values()
    driver.init_concentrations(sed, iv)
    assert sed.conc.shape == (NTR, K, sed.ncol) and sed.conc.flags.c_contiguous
    for n in range(NTR):   # :455-467
        for k in range(K):
            for c in range(sed.ncol):
                want = 1.0e20 if sed.mask[k, c] > 0 else iv[n] / sed.porosity[k, c]
                assert sed.conc[n, k, c] == want
    # update_porosity(reinitialize_concentrations) reuses the last values
    sed.porosity = sed.porosity.copy()
    sed.porosity[0] = 0.5
    driver.update_porosity(sed, reinitialize_concentrations=True)
    np.testing.assert_array_equal(sed.conc[:, 0, 0], iv / 0.5)
    with pytest.raises(ValueError):
        driver.init_concentrations(sed, iv[:5])
    fresh = _sed(knum=K)
    with pytest.raises(ValueError, match="no initial values"):
        driver.init_concentrations(fresh)


# ---------------------------------------------------------------- GPU path

def _coupled_sed(profile, precision):
    """A 5 x 3 grid of 16 layers with masked tails, one land column, the
    namelist defaults but for the bioturbation profile, bottom water and
    POC fluxes in the ranges of the synthetic workloads."""
    K, ncol = 16, 15
    kact = np.array([16, 16, 11, 0, 16, 7, 16, 16, 2, 16, 13, 16, 16, 5, 16])
    sed = _sed(inum=5, jnum=3, knum=K, dzmin=0.003, masked=_tail_mask(K, kact),
               nml=dict(bioturbation_profile=profile))
    sed.precision = precision
    driver.init_concentrations(sed, _initial_values())
    col = np.arange(ncol)
    sed.bdys[0] = 5.0 + 0.5 * col                       # temperature
    sed.bdys[1 + 6] = 200.0 + 5.0 * col                 # O2
    sed.bdys[1 + 7] = 10.0 + col                        # NO3
    sed.bdys[1 + 8] = 3.0                               # NH4
    sed.bdys[1 + 10] = 0.8                              # PO4
    poc = (5.0 + 3.0 * col) / 86400.0
    sed.fluxes[0] = sed.fluxes[1] = 0.5 * poc
    sed.fluxes[2] = sed.fluxes[3] = 0.5 * poc * 16.0 / 106.0
    sed.fluxes[4] = poc / 106.0
    return sed


@pytest.mark.gpu
@pytest.mark.parametrize("profile", [1, 2, 3])
@pytest.mark.parametrize("method", [ADAPTIVE_EULER, RUNGE_KUTTA_4])
def test_driver_ode_solver_fp64_matches_oracle(oracle_mod, profile, method):
    """Bit for bit for the static profiles.  Profile 3 takes CUDA's pow,
    which may differ from the CPU's in the last bit: 1e-9 relative there."""
    sed = _coupled_sed(profile, capi.SED_FP64)

    def same(got, want):
        if profile != 3:
            np.testing.assert_array_equal(got, want)
        else:
            np.testing.assert_allclose(got, want, rtol=1e-9, atol=0.0)

    cs = sed.to_columns()
    ref = np.ascontiguousarray(sed.conc.copy())
    om = oracle_mod.OracleModel(cs)
    fl_ref = sed.fluxes.copy()
    dt = 3600.0 if method == ADAPTIVE_EULER else 60.0
    for _ in range(4):
        driver.ode_solver(sed, dt, method)
        rc, _, fl_ref = om.run(ref, nsteps=1, dt=dt, method=method, fluxes=fl_ref)
        assert rc == 0
        act = np.arange(sed.knum)[:, None] < sed.kact()[None, :]
        same(sed.conc[:, act], ref[:, act])
    # masked cells keep the missing value
    assert np.all(sed.conc[:, sed.mask > 0] == 1.0e20)
    rhs = driver.get_rhs(sed)
    rref, _, _ = om.get_rhs(sed.conc)
    scale = np.abs(rref[:, act]).max(axis=1, keepdims=True)
    if profile != 3:
        np.testing.assert_array_equal(rhs[:, act], rref[:, act])
    else:
        assert np.max(np.abs(rhs[:, act] - rref[:, act]) / scale) < 1e-13
    sed.solver().close()


@pytest.mark.gpu
def test_driver_ode_solver_fp32_close_to_oracle(oracle_mod):
    sed = _coupled_sed(1, capi.SED_FP32)
    sed.atol = synth.ATOL
    cs = sed.to_columns()
    assert cs.driver.atol == synth.ATOL
    ref = np.ascontiguousarray(sed.conc.copy())
    driver.ode_solver(sed, 3600.0, ADAPTIVE_EULER)
    rc, _, _ = oracle_mod.OracleModel(cs).run(ref, nsteps=1, dt=3600.0,
                                              method=ADAPTIVE_EULER)
    assert rc == 0
    act = np.arange(sed.knum)[:, None] < sed.kact()[None, :]
    got, want = sed.conc[:, act], ref[:, act]
    scale = np.abs(want).max(axis=1, keepdims=True) + 1e-30
    assert np.max(np.abs(got - want) / scale) < 1e-3
    sed.solver().close()


def test_last_min_dt_diagnostics_mirror():
    """type_rhs_driver's last_min_dt starts at the default-real 1e20 and the
    cell at -99 (solver_library.F90:44-45); a call lowers it to the grid's
    smallest accepted substep, at (i, j) of the first column in Fortran
    order that took it, and a later call with larger substeps keeps it."""
    from sedgpu import driver
    sed = driver.TypeSed(4, 3, 10)
    assert sed.last_min_dt == float(np.float32(1e20))
    assert sed.last_min_dt_grid_cell == [-99, -99, -99, -99]
    assert sed.adaptive_solver_diagnostics is False
    md = np.full(12, 900.0)
    md[[2, 7]] = 0.0          # land, or no accepted substep
    md[6] = 56.25             # col 6 = (i 3, j 2)
    md[9] = 56.25
    driver.update_min_dt(sed, md)
    assert sed.last_min_dt == 56.25 and sed.last_min_dt_grid_cell == [3, 2, -99, -99]
    driver.update_min_dt(sed, np.full(12, 225.0))
    assert sed.last_min_dt == 56.25 and sed.last_min_dt_grid_cell == [3, 2, -99, -99]
    driver.update_min_dt(sed, np.zeros(12))
    assert sed.last_min_dt == 56.25
