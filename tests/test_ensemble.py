"""Ensembles: an OMEXDIA+P parameter set per column (sed_set_column_bgc).

The reference's rates take one parameter set (fabm_sed.nml); many sets run
here as the columns of one grid.  The per-column table is derived from each
column's set exactly as the handle's own Params, so:
  - a table that repeats the handle's set gives the uniform run's bits;
  - every column of an ensemble equals a run of its set alone, bit for bit;
  - FP64 state equals the oracle with the same per-column sets;
  - the ensemble spin-up (SED_SPINUP_ALL) equals ordinary steps.
The oracle side (CPU) checks the same properties of the restatement."""
import numpy as np
import pytest

from cases import small
from sedgpu import capi
from sedgpu.model import ADAPTIVE_EULER, BGC_NAMES, RUNGE_KUTTA_4

SETS = (dict(), dict(rLabile=0.1, ksO2oxic=5.0), dict(rSemilabile=0.004, rnit=50.0),
        dict(CprodMax=4000.0, PAds=0.05, NH3Ads=1.3))


def ensemble(cs, sets=SETS):
    """Columns take the sets in turn; returns the table and each column's set."""
    tab = cs.bgc_columns().copy()
    which = np.arange(cs.ncol) % len(sets)
    for c in range(cs.ncol):
        for k, v in sets[which[c]].items():
            tab[BGC_NAMES.index(k), c] = v
    return tab, which


def with_set(cs, overrides):
    out = cs.copy()
    out.bgc.update(overrides)
    out.bgc_col = None
    return out


# ---------------------------------------------------------------- CPU

def test_oracle_table_of_the_handle_set_is_the_uniform_run(oracle_mod):
    cs = small(ncol=10, K=14, seed=21)
    ref = cs.conc.copy()
    oracle_mod.OracleModel(cs).run(ref, nsteps=3, percol=True, nthreads=1)
    e = cs.copy()
    e.bgc_col = e.bgc_columns()
    got = e.conc.copy()
    oracle_mod.OracleModel(e).run(got, nsteps=3, percol=True, nthreads=1)
    np.testing.assert_array_equal(got, ref)


def test_oracle_ensemble_columns_equal_separate_runs(oracle_mod):
    cs = small(ncol=12, K=14, seed=22)
    e = cs.copy()
    e.bgc_col, which = ensemble(cs)
    got = e.conc.copy()
    oracle_mod.OracleModel(e).run(got, nsteps=3, percol=True, nthreads=2)
    for i, ov in enumerate(SETS):
        cols = np.flatnonzero(which == i)
        one = with_set(cs, ov)
        ref = one.conc.copy()
        oracle_mod.OracleModel(one).run(ref, nsteps=3, percol=True, nthreads=1)
        np.testing.assert_array_equal(got[:, :, cols], ref[:, :, cols])
    base = cs.conc.copy()
    oracle_mod.OracleModel(cs).run(base, nsteps=3, percol=True, nthreads=1)
    for i in range(1, len(SETS)):   # every other set changes its columns
        assert not np.array_equal(got[:, :, which == i], base[:, :, which == i])


# ---------------------------------------------------------------- GPU

def gpu(cs, nsteps, precision, method=ADAPTIVE_EULER, table=None):
    s = capi.Solver(cs, precision=precision)
    if table is not None:
        s.set_column_bgc(table)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(nsteps, method=method)
    out = s.get_state()
    s.close()
    return out, st


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [capi.SED_FP32, capi.SED_FP64])
def test_uniform_table_gives_the_uniform_bits(precision):
    cs = small(ncol=40, K=20, kmin=5, seed=23, land=0.1)
    ref, _ = gpu(cs, 4, precision)
    got, _ = gpu(cs, 4, precision, table=cs.bgc_columns())
    np.testing.assert_array_equal(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [ADAPTIVE_EULER, RUNGE_KUTTA_4])
def test_ensemble_columns_equal_separate_runs_fp32(method):
    cs = small(ncol=48, K=33, kmin=4, seed=24, land=0.1)   # both depth classes
    tab, which = ensemble(cs)
    got, st = gpu(cs, 3, capi.SED_FP32, method=method, table=tab)
    for i, ov in enumerate(SETS):
        ref, _ = gpu(with_set(cs, ov), 3, capi.SED_FP32, method=method)
        cols = np.flatnonzero(which == i)
        np.testing.assert_array_equal(got[:, :, cols], ref[:, :, cols])
    assert st["column_steps"] == 3 * cs.n_active


@pytest.mark.gpu
@pytest.mark.parametrize("profile3,bc4", [(True, False), (False, True), (True, True)])
def test_ensemble_with_profile3_and_cascade(profile3, bc4):
    """The ENS kernels of the other template branches: TOC-dependent
    bioturbation and the capped particulate flux cascade."""
    cs = small(ncol=24, K=20, seed=28)
    if profile3:
        cs.driver.bioturbation_profile = 3
    if bc4:   # a cap that binds, so the cascade moves material down
        cs.driver.bcup_particulate = 4
        cs.flux_cap[:] = 2e-5 * cs.dz / cs.dz[0]
        # 50x deposition with profile 3 drives the reference algorithm (and
        # the oracle) to NaN within two steps; profile 3 keeps the fluxes
        for n in range(6):
            cs.fluxes[n] *= 1.0 if profile3 else 50.0
    tab, which = ensemble(cs)
    got, _ = gpu(cs, 2, capi.SED_FP32, table=tab)
    for i, ov in enumerate(SETS):
        ref, _ = gpu(with_set(cs, ov), 2, capi.SED_FP32)
        cols = np.flatnonzero(which == i)
        np.testing.assert_array_equal(got[:, :, cols], ref[:, :, cols])


@pytest.mark.gpu
def test_ensemble_fp64_matches_oracle(oracle_mod):
    cs = small(ncol=32, K=24, kmin=3, seed=25)
    cs.bgc_col, _ = ensemble(cs)
    out, st = gpu(cs, 3, capi.SED_FP64, table=cs.bgc_col)
    ref = cs.conc.copy()
    rc, sref, _ = oracle_mod.OracleModel(cs).run(ref, nsteps=3, percol=True, nthreads=1)
    assert rc == 0
    a = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    np.testing.assert_array_equal(out[:, a], ref[:, a])
    assert st["attempts"] == sref["attempts"]


@pytest.mark.gpu
def test_ensemble_spinup_equals_steps():
    cs = small(ncol=64, K=30, seed=26)
    tab, _ = ensemble(cs)
    s = capi.Solver(cs)
    s.set_column_bgc(tab)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.spinup(60, capi.SED_SPINUP_ALL)
    spun = s.get_state()
    s.close()
    ref, _ = gpu(cs, 60, capi.SED_FP32, table=tab)
    np.testing.assert_array_equal(spun, ref)
    assert st["column_steps"] == 60 * cs.n_active


@pytest.mark.gpu
def test_ensemble_refusals_and_reset():
    cs = small(ncol=16, K=12, seed=27)
    tab, _ = ensemble(cs)
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_column_bgc(tab)
    with pytest.raises(capi.SedError) as e:
        s.get_rhs(cs.conc)
    assert e.value.code == capi.SED_E_STATE
    with pytest.raises(capi.SedError) as e:
        s.set_tuning(tile_columns=(16, 16))
    assert e.value.code == capi.SED_E_ARG
    bad = tab.copy()
    bad[0, 3] = -1.0
    with pytest.raises(capi.SedError) as e:
        s.set_column_bgc(bad)
    assert e.value.code == capi.SED_E_ARG
    s.set_column_bgc(None)          # back to the handle's set
    s.set_state(cs.conc)
    s.step(2)
    got = s.get_state()
    s.close()
    ref, _ = gpu(cs, 2, capi.SED_FP32)
    np.testing.assert_array_equal(got, ref)
    g = capi.Solver(cs, cut_scope=capi.SED_CUT_GLOBAL)
    with pytest.raises(capi.SedError) as e:
        g.set_column_bgc(tab)
    assert e.value.code == capi.SED_E_ARG
    g.close()
