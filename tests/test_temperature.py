"""Temperature-dependent OMEXDIA+P rates (sed_params.temp_activation).

The reference hands the column temperature to the reaction model at every
right-hand side (fabm_sediment_driver.F90:613); the model's own rate law
lives in FABM, outside the tree.  Here temp_activation > 0 multiplies the
microbial rate constants (rLabile, rSemilabile, CprodMax, rnit, rODUox) by
exp(-temp_activation (1/(T+273) - 1/288)), the Arrhenius form and 288 K
reference of the driver's bioturbation factor f_T (:648).

CPU: the oracle's rates scale by that factor and only those; at 15 degC the
factor is exactly 1, so a run there equals a run without the option.
GPU: FP64 equals the oracle bit for bit at two temperature fields (cold and
warm, varying per column), with per-column parameter sets too, and in the
column spin-up; FP32 is within 1e-3 of it; at 15 degC the option gives the
uniform run's bits."""
import numpy as np
import pytest

from cases import small
from conftest import relerr
from sedgpu import capi
from sedgpu.model import BGC_NAMES

TA = 4500.0      # the driver's activation temperature for bioturbation
FP32_TOL = 1e-3


def factor(T, ta=TA):
    return np.exp(-ta * (1.0 / (T + 273.0) - (1.0 / 288.0)))


def with_temperature(cs, T, ta=TA):
    out = cs.copy()
    out.driver.temp_activation = ta
    out.bdys = np.array(cs.bdys, dtype=np.float64, copy=True)
    out.bdys[0] = T
    return out


def fields(ncol):
    """Cold (2..10 degC) and warm (18..28 degC) temperature fields."""
    i = np.arange(ncol)
    return {"cold": 2.0 + 8.0 * i / max(ncol - 1, 1),
            "warm": 28.0 - 10.0 * i / max(ncol - 1, 1)}


def active(cs, c):
    a = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    return c[:, a]


# ---------------------------------------------------------------- CPU

def test_oracle_rates_scale_by_the_factor(oracle_mod):
    cs = small(ncol=2, K=4, seed=31)
    cell = np.array(cs.conc[:, 1, 0], dtype=np.float64)
    r1, dn1 = oracle_mod.omexdia_rates(cs.bgc, cell)
    for T in (4.0, 24.0):
        f = factor(T)
        rf, dnf = oracle_mod.omexdia_rates(cs.bgc, cell, f)
        # detritus decay, mineralisation, nitrification, ODU oxidation scale
        np.testing.assert_allclose(rf[:5], f * r1[:5], rtol=1e-13)
        assert dnf == pytest.approx(f * dn1, rel=1e-13)
        # adsorption is not microbial
        assert rf[5] == r1[5]
        assert (f > 1.0) == (T > 15.0)
    # a factor of 1 is the rate law without temperature, bit for bit
    r, _ = oracle_mod.omexdia_rates(cs.bgc, cell, 1.0)
    np.testing.assert_array_equal(r, r1)


def test_oracle_reference_temperature_is_the_plain_run(oracle_mod):
    cs = small(ncol=8, K=10, seed=32)
    cs.bdys = np.array(cs.bdys, dtype=np.float64, copy=True)
    cs.bdys[0] = 15.0
    ref = cs.conc.copy()
    oracle_mod.OracleModel(cs).run(ref, nsteps=3, percol=True, nthreads=1)
    t = with_temperature(cs, 15.0)
    got = t.conc.copy()
    oracle_mod.OracleModel(t).run(got, nsteps=3, percol=True, nthreads=1)
    np.testing.assert_array_equal(got, ref)


def test_oracle_warm_columns_mineralise_faster(oracle_mod):
    cs = small(ncol=6, K=10, seed=33)
    out = {}
    for name, T in (("cold", 5.0), ("warm", 25.0)):
        t = with_temperature(cs, T)
        c = t.conc.copy()
        rc, _, _ = oracle_mod.OracleModel(t).run(c, nsteps=4, percol=True, nthreads=1)
        assert rc == 0
        out[name] = c
    # labile detritus carbon: less left in every layer of the warm run
    assert (out["warm"][0] < out["cold"][0]).all()


# ---------------------------------------------------------------- GPU

def gpu(cs, nsteps, precision, table=None):
    s = capi.Solver(cs, precision=precision)
    if table is not None:
        s.set_column_bgc(table)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(nsteps)
    out = s.get_state()
    s.close()
    return out, st


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["cold", "warm"])
def test_fp64_matches_oracle(oracle_mod, which):
    cs = small(ncol=40, K=33, kmin=4, seed=34, land=0.1)   # both depth classes
    t = with_temperature(cs, fields(cs.ncol)[which])
    out, st = gpu(t, 3, capi.SED_FP64)
    ref = t.conc.copy()
    rc, sref, _ = oracle_mod.OracleModel(t).run(ref, nsteps=3, percol=True, nthreads=1)
    assert rc == 0
    np.testing.assert_array_equal(active(t, out), active(t, ref))
    assert st["attempts"] == sref["attempts"]
    # the option changed the run
    plain, _ = gpu(cs, 3, capi.SED_FP64)
    assert not np.array_equal(active(cs, plain), active(t, out))


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["cold", "warm"])
def test_fp32_within_tolerance(oracle_mod, which):
    cs = small(ncol=40, K=30, kmin=6, seed=35, land=0.1)
    t = with_temperature(cs, fields(cs.ncol)[which])
    out, _ = gpu(t, 1, capi.SED_FP32)
    ref = t.conc.copy()
    oracle_mod.OracleModel(t).run(ref, nsteps=1, percol=True, nthreads=1)
    err = relerr(active(t, out), active(t, ref))
    assert err.max() < FP32_TOL, err


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [capi.SED_FP32, capi.SED_FP64])
def test_reference_temperature_gives_the_uniform_bits(precision):
    cs = small(ncol=24, K=20, kmin=5, seed=36, land=0.1)
    cs.bdys = np.array(cs.bdys, dtype=np.float64, copy=True)
    cs.bdys[0] = 15.0
    ref, _ = gpu(cs, 3, precision)
    got, _ = gpu(with_temperature(cs, 15.0), 3, precision)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.gpu
def test_with_column_sets_fp64_matches_oracle(oracle_mod):
    cs = small(ncol=32, K=24, kmin=3, seed=37)
    t = with_temperature(cs, fields(cs.ncol)["warm"])
    tab = t.bgc_columns().copy()
    tab[BGC_NAMES.index("rLabile"), ::2] = 0.1
    tab[BGC_NAMES.index("rnit"), 1::3] = 50.0
    t.bgc_col = tab
    out, st = gpu(t, 3, capi.SED_FP64, table=tab)
    ref = t.conc.copy()
    rc, sref, _ = oracle_mod.OracleModel(t).run(ref, nsteps=3, percol=True, nthreads=1)
    assert rc == 0
    np.testing.assert_array_equal(active(t, out), active(t, ref))
    assert st["attempts"] == sref["attempts"]


@pytest.mark.gpu
def test_column_spinup_fp64_matches_oracle(oracle_mod):
    cs = with_temperature(small(ncol=12, K=16, seed=38), fields(12)["cold"])
    col, n = 5, 30
    b1 = np.array(cs.bdys[:, col], dtype=np.float64)
    f1 = np.array(cs.fluxes[:, col], dtype=np.float64)
    b1[0] = 22.0   # the spin-up temperature, not the column's own
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.spinup(n, capi.SED_SPINUP_COLUMN, column=col, bdys1=b1, fluxes1=f1)
    out = s.get_state()
    # the handle's own rates were put back: one more step equals a fresh
    # handle's step from the same state
    s.step(1)
    nxt = s.get_state()
    s.close()
    sub = cs.subset([col])
    sub.bdys = b1[:, None].copy()
    sub.fluxes = f1[:, None].copy()
    c = np.ascontiguousarray(cs.conc[:, :, [col]])
    rc, sref, _ = oracle_mod.OracleModel(sub).run(c, nsteps=n, percol=True)
    assert rc == 0
    assert st["attempts"] == sref["attempts"]
    np.testing.assert_array_equal(out[:, :, col], c[:, :, 0])
    t = capi.Solver(cs, precision=capi.SED_FP64)
    t.set_forcing()
    t.set_state(out)
    t.step(1)
    np.testing.assert_array_equal(nxt, t.get_state())
    t.close()


@pytest.mark.gpu
def test_refusals():
    cs = with_temperature(small(ncol=8, K=10, seed=39), 10.0)
    with pytest.raises(capi.SedError):
        capi.Solver(cs, cut_scope=capi.SED_CUT_GLOBAL)
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    with pytest.raises(capi.SedError):
        s.get_rhs(cs.conc)
    with pytest.raises(capi.SedError):
        s.set_tuning(tile_columns=(8, 8))
    s.close()
