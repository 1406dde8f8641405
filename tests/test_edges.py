"""Edge cases of the sediment path on the GPU, FP64 state against the oracle
bit for bit: the depth-class boundaries (1, 31, 32, 33, 63, 64, 65 and the
maximum 127 active layers, where a warp's lanes hold one, two or four
layers), a single
column, a grid without any active column, and the column counts that leave
partial warps, tiles and segments."""
import numpy as np
import pytest

from cases import small
from sedgpu import capi
from sedgpu.model import ADAPTIVE_EULER, RUNGE_KUTTA_4

pytestmark = pytest.mark.gpu


def run_both(oracle_mod, cs, nsteps=3, method=ADAPTIVE_EULER, precision=capi.SED_FP64):
    s = capi.Solver(cs, precision=precision)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(nsteps, method=method)
    out = s.get_state()
    fl = s.fluxes()
    s.close()
    ref = cs.conc.copy()
    rc, sref, fref = oracle_mod.OracleModel(cs).run(ref, nsteps=nsteps, method=method,
                                                    percol=True, nthreads=1)
    assert rc == 0
    return out, fl, st, ref, fref, sref


def active(cs):
    return np.arange(cs.kmax)[:, None] < cs.kact[None, :]


@pytest.mark.parametrize("K", [1, 2, 31, 32, 33, 63, 64, 65, 127])
def test_depth_class_edges(oracle_mod, K):
    cs = small(ncol=37, K=K, kmin=1, land=0.2, seed=11)
    kact = cs.kact.copy()
    for i, k in enumerate((K, 0, min(K, 31), min(K, 32), 1, min(K, 63), min(K, 64))):
        kact[i] = k
    cs.kact = kact
    out, fl, st, ref, fref, sref = run_both(oracle_mod, cs)
    a = active(cs)
    np.testing.assert_array_equal(out[:, a], ref[:, a])
    np.testing.assert_array_equal(fl[:, cs.kact > 0], fref[:, cs.kact > 0])
    assert st["attempts"] == sref["attempts"]
    assert st["column_steps"] == 3 * int(np.count_nonzero(cs.kact))
    # FP32 state on the same columns stays close
    out32, _, _, _, _, _ = run_both(oracle_mod, cs, nsteps=1, precision=capi.SED_FP32)
    ref1 = cs.conc.copy()
    oracle_mod.OracleModel(cs).run(ref1, nsteps=1, percol=True, nthreads=1)
    for n in range(ref1.shape[0]):
        r = ref1[n][a]
        floor = 1e-4 * max(np.abs(r).max(), 1e-300)
        assert np.max(np.abs(out32[n][a] - r) / (np.abs(r) + floor)) < 1e-3


def test_single_column(oracle_mod):
    cs = small(ncol=1, K=20, seed=4)
    out, fl, st, ref, fref, _ = run_both(oracle_mod, cs, nsteps=4)
    np.testing.assert_array_equal(out[:, active(cs)], ref[:, active(cs)])
    np.testing.assert_array_equal(fl, fref)
    assert st["column_steps"] == 4


def test_grid_without_active_columns():
    cs = small(ncol=8, K=10, land=1.0)
    assert cs.n_active == 0
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(2)
    assert st["column_steps"] == 0 and st["attempts"] == 0
    np.testing.assert_array_equal(s.get_state(), cs.conc)
    c = cs.conc.copy()
    fl = cs.fluxes.copy()
    s.ode_solver(c, cs.bdys, fl, cs.dt, ADAPTIVE_EULER)
    np.testing.assert_array_equal(c, cs.conc)
    s.close()


@pytest.mark.parametrize("ncol", [31, 33, 65, 1000])
def test_partial_warps_tiles_and_segments(oracle_mod, ncol):
    cs = small(ncol=ncol, K=12, kmin=3, land=0.1, seed=ncol)
    out, fl, st, ref, fref, _ = run_both(oracle_mod, cs, nsteps=2, method=RUNGE_KUTTA_4)
    a = active(cs)
    np.testing.assert_array_equal(out[:, a], ref[:, a])
    np.testing.assert_array_equal(fl[:, cs.kact > 0], fref[:, cs.kact > 0])


def test_deep_columns_rhs_and_fixed_methods(oracle_mod):
    """Columns of 64..127 layers (four per lane): the right-hand side, RK4
    and the drop-in call equal the oracle in FP64 bit for bit, beside
    shallower columns on the same grid."""
    cs = small(ncol=40, K=100, kmin=40, land=0.1, seed=5)
    assert (cs.kact > 63).any() and ((cs.kact > 31) & (cs.kact <= 63)).any()
    a = active(cs)
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    rhs, fl = s.get_rhs(cs.conc)
    s.close()
    ref, fref, _ = oracle_mod.OracleModel(cs).get_rhs(cs.conc)
    np.testing.assert_array_equal(rhs[:, a], ref[:, a])
    np.testing.assert_array_equal(fl[:, cs.kact > 0], fref[:, cs.kact > 0])
    out, _, _, sref_state, _, _ = run_both(oracle_mod, cs, nsteps=2, method=RUNGE_KUTTA_4)
    np.testing.assert_array_equal(out[:, a], sref_state[:, a])
    # the drop-in call (host arrays in and out)
    s = capi.Solver(cs, precision=capi.SED_FP64)
    c = cs.conc.copy()
    f = cs.fluxes.copy()
    s.ode_solver(c, cs.bdys, f, cs.dt, ADAPTIVE_EULER)
    s.close()
    r1 = cs.conc.copy()
    oracle_mod.OracleModel(cs).run(r1, nsteps=1, percol=True, nthreads=1)
    np.testing.assert_array_equal(c[:, a], r1[:, a])


def test_deep_columns_refuse_per_column_sets():
    """Per-column parameter sets step only columns of at most 63 layers."""
    cs = small(ncol=8, K=80, seed=2)
    s = capi.Solver(cs)
    with pytest.raises(capi.SedError):
        s.set_column_bgc(cs.bgc_columns().copy())
    s.close()
