"""The surrogate coupling step (sed_step_surrogate).  Each step gates every
column with its first plain attempt (the whole step at once); the network
proposes states for the columns that attempt rejects, a residual test with
the plain right-hand side takes or rejects each proposal, and the rest are
stepped by the plain solver.

Checked: with tol = 0 the step is exactly the plain solver's; with a
tolerance everything meets, gated-out columns are exactly the plain step's
and the others exactly the network's proposal; in between, every column is
one or the other; and the trained network beats an untrained one on held-out
rows."""
import numpy as np
import pytest

from conftest import relerr
from sedgpu import capi, synth
from sedgpu import surrogate as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    train = synth.make_workload("surrogate_200k", cols=np.arange(4096))
    test = synth.make_workload("surrogate_200k", cols=np.arange(150000, 151024))
    sur, rep = S.train_surrogate(train, test, nsteps=48, every=3, warm=12, train_steps=400,
                                 batch=2048, log_every=100, test_nsteps=36)
    grid = synth.make_workload("surrogate_200k", cols=np.arange(100000, 100512))
    s = capi.Solver(grid)
    s.set_forcing()
    s.set_state(grid.conc)
    s.step(24)
    state = s.get_state()
    s.close()
    yield sur, rep, grid, state
    sur.close()


def _one_step(grid, state, sur=None, tol=None):
    s = capi.Solver(grid)
    s.set_forcing()
    s.set_state(state)
    st = s.step(1) if sur is None else S.step_surrogate(s, sur, 1, tol=tol)
    out = s.get_state()
    att = s.attempts()
    s.close()
    return out, st, att


def test_training_rows_and_loss(trained):
    sur, rep, grid, state = trained
    assert rep["rows"] > 0 and not rep["rows_full"]
    log = rep["loss_log"]
    assert log[-1][1] < 0.5 * log[0][1], log


def test_nothing_accepted_is_the_plain_step(trained):
    sur, rep, grid, state = trained
    plain, _, att = _one_step(grid, state)
    out, st, _ = _one_step(grid, state, sur, tol=0.0)
    assert st["surrogate_columns"] == 0
    assert st["column_steps"] == grid.n_active
    # some columns are gated out, some go through the network
    assert 0 < np.sum(att[grid.kact > 0] > 1) < grid.n_active
    np.testing.assert_array_equal(out, plain)


def test_gemm_engine_step_takes_the_host_count_path(trained):
    """With the mma.sync network the step reads the gate's count on the host
    (its GEMM grids need it): tol 0 is still the plain step bit for bit, and
    a tolerance everything meets takes exactly the gated-out columns."""
    sur, rep, grid, state = trained
    plain, _, att = _one_step(grid, state)
    sur.lib.sed_sur_set_tensor_cores(sur.h, 0)
    try:
        out, st, _ = _one_step(grid, state, sur, tol=0.0)
        np.testing.assert_array_equal(out, plain)
        _, st, _ = _one_step(grid, state, sur, tol=1e30)
        assert st["surrogate_columns"] == int(np.sum((att > 1) & (grid.kact > 0)))
    finally:
        sur.lib.sed_sur_set_tensor_cores(sur.h, 1)


def test_everything_accepted(trained):
    sur, rep, grid, state = trained
    plain, _, att = _one_step(grid, state)
    out, st, _ = _one_step(grid, state, sur, tol=1e30)
    heavy = (att > 1) & (grid.kact > 0)
    cheap = (att == 1) & (grid.kact > 0)
    assert st["surrogate_columns"] == int(heavy.sum())
    assert st["column_steps"] == grid.n_active
    # gated-out columns: the plain step, bit for bit
    np.testing.assert_array_equal(out[:, :, cheap], plain[:, :, cheap])
    # the others: the network's proposal (host rows vs device rows differ in
    # the BF16 rounding of the features)
    prop = sur.next_state(state[:, :, heavy].astype(np.float64),
                          S.forcing_rows(grid)[:, heavy])
    assert relerr(out[:, :, heavy], prop).max() < 5e-2


def test_mixed_columns_are_one_or_the_other(trained):
    sur, rep, grid, state = trained
    plain, _, _ = _one_step(grid, state)
    full, _, _ = _one_step(grid, state, sur, tol=1e30)
    # a tolerance between the proposals' smallest and largest residuals
    out, st, _ = _one_step(grid, state, sur, tol=30.0)
    same_plain = np.all(out == plain, axis=(0, 1))
    same_sur = np.all(out == full, axis=(0, 1))
    assert np.all(same_plain | same_sur)
    assert st["surrogate_columns"] == int(np.sum(same_sur & ~same_plain))


def test_trained_network_beats_untrained(trained):
    """What training adds: on held-out rows the trained network's error is
    far below that of the same network at its initial weights."""
    sur, rep, grid, state = trained
    ho = rep["held_out"]
    fresh = S.Surrogate(grid.kmax, batch=2048, seed=11)
    fresh.set_norm(sur.norm)
    test = synth.make_workload("surrogate_200k", cols=np.arange(150000, 151024))
    rows = S.collect_rows(test, 36, 3, warm=12, c0=sur.norm.c0)
    base = S.evaluate(fresh, rows)
    fresh.close()
    print(f"held-out mse trained {ho['mse_standardised']:.4f} untrained "
          f"{base['mse_standardised']:.4f}; median row max rel err trained "
          f"{ho['row_max_rel_err_quantiles'][50]:.3e} untrained "
          f"{base['row_max_rel_err_quantiles'][50]:.3e}")
    assert ho["mse_standardised"] < 0.5 * base["mse_standardised"]
    assert ho["row_max_rel_err_quantiles"][50] < base["row_max_rel_err_quantiles"][50]


@pytest.fixture(scope="module")
def segmented(trained):
    """A grid of several column segments (the drop-in call's chunks) ten
    coupling steps in."""
    grid = synth.make_workload("surrogate_200k", cols=np.arange(100000, 140000))
    s = capi.Solver(grid)
    s.set_forcing()
    s.set_state(grid.conc)
    s.step(10)
    state = s.get_state()
    s.close()
    return grid, state


@pytest.mark.parametrize("tol", [0.0, 1e-3, 1e30])
def test_drop_in_call_equals_device_resident_step(trained, segmented, tol):
    """sed_ode_solver_surrogate (host arrays, copies pipelined over the
    column segments) equals sed_set_state + sed_step_surrogate +
    sed_get_state bit for bit: state, surface fluxes and statistics."""
    sur = trained[0]
    grid, state = segmented
    a = capi.Solver(grid)
    a.set_forcing()
    a.set_state(state)
    sa = S.step_surrogate(a, sur, 1, tol=tol)
    out_a = a.get_state()
    fl_a = a.fluxes()
    a.close()
    b = capi.Solver(grid)
    assert b.tuning().segments > 1
    conc = np.array(state, dtype=np.float64, copy=True)
    fluxes = np.array(grid.fluxes, dtype=np.float64, copy=True)
    sb = S.ode_solver_surrogate(b, sur, conc, grid.bdys, fluxes, tol=tol)
    b.close()
    np.testing.assert_array_equal(conc, out_a)
    np.testing.assert_array_equal(fluxes, fl_a)
    for k in ("surrogate_columns", "column_steps", "attempts", "accepted"):
        assert sa[k] == sb[k], k
    if tol == 1e30:
        assert sb["surrogate_columns"] > 0
