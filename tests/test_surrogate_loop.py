"""The surrogate coupling step (sed_step_surrogate): a network trained by the
library's kernels on solver-generated pairs proposes every column's state;
columns whose backward-Euler defect exceeds the tolerance fall back to the
plain solver.  Checked: with a tolerance nothing meets, the step is exactly
the plain solver's; with one everything meets, it is exactly the network's
proposal; in between, every column is one or the other.  The ablation test
records what the network gains over the plain method."""
import numpy as np
import pytest

from conftest import relerr
from sedgpu import capi, synth
from sedgpu import surrogate as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    cs = synth.make_workload("surrogate_200k", cols=np.arange(2048))
    pairs = S.generate_pairs(cs, nsteps=36, samples=8, warm=12, seed=3)
    nz = S.fit_normalizer(pairs, cs.kmax)
    X, Y = S.training_arrays(pairs, nz)
    sur = S.Surrogate(cs.kmax, batch=2048)
    sur.set_norm(nz)
    log = sur.train(X, Y, steps=300, lr=1e-3, log_every=100)
    assert log[-1][1] < log[0][1]
    grid = synth.make_workload("surrogate_200k", cols=np.arange(100000, 100512))
    s = capi.Solver(grid)
    s.set_forcing()
    s.set_state(grid.conc)
    s.step(24)
    state = s.get_state()
    s.close()
    yield sur, grid, state
    sur.close()


def _one_step(grid, state, sur=None, tol=None):
    s = capi.Solver(grid)
    s.set_forcing()
    s.set_state(state)
    st = s.step(1) if sur is None else S.step_surrogate(s, sur, 1, tol=tol)
    out = s.get_state()
    s.close()
    return out, st


def test_nothing_accepted_is_the_plain_step(trained):
    sur, grid, state = trained
    plain, _ = _one_step(grid, state)
    out, st = _one_step(grid, state, sur, tol=1e-30)
    assert st["surrogate_columns"] == 0
    assert st["column_steps"] == grid.n_active
    np.testing.assert_array_equal(out, plain)


def test_everything_accepted_is_the_proposal(trained):
    sur, grid, state = trained
    out, st = _one_step(grid, state, sur, tol=1e30)
    assert st["surrogate_columns"] == grid.n_active
    prop = sur.next_state(state.astype(np.float64), S.forcing_rows(grid))
    assert relerr(out, prop).max() < 5e-2


def test_warp_direct_fallback_is_the_plain_step(trained):
    sur, grid, state = trained
    plain, _ = _one_step(grid, state)
    s = capi.Solver(grid)
    s.set_tuning(tile_columns=(0, 0))
    s.set_forcing()
    s.set_state(state)
    st = S.step_surrogate(s, sur, 1, tol=1e-30)
    out = s.get_state()
    s.close()
    assert st["surrogate_columns"] == 0
    np.testing.assert_array_equal(out, plain)


def test_mixed_columns_are_one_or_the_other(trained):
    sur, grid, state = trained
    plain, _ = _one_step(grid, state)
    full, _ = _one_step(grid, state, sur, tol=1e30)
    out, st = _one_step(grid, state, sur, tol=0.3)
    same_plain = np.all(out == plain, axis=(0, 1))
    same_sur = np.all(out == full, axis=(0, 1))
    assert np.all(same_plain | same_sur)
    assert st["surrogate_columns"] == int(np.sum(same_sur & ~same_plain))


def test_ablation_gain_over_plain(trained):
    """What the trained network adds: the fraction of columns it takes at
    the 1e-3 residual tolerance and the error of its proposals against the
    plain solver.  For this reference algorithm (explicit Euler substeps in a
    limit cycle) the 1e-3 test accepts no proposal, so the gain is zero;
    the test records that instead of assuming a speed-up."""
    sur, grid, state = trained
    plain, _ = _one_step(grid, state)
    out, st = _one_step(grid, state, sur, tol=1e-3)
    frac = st["surrogate_columns"] / grid.n_active
    prop = sur.next_state(state.astype(np.float64), S.forcing_rows(grid))
    err = relerr(prop, plain)
    print(f"surrogate share at tol 1e-3: {frac:.4f}; proposal max rel err {err.max():.3e}")
    assert 0.0 <= frac <= 1.0
    # accepted columns, if any, are the network's; the rest the plain solver's
    if frac == 0.0:
        np.testing.assert_array_equal(out, plain)
