"""GPU parity on the larger workloads' own column distributions, in their
developed regime (ten simulated days in, where most of the solver's work
lies: a quarter of the columns then take hundreds of substeps per coupling
step).

- 2048 x 2048 workload (30 % land, 30 layers, log-uniform deposition): its
  64 x 64 regular subsample.  The FP64 device path equals the oracle bit for
  bit over two days from the initial state; from the day-10 state one FP32
  coupling step is within 1e-3 of the oracle's.
- 1024 x 1024 uneven workload (10..60 layers, 30 % land): 3000 columns
  spread over the grid (over 2048 active), among them columns of 32..60
  layers (two layers per lane); from the day-10 state one FP32 step is
  within 1e-3 of the oracle's and one FP64 step equals it bit for bit.

The reference algorithm amplifies a rounding difference ~100x per step
(tests/test_oracle.py::test_reference_amplifies_one_ulp), so FP32 is
compared one coupling step at a time from a shared state."""
import numpy as np
import pytest

from conftest import relerr
from sedgpu import capi, synth

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-3


def grid_sample(inum, jnum, n=64):
    si, sj = inum // n, jnum // n
    i = si // 2 + si * np.arange(n)
    j = sj // 2 + sj * np.arange(n)
    return (i[None, :] + inum * j[:, None]).ravel()


def develop(cs, nsteps):
    """The state after nsteps FP32 device steps from the initial state."""
    s = capi.Solver(cs, precision=capi.SED_FP32)
    s.set_forcing()
    s.set_state(cs.conc)
    s.step(nsteps)
    out = s.get_state()
    s.close()
    return out


def one_step(cs, state, precision):
    s = capi.Solver(cs, precision=precision)
    s.set_forcing()
    s.set_state(state)
    st = s.step(1)
    out = s.get_state()
    s.close()
    return out, st


def oracle_step(oracle_mod, cs, state, nsteps=1):
    c = np.array(state, dtype=np.float64, copy=True)
    rc, st, _ = oracle_mod.OracleModel(cs).run(c, nsteps=nsteps, percol=True)
    assert rc == 0
    return c, st


def active(cs, c):
    K = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    return c[:, K]


@pytest.fixture(scope="module")
def sub2048():
    cols = grid_sample(2048, 2048)
    cs = synth.make_workload("surrogate_2048x2048", cols=cols)
    assert 0 < cs.n_active < len(cols)   # land among them
    return cs


def test_2048_subsample_fp64_bit_exact_two_days(oracle_mod, sub2048):
    cs = sub2048
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    s.set_state(cs.conc)
    s.step(48)
    out = s.get_state()
    s.close()
    ref, _ = oracle_step(oracle_mod, cs, cs.conc, nsteps=48)
    np.testing.assert_array_equal(active(cs, out), active(cs, ref))


def test_2048_subsample_fp32_day10(oracle_mod, sub2048):
    cs = sub2048
    state = develop(cs, 240)
    out, st = one_step(cs, state, capi.SED_FP32)
    ref, sref = oracle_step(oracle_mod, cs, state)
    # the developed regime: many columns take hundreds of substeps
    assert st["attempts"] / st["column_steps"] > 50, st
    assert sref["attempts"] / cs.n_active > 50, sref
    err = relerr(active(cs, out), active(cs, ref))
    assert err.max() < FP32_TOL, err


def test_uneven_1024_developed_fp32_and_fp64(oracle_mod):
    cols = np.arange(0, 1024 * 1024, (1024 * 1024) // 3000)[:3000]
    cs = synth.make_workload("uneven_1024x1024", cols=cols)
    deep = cs.kact >= 32
    assert cs.n_active >= 2048 and deep.sum() >= 1000 and (cs.kact == 0).any()
    state = develop(cs, 240)
    ref, _ = oracle_step(oracle_mod, cs, state)
    out32, st = one_step(cs, state, capi.SED_FP32)
    assert st["column_steps"] == cs.n_active
    err = relerr(active(cs, out32), active(cs, ref))
    assert err.max() < FP32_TOL, err
    # the two-layers-per-lane columns on their own
    sub = cs.subset(np.nonzero(deep)[0])
    err_deep = relerr(active(sub, out32[:, :, deep]), active(sub, ref[:, :, deep]))
    assert err_deep.max() < FP32_TOL, err_deep
    out64, _ = one_step(cs, state, capi.SED_FP64)
    np.testing.assert_array_equal(active(cs, out64), active(cs, ref))
