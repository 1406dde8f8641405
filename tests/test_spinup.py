"""Spin-up (sed_spinup, fabm_sediment_component.F90:557-632).

The column mode integrates one column of the grid alone with the spin-up
forcing and copies its profile into every other active column; on FP64 state
that column equals the oracle's 1-column run bit for bit.  The all-columns
mode equals the same number of ordinary coupling steps."""
import numpy as np
import pytest

from sedgpu import capi, synth
from sedgpu.model import NTR

pytestmark = pytest.mark.gpu


def spinup_forcing(cs, col):
    """A spin-up forcing unlike the column's own: the namelist's uniform
    bottom water and deposition fluxes of a 1-column run."""
    b = np.array(cs.bdys[:, col], dtype=np.float64)
    f = np.array(cs.fluxes[:, col], dtype=np.float64)
    b[0] = 10.0
    b[1 + 6:] = [250.0, 20.0, 5.0, 0.0, 1.0]
    f[:6] *= 1.5
    return b, f


@pytest.mark.parametrize("column", [37, -1])
def test_column_spinup_fp64_matches_oracle(oracle_mod, column):
    cs = synth.make_workload("plain_cpu_10x10")
    n = 50
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    s.set_state(cs.conc)
    col = 0 if column < 0 else column   # -1: the first column with the most layers
    b1, f1 = spinup_forcing(cs, col)
    st = s.spinup(n, capi.SED_SPINUP_COLUMN, column=column, bdys1=b1, fluxes1=f1)
    out = s.get_state()
    assert st["column_steps"] == n
    sub = cs.subset([col])
    sub.bdys = b1[:, None].copy()
    sub.fluxes = f1[:, None].copy()
    c = np.ascontiguousarray(cs.conc[:, :, [col]])
    rc, sref, _ = oracle_mod.OracleModel(sub).run(c, nsteps=n, percol=True)
    assert rc == 0
    assert st["attempts"] == sref["attempts"]
    np.testing.assert_array_equal(out[:, :, col], c[:, :, 0])
    # the profile in every other column (all have the same layers here)
    np.testing.assert_array_equal(out, np.repeat(c, cs.ncol, axis=2))
    # the handle's forcing was left as it was: one more step equals a fresh
    # handle's step from the same state
    s.step(1)
    nxt = s.get_state()
    s.close()
    t = capi.Solver(cs, precision=capi.SED_FP64)
    t.set_forcing()
    t.set_state(out)
    t.step(1)
    np.testing.assert_array_equal(nxt, t.get_state())
    t.close()


def test_column_spinup_uneven_copies_min_layers():
    cols = np.arange(0, 1024 * 1024, 1024 * 1024 // 200)[:200]
    cs = synth.make_workload("uneven_1024x1024", cols=cols)
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    col = int(np.argmax(cs.kact))
    b1, f1 = spinup_forcing(cs, col)
    s.spinup(30, capi.SED_SPINUP_COLUMN, column=-1, bdys1=b1, fluxes1=f1)
    out = s.get_state()
    s.close()
    Kc = int(cs.kact[col])
    for c in range(cs.ncol):
        K = int(cs.kact[c])
        if K == 0:
            np.testing.assert_array_equal(out[:, :, c], cs.conc[:, :, c])
            continue
        m = min(K, Kc)
        np.testing.assert_array_equal(out[:, :m, c], out[:, :m, col])
        np.testing.assert_array_equal(out[:, m:, c], cs.conc[:, m:, c])


@pytest.mark.parametrize("precision", [capi.SED_FP32, capi.SED_FP64])
def test_all_columns_spinup_equals_steps(precision):
    cols = np.arange(0, 1024 * 1024, 1024 * 1024 // 300)[:300]
    cs = synth.make_workload("uneven_1024x1024", cols=cols)
    n = 30   # one launch of 24 steps, one of 6
    a = capi.Solver(cs, precision=precision)
    a.set_forcing()
    a.set_state(cs.conc)
    sa = a.spinup(n, capi.SED_SPINUP_ALL)
    b = capi.Solver(cs, precision=precision)
    b.set_forcing()
    b.set_state(cs.conc)
    sb = b.step(n)
    np.testing.assert_array_equal(a.get_state(), b.get_state())
    np.testing.assert_array_equal(a.fluxes(), b.fluxes())
    np.testing.assert_array_equal(a.attempts(), b.attempts())
    for k in ("attempts", "accepted", "column_steps", "max_col_attempts"):
        assert sa[k] == sb[k], k
    a.close()
    b.close()


def test_spinup_argument_errors():
    cs = synth.make_workload("plain_cpu_10x10")
    s = capi.Solver(cs)
    s.set_forcing()
    with pytest.raises(capi.SedError) as e:
        s.spinup(4, capi.SED_SPINUP_ALL)          # no state yet
    assert e.value.code == capi.SED_E_STATE
    s.set_state(cs.conc)
    with pytest.raises(capi.SedError) as e:
        s.spinup(4, capi.SED_SPINUP_COLUMN)       # no spin-up forcing
    assert e.value.code == capi.SED_E_ARG
    b1, f1 = spinup_forcing(cs, 0)
    with pytest.raises(capi.SedError) as e:
        s.spinup(4, capi.SED_SPINUP_COLUMN, column=cs.ncol, bdys1=b1, fluxes1=f1)
    assert e.value.code == capi.SED_E_ARG
    s.close()
