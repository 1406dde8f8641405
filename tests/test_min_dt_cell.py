"""type_rhs_driver's last_min_dt and last_min_dt_grid_cell on the device
(solver_library.F90:43-45, :129-136): with adaptive_solver_diagnostics set,
the grid-wide cut records every accepted substep smaller than the smallest
so far, and the (i, j, k, n) of the smallest relative change (c1 - c) / c in
it, as gfortran's MINLOC takes it (first in element order, NaN skipped).
The FP64 device path equals the oracle's orc_ode_solver_diag call for call,
on a grid with land columns (zero state: NaN quotients) and masked bottom
tails."""
import numpy as np
import pytest

from sedgpu import capi, synth

pytestmark = pytest.mark.gpu


def diag_case():
    cs = synth.make_columns(inum=5, jnum=3, kmin=6, kmax=10, total=0.18, land=0.25,
                            poc="loguniform", days=1, seed=41, name="diag5x3")
    cs.conc[:, :, cs.kact == 0] = 0.0
    cs.driver.adaptive_solver_diagnostics = True
    return cs


def test_fp64_matches_oracle_call_for_call(oracle_mod):
    cs = diag_case()
    s = capi.Solver(cs, precision=capi.SED_FP64, cut_scope=capi.SED_CUT_GLOBAL, epilogue=False)
    s.set_forcing()
    s.set_state(cs.conc)
    last, cell = s.min_dt_grid_cell()
    assert cell == (-99, -99, -99, -99) and last == float(np.float32(1e20))
    om = oracle_mod.OracleModel(cs)
    d = om.new_diag()
    ref = cs.conc.copy()
    seen = set()
    for step in range(6):
        s.step(1)
        rc, _, _ = om.ode_solver_diag(ref, d)
        assert rc == 0
        last, cell = s.min_dt_grid_cell()
        assert last == d.last_min_dt and cell == d.cell(), (step, cell, d.cell())
        seen.add(cell)
    np.testing.assert_array_equal(s.get_state(), ref)
    s.close()
    assert last < cs.dt                     # the grid did cut
    i, j, k, n = cell
    assert cs.kact[(i - 1) + cs.inum * (j - 1)] >= k   # an active cell


def test_requires_grid_wide_cut_and_the_flag():
    cs = diag_case()
    s = capi.Solver(cs)                     # per-column cuts
    with pytest.raises(capi.SedError):
        s.min_dt_grid_cell()
    s.close()
    cs.driver.adaptive_solver_diagnostics = False
    s = capi.Solver(cs, cut_scope=capi.SED_CUT_GLOBAL)
    with pytest.raises(capi.SedError):
        s.min_dt_grid_cell()
    s.close()
