"""CPU tests of the FP64 oracle: known-answer tests of the stepper built from
the reference's own solver test and source, conservation and steady-state
properties of the transport, and the golden regression vectors."""
import os

import numpy as np
import pytest

from cases import constant_rhs_case, decay_case, no_reactions, no_transport, small
from sedgpu import synth
from sedgpu.model import (ADAPTIVE_EULER, EULER, NTR, RUNGE_KUTTA_4,
                          RUNGE_KUTTA_4_38)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("method", [EULER, RUNGE_KUTTA_4, ADAPTIVE_EULER,
                                    RUNGE_KUTTA_4_38])
@pytest.mark.parametrize("percol", [True, False])
def test_constant_rhs_exact(oracle_mod, method, percol):
    # src/test/test_Solver.F90:36-43: a constant rhs is integrated exactly
    cs = constant_rhs_case()
    om = oracle_mod.OracleModel(cs)
    c0 = cs.conc.copy()
    rhs, _, _ = om.get_rhs(c0)
    assert np.all(rhs[:, 1:, :] == 0.0)
    assert np.all(rhs[6:] == 0.0)
    c = c0.copy()
    nsteps, dt = 5, 600.0
    rc, st, _ = om.run(c, nsteps=nsteps, dt=dt, method=method, percol=percol)
    assert rc == 0
    expect = c0.copy()
    for _ in range(nsteps):
        expect = expect + dt * rhs
    np.testing.assert_allclose(c, expect, rtol=1e-13, atol=0)


def test_constant_rhs_is_flux_over_volume(oracle_mod):
    cs = constant_rhs_case()
    om = oracle_mod.OracleModel(cs)
    rhs, _, _ = om.get_rhs(cs.conc)
    top = cs.fluxes[:6] / (cs.phi[0] * cs.dz[0])
    np.testing.assert_allclose(rhs[:6, 0, :], top, rtol=1e-14)


@pytest.mark.parametrize("percol", [True, False])
def test_adaptive_cut_sequence(oracle_mod, percol):
    # solver_library.F90:121-127: c1 = c(1 - 8) and c(1 - 2) are rejected,
    # c(1 - 0.5) is accepted -> 2 cuts, 16 accepted substeps of dt/16.
    cs = decay_case()
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    rc, st, _ = om.run(c, nsteps=1, method=ADAPTIVE_EULER, percol=percol)
    assert rc == 0
    assert st["min_dt"] == cs.dt / 16
    if percol:
        assert st["accepted"] == 16 * cs.ncol
        assert st["attempts"] == 18 * cs.ncol
        assert st["max_col_attempts"] == 18
    else:
        assert st["accepted"] == 16 and st["attempts"] == 18
    np.testing.assert_allclose(c[0], cs.conc[0] * 0.5 ** 16, rtol=1e-12)


def test_dt_min_accepts_bad_step(oracle_mod):
    # the dt_min guard (:126): once dt_red <= dt_min the step is accepted
    cs = decay_case(lam_dt=8.0)
    cs.driver.dt_min = cs.dt / 4   # 900 s is the smallest cut
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    rc, st, _ = om.run(c, nsteps=1, method=ADAPTIVE_EULER, percol=True)
    assert rc == 0
    assert st["min_dt"] == cs.dt / 4
    assert st["accepted"] == 4 * cs.ncol
    # each accepted substep multiplies by 1 - 2 = -1: four of them give +c0
    np.testing.assert_allclose(c[0], cs.conc[0], rtol=1e-12)


def test_substep_cap_reported(oracle_mod):
    cs = decay_case()
    cs.driver.max_attempts = 3
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    rc, st, _ = om.run(c, nsteps=1, method=ADAPTIVE_EULER, percol=True)
    assert rc == -3 and st["capped"] == cs.ncol


@pytest.mark.parametrize("bcup", [1, 2])
def test_transport_conserves_mass(oracle_mod, bcup):
    # diff3d :818-820 + no-flux bottom: inventory changes by the surface flux
    cs = no_reactions(small(8, 15, seed=11))
    cs.driver.bcup_dissolved = bcup
    if bcup == 1:
        cs.fluxes[6:] = 1e-5
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    inv0 = om.inventory(c)
    _, fl, _ = om.get_rhs(c)
    rc, st, _ = om.run(c, nsteps=1, dt=60.0, method=EULER, percol=True)
    inv1 = om.inventory(c)
    expect = inv0 + 60.0 * fl
    np.testing.assert_allclose(inv1, expect, rtol=1e-11)


def test_dirichlet_steady_state_uniform(oracle_mod):
    # Dirichlet top, no-flux bottom, no reactions: the dissolved profiles
    # relax to the bottom-water value.  The coupling step is short enough for
    # explicit Euler to be stable (at 3600 s the positivity limiter of
    # solver_library.F90:121 accepts 900 s steps that are oscillatory for the
    # 1 mm top layers, and the profile settles into a bounded limit cycle).
    cs = no_reactions(small(3, 6, seed=2, total=0.0061))
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    rc, st, _ = om.run(c, nsteps=4000, dt=120.0, method=ADAPTIVE_EULER,
                       percol=True)
    assert rc == 0
    for n in range(6, NTR):
        np.testing.assert_allclose(c[n], np.broadcast_to(cs.bdys[n + 1], c[n].shape),
                                   rtol=2e-3, atol=1e-6)


def test_reaction_budgets_close(oracle_mod):
    # P moves between pools without loss; N is lost only by denitrification
    import oracle as O
    rng = np.random.default_rng(0)
    for _ in range(50):
        c = rng.uniform(0.0, 300.0, NTR)
        r, dn = O.omexdia_rates(synth.BGC_DEFAULTS, c)
        assert abs(r[4] + r[5] + r[10]) <= 1e-15 * np.abs(r[[4, 5, 10]]).max() + 1e-300
        n_sum = r[2] + r[3] + r[7] + r[8]
        assert abs(n_sum + 0.8 * dn) <= 1e-12 * (np.abs(r).max() + 1e-30)


def test_atol_floor(oracle_mod):
    """The positivity test ignores cells whose value is within atol of zero:
    a cell at 1e-20 decaying at lam*dt = 8 forces the cut sequence with
    atol = 0 (the reference's test) and none with atol = 1e-12."""
    cs = decay_case()
    cs.conc[0] = 1e-20
    cs.conc[1:6] = 0.0
    for atol, accepted in ((0.0, 16), (1e-12, 1)):
        cs.driver.atol = atol
        c = cs.conc.copy()
        rc, st, _ = oracle_mod.OracleModel(cs).run(c, nsteps=1, percol=True)
        assert st["accepted"] == accepted * cs.ncol, (atol, st)


def test_percol_equals_single_column_runs(oracle_mod):
    # per-column mode: each column's result does not depend on the others
    cs = small(6, 10, seed=4, days=1)
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    om.run(c, nsteps=6, method=ADAPTIVE_EULER, percol=True)
    for col in (0, 3, 5):
        sub = cs.subset(np.array([col]))
        cc = sub.conc.copy()
        oracle_mod.OracleModel(sub).run(cc, nsteps=6, method=ADAPTIVE_EULER,
                                        percol=False)
        np.testing.assert_array_equal(cc[:, :, 0], c[:, :, col])


def test_linear_grid_matches_reference_formula(oracle_mod):
    from sedgpu import driver
    dz, zc, zi, dzc = oracle_mod.init_grid_linear(24, 0.003)
    g = driver.SedGrid(1, 1, 24, 0.003)
    driver.init_grid(g)
    np.testing.assert_allclose(g.dz[:, 0], dz, rtol=1e-15)
    np.testing.assert_allclose(g.dzc[:, 0], dzc, rtol=1e-13)
    fac = 0.18 / ((24 + 1) / 2.0 * 0.003) - 1.0
    assert dz[-1] == pytest.approx(fac * 0.003, rel=1e-14)


def test_bcup4_cascade(oracle_mod):
    # diff3d :791-802 with a flux larger than the first caps
    K = 5
    cap = np.array([1.0, 2.0, 0.5, 0.5, 0.5])
    C = np.zeros(K)
    ones = np.ones(K)
    flux, dC = oracle_mod.diff3d(C, 0.0, 3.2, 4, 0 * ones, ones, ones,
                                 np.ones(K - 1), flux_cap=cap)
    # rest: 3.2-1=2.2 -> F2 += 2.2; 2.2-2=0.2 -> F3 += 0.2; 0.2-0.5<0 stop
    np.testing.assert_allclose(flux[:K + 1], [3.2, 2.2, 0.2, 0.0, 0.0, 0.0])
    flux, dC = oracle_mod.diff3d(C, 0.0, 10.0, 4, 0 * ones, ones, ones,
                                 np.ones(K - 1), flux_cap=cap)
    # all caps exceeded: rests 9, 7, 6.5, 6, 5.5; the last added to F(K)
    np.testing.assert_allclose(flux[:K + 1], [10.0, 9.0, 7.0, 6.5, 6.0 + 5.5, 0.0])


def _golden_files():
    if not os.path.isdir(GOLDEN):
        return []
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))


@pytest.mark.parametrize("fname", _golden_files())
def test_golden_regression(oracle_mod, fname):
    """The oracle reproduces the committed fixtures (tests/golden/make_golden.py)."""
    import make_golden_cases
    g = np.load(os.path.join(GOLDEN, fname))
    cs = make_golden_cases.case(str(g["case"]))
    out = make_golden_cases.run_oracle(oracle_mod, cs, str(g["case"]))
    for key in out:
        np.testing.assert_allclose(out[key], g[key], rtol=1e-11, atol=1e-300,
                                   err_msg=key)


def test_reference_amplifies_one_ulp(oracle_mod):
    """The reference's positivity-limited Euler accepts 900 s substeps that
    are unstable for the 1 mm surface layers, so a 1-ulp change of the
    initial state grows by orders of magnitude within days: long-horizon
    parity is only possible for a bit-identical implementation."""
    from conftest import relerr
    cs = synth.make_workload("plain_cpu_10x10")
    cs.driver.atol = 0.0
    om = oracle_mod.OracleModel(cs)
    a = cs.conc.copy()
    b = cs.conc * (1.0 + 2.0 ** -52)
    om.run(a, nsteps=24, percol=True)
    om.run(b, nsteps=24, percol=True)
    assert relerr(a, b).max() > 1e-6


def test_bioturbation_profile3_matches_formula(oracle_mod):
    """Profile 3 equals the static profile whose factor is the Zhang & Wirtz
    formula evaluated on the same state, with bioturbation = f_T = 1 (the
    reference sets both to one, get_rhs :622-623; at T = 15 C the static
    path's f_T is exactly one)."""
    from cases import zhang_wirtz_factor
    cs = synth.make_workload("plain_cpu_10x10")
    cs.bdys[0] = 15.0
    b3 = cs.copy()
    b3.driver.bioturbation_profile = 3
    r3, f3, _ = oracle_mod.OracleModel(b3).get_rhs(cs.conc)
    st = cs.copy()
    st.biofac = zhang_wirtz_factor(cs, cs.conc)
    st.driver.bioturbation = 1.0
    rs, fs, _ = oracle_mod.OracleModel(st).get_rhs(cs.conc)
    scale = np.abs(rs).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(r3 - rs) / scale) < 1e-12
    np.testing.assert_allclose(f3, fs, rtol=1e-12, atol=0)
    # and the factor changes the transport: profile 3 is not the static one
    r1, _, _ = oracle_mod.OracleModel(cs).get_rhs(cs.conc)
    assert np.max(np.abs(r3 - r1) / scale) > 1e-6


def test_assemble_bc_matches_reference_formulas(oracle_mod):
    """orc_assemble_bc against get_boundary_conditions' formulas
    (fabm_sediment_component.F90:1978,1986,2012-2014) written in numpy."""
    from cases import pelagic_fields
    cs = synth.make_workload("plain_cpu_10x10")
    cs.driver.bcup_dissolved = 1
    T, surf, vel = pelagic_fields(cs)
    present = np.ones(NTR, dtype=np.int32)
    present[[1, 8]] = 0
    bd, fl = oracle_mod.OracleModel(cs).assemble_bc(cs.conc, T, surf, vel, present)
    d = cs.driver
    np.testing.assert_array_equal(bd[0], T)
    for n in range(NTR):
        if not present[n]:
            np.testing.assert_array_equal(fl[n], cs.fluxes[n])
            np.testing.assert_array_equal(bd[n + 1], cs.bdys[n + 1])
        elif n < 6:
            np.testing.assert_array_equal(fl[n], -surf[n] * vel[n])
        else:
            np.testing.assert_array_equal(bd[n + 1], surf[n])
            est = (-(cs.conc[n, 0] - surf[n]) / cs.dz[0] *
                   (d.bioturbation + d.diffusivity + T * 0.035) * cs.phi[0] / 86400.0 / 10000.0)
            np.testing.assert_allclose(fl[n], est, rtol=1e-14, atol=0)
    cs.driver.bcup_dissolved = 2
    _, fl2 = oracle_mod.OracleModel(cs).assemble_bc(cs.conc, T, surf, vel)
    assert np.all(fl2[6:] == 0.0)


def numpy_adaptive_diag(om, cs, conc, dt, last_min_dt, cell):
    """Grid-wide ADAPTIVE_EULER with adaptive_solver_diagnostics restated in
    numpy over the oracle's right-hand side (solver_library.F90:104-140):
    on an accepted substep with dt_red < last_min_dt, last_min_dt = dt_red
    and the cell is minloc((c1 - c)/c) over the whole (i,j,k,n) array,
    NaN quotients skipped (gfortran's MINLOC)."""
    m = om.m
    keep = 1.0 + m.relative_change_min
    active = (np.arange(cs.kmax)[:, None] < cs.kact[None, :])[None].repeat(NTR, axis=0)
    fl = np.array(cs.fluxes, dtype=np.float64, copy=True)
    dt_int, dt_red = 0.0, dt
    while dt_int < dt:
        rhs, fl, _ = om.get_rhs(conc, fl)
        c1 = np.where(active, conc + dt_red * rhs, conc)
        reject = bool(np.any((c1 - keep * conc < -m.atol) & active))
        if reject and dt_red > m.dt_min:
            dt_red = dt_red * 0.25
            continue
        if dt_red < last_min_dt:
            last_min_dt = dt_red
            with np.errstate(divide="ignore", invalid="ignore"):
                v = (c1 - conc) / conc
            shape = (NTR, cs.kmax, cs.jnum, cs.inum)
            flat = v.reshape(shape).ravel()
            pos = 0 if np.isnan(flat).all() else int(np.nanargmin(flat))
            n, k, j, i = np.unravel_index(pos, shape)
            cell = (int(i) + 1, int(j) + 1, int(k) + 1, int(n) + 1)
        conc[active] = c1[active]
        dt_int = dt_int + dt_red
    return last_min_dt, cell


def test_last_min_dt_grid_cell_matches_numpy_restatement(oracle_mod):
    """a1: type_rhs_driver's last_min_dt and last_min_dt_grid_cell, carried
    across calls, with land columns (zero state: NaN quotients) and masked
    bottom tails in the grid."""
    cs = synth.make_columns(inum=5, jnum=3, kmin=6, kmax=10, total=0.18, land=0.25,
                            poc="loguniform", days=1, seed=41, name="diag5x3")
    cs.conc[:, :, cs.kact == 0] = 0.0
    om = oracle_mod.OracleModel(cs)
    d = om.new_diag()
    assert d.cell() == (-99, -99, -99, -99)
    assert d.last_min_dt == float(np.float32(1e20))
    got = cs.conc.copy()
    ref = cs.conc.copy()
    last, cell = d.last_min_dt, d.cell()
    for step in range(4):
        rc, st, _ = om.ode_solver_diag(got, d)
        assert rc == 0
        last, cell = numpy_adaptive_diag(om, cs, ref, cs.dt, last, cell)
        np.testing.assert_array_equal(got, ref)
        assert d.last_min_dt == last and d.cell() == cell, (step, d.cell(), cell)
    assert d.last_min_dt < cs.dt                 # the grid did cut
    i, j, k, n = d.cell()
    assert cs.kact[(i - 1) + cs.inum * (j - 1)] >= k   # an active cell


def test_last_min_dt_grid_cell_of_a_uniform_decay(oracle_mod):
    """Labile carbon alone decays at lam with lam*dt = 8: the cut sequence
    is fixed (dt/16 is the first accepted substep), and the smallest
    relative change is labile carbon's (tracer 1)."""
    cs = decay_case(ncol=4, K=3, lam_dt=8.0)
    om = oracle_mod.OracleModel(cs)
    d = om.new_diag()
    c = cs.conc.copy()
    rc, st, _ = om.ode_solver_diag(c, d)
    assert rc == 0
    assert d.last_min_dt == cs.dt / 16.0
    assert d.cell()[3] in (1, 3)    # labile detritus C or N (the same rate)
