"""GPU parity of the CUDA library (through the C ABI) against the FP64 oracle.

FP64 device state evaluates the reference's arithmetic in the oracle's
operation order and must reproduce it bit for bit over any horizon.  FP32
device state must stay within 1e-3 per-tracer relative error (relative to
|ref| plus a floor of 1e-4 x the tracer's largest value, since deep O2 / NO3
fall to ~0) over short horizons and for every coupling step started from the
same state.  Over long horizons no implementation that is not bit-identical
can track the reference: its positivity-limited Euler accepts unstable
substeps that amplify a 1-ulp difference to 1e-2 within ~24 coupling steps
(tests/test_oracle.py::test_reference_amplifies_one_ulp).
"""
import numpy as np
import pytest

from cases import constant_rhs_case, decay_case, no_reactions, pelagic_fields, small
from conftest import relerr
from sedgpu import capi, synth
from sedgpu.model import (ADAPTIVE_EULER, EULER, NTR, RUNGE_KUTTA_4,
                          RUNGE_KUTTA_4_38)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9
FP32_TOL = 1e-3


def run_gpu(cs, nsteps, method=ADAPTIVE_EULER, dt=None, precision=capi.SED_FP32,
            cut=capi.SED_CUT_PER_COLUMN, budgets=False):
    s = capi.Solver(cs, precision=precision, cut_scope=cut, budgets=budgets)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(nsteps, dt=dt, method=method)
    out = s.get_state()
    fl = s.fluxes()
    att = s.attempts()
    bud = s.budgets() if budgets else None
    s.close()
    return out, fl, st, att, bud


def run_oracle(oracle_mod, cs, nsteps, method=ADAPTIVE_EULER, dt=None, percol=True):
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    rc, st, fl = om.run(c, nsteps=nsteps, dt=dt, method=method, percol=percol)
    assert rc == 0
    return c, fl, st


def active(cs, c):
    """Active cells only, as [ntr][cells]."""
    K = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    return c[:, K]


def test_rhs_fp64_matches_oracle(oracle_mod):
    cs = synth.make_workload("plain_cpu_10x10")
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    rhs, fl = s.get_rhs(cs.conc)
    s.close()
    ref, fref, _ = oracle_mod.OracleModel(cs).get_rhs(cs.conc)
    np.testing.assert_array_equal(rhs, ref)
    np.testing.assert_array_equal(fl, fref)


def test_rhs_fp32_matches_oracle(oracle_mod):
    cs = synth.make_workload("plain_cpu_10x10")
    s = capi.Solver(cs, precision=capi.SED_FP32)
    s.set_forcing()
    rhs, fl = s.get_rhs(cs.conc)
    s.close()
    ref, _, _ = oracle_mod.OracleModel(cs).get_rhs(cs.conc)
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(rhs - ref) / scale) < 2e-5


@pytest.mark.parametrize("atol", [0.0, 1e-12])
def test_adaptive_percol_fp64_bit_exact(oracle_mod, atol):
    # atol = 0 is the reference's positivity test (solver_library.F90:121)
    cs = synth.make_workload("plain_cpu_10x10")
    cs.driver.atol = atol
    n = 72
    out, fl, st, att, _ = run_gpu(cs, n, precision=capi.SED_FP64)
    ref, fref, sref = run_oracle(oracle_mod, cs, n)
    np.testing.assert_array_equal(out, ref)
    np.testing.assert_array_equal(fl, fref)
    assert st["attempts"] == sref["attempts"]
    assert st["accepted"] == sref["accepted"]


def teacher_forced(oracle_mod, cs, state, gpu_next, cols=None):
    """Relative error of one GPU coupling step against one oracle step from
    the same state."""
    sub = cs if cols is None else cs.subset(cols)
    start = state if cols is None else state[:, :, cols]
    sub = sub.copy()
    sub.conc = np.ascontiguousarray(start)
    ref, _, _ = run_oracle(oracle_mod, sub, 1)
    nxt = gpu_next if cols is None else gpu_next[:, :, cols]
    return relerr(active(sub, nxt), active(sub, ref))


def test_adaptive_percol_fp32(oracle_mod):
    cs = synth.make_workload("plain_cpu_10x10")
    s = capi.Solver(cs, precision=capi.SED_FP32)
    s.set_forcing()
    s.set_state(cs.conc)
    s.step(1)
    out1 = s.get_state()
    ref1, _, _ = run_oracle(oracle_mod, cs, 1)
    err = relerr(active(cs, out1), active(cs, ref1))
    assert err.max() < FP32_TOL, err
    # every later step, started from the GPU's own state (over several steps
    # the reference dynamics amplify any rounding difference ~100x per step)
    state = out1
    for step in range(1, 48):
        s.step(1)
        nxt = s.get_state()
        if step % 7 == 6:
            e = teacher_forced(oracle_mod, cs, state, nxt)
            assert e.max() < FP32_TOL, (step, e)
        state = nxt
    s.close()


def test_adaptive_global_cut_10x10(oracle_mod):
    # the reference's own semantics: one cut for the whole grid, its test
    cs = synth.make_workload("plain_cpu_10x10")
    cs.driver.atol = 0.0
    n = 12
    out, fl, st, _, _ = run_gpu(cs, n, precision=capi.SED_FP64,
                                cut=capi.SED_CUT_GLOBAL)
    ref, fref, sref = run_oracle(oracle_mod, cs, n, percol=False)
    np.testing.assert_array_equal(out, ref)
    assert st["accepted"] == sref["accepted"] * cs.n_active


@pytest.mark.parametrize("method", [EULER, RUNGE_KUTTA_4, RUNGE_KUTTA_4_38])
def test_fixed_methods(oracle_mod, method):
    cs = small(32, 20, seed=9)
    out, fl, st, _, _ = run_gpu(cs, 30, method=method, dt=60.0,
                                precision=capi.SED_FP64)
    ref, fref, _ = run_oracle(oracle_mod, cs, 30, method=method, dt=60.0)
    np.testing.assert_array_equal(out, ref)
    np.testing.assert_array_equal(fl, fref)
    out32, _, _, _, _ = run_gpu(cs, 30, method=method, dt=60.0)
    assert relerr(active(cs, out32), active(cs, ref)).max() < FP32_TOL


def test_uneven_columns_and_land(oracle_mod):
    cols = np.arange(0, 1024 * 1024, 1024 * 1024 // 300)[:300]
    cs = synth.make_workload("uneven_1024x1024", cols=cols)
    assert (cs.kact == 0).any() and (cs.kact > 32).any() and (cs.kact <= 32).any()
    n = 24
    out, fl, st, att, _ = run_gpu(cs, n, precision=capi.SED_FP64)
    ref, fref, sref = run_oracle(oracle_mod, cs, n)
    np.testing.assert_array_equal(out, ref)
    # land columns and inactive layers are returned untouched
    land = cs.kact == 0
    np.testing.assert_array_equal(out[:, :, land], cs.conc[:, :, land])
    assert np.all(att[land] == 0) and np.all(att[~land] > 0)
    out32, _, _, _, _ = run_gpu(cs, 4, precision=capi.SED_FP32)
    ref4, _, _ = run_oracle(oracle_mod, cs, 4)
    err32 = relerr(active(cs, out32), active(cs, ref4))
    assert err32.max() < FP32_TOL, err32


def test_bcup_variants(oracle_mod):
    cs = small(24, 16, seed=21)
    cs.driver.bcup_dissolved = 1
    cs.fluxes[6:] = -2e-6
    cs.driver.bcup_particulate = 4
    cs.flux_cap[:] = 2e-5 * cs.dz / cs.dz[0]
    cs.driver.mol_diff_mode = 0
    for n in range(6):
        cs.fluxes[n] *= 50.0
    out, fl, st, _, _ = run_gpu(cs, 8, precision=capi.SED_FP64)
    ref, fref, _ = run_oracle(oracle_mod, cs, 8)
    np.testing.assert_array_equal(out, ref)
    out32, _, _, _, _ = run_gpu(cs, 2, precision=capi.SED_FP32)
    ref2, _, _ = run_oracle(oracle_mod, cs, 2)
    assert relerr(active(cs, out32), active(cs, ref2)).max() < FP32_TOL


def test_constant_rhs_exact_on_gpu():
    cs = constant_rhs_case()
    for method in (EULER, RUNGE_KUTTA_4, ADAPTIVE_EULER, RUNGE_KUTTA_4_38):
        out, _, _, _, _ = run_gpu(cs, 5, method=method, dt=600.0,
                                  precision=capi.SED_FP64)
        rhs_top = cs.fluxes[:6] / (cs.phi[0] * cs.dz[0])
        expect = cs.conc.copy()
        expect[:6, 0, :] += 5 * 600.0 * rhs_top
        np.testing.assert_allclose(out, expect, rtol=1e-13)


def test_cut_sequence_on_gpu():
    cs = decay_case()
    for prec in (capi.SED_FP64, capi.SED_FP32):
        out, _, st, att, _ = run_gpu(cs, 1, precision=prec)
        assert st["attempts"] == 18 * cs.ncol
        assert st["accepted"] == 16 * cs.ncol
        assert st["min_dt"] == cs.dt / 16
        assert np.all(att == 18)


def test_drop_in_ode_solver_host_arrays(oracle_mod):
    # sed_ode_solver: host FP64 arrays in and out, as ode_solver + epilogue
    cs = synth.make_workload("plain_cpu_10x10")
    s = capi.Solver(cs, precision=capi.SED_FP64)
    conc = cs.conc.copy()
    fl = cs.fluxes.copy()
    for _ in range(6):
        s.ode_solver(conc, cs.bdys, fl, cs.dt, ADAPTIVE_EULER)
    s.close()
    ref, fref, _ = run_oracle(oracle_mod, cs, 6)
    np.testing.assert_array_equal(conc, ref)
    np.testing.assert_array_equal(fl, fref)


def test_budgets_fp64(oracle_mod):
    cs = small(64, 30, seed=13, total=0.2)
    out, fl, st, att, bud = run_gpu(cs, 4, precision=capi.SED_FP32, budgets=True)
    invP, resP, invN, resN = bud
    assert np.all(invP > 0) and np.all(invN > 0)
    # FP32 state: the residual of the last step is at rounding level
    assert np.max(np.abs(resP) / invP) < 1e-5
    assert np.max(np.abs(resN) / invN) < 1e-5


def test_status_codes():
    cs = decay_case()
    cs.driver.max_attempts = 3
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    rc, st = s.step(1, raise_on_error=False)
    assert rc == capi.SED_E_SUBSTEP_CAP and st["capped_columns"] == cs.ncol
    s.close()
    # NaN in the input state surfaces as SED_E_NAN, the context stays usable
    cs = small(8, 10, seed=1)
    bad = cs.conc.copy()
    bad[6, 3, 2] = np.nan
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(bad)
    rc, st = s.step(1, raise_on_error=False)
    assert rc == capi.SED_E_NAN and st["nan_cells"] >= 1
    s.set_state(cs.conc)
    rc, st = s.step(1, raise_on_error=False)
    assert rc == capi.SED_OK
    s.close()
    # call order and argument checks
    lib = capi.load()
    p = capi.params_from(cs)
    h = capi._H()
    import ctypes
    assert lib.sed_create(ctypes.byref(p), 4, 4, capi.SED_KMAX_LIMIT + 1, 11,
                          ctypes.byref(h)) == capi.SED_E_ARG
    assert lib.sed_create(ctypes.byref(p), 4, 4, 10, 12, ctypes.byref(h)) == capi.SED_E_ARG
    p.bcup_dissolved = 7
    assert lib.sed_create(ctypes.byref(p), 4, 4, 10, 11, ctypes.byref(h)) == capi.SED_E_ARG
    s = capi.Solver(cs)
    rc = lib.sed_step(s.h, 3600.0, 2, 1, None)
    assert rc == capi.SED_E_STATE
    s.close()


def test_full_size_workload_properties(oracle_mod):
    """256 x 256 x 30 for 48 coupling steps on the GPU; a column subsample is
    rerun by the oracle (per-column cuts make any subset exact)."""
    cs = synth.make_workload("plain_gpu_256x256")
    n = 48
    s = capi.Solver(cs, precision=capi.SED_FP32, budgets=True)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(n - 1)
    prev = s.get_state()
    st1 = s.step(1)
    out = s.get_state()
    bud = s.budgets()
    s.close()
    assert np.isfinite(out).all() and (out >= 0).all()
    assert st["column_steps"] + st1["column_steps"] == cs.ncol * n
    assert np.max(np.abs(bud[1]) / bud[0]) < 1e-4
    assert np.max(np.abs(bud[3]) / bud[2]) < 1e-4
    cols = np.random.default_rng(3).choice(cs.ncol, 256, replace=False)
    e = teacher_forced(oracle_mod, cs, prev, out, cols)
    assert e.max() < FP32_TOL, e


def with_profile3(cs):
    cs = cs.copy()
    cs.driver.bioturbation_profile = 3
    return cs


@pytest.mark.parametrize("workload", ["plain_cpu_10x10", "uneven"])
def test_bioturbation_profile3(oracle_mod, workload):
    """Zhang & Wirtz bioturbation recomputed at every right-hand side.  FP64
    keeps the reference's operation order but takes CUDA's pow, which may
    differ from the CPU's in the last bit, so FP64 is compared at 1e-13 per
    right-hand side and 1e-9 after two steps instead of bit for bit."""
    if workload == "uneven":   # both depth classes and land
        cols = np.arange(0, 1024 * 1024, 1024 * 1024 // 200)[:200]
        cs = with_profile3(synth.make_workload("uneven_1024x1024", cols=cols))
    else:
        cs = with_profile3(synth.make_workload(workload))
    ref, fref, _ = oracle_mod.OracleModel(cs).get_rhs(cs.conc)
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
    for prec, tol in ((capi.SED_FP64, 1e-13), (capi.SED_FP32, 1e-4)):
        s = capi.Solver(cs, precision=prec)
        s.set_forcing()
        rhs, fl = s.get_rhs(cs.conc)
        s.close()
        assert np.max(np.abs(rhs - ref) / scale) < tol, prec
    out64, _, _, _, _ = run_gpu(cs, 2, precision=capi.SED_FP64)
    ref2, _, _ = run_oracle(oracle_mod, cs, 2)
    assert relerr(active(cs, out64), active(cs, ref2)).max() < 1e-9
    out32, _, _, _, _ = run_gpu(cs, 1, precision=capi.SED_FP32)
    ref1, _, _ = run_oracle(oracle_mod, cs, 1)
    err = relerr(active(cs, out32), active(cs, ref1))
    assert err.max() < FP32_TOL, err
    # the TOC-dependent factor changes the result against the static profile
    plain = cs.copy()
    plain.driver.bioturbation_profile = 1
    static, _, _, _, _ = run_gpu(plain, 2, precision=capi.SED_FP64)
    assert relerr(active(cs, static), active(cs, out64)).max() > 1e-6


@pytest.mark.parametrize("bcup", [1, 2])
def test_boundary_assembly_on_device(oracle_mod, bcup):
    """sed_set_boundary equals get_boundary_conditions (the oracle's
    orc_assemble_bc) bit for bit on FP64 state, absent tracers keep their
    values, and the step that follows equals the oracle's step."""
    cs = synth.make_workload("uneven_1024x1024",
                             cols=np.arange(0, 1024 * 1024, 1024 * 1024 // 150)[:150])
    cs.driver.bcup_dissolved = bcup
    T, surf, vel = pelagic_fields(cs)
    present = np.ones(NTR, dtype=np.int32)
    present[[2, 9]] = 0
    om = oracle_mod.OracleModel(cs)
    bref, fref = om.assemble_bc(cs.conc, T, surf, vel, present)
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    s.set_state(cs.conc)
    s.set_boundary(T, surf, vel, present)
    bd, fl = s.boundary()
    np.testing.assert_array_equal(bd, bref)
    np.testing.assert_array_equal(fl, fref)
    s.step(1)
    out = s.get_state()
    fl_out = s.fluxes()
    s.close()
    c = cs.conc.copy()
    sub = cs.copy()
    sub.bdys, sub.fluxes = bref, fref
    rc, _, fl_ref = oracle_mod.OracleModel(sub).run(c, nsteps=1)
    assert rc == 0
    np.testing.assert_array_equal(out, c)
    np.testing.assert_array_equal(fl_out, fl_ref)
    # FP32 state: the estimate is formed in FP64 from the FP32 first layer,
    # i.e. the oracle's on the state rounded to FP32 (c0 - cb cancels, so
    # the rounding of c0 shows at ~1e-4 against the FP64-state estimate)
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    s.set_boundary(T, surf, vel, present)
    bd32, fl32 = s.boundary()
    s.close()
    c32 = cs.conc.astype(np.float32).astype(np.float64)
    _, fref32 = om.assemble_bc(c32, T, surf, vel, present)
    np.testing.assert_array_equal(bd32, bref)
    np.testing.assert_allclose(fl32, fref32, rtol=1e-12, atol=0)


def test_boundary_assembly_errors():
    cs = synth.make_workload("plain_cpu_10x10")
    cs.driver.bcup_dissolved = 1
    T, surf, vel = pelagic_fields(cs)
    s = capi.Solver(cs)
    with pytest.raises(capi.SedError) as e:
        s.set_boundary(T, surf, vel)   # the flux estimate needs the state
    assert e.value.code == capi.SED_E_STATE
    s.set_state(cs.conc)
    with pytest.raises(capi.SedError) as e:
        s.set_boundary(T, surf, None)  # particulates present, no velocity
    assert e.value.code == capi.SED_E_ARG
    only_dissolved = np.array([0] * 6 + [1] * 5, dtype=np.int32)
    s.set_boundary(T, surf, None, only_dissolved)
    s.close()


@pytest.mark.parametrize("cut", [capi.SED_CUT_PER_COLUMN, capi.SED_CUT_GLOBAL])
def test_min_dt_per_column(oracle_mod, cut):
    """The smallest accepted substep of every column in the last step (the
    per-column form of last_min_dt, solver_library.F90:130-136) equals the
    oracle's, column by column (per-column cut) or grid-wide (global cut)."""
    cs = synth.make_workload("plain_cpu_10x10")
    n = 30
    s = capi.Solver(cs, precision=capi.SED_FP64, cut_scope=cut)
    s.set_forcing()
    s.set_state(cs.conc)
    s.step(n - 1)
    before = s.get_state()
    st = s.step(1)
    md = s.min_dt()
    s.close()
    assert md.min() == st["min_dt"]
    if cut == capi.SED_CUT_GLOBAL:
        sub = cs.copy()
        sub.conc = before
        c = before.copy()
        rc, sref, _ = oracle_mod.OracleModel(sub).run(c, nsteps=1, percol=False)
        assert np.all(md == sref["min_dt"])
        return
    for col in (0, 17, 42, 99):
        sub = cs.subset([col])
        c = np.ascontiguousarray(before[:, :, [col]])
        rc, sref, _ = oracle_mod.OracleModel(sub).run(c, nsteps=1, percol=True)
        assert rc == 0
        assert md[col] == sref["min_dt"], col


def test_pinned_host_arrays_give_the_same_drop_in_result():
    """The drop-in call on arrays from sed_host_alloc (pinned host memory)
    equals the call on ordinary arrays, bit for bit."""
    cs = synth.make_workload("plain_cpu_10x10")
    out = []
    for pinned in (False, True):
        if pinned:
            conc = capi.host_empty(cs.conc.shape)
            conc[:] = cs.conc
            fl = capi.host_empty(cs.fluxes.shape)
            fl[:] = cs.fluxes
        else:
            conc = cs.conc.copy()
            fl = cs.fluxes.copy()
        s = capi.Solver(cs)
        for _ in range(3):
            s.ode_solver(conc, cs.bdys, fl, cs.dt)
        s.close()
        out.append((np.array(conc), np.array(fl)))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_attempt_histogram_counts_the_attempt_array():
    """sed_get_attempt_histogram bins the last step's per-column attempts
    (power-of-two bins, land and empty slots excluded) exactly as the
    attempt array itself gives them, for uneven columns and land."""
    cs = synth.make_workload("uneven_1024x1024", cols=np.arange(0, 1024 * 1024, 997)[:800])
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    for _ in range(3):
        s.step(4)
        att = s.attempts()[cs.kact > 0]
        bins = np.zeros(capi.SED_HIST_BINS, dtype=np.int64)
        for a in att:
            b = 0 if a <= 0 else min(int(a).bit_length(), capi.SED_HIST_BINS - 1)
            bins[b] += 1
        np.testing.assert_array_equal(s.attempt_histogram(), bins)
    s.close()
