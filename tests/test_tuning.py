"""Launch tuning, the pipelined drop-in call and the autotuner.

Every tuning is a pure launch choice over a fixed slot layout, so the state
after a step must be bit-identical under any tile width, block size and
pipeline depth; the pipelined sed_ode_solver must equal the unpipelined one
(and, with FP64 state, the oracle) bit for bit; the autotuner must leave the
state it found untouched."""
import ctypes

import numpy as np
import pytest

from sedgpu import capi, synth
from sedgpu.model import ADAPTIVE_EULER, RUNGE_KUTTA_4

pytestmark = pytest.mark.gpu


def uneven(n=20000):
    """Land, and both depth classes (10..60 layers): two column segments."""
    return synth.make_workload("uneven_1024x1024", cols=np.arange(n))


def plain(n=40000):
    """Uniform 30-layer columns: eight column segments."""
    return synth.make_workload("plain_gpu_256x256", cols=np.arange(n))


def stepped(cs, nsteps, tuning=None, method=ADAPTIVE_EULER, precision=capi.SED_FP32):
    s = capi.Solver(cs, precision=precision)
    if tuning:
        s.set_tuning(**tuning)
    s.set_forcing()
    s.set_state(cs.conc)
    s.step(nsteps, method=method)
    out, fl, att = s.get_state(), s.fluxes(), s.attempts()
    s.close()
    return out, fl, att


def test_default_tuning_and_segments():
    s = capi.Solver(uneven())
    t = s.tuning().as_dict()
    s.close()
    assert t["tile_columns"] == [0, 0] and t["threads"] == [128, 128]
    s64 = capi.Solver(uneven(), precision=capi.SED_FP64)
    t64 = s64.tuning().as_dict()
    s64.close()
    assert t64["tile_columns"] == [32, 16] and t64["threads"] == [256, 256]
    assert t["segments"] == 2 and t["pipeline_chunks"] == 2
    s = capi.Solver(plain())
    assert s.tuning().segments == 8 and s.tuning().pipeline_chunks == 4
    s.close()
    s = capi.Solver(synth.make_workload("plain_cpu_10x10"))
    assert s.tuning().segments == 1 and s.tuning().pipeline_chunks == 1
    s.close()


@pytest.mark.parametrize("tuning", [
    dict(tile_columns=(32, 16), threads=(256, 256)),
    dict(tile_columns=(0, 0), threads=(128, 64)),
    dict(tile_columns=(0, 16), threads=(256, 256)),
    dict(tile_columns=(8, 8), threads=(64, 128)),
    dict(tile_columns=(64, 32), threads=(256, 192)),
    dict(tile_columns=(16, 8), threads=(128, 64), blocks_per_sm=(1, 1)),
])
def test_any_tuning_is_bit_identical(tuning):
    cs = uneven()
    ref = stepped(cs, 2)
    got = stepped(cs, 2, tuning)
    for r, g in zip(ref, got):
        np.testing.assert_array_equal(g, r)


@pytest.mark.parametrize("tiles", [(8, 16), (0, 0)])
def test_tuning_is_bit_identical_fixed_method(tiles):
    cs = plain(12000)
    ref = stepped(cs, 1, method=RUNGE_KUTTA_4)
    got = stepped(cs, 1, dict(tile_columns=tiles, threads=(64, 256)), method=RUNGE_KUTTA_4)
    for r, g in zip(ref, got):
        np.testing.assert_array_equal(g, r)


def test_warp_direct_with_profile3_and_cascade():
    cs = uneven(12000)
    cs.driver.bioturbation_profile = 3
    cs.driver.bcup_particulate = 4
    ref = stepped(cs, 2)
    got = stepped(cs, 2, dict(tile_columns=(0, 0), threads=(128, 128)))
    for r, g in zip(ref, got):
        np.testing.assert_array_equal(g, r)


def test_warp_direct_rhs():
    cs = uneven(9000)
    s = capi.Solver(cs)
    s.set_forcing()
    ref = s.get_rhs(cs.conc)
    s.set_tuning(tile_columns=(0, 0))
    got = s.get_rhs(cs.conc)   # rhs kind served by the 32-column tile kernel
    s.close()
    for r, g in zip(ref, got):
        np.testing.assert_array_equal(g, r)


def test_warp_direct_fp64_matches_oracle(oracle_mod):
    cols = np.arange(0, 1024 * 1024, 1024 * 1024 // 300)[:300]
    cs = synth.make_workload("uneven_1024x1024", cols=cols)
    out, _, _ = stepped(cs, 6, dict(tile_columns=(0, 0)), precision=capi.SED_FP64)
    c = cs.conc.copy()
    rc, _, _ = oracle_mod.OracleModel(cs).run(c, nsteps=6, percol=True)
    assert rc == 0
    np.testing.assert_array_equal(out, c)


def drop_in(cs, chunks, nsteps=2, precision=capi.SED_FP32, tiles=None):
    s = capi.Solver(cs, precision=precision)
    s.set_tuning(pipeline_chunks=chunks)
    if tiles:
        s.set_tuning(tile_columns=tiles)
    conc = cs.conc.copy()
    fl = np.array(cs.fluxes, dtype=np.float64, copy=True)
    stats = []
    for _ in range(nsteps):
        stats.append(s.ode_solver(conc, cs.bdys, fl, cs.dt))
    att = s.attempts()
    s.close()
    return conc, fl, att, stats


@pytest.mark.parametrize("make", [plain, uneven])
def test_pipelined_ode_solver_matches_unpipelined(make):
    cs = make()
    nseg = capi.Solver(cs).tuning().segments
    ref = drop_in(cs, 1)
    p = 2
    while p <= nseg:
        got = drop_in(cs, p, tiles=(0, 0) if p == 2 else None)
        for r, g in zip(ref[:3], got[:3]):
            np.testing.assert_array_equal(g, r)
        for a, b in zip(ref[3], got[3]):
            for k in ("attempts", "accepted", "column_steps", "max_col_attempts"):
                assert a[k] == b[k]
        p *= 2
    # the untouched land columns come back as they went
    land = cs.kact == 0
    if land.any():
        np.testing.assert_array_equal(ref[0][:, :, land], cs.conc[:, :, land])


def test_pipelined_fp64_matches_oracle(oracle_mod):
    cs = plain(9000)
    conc, fl, _, _ = drop_in(cs, 2, nsteps=1, precision=capi.SED_FP64)
    om = oracle_mod.OracleModel(cs)
    c = cs.conc.copy()
    rc, _, fref = om.run(c, nsteps=1, percol=True, nthreads=8)
    assert rc == 0
    np.testing.assert_array_equal(conc, c)
    np.testing.assert_array_equal(fl[6:], fref[6:])


def test_autotune_restores_state_and_keeps_results():
    cs = uneven()
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    s.step(1)
    before = s.get_state()
    fl_before = s.fluxes()
    t = s.autotune(flags=capi.SED_TUNE_PIPELINE | capi.SED_TUNE_CAP)
    np.testing.assert_array_equal(s.get_state(), before)
    np.testing.assert_array_equal(s.fluxes(), fl_before)
    assert t["trials"] > 0 and t["step_ms"] > 0 and t["ode_solver_ms"] > 0
    assert all(c in (0, 8, 16, 32, 64) for c in t["tile_columns"])
    assert all(th in (64, 128, 256) for th in t["threads"])
    assert t["segments"] % t["pipeline_chunks"] == 0
    assert t["max_attempts"] >= 64
    cur = s.tuning().as_dict()
    for k in ("tile_columns", "threads", "pipeline_chunks", "max_attempts"):
        assert cur[k] == t[k]
    s.step(1)
    tuned = s.get_state()
    s.close()
    # the same two steps under the default tuning
    ref, _, _ = stepped(cs, 2)
    np.testing.assert_array_equal(tuned, ref)
    print("autotuned:", t)


def test_set_tuning_rejects_bad_values():
    s = capi.Solver(uneven(6000))
    good = s.tuning()
    for field, value in [("tile_columns", (12, 16)), ("threads", (96, 256)),
                         ("threads", (512, 256)), ("blocks_per_sm", (-1, 0)),
                         ("pipeline_chunks", 3), ("max_attempts", 0)]:
        t = capi.SedTuning.from_buffer_copy(good)
        if isinstance(getattr(t, field), ctypes.Array):
            getattr(t, field)[:] = list(value)
        else:
            setattr(t, field, value)
        rc = s.lib.sed_set_tuning(s.h, ctypes.byref(t))
        assert rc == capi.SED_E_ARG, (field, value, rc)
    assert s.tuning().as_dict() == good.as_dict()
    s.close()
