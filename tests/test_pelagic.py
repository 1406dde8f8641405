"""The pelagic driver path (include/mossco_pel.h).

CPU: the oracle (oracle/pel_oracle.c) against closed-form statements of the
reference's pieces -- the light loop of fabm_pelagic_driver.F90:774-814,
the gotm_npzd rates, the Run's internal-step schedule and epilogue of
fabm_pelagic_component.F90:2061-2240 -- and invariants: the four rates sum
to zero, so a Run changes a column's nitrogen only by its boundary fluxes.
The library exports every function mossco_pel.h declares.

GPU: the CUDA path through the C ABI against the oracle.  The FP64 device
path uses the oracle's own exp (Cody-Waite + Taylor, every step one IEEE
rounding), so FP64 results are bit for bit; FP32 is compared at 1e-4 of
each tracer's largest value after a Run.
"""
import math
import re
import subprocess

import numpy as np
import pytest

from sedgpu import build, capi, pelagic
from sedgpu.model import ADAPTIVE_EULER, EULER, RUNGE_KUTTA_4, RUNGE_KUTTA_4_38

pel_oracle = pytest.importorskip("pel_oracle")

METHODS = [EULER, RUNGE_KUTTA_4, ADAPTIVE_EULER, RUNGE_KUTTA_4_38]


@pytest.fixture(scope="module")
def po():
    pel_oracle.build()
    return pel_oracle


def small(cols=64, seed=0):
    return pelagic.make_pelagic_workload(
        "pelagic_cpu_16x16", cols=np.arange(0, 256, 256 // cols)[:cols], seed=seed)


def stiff(pcs):
    """Rates and steps that make the adaptive method cut: a day per
    internal step with fast grazing and uptake."""
    pcs = pcs.copy()
    pcs.npzd.update(rmax=6.0, gmax=4.0, Iv=2.0, rpdl=0.8)
    pcs.t_couple, pcs.dt = 3 * 86400.0, 86400.0
    return pcs


# ---------------------------------------------------------------- CPU

def test_exp_within_one_ulp_of_libm(po):
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-700, 700, 4000), rng.uniform(-2, 2, 4000),
                         [0.0, 1.0, -1.0, 1e-300, -1e-300, 700.0, -706.9]])
    for x in xs:
        want = math.exp(x)
        got = po.pel_exp(x)
        assert abs(got - want) <= math.ulp(want), x
    assert po.pel_exp(0.0) == 1.0
    assert po.pel_exp(-800.0) == 0.0 and math.isinf(po.pel_exp(800.0))
    assert math.isnan(po.pel_exp(float("nan")))


def npzd_formula(npzd, c, par, iopt):
    """gotm_npzd rates (per second) from the published model, numpy."""
    day = 86400.0
    n, p, z, d = c
    rpd = np.where(par >= npzd["I_min"], npzd["rpdu"], npzd["rpdl"]) / day
    fnp = npzd["rmax"] / day * par / iopt * np.exp(1.0 - par / iopt) * n / (npzd["alpha"] + n) * (p + npzd["p0"])
    fpz = npzd["gmax"] / day * (1.0 - np.exp(-npzd["Iv"] ** 2 * p ** 2)) * (z + npzd["z0"])
    r = [-fnp + npzd["rpn"] / day * p + npzd["rzn"] / day * z + npzd["rdn"] / day * d,
         fnp - fpz - npzd["rpn"] / day * p - rpd * p,
         fpz - npzd["rzn"] / day * z - npzd["rzd"] / day * z,
         rpd * p + npzd["rzd"] / day * z - npzd["rdn"] / day * d]
    return np.array(r)


def test_rates_match_formula_and_conserve(po):
    pcs = small()
    o = po.PelOracle(pcs)
    par = o.light(pcs.conc)
    rhs = o.get_rhs(pcs.conc, par)
    w = pcs.water()
    iopt = np.maximum(0.25 * pcs.I_0, pcs.npzd["I_min"])[None, :]
    want = npzd_formula(pcs.npzd, pcs.conc, par, iopt)
    scale = np.abs(want[:, w]).max(axis=1, keepdims=True)
    assert np.max(np.abs(rhs[:, w] - want[:, w]) / scale) < 1e-13
    assert np.all(rhs[:, ~w] == 0.0)
    assert np.max(np.abs(rhs[:, w].sum(axis=0))) < 1e-15 * scale.max() * 10
    # below I_min the mortality is rpdl, above rpdu
    assert (par[w] < pcs.npzd["I_min"]).any() and (par[w] >= pcs.npzd["I_min"]).any()


def test_light_matches_reference_loop(po):
    pcs = small(16)
    pcs.mask = pcs.mask.copy()
    pcs.mask[:3, 1] = 1          # masked bottom cells of a water column
    o = po.PelOracle(pcs)
    par = o.light(pcs.conc)
    K = pcs.knum
    for col in range(pcs.ncol):
        bioext = [0.0] * K        # fabm_pelagic_driver.F90:784-799
        ext = lambda k: pcs.npzd["kc"] * (pcs.npzd["p0"] + pcs.conc[1, k, col] + pcs.conc[3, k, col])  # noqa: E731
        bg = pcs.background_extinction
        h = lambda k: pcs.layer_height[k, col] if pcs.mask[k, col] == 0 else 0.0  # noqa: E731
        for k in range(K - 1, 0, -1):
            bioext[k] = bioext[k] + (ext(k) + bg) * 0.5 * h(k)
            bioext[k - 1] = bioext[k] + (ext(k) + bg) * 0.5 * h(k)
        bioext[0] = bioext[0] + (ext(0) + bg) * 0.5 * h(0)
        localpar = pcs.I_0[col] * (1.0 - pcs.albedo[col])
        want = localpar * np.exp(-np.array(bioext))
        np.testing.assert_allclose(par[:, col], want, rtol=1e-14, atol=0)


def test_run_schedule_and_fluxes(po):
    """Internal steps 360, 360, 280 s for a 1000 s Run; the nitrogen of each
    column changes by exactly its boundary fluxes times the Run."""
    pcs = small()
    o = po.PelOracle(pcs)
    c = pcs.conc.copy()
    inv0 = pcs.inventory(c)
    rc, st, _ = o.run(c, t_couple=1000.0, dt=360.0, method=RUNGE_KUTTA_4, nthreads=1)
    assert rc == 0
    cells = int(pcs.water().sum())
    assert st["attempts"] == 3 * cells and st["min_dt"] == 280.0
    w = pcs.water().any(axis=0)
    change = (pcs.bottom_flux.sum(axis=0) + pcs.surface_flux.sum(axis=0)) * 1000.0
    err = np.abs(pcs.inventory(c) - inv0 - change)[w]
    assert err.max() < 1e-12 * np.abs(inv0[w]).max()


def test_soil_flux_guard_and_clip(po):
    pcs = small(8)
    pcs.bottom_flux = None
    pcs.surface_flux = None
    pcs.soil_flux = np.zeros((4, pcs.ncol))
    pcs.soil_flux[3] = -1.0e3      # would empty the bottom detritus: skipped
    pcs.soil_flux[0] = 1.0e-3      # added
    pcs.minimum = np.array([0.0, 0.5, 0.0, 0.0])   # clip phytoplankton at 0.5
    o = po.PelOracle(pcs)
    c = pcs.conc.copy()
    ref = pcs.conc.copy()
    o2 = po.PelOracle(dataclass_without_fluxes(pcs))
    rc, _, _ = o.run(c, t_couple=360.0, dt=360.0, method=EULER, nthreads=1)
    rc2, _, _ = o2.run(ref, t_couple=360.0, dt=360.0, method=EULER, nthreads=1)
    assert rc == 0 and rc2 == 0
    w = pcs.water()
    wc = w[0]
    h0 = pcs.layer_height[0]
    np.testing.assert_allclose(c[0, 0, wc], ref[0, 0, wc] + 1.0e-3 * 360.0 / h0[wc], rtol=1e-12)
    np.testing.assert_array_equal(c[3, 0, wc], ref[3, 0, wc])
    assert np.all(c[1][w] >= 0.5)


def dataclass_without_fluxes(pcs):
    q = pcs.copy()
    q.soil_flux = None
    return q


def test_adaptive_cuts_and_grid_scope(po):
    """The stiff case cuts; the grid-wide any() takes the smallest cut of any
    cell for every cell, so it needs at least as many accepted substeps per
    cell; a grid of one water cell gives the same result under both."""
    pcs = stiff(small(16))
    c1 = pcs.conc.copy()
    rc, st, _ = po.PelOracle(pcs, cut_scope=0).run(c1, method=ADAPTIVE_EULER, nthreads=1)
    assert rc == 0 and st["min_dt"] < pcs.dt and st["max_cell_attempts"] > 1
    c2 = pcs.conc.copy()
    rc, sg, _ = po.PelOracle(pcs, cut_scope=1).run(c2, method=ADAPTIVE_EULER, nthreads=1)
    assert rc == 0 and sg["min_dt"] == st["min_dt"]
    one = pcs.subset([int(np.flatnonzero(pcs.water().any(axis=0))[0])])
    one.mask = np.ones_like(one.mask)
    one.mask[one.knum // 2, 0] = 0
    a, b = one.conc.copy(), one.conc.copy()
    po.PelOracle(one, cut_scope=0).run(a, method=ADAPTIVE_EULER, nthreads=1)
    po.PelOracle(one, cut_scope=1).run(b, method=ADAPTIVE_EULER, nthreads=1)
    w = one.water()
    np.testing.assert_array_equal(a[:, w], b[:, w])


def test_threads_do_not_change_results(po):
    pcs = small()
    a, b = pcs.conc.copy(), pcs.conc.copy()
    po.PelOracle(pcs).run(a, nthreads=1)
    po.PelOracle(pcs).run(b, nthreads=4)
    np.testing.assert_array_equal(a, b)


def test_library_exports_pelagic_abi():
    path = build.build()
    text = open(f"{build.INCLUDE}/mossco_pel.h").read()
    declared = sorted(set(re.findall(r"\b(pel_[a-z_]+)\s*\(", text)))
    assert len(declared) == 14
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True,
                         text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    for name in declared:
        assert name in exported and name in pelagic.PEL_SIGNATURES, name


def test_param_struct_layout():
    p = pelagic.default_params()
    assert p.rmax == 1.0 and p.I_min == 25.0 and p.Iv == 1.1
    assert abs(p.background_extinction - 1.0 / 7.9) < 1e-15
    assert p.dt_min == 1e-8 and p.relative_change_min == -0.9
    assert p.precision == capi.SED_FP32 and p.cut_scope == pelagic.PEL_CUT_PER_CELL


def test_workload_is_seeded_and_column_addressable():
    a = pelagic.make_pelagic_workload("pelagic_cpu_16x16")
    b = pelagic.make_pelagic_workload("pelagic_cpu_16x16", cols=[5, 17, 200])
    np.testing.assert_array_equal(a.conc[:, :, [5, 17, 200]], b.conc)
    np.testing.assert_array_equal(a.layer_height[:, [5, 17, 200]], b.layer_height)
    assert 0.1 < 1 - a.water_columns() / a.ncol < 0.35


def test_open_boundary_values_in_the_oracle(po):
    """The Run's vertically homogeneous boundary values
    (fabm_pelagic_component.F90:2115-2155): an open-boundary column takes the
    value of every tracer that has one after each internal step's bottom
    fluxes, before the surface fluxes and the clip; other columns, and
    tracers without a value, are stepped as without boundaries."""
    pcs = small(32, seed=4)
    assert pcs.soil_flux is None and pcs.surface_flux is not None
    water = np.flatnonzero(pcs.water().all(axis=0))
    obc = water[[0, 3, 7]]
    ob = np.zeros(pcs.ncol, dtype=np.int32)
    ob[obc] = 1
    bv = np.full((4, pcs.ncol), np.nan)
    bv[0], bv[3] = 7.5, 0.25
    for cut in (0, 1):
        ref = pcs.conc.copy()
        assert po.PelOracle(pcs, cut_scope=cut).run(ref, nthreads=1)[0] == 0
        got = pcs.conc.copy()
        assert po.PelOracle(pcs, cut_scope=cut, open_boundary=ob,
                            boundary_value=bv).run(got, nthreads=1)[0] == 0
        rest = np.setdiff1d(np.arange(pcs.ncol), obc)
        if cut == 0:    # per-cell cuts: the other columns do not see them
            np.testing.assert_array_equal(got[:, :, rest], ref[:, :, rest])
        K = pcs.knum
        top = K - 1
        h = pcs.dt if pcs.t_couple % pcs.dt == 0 else pcs.t_couple % pcs.dt
        for c in obc:
            np.testing.assert_array_equal(got[0, :top, c], 7.5)
            np.testing.assert_array_equal(got[3, :top, c], 0.25)
            ht = pcs.layer_height[top, c]
            assert got[0, top, c] == 7.5 + pcs.surface_flux[0, c] * h / ht
            assert got[3, top, c] == 0.25 + pcs.surface_flux[3, c] * h / ht
            assert not np.array_equal(got[1, :, c], pcs.conc[1, :, c])


# ---------------------------------------------------------------- GPU

def gpu_run(pcs, precision, cut=pelagic.PEL_CUT_PER_CELL, nruns=1, method=None):
    s = pelagic.PelagicSolver(pcs, precision=precision, cut_scope=cut)
    s.set_state(pcs.conc)
    st = s.step(nruns, method=method)
    out = s.get_state()
    s.close()
    return out, st


def oracle_run(po, pcs, cut=0, nruns=1, method=None):
    c = pcs.conc.copy()
    rc, st, par = po.PelOracle(pcs, cut_scope=cut).run(c, method=method, nruns=nruns)
    assert rc == 0
    return c, st, par


@pytest.mark.gpu
@pytest.mark.parametrize("method", METHODS)
def test_run_fp64_bit_exact(po, method):
    pcs = small(256)
    out, st = gpu_run(pcs, capi.SED_FP64, nruns=2, method=method)
    ref, sref, _ = oracle_run(po, pcs, nruns=2, method=method)
    w = pcs.water()
    np.testing.assert_array_equal(out[:, w], ref[:, w])
    np.testing.assert_array_equal(out[:, ~w], pcs.conc[:, ~w])   # masked untouched
    assert st["attempts"] == sref["attempts"]
    assert st["column_steps"] == 2 * pcs.water_columns()


@pytest.mark.gpu
@pytest.mark.parametrize("cut", [pelagic.PEL_CUT_PER_CELL, pelagic.PEL_CUT_GLOBAL])
def test_adaptive_cuts_fp64_bit_exact(po, cut):
    pcs = stiff(small(64))
    out, st = gpu_run(pcs, capi.SED_FP64, cut=cut, method=ADAPTIVE_EULER)
    ref, sref, _ = oracle_run(po, pcs, cut=cut, method=ADAPTIVE_EULER)
    w = pcs.water()
    np.testing.assert_array_equal(out[:, w], ref[:, w])
    assert st["attempts"] == sref["attempts"] and st["min_dt"] == sref["min_dt"]
    assert st["max_cell_attempts"] == sref["max_cell_attempts"] > 1


@pytest.mark.gpu
def test_run_fp32_close(po):
    pcs = small(256)
    out, _ = gpu_run(pcs, capi.SED_FP32, nruns=4)
    ref, _, _ = oracle_run(po, pcs, nruns=4)
    w = pcs.water()
    scale = np.abs(ref[:, w]).max(axis=1, keepdims=True)
    assert np.max(np.abs(out[:, w] - ref[:, w]) / scale) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [capi.SED_FP64, capi.SED_FP32])
def test_light_rhs_and_drop_in_ode_solver(po, precision):
    pcs = small(128)
    o = po.PelOracle(pcs)
    s = pelagic.PelagicSolver(pcs, precision=precision)
    par = s.light(pcs.conc)
    rpar = o.light(pcs.conc)
    rhs = s.get_rhs(pcs.conc)
    rrhs = o.get_rhs(pcs.conc, rpar)
    c = pcs.conc.copy()
    st = s.ode_solver(c, 360.0, RUNGE_KUTTA_4)
    ref = pcs.conc.copy()
    rc, _ = o.ode_solver(ref, rpar, 360.0, RUNGE_KUTTA_4)
    assert rc == 0
    w = pcs.water()
    if precision == capi.SED_FP64:
        np.testing.assert_array_equal(par, rpar)
        np.testing.assert_array_equal(rhs, rrhs)
        np.testing.assert_array_equal(c[:, w], ref[:, w])
    else:
        # FP32 optical depth summed over up to 20 half layers: ~1e-5 relative
        np.testing.assert_allclose(par[w], rpar[w], rtol=5e-5, atol=1e-9)
        scale = np.abs(rrhs[:, w]).max(axis=1, keepdims=True)
        assert np.max(np.abs(rhs[:, w] - rrhs[:, w]) / scale) < 1e-5
        assert np.max(np.abs(c[:, w] - ref[:, w]) / np.abs(ref[:, w]).max(axis=1, keepdims=True)) < 1e-5
    assert st["attempts"] == int(w.sum())
    s.close()


@pytest.mark.gpu
def test_host_run_equals_device_run_and_keeps_state(po):
    pcs = small(128)
    s = pelagic.PelagicSolver(pcs, precision=capi.SED_FP64)
    s.set_state(pcs.conc)
    c = pcs.conc.copy()
    s.run(c)                              # host arrays
    np.testing.assert_array_equal(s.get_state(), pcs.conc)   # resident untouched
    s.run()                               # device state
    np.testing.assert_array_equal(s.get_state(), c)
    s.close()


@pytest.mark.gpu
def test_errors_and_call_order():
    pcs = small(16)
    s = pelagic.PelagicSolver(pcs)
    with pytest.raises(capi.SedError) as e:
        s.get_rhs(pcs.conc)              # no PAR yet
    assert e.value.code == capi.SED_E_STATE
    with pytest.raises(capi.SedError) as e:
        s.step(1)                        # no state
    assert e.value.code == capi.SED_E_STATE
    s.set_state(pcs.conc)
    with pytest.raises(capi.SedError) as e:
        s.step(1, method=7)
    assert e.value.code == capi.SED_E_ARG
    bad = pcs.conc.copy()
    bad[2, 3, int(np.flatnonzero(pcs.water()[3])[0])] = np.nan
    rc, st = s.run(bad, raise_on_error=False)
    assert rc == capi.SED_E_NAN and st["nan_cells"] >= 1
    capped = stiff(pcs)
    capped.max_attempts = 2
    s2 = pelagic.PelagicSolver(capped, precision=capi.SED_FP64)
    rc, st = s2.run(capped.conc.copy(), method=ADAPTIVE_EULER, raise_on_error=False)
    assert rc == capi.SED_E_SUBSTEP_CAP and st["capped_cells"] > 0
    s.close()
    s2.close()


@pytest.mark.gpu
def test_driver_mirror_sequence(po):
    """TypePelagic: initialize_domain, initialize_concentrations, light,
    get_rhs, ode_solver, as a caller of the reference's driver would."""
    K, inum, jnum = 12, 4, 3
    pf = pelagic.TypePelagic(inum, jnum, K, precision=capi.SED_FP64)
    depth = np.linspace(8.0, 40.0, inum * jnum)
    zi = np.linspace(0.0, 1.0, K + 1)[:, None] * depth[None, :]
    pf.initialize_domain(zi)
    pf.initialize_concentrations((4.5, 0.5, 0.2, 4.5))
    pf.I_0 = np.full(inum * jnum, 120.0)
    par = pf.light()
    assert par.shape == (K, inum * jnum) and np.all(np.diff(par, axis=0) > 0)  # brighter upwards
    rhs = pf.get_rhs()
    pcs = pf._pcs().copy()
    o = po.PelOracle(pcs)
    rpar = o.light(pcs.conc)
    np.testing.assert_array_equal(par, rpar)
    np.testing.assert_array_equal(rhs, o.get_rhs(pcs.conc, rpar))
    pf.ode_solver(600.0, RUNGE_KUTTA_4)
    ref = pcs.conc.copy()
    o.ode_solver(ref, rpar, 600.0, RUNGE_KUTTA_4)
    np.testing.assert_array_equal(pf.conc, ref)


def column_stack(K, ncol=40, seed=5):
    """ncol water columns of K layers (one masked column, one column with a
    masked bottom segment), values in the synthetic workload's ranges."""
    rng = np.random.default_rng(seed)
    h = np.repeat(rng.uniform(0.2, 3.0, ncol)[None, :], K, axis=0)
    conc = np.stack([rng.uniform(2, 10, (K, ncol)), rng.uniform(0.05, 2, (K, ncol)),
                     rng.uniform(0.02, 0.5, (K, ncol)), rng.uniform(0.5, 3.5, (K, ncol))])
    mask = np.zeros((K, ncol), dtype=np.int32)
    mask[:, 3] = 1
    mask[:K // 2, 7] = 1
    bfl = np.zeros((4, ncol))
    bfl[0] = rng.uniform(0, 3, ncol) / 86400.0
    return pelagic.PelColumnSet(inum=ncol, jnum=1, knum=K, layer_height=h, conc=conc,
                                I_0=rng.uniform(0, 250, ncol), mask=mask,
                                albedo=rng.uniform(0.05, 0.1, ncol), bottom_flux=bfl)


@pytest.mark.gpu
@pytest.mark.parametrize("K", [1, 2, 33, 300])
def test_layer_counts_fp64_bit_exact(po, K):
    pcs = column_stack(K)
    for method in (RUNGE_KUTTA_4, ADAPTIVE_EULER):
        out, st = gpu_run(pcs, capi.SED_FP64, method=method)
        ref, sref, _ = oracle_run(po, pcs, method=method)
        w = pcs.water()
        np.testing.assert_array_equal(out[:, w], ref[:, w])
        np.testing.assert_array_equal(out[:, ~w], pcs.conc[:, ~w])
        assert st["attempts"] == sref["attempts"]


@pytest.mark.gpu
def test_soil_flux_guard_and_clip_fp64_bit_exact(po):
    """The epilogue's third flux field (added unless the bottom cell would go
    negative) and a nonzero clip floor on the device, against the oracle."""
    pcs = small(64)
    pcs.soil_flux = np.zeros((4, pcs.ncol))
    pcs.soil_flux[3] = -0.005                 # removes more than some cells hold
    pcs.soil_flux[0] = 2.0e-4
    pcs.minimum = np.array([0.0, 0.3, 0.0, 0.0])
    for method in (EULER, RUNGE_KUTTA_4):
        out, _ = gpu_run(pcs, capi.SED_FP64, method=method, nruns=2)
        ref, _, _ = oracle_run(po, pcs, method=method, nruns=2)
        w = pcs.water()
        np.testing.assert_array_equal(out[:, w], ref[:, w])
        assert np.all(out[1][w] >= 0.3)


@pytest.mark.gpu
@pytest.mark.parametrize("cut", [pelagic.PEL_CUT_PER_CELL, pelagic.PEL_CUT_GLOBAL])
def test_open_boundary_values_fp64_bit_exact(po, cut):
    """The Run's vertically homogeneous open-boundary values
    (fabm_pelagic_component.F90:2115-2155) on the device: after every
    internal step's bottom fluxes an open column takes the value of every
    tracer that has one.  FP64 equals the oracle bit for bit for both cut
    scopes and every method; FP32 is close; clearing the boundaries gives
    the run without them."""
    pcs = small(96, seed=9)
    water = np.flatnonzero(pcs.water().all(axis=0))
    ob = np.zeros(pcs.ncol, dtype=np.int32)
    ob[water[[0, 5, 11, 40]]] = 1
    bv = np.full((4, pcs.ncol), np.nan)
    bv[0], bv[3] = 7.5, 0.25
    bv[1, ob != 0] = np.linspace(0.1, 0.4, int(ob.sum()))

    def device(precision, method, open_=True):
        s = pelagic.PelagicSolver(pcs, precision=precision, cut_scope=cut)
        if open_:
            s.set_open_boundary(ob, bv)
        s.set_state(pcs.conc)
        st = s.step(2, method=method)
        out = s.get_state()
        if open_:   # cleared: the next Run has no boundary values
            s.set_open_boundary(None)
        s.close()
        return out, st

    w = pcs.water()
    for method in (EULER, RUNGE_KUTTA_4, ADAPTIVE_EULER):
        out, st = device(capi.SED_FP64, method)
        ref = pcs.conc.copy()
        rc, sref, _ = po.PelOracle(pcs, cut_scope=cut, open_boundary=ob,
                                   boundary_value=bv).run(ref, method=method, nruns=2)
        assert rc == 0
        np.testing.assert_array_equal(out[:, w], ref[:, w])
        assert st["attempts"] == sref["attempts"]
        plain, _ = device(capi.SED_FP64, method, open_=False)
        assert not np.array_equal(plain[:, w], out[:, w])
    out32, _ = device(capi.SED_FP32, RUNGE_KUTTA_4)
    ref = pcs.conc.copy()
    po.PelOracle(pcs, cut_scope=cut, open_boundary=ob, boundary_value=bv).run(
        ref, method=RUNGE_KUTTA_4, nruns=2)
    scale = np.abs(ref[:, w]).max(axis=1, keepdims=True)
    assert np.max(np.abs(out32[:, w] - ref[:, w]) / scale) < 1e-4
