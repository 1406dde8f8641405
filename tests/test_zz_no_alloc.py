"""sed_ode_solver_noalloc against the handle-based sed_ode_solver.

The no-allocation entry point serves callers that cannot allocate device
memory (their framework owns the GPU's pool, or they cannot keep a solver
handle alive): it runs the tile form of the column kernel with every device
buffer in a static device array.  The per-column arithmetic of every FP32
kernel of the library is the same, so its results must equal the
handle-based drop-in bit for bit, call after call.  This file is collected
last so that a failure here leaves every other test already run; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from sedgpu import capi, synth
from sedgpu.model import ADAPTIVE_EULER

pytestmark = pytest.mark.gpu


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def noalloc_step(cs, params, conc, fluxes, dt, method=ADAPTIVE_EULER):
    lib = capi.load()
    st = capi.SedStats()
    kact = np.ascontiguousarray(cs.kact, dtype=np.int32)
    rc = lib.sed_ode_solver_noalloc(
        ctypes.byref(params), cs.inum, cs.jnum, cs.kmax,
        _p(np.ascontiguousarray(cs.dz)), _p(np.ascontiguousarray(cs.dzc)),
        _p(np.ascontiguousarray(cs.phi)), _p(np.ascontiguousarray(cs.phi_i)),
        _p(np.ascontiguousarray(cs.biofac)), _p(np.ascontiguousarray(cs.flux_cap)),
        _p(kact, ctypes.c_int), _p(conc), _p(np.ascontiguousarray(cs.bdys)),
        _p(fluxes), float(dt), int(method), ctypes.byref(st))
    return rc, st.as_dict()


def active(cs, c):
    K = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    return c[:, K]


def deep_grid():
    """Columns of 20..100 active layers: every depth class, four layers per
    lane in the deepest."""
    return synth.make_columns(inum=40, jnum=1, kmin=20, kmax=100, total=0.3, land=0.1,
                              poc="uniform", days=1, seed=3, name="deep40x100")


@pytest.mark.parametrize("workload,cols", [
    ("plain_cpu_10x10", None),
    ("uneven_1024x1024", np.arange(0, 1024 * 1024, 3499)[:300]),
    ("deep", None),
])
def test_noalloc_matches_handle_two_calls(workload, cols):
    cs = deep_grid() if workload == "deep" else synth.make_workload(workload, cols=cols)
    params = capi.params_from(cs, capi.SED_FP32)
    ref_conc = cs.conc.copy()
    ref_fl = cs.fluxes.copy()
    new_conc = cs.conc.copy()
    new_fl = cs.fluxes.copy()
    with capi.Solver(cs, params=capi.params_from(cs, capi.SED_FP32)) as s:
        for call in range(2):
            st_ref = s.ode_solver(ref_conc, cs.bdys, ref_fl, cs.dt, ADAPTIVE_EULER)
            rc, st = noalloc_step(cs, params, new_conc, new_fl, cs.dt)
            assert rc == capi.SED_OK, (call, rc)
            np.testing.assert_array_equal(active(cs, new_conc), active(cs, ref_conc))
            np.testing.assert_array_equal(new_fl, ref_fl)
            assert st["column_steps"] == st_ref["column_steps"] == cs.n_active
            assert st["gpu_launches"] > 0
    # land columns and inactive layers are handed back untouched
    land = cs.kact == 0
    np.testing.assert_array_equal(new_conc[:, :, land], cs.conc[:, :, land])


def test_noalloc_rejects_oversized_grid():
    cs = synth.make_workload("plain_cpu_10x10")
    params = capi.params_from(cs, capi.SED_FP32)
    lib = capi.load()
    st = capi.SedStats()
    big = 30000  # columns of 20 layers (~3.2 KB each): more than 64 MiB
    dz = np.ones((20, big))
    conc = np.ones((11, 20, big))
    fl = np.zeros((11, big))
    bd = np.ones((12, big))
    rc = lib.sed_ode_solver_noalloc(
        ctypes.byref(params), big, 1, 20, _p(dz), _p(dz[:19].copy()),
        _p(0.8 * dz), _p(0.8 * dz), _p(dz), None, None, _p(conc), _p(bd),
        _p(fl), 3600.0, ADAPTIVE_EULER, ctypes.byref(st))
    assert rc == capi.SED_E_TOO_LARGE
    assert lib.sed_error_string(rc).decode().startswith("grid exceeds")
