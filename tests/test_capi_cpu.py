"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, exports
every function include/mossco_sed.h declares, and refuses work without a
GPU instead of computing anything on the host."""
import ctypes
import subprocess

import numpy as np
import pytest

from conftest import gpu_available
from sedgpu import build, capi, synth
from sedgpu.model import NTR, TRACERS


@pytest.fixture(scope="module")
def lib():
    return capi.load()


def test_exports_every_declared_function(lib):
    declared = capi.header_functions()
    assert len(declared) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    for name in declared:
        assert name in exported, name
        assert name in capi.SIGNATURES, name
        getattr(lib, name)


def test_param_struct_layout(lib):
    p = capi.default_params()
    assert p.bcup_dissolved == 2 and p.bcup_particulate == 1
    assert p.relative_change_min == -0.9 and p.dt_min == 1e-9
    assert p.rnit == 200.0 and p.PAdsODU == 70.0
    assert p.epilogue == 1 and p.precision == capi.SED_FP32


def test_tracer_table(lib):
    for n in range(NTR):
        assert lib.sed_tracer_name(n).decode() == TRACERS[n]
        assert lib.sed_tracer_is_particulate(n) == (1 if n < 6 else 0)
    assert lib.sed_error_string(capi.SED_E_NAN).decode() == "NaN in state"


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU path")
def test_no_device_refuses(lib):
    cs = synth.make_workload("plain_cpu_10x10")
    with pytest.raises(capi.SedError) as e:
        capi.Solver(cs)
    assert e.value.code == capi.SED_E_NODEVICE


def test_bad_sizes_rejected_before_device(lib):
    p = capi.default_params()
    h = capi._H()
    assert lib.sed_create(ctypes.byref(p), 0, 4, 10, NTR, ctypes.byref(h)) == capi.SED_E_ARG
    assert lib.sed_create(ctypes.byref(p), 4, 4, capi.SED_KMAX_LIMIT + 1, NTR,
                          ctypes.byref(h)) == capi.SED_E_ARG
    assert lib.sed_create(ctypes.byref(p), 4, 4, 10, 12, ctypes.byref(h)) == capi.SED_E_ARG
    assert lib.sed_create(None, 4, 4, 10, NTR, ctypes.byref(h)) == capi.SED_E_ARG


def test_host_allocator_checks_its_arguments(lib):
    """sed_host_alloc refuses a null result pointer or zero bytes, and
    without a device it answers SED_E_NODEVICE with a null pointer."""
    p = ctypes.c_void_p(123)
    assert lib.sed_host_alloc(0, ctypes.byref(p)) == capi.SED_E_ARG
    assert p.value is None
    assert lib.sed_host_alloc(16, None) == capi.SED_E_ARG
    assert lib.sed_host_free(None) == capi.SED_E_ARG
    rc = lib.sed_host_alloc(16, ctypes.byref(p))
    if rc == capi.SED_OK:       # a GPU is present: the memory is usable
        assert p.value is not None
        assert lib.sed_host_free(p) == capi.SED_OK
    else:
        assert rc == capi.SED_E_NODEVICE and p.value is None


def test_synth_subset_is_counter_based():
    full = synth.make_workload("uneven_1024x1024", cols=np.arange(0, 5000))
    sub = synth.make_workload("uneven_1024x1024", cols=np.array([17, 4242, 999]))
    for name in ("kact", "dz", "phi", "bdys", "fluxes", "conc"):
        a = getattr(full, name)
        b = getattr(sub, name)
        np.testing.assert_array_equal(a[..., [17, 4242, 999]], b, err_msg=name)


def test_synth_workload_shapes():
    cs = synth.make_workload("plain_cpu_10x10")
    assert cs.ncol == 100 and cs.kmax == 20 and cs.nsteps == 240
    assert abs(cs.dz[:, 0].sum() - 0.18) < 1e-12
    assert abs(cs.dz[1, 0] / cs.dz[0, 0] - 1.19699) < 1e-4
    cs = synth.make_workload("plain_gpu_256x256", cols=np.arange(4))
    assert cs.kmax == 30 and abs(cs.dz[:, 0].sum() - 0.2) < 1e-12
    assert abs(cs.dz[1, 0] / cs.dz[0, 0] - 1.11026) < 1e-4
    # porosity and bottom-water ranges of the workload definition
    assert np.allclose(cs.phi, 0.7 + 0.2 * np.exp(-cs.zc / 0.02))
    assert (150 <= cs.bdys[7]).all() and (cs.bdys[7] <= 300).all()
    cs = synth.make_workload("uneven_1024x1024", cols=np.arange(20000))
    land = (cs.kact == 0).mean()
    assert 0.27 < land < 0.33
    act = cs.kact[cs.kact > 0]
    assert act.min() == 10 and act.max() == 60
    # the soil under the pelagic grid of the coupling measurement: 15 layers
    # (examples/standalone/omexdia_p/run_sed.nml:34), 0.18 m, 30 % land
    cs = synth.make_workload("soil_1024x1024", cols=np.arange(20000))
    assert cs.kmax == 15 and 0.27 < (cs.kact == 0).mean() < 0.33
    assert set(np.unique(cs.kact)) <= {0, 15}
    assert abs(cs.dz[:, np.flatnonzero(cs.kact)[0]].sum() - 0.18) < 1e-12
