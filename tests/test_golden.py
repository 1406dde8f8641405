"""The reference's standalone one-column OMEXDIA+P example
(examples/standalone/omexdia_p, run_sed.nml and fabm_sed.nml) as a golden
fixture (tests/golden/omexdia_p_example.json, written by
tests/golden/make_golden.py from the reference's files).

The fixture holds the example's inputs as the reference's namelists give
them and the FP64 oracle's state after 24 of its 360 s steps.  CPU: the
package's parameter defaults are the example's, and the oracle reproduces
the stored state bit for bit (on the machine type that wrote it).  GPU: the
FP64 device path equals the oracle on the same inputs bit for bit, and the
stored state to 1e-9 (host libm values may differ between machine types in
the last bit)."""
import json
import os
import sys

import numpy as np
import pytest

from sedgpu import capi
from sedgpu.model import ADAPTIVE_EULER, BGC_DEFAULTS, BGC_NAMES

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import golden_case  # noqa: E402


@pytest.fixture(scope="module")
def fixture():
    with open(os.path.join(HERE, "omexdia_p_example.json")) as f:
        return json.load(f)


def test_package_defaults_are_the_example_parameters(fixture):
    p = fixture["hzg_omexdia_p"]
    for name in BGC_NAMES:
        assert BGC_DEFAULTS[name] == p[name], name
    run = fixture["run_nml"]
    assert run["ode_method"] == ADAPTIVE_EULER and run["dt"] == 360.0


def test_example_column_is_built_as_the_reference_does(fixture):
    cs = golden_case.column_set(fixture)
    K = int(fixture["run_nml"]["numlayers"])
    assert cs.kmax == K and cs.ncol == 1 and cs.kact[0] == K
    assert cs.driver.bcup_dissolved == 1 and cs.driver.dt_min == 1.0
    # bioturbation profile 0 keeps the factor at 1; initial values per pore water
    np.testing.assert_array_equal(cs.biofac, np.ones_like(cs.biofac))
    assert cs.conc[0, 0, 0] == fixture["hzg_omexdia_p"]["ldetC_init"] / cs.phi[0, 0]


def test_oracle_reproduces_the_golden_state(oracle_mod, fixture):
    cs = golden_case.column_set(fixture)
    c = cs.conc.copy()
    rc, st, fl = oracle_mod.OracleModel(cs).run(c, nsteps=fixture["nsteps"], percol=True,
                                                nthreads=1)
    assert rc == 0
    assert st["attempts"] == fixture["attempts"]
    np.testing.assert_array_equal(c[:, :, 0], np.array(fixture["state"]))
    np.testing.assert_array_equal(fl[:, 0], np.array(fixture["fluxes"]))


@pytest.mark.gpu
def test_fp64_device_reproduces_the_example(oracle_mod, fixture):
    cs = golden_case.column_set(fixture)
    s = capi.Solver(cs, precision=capi.SED_FP64)
    s.set_forcing()
    s.set_state(cs.conc)
    st = s.step(fixture["nsteps"], method=ADAPTIVE_EULER)
    out = s.get_state()[:, :, 0]
    s.close()
    ref = cs.conc.copy()
    rc, sref, _ = oracle_mod.OracleModel(cs).run(ref, nsteps=fixture["nsteps"], percol=True,
                                                 nthreads=1)
    assert rc == 0
    np.testing.assert_array_equal(out, ref[:, :, 0])
    assert st["attempts"] == sref["attempts"]
    gold = np.array(fixture["state"])
    scale = np.abs(gold).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(out - gold) / scale) < 1e-9


def test_pelagic_defaults_are_the_example_gotm_npzd():
    """The pelagic path's gotm_npzd parameters and initial values are those
    of the reference's fabm0d examples (tests/golden/gotm_npzd_example.json)."""
    from sedgpu import pelagic
    with open(os.path.join(HERE, "gotm_npzd_example.json")) as f:
        nml = json.load(f)["gotm_npzd"]
    for name in pelagic.NPZD_NAMES:
        assert pelagic.NPZD_DEFAULTS[name] == nml[name], name
    assert pelagic.NPZD_INITIAL == (nml["n_initial"], nml["p_initial"], nml["z_initial"],
                                    nml["d_initial"])
