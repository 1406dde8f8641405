"""Pelagic -> soil coupling (include/mossco_cpl.h) against the connector oracle.

The reference maps the pelagic state's bottom layer to the soil's surface
fields in pelagic_soil_connector's Run
(src/mediators/pelagic_soil_connector.F90:176-2122) and the sediment
component turns them into bdys / fluxes (get_boundary_conditions,
src/components/fabm_sediment_component.F90:1865-2030).  CPU tests check the
oracle (oracle/cpl_oracle.c) against a vectorised restatement written here
from the same source lines, the connector's default-real literals and the
library's exports.  GPU tests check the device coupling bit for bit against
the oracle for FP64 and FP32 pelagic state, after device-resident steps, and
a coupled pelagic / soil loop against the same loop routed through the host.
"""
import os
import subprocess

import numpy as np
import pytest

from cases import small
from sedgpu import build, capi, coupling, pelagic

pel_oracle = pytest.importorskip("pel_oracle")

NPZD = dict(detN=3, din=0)
# field tables that reach every branch of the Run with gotm_npzd's four
# tracers standing in for the other models' fields
FIELD_SETS = [
    NPZD,
    dict(detN=3, detC=2, nitrate=0, ammonium=1),            # C:N from detC, critical detritus
    dict(detN=3, detP=2, din=0, nitrate=1, oxygen=2, odu=1),
    dict(detN=3, din=0, ammonium=2, odu=1),                 # deficit split
    dict(nitrate=0, oxygen=2),                              # no detritus, oxygen only
    dict(ammonium=1),                                       # DIN from 2 x ammonium
]


@pytest.fixture(scope="module")
def po():
    pel_oracle.build()
    return pel_oracle


def pel_case(ncol, seed=0):
    return pelagic.make_pelagic_workload("pelagic_cpu_16x16", cols=np.arange(ncol), seed=seed)


def numpy_run(conc, fields, p, as_named, depth=None, tke=None, velocity_in=None):
    """The Run restated with whole-array numpy expressions."""
    b = {k: conc[v, 0, :] for k, v in fields.items() if v >= 0}
    ncol = conc.shape[2]
    S = np.zeros((11, ncol))
    V = np.zeros((11, ncol))
    if velocity_in is not None:
        V[:6] = velocity_in[:6]
    f1e5, f1e3, f9e9 = float(np.float32(1e-5)), float(np.float32(1e-3)), float(np.float32(9e9))
    if "oxygen" in b and "odu" in b:
        S[6], S[9] = b["oxygen"], b["odu"]
    elif "odu" in b:
        S[6], S[9] = np.maximum(0.0, -b["odu"]), np.maximum(0.0, b["odu"])
    elif "oxygen" in b:
        S[6] = b["oxygen"]
    CN = np.full(ncol, 106.0 / 16.0)
    if "detN" in b and "detC" in b:
        CN = b["detC"] / (f1e5 + b["detN"])
    fl = (1.0 - p["NC_sdet"] * CN) / (p["NC_ldet"] - p["NC_sdet"])
    rl = fl * p["NC_ldet"]
    hi = fl > CN
    fl, rl = np.where(hi, CN, fl), np.where(hi, 1.0, rl)
    lo = fl < 0.0
    fl, rl = np.where(lo, 0.0, fl), np.where(lo, 0.0, rl)
    fs, rs = CN - fl, 1.0 - rl
    fe = np.ones(ncol)
    hsd = p["half_sedimentation_depth"]
    if depth is not None and hsd > f1e3:
        fe = fe * (depth * depth) / (depth * depth + hsd * hsd)
    if tke is not None and p["half_sedimentation_tke"] < f9e9:
        fe = fe * p["half_sedimentation_tke"] / (tke + p["half_sedimentation_tke"])
    fe = fe + p["sinking_factor_min"] / p["sinking_factor"]
    if "detC" in b and f1e3 < p["critical_detritus"] < f9e9:
        x = b["detC"] / p["critical_detritus"]
        fe = fe * 1.0 / (1.0 + (x * x) * (x * x))
    cN, cP = p["convertN"], p["convertP"]
    if "detN" in b:
        N = b["detN"]
        w = p["sinking_factor"] * fe * N
        for row, fac in zip((0, 1, 2, 3), (fl, fs, rl, rs)):
            if as_named:
                S[row], V[row] = fac * cN * N, w
            else:
                S[row] = w
        S[4], V[4] = 1.0 / 16.0 * cN * N, w
    if "detP" in b:
        S[4] = b["detP"]
    hN, hA, hD = "nitrate" in b, "ammonium" in b, "din" in b
    z = np.zeros(ncol)
    Nt, A, D = b.get("nitrate", z), b.get("ammonium", z), b.get("din", z)
    S[8] = (cN * A if hA else cN * (D - Nt) if hD and hN else cN * 0.5 * D if hD else cN * Nt)
    nit = (cN * Nt if hN else cN * (D - A) if hA and hD else cN * 0.5 * D if hD else cN * A)
    if as_named:
        S[7] = nit
    else:        # the nitrate block writes through the ammonium field
        S[8] = nit
    din = D if hD else Nt + A if hA and hN else 2 * A if hA else 2 * Nt
    S[10] = cP * (1.0 / 16.0 * cN * din)
    return S, V


# ---------------------------------------------------------------- CPU

def test_library_exports_coupling_abi():
    path = build.build()
    declared = coupling.header_functions()
    assert declared == ["cpl_default_params", "cpl_npzd_fields", "cpl_pelagic_soil",
                        "cpl_soil_default_params", "cpl_soil_pelagic"]
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for name in declared:
        assert name in exported and name in coupling.CPL_SIGNATURES, name


def test_defaults_are_the_connectors_literals(po):
    p = coupling.default_params()
    assert p.sinking_factor == 0.3 and p.NC_ldet == 0.23 and p.NC_sdet == 0.01
    # 0.02 and 0.1 are default-real literals in the reference (:43-44)
    assert p.sinking_factor_min == float(np.float32(0.02)) != 0.02
    assert p.half_sedimentation_depth == float(np.float32(0.1)) != 0.1
    assert p.half_sedimentation_tke == 1000.0 and p.critical_detritus == 60.0
    assert p.mode == coupling.CPL_AS_RUN
    od = po.cpl_defaults()
    for n in coupling.PARAM_NAMES:
        assert getattr(p, n) == od[n], n
    f = coupling.npzd_fields()
    assert (f.detN, f.din) == (3, 0)
    assert all(getattr(f, n) == -1 for n in coupling.FIELD_NAMES if n not in ("detN", "din"))


def test_null_handles_are_refused():
    L = coupling.load()
    p, f = coupling.default_params(), coupling.npzd_fields()
    st = coupling.CplStats()
    st.gpu_launches = 7
    assert L.cpl_pelagic_soil(None, None, p, f, None, None, None, None, None, None,
                              None, st) == capi.SED_E_ARG
    assert st.gpu_launches == 0   # cleared on entry
    st.gpu_launches = 7
    assert L.cpl_soil_pelagic(None, None, coupling.soil_default_params(), f, None, None,
                              st) == capi.SED_E_ARG
    assert st.gpu_launches == 0


@pytest.mark.parametrize("fields", FIELD_SETS)
@pytest.mark.parametrize("as_named", [False, True])
def test_oracle_matches_numpy_restatement(po, fields, as_named):
    pcs = pel_case(40, seed=3)
    conc = pcs.conc.copy()
    rng = np.random.default_rng(5)
    conc[2, 0] *= rng.uniform(0.0, 40.0, conc.shape[2])   # C:N over the clamps
    conc[1, 0] -= 1.5                                       # a deficit of both signs
    depth = rng.uniform(0.02, 40.0, conc.shape[2])
    tke = rng.uniform(0.0, 3e3, conc.shape[2])
    vin = rng.uniform(-1e-4, 0.0, (6, conc.shape[2]))
    p = po.cpl_defaults()
    p.update(convertN=1.1, convertP=0.9)
    for d, t in ((None, None), (depth, tke)):
        rc, S, V, present = po.cpl_run(conc, fields, p, as_named, d, t, vin)
        assert rc == 0
        S2, V2 = numpy_run(conc, fields, p, as_named, d, t, vin)
        np.testing.assert_array_equal(S, S2)
        np.testing.assert_array_equal(V, V2)
        assert present[8] == present[10] == 1 and present[7] == int(as_named)
        assert present[5] == 0
        assert present[0] == ("detN" in fields)


def test_oracle_run_as_written_overwrites_the_concentrations(po):
    """CPL_AS_RUN: the four C / N concentration fields carry the velocity
    formula and their velocities stay as they were; AS_NAMED splits by C:N."""
    pcs = pel_case(16)
    p = po.cpl_defaults()
    rc, S, V, _ = po.cpl_run(pcs.conc, NPZD, p, False)
    N = pcs.conc[3, 0]
    w = p["sinking_factor"] * (1.0 + p["sinking_factor_min"] / p["sinking_factor"]) * N
    for row in range(4):
        np.testing.assert_array_equal(S[row], w)
        assert not V[row].any()
    np.testing.assert_array_equal(V[4], w)
    np.testing.assert_array_equal(S[4], 1.0 / 16.0 * N)
    rc, S, V, _ = po.cpl_run(pcs.conc, NPZD, p, True)
    # Redfield C:N 6.625 with NC_ldet 0.23, NC_sdet 0.01: fac_ldet = 0.93375/0.22
    fl = (1.0 - 0.01 * 6.625) / 0.22
    np.testing.assert_allclose(S[0], fl * N, rtol=1e-15)
    np.testing.assert_allclose(S[0] + S[1], 6.625 * N, rtol=1e-14)
    np.testing.assert_allclose(S[2] + S[3], N, rtol=1e-14)
    np.testing.assert_array_equal(V[:5], np.repeat(w[None], 5, axis=0))
    # gotm_npzd has DIN only: half of it as nitrate, half as ammonium
    np.testing.assert_array_equal(S[7], 0.5 * pcs.conc[0, 0])
    np.testing.assert_array_equal(S[8], S[7])
    np.testing.assert_array_equal(S[10], 1.0 / 16.0 * pcs.conc[0, 0])
    # as written, the nitrate value lands in the ammonium field and the
    # nitrate field is not written (pelagic_soil_connector.F90:1863-1935)
    rc, S, V, present = po.cpl_run(pcs.conc, dict(din=0, nitrate=1), p, False)
    np.testing.assert_array_equal(S[8], pcs.conc[1, 0])
    assert not S[7].any() and present[7] == 0 and present[8] == 1
    rc, S, V, present = po.cpl_run(pcs.conc, dict(din=0, nitrate=1), p, True)
    np.testing.assert_array_equal(S[7], pcs.conc[1, 0])
    np.testing.assert_array_equal(S[8], pcs.conc[0, 0] - pcs.conc[1, 0])
    assert present[7] == present[8] == 1


def test_oracle_without_nitrogen_is_not_found(po):
    rc, *_ = po.cpl_run(pel_case(8).conc, dict(detN=3), po.cpl_defaults(), False)
    assert rc == -1


# the reverse Run's field tables (pelagic rows of the fields it writes)
SOIL_FIELD_SETS = [
    NPZD,                                                   # gotm_npzd: DIN and detN
    dict(nitrate=0, ammonium=1, dip=2, detC=3),
    dict(din=0, oxygen=1, odu=2, detP=3),
    dict(odu=1, detN=3),                                    # deficit as odu - oxygen
    dict(oxygen=2, din=0),                                  # oxygen - odu
]


def numpy_soil_run(fluxes, fields, p, bfl_in):
    """The reverse Run restated with whole-array numpy expressions."""
    up = -fluxes
    out = bfl_in.copy()
    year = float(np.float32(86400.0) * np.float32(365.0))
    g = {k: v for k, v in fields.items() if v >= 0}
    if "nitrate" in g:
        out[g["nitrate"]] = up[7]
    if "ammonium" in g:
        out[g["ammonium"]] = p["convertN"] * up[8]
    if "din" in g:
        out[g["din"]] = (up[8] + up[7] + p["dinflux_const"] / year) * p["convertN"]
    if "dip" in g:
        out[g["dip"]] = p["convertP"] * (up[10] + p["dipflux_const"] / year)
    if "odu" in g and "oxygen" in g:
        out[g["odu"]], out[g["oxygen"]] = up[9], up[6]
    elif "odu" in g:
        out[g["odu"]] = up[9] - up[6]
    elif "oxygen" in g:
        out[g["oxygen"]] = up[6] - up[9]
    if "detN" in g:
        out[g["detN"]] = 0.0 + up[2] + up[3]
    if "detC" in g:
        out[g["detC"]] = 0.0 + up[0] + up[1]
    if "detP" in g:          # 'detritus*phosphorous': no soil name matches
        out[g["detP"]] = 0.0
    return out


def test_soil_defaults_are_the_connectors_literals(po):
    p = coupling.soil_default_params()
    od = po.cpl_soil_defaults()
    assert (p.dinflux_const, p.dipflux_const, p.convertN, p.convertP) == (0.0, -1.0, 1.0, 1.0)
    assert (p.NC_ldet, p.NC_sdet) == (0.2, 0.04)
    for n in coupling.SOIL_PARAM_NAMES:
        assert getattr(p, n) == od[n], n


@pytest.mark.parametrize("fields", SOIL_FIELD_SETS)
def test_soil_oracle_matches_numpy_restatement(po, fields):
    rng = np.random.default_rng(9)
    ncol = 50
    fluxes = rng.normal(0.0, 1e-5, (11, ncol))
    bfl_in = rng.normal(0.0, 1e-6, (4, ncol))
    p = po.cpl_soil_defaults()
    p.update(convertN=1.3, convertP=0.7, dinflux_const=2.5)
    got, present = po.cpl_soil_run(fluxes, fields, p, bfl_in)
    np.testing.assert_array_equal(got, numpy_soil_run(fluxes, fields, p, bfl_in))
    for name, row in fields.items():
        assert present[row] == 1, name
    assert present.sum() == len(fields)


HARNESS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cpl_map_harness.cu")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    """The kernels' per-column functions (csrc/cpl_map.cuh) compiled for the
    host with nvcc, as tests/cpl_map_harness.cu drives them."""
    exe = tmp_path_factory.mktemp("cplmap") / "harness"
    r = subprocess.run([build.nvcc(), *build.ARCH, "-std=c++17", "-O2", "-Xcompiler",
                        "-ffp-contract=off", "-I", build.CSRC, HARNESS, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def _hex(values):
    return " ".join(float(v).hex() for v in np.ravel(values))


def _fields_line(d):
    return " ".join(str(int(d.get(n, -1))) for n in coupling.FIELD_NAMES)


@pytest.mark.parametrize("as_named", [False, True])
def test_kernel_arithmetic_on_the_host_matches_the_oracle(po, harness, as_named):
    """The forward kernel's per-column function, run on the host, equals the
    connector oracle bit for bit over every field table, with and without
    water depth and turbulence."""
    pcs = pel_case(40, seed=5)
    conc = pcs.conc.copy()
    rng = np.random.default_rng(8)
    conc[2, 0] *= rng.uniform(0.0, 40.0, conc.shape[2])
    conc[1, 0] -= 1.5
    ncol = conc.shape[2]
    depth = rng.uniform(0.02, 40.0, ncol)
    tke = rng.uniform(0.0, 3e3, ncol)
    vin = rng.uniform(-1e-4, 0.0, (6, ncol))
    p = po.cpl_defaults()
    p.update(convertN=1.1, convertP=0.9)
    cases, refs = [], []
    for fields in FIELD_SETS:
        for d, t in ((None, None), (depth, tke)):
            lines = ["F", _hex([p[n] for n in coupling.PARAM_NAMES]) + f" {int(as_named)}",
                     _fields_line(fields), f"{int(d is not None)} {int(t is not None)} {ncol}"]
            for c in range(ncol):
                lines.append(_hex(list(conc[:, 0, c]) + [0.0 if d is None else d[c],
                                                          0.0 if t is None else t[c]]))
            cases.append("\n".join(lines))
            refs.append(po.cpl_run(conc, fields, p, as_named, d, t, vin))
    out = subprocess.run([harness], input="\n".join(cases) + "\n", capture_output=True,
                         text=True, check=True).stdout.split("\n")
    row = 0
    for rc, S, V, present in refs:
        assert rc == 0
        for c in range(ncol):
            tok = out[row].split()
            row += 1
            got = np.array([float.fromhex(x) for x in tok[:11]])
            srows, w, vrows = int(tok[11]), float.fromhex(tok[12]), int(tok[13])
            np.testing.assert_array_equal(got, S[:, c])
            assert [int((srows >> n) & 1) for n in range(11)] == list(present)
            v = vin[:, c].copy()
            for n in range(6):
                if (vrows >> n) & 1:
                    v[n] = w
            np.testing.assert_array_equal(v, V[:6, c])


def test_reverse_kernel_arithmetic_on_the_host_matches_the_oracle(po, harness):
    rng = np.random.default_rng(12)
    ncol = 30
    fluxes = rng.normal(0.0, 1e-5, (11, ncol))
    bfl_in = rng.normal(0.0, 1e-6, (4, ncol))
    p = po.cpl_soil_defaults()
    p.update(convertN=1.3, convertP=0.7, dinflux_const=2.5)
    cases, refs = [], []
    for fields in SOIL_FIELD_SETS:
        lines = ["R", _hex([p[n] for n in coupling.SOIL_PARAM_NAMES]), _fields_line(fields),
                 str(ncol)]
        for c in range(ncol):
            lines.append(_hex(list(fluxes[:, c]) + list(bfl_in[:, c])))
        cases.append("\n".join(lines))
        refs.append(po.cpl_soil_run(fluxes, fields, p, bfl_in)[0])
    out = subprocess.run([harness], input="\n".join(cases) + "\n", capture_output=True,
                         text=True, check=True).stdout.split("\n")
    row = 0
    for ref in refs:
        for c in range(ncol):
            got = [float.fromhex(x) for x in out[row].split()]
            row += 1
            np.testing.assert_array_equal(got, ref[:, c])


# ---------------------------------------------------------------- GPU

def handles(ncol, pel_precision, sed_precision=capi.SED_FP32, seed=0):
    pcs = pel_case(ncol, seed=seed)
    cs = small(ncol=ncol, K=14, seed=seed + 1)
    pel = pelagic.PelagicSolver(pcs, precision=pel_precision)
    pel.set_state(pcs.conc)
    sed = capi.Solver(cs, precision=sed_precision)
    sed.set_state(cs.conc)
    return pcs, cs, pel, sed


def fields_struct(d):
    return coupling.CplFields(*[int(d.get(n, -1)) for n in coupling.FIELD_NAMES])


@pytest.mark.gpu
@pytest.mark.parametrize("pel_precision", [capi.SED_FP64, capi.SED_FP32])
@pytest.mark.parametrize("fields", FIELD_SETS)
@pytest.mark.parametrize("as_named", [False, True])
def test_device_coupling_bit_exact(po, pel_precision, fields, as_named):
    ncol = 300
    pcs, cs, pel, sed = handles(ncol, pel_precision)
    rng = np.random.default_rng(11)
    T = rng.uniform(2.0, 20.0, ncol)
    depth = rng.uniform(0.05, 60.0, ncol)
    tke = rng.uniform(0.0, 2e3, ncol)
    vin = np.zeros((capi.NTR, ncol))
    vin[:6] = rng.uniform(-2e-4, 0.0, (6, ncol))
    p = coupling.default_params(mode=int(as_named), convertN=1.1)
    S, V, present = coupling.pelagic_soil(pel, sed, T, depth, tke, vin, params=p,
                                          fields=fields_struct(fields))
    state = pel.get_state()   # the bits the device holds (FP32-rounded when FP32)
    po_p = {n: getattr(p, n) for n in coupling.PARAM_NAMES}
    rc, S0, V0, P0 = po.cpl_run(state, fields, po_p, as_named, depth, tke, vin)
    assert rc == 0
    np.testing.assert_array_equal(present, P0)
    np.testing.assert_array_equal(S, S0)
    np.testing.assert_array_equal(V[:6], V0[:6])
    bd, fl = sed.boundary()
    # the same boundary through the host route
    ref = capi.Solver(cs, precision=capi.SED_FP32)
    ref.set_state(cs.conc)
    ref.set_boundary(T, S0, V0, P0)
    bd0, fl0 = ref.boundary()
    np.testing.assert_array_equal(bd, bd0)
    np.testing.assert_array_equal(fl, fl0)
    for s in (pel, sed, ref):
        s.close()


@pytest.mark.gpu
def test_coupling_reads_the_stepped_device_state(po):
    """cpl_pelagic_soil after pel_step (no host copy in between) sees the
    stepped state: the event orders the sediment stream after the pelagic
    one."""
    pcs, cs, pel, sed = handles(256, capi.SED_FP32, seed=4)
    T = np.full(256, 10.0)
    for _ in range(3):
        pel.step(2)
        st = coupling.CplStats()
        S, V, present = coupling.pelagic_soil(pel, sed, T, stats=st)
        assert st.gpu_launches == 3 and st.columns == 256   # mapping, assembly, forcing rows
        assert 0.0 < st.kernel_ms <= st.device_ms
        rc, S0, V0, _ = po.cpl_run(pel.get_state(), NPZD, po.cpl_defaults(), False)
        np.testing.assert_array_equal(S, S0)
        np.testing.assert_array_equal(V[:6], V0[:6])
    pel.close()
    sed.close()


@pytest.mark.gpu
@pytest.mark.parametrize("sed_precision", [capi.SED_FP32, capi.SED_FP64])
def test_coupled_loop_equals_host_route(po, sed_precision):
    """pel_step -> cpl_pelagic_soil -> sed_step for a few coupling steps
    equals the loop that takes the pelagic state to the host, maps it with
    the oracle and calls sed_set_boundary."""
    ncol = 128
    pcs, cs, pel, sed = handles(ncol, capi.SED_FP32, sed_precision, seed=6)
    _, _, pel2, sed2 = handles(ncol, capi.SED_FP32, sed_precision, seed=6)
    T = np.linspace(4.0, 16.0, ncol)
    depth = np.linspace(1.0, 50.0, ncol)
    for _ in range(3):
        pel.step(1)
        coupling.pelagic_soil(pel, sed, T, depth)
        sed.step(1)
        pel2.step(1)
        rc, S0, V0, P0 = po.cpl_run(pel2.get_state(), NPZD, po.cpl_defaults(), False, depth)
        sed2.set_boundary(T, S0, V0, P0)
        sed2.step(1)
    np.testing.assert_array_equal(pel.get_state(), pel2.get_state())
    np.testing.assert_array_equal(sed.get_state(), sed2.get_state())
    for s in (pel, sed, pel2, sed2):
        s.close()


@pytest.mark.gpu
def test_coupling_errors():
    pcs, cs, pel, sed = handles(64, capi.SED_FP32)
    T = np.full(64, 10.0)
    with pytest.raises(capi.SedError) as e:
        coupling.pelagic_soil(pel, sed, T, fields=fields_struct(dict(detN=3)))
    assert e.value.code == capi.SED_E_ARG
    with pytest.raises(capi.SedError) as e:
        coupling.pelagic_soil(pel, sed, T, fields=fields_struct(dict(detN=7, din=0)))
    assert e.value.code == capi.SED_E_ARG
    with pytest.raises(capi.SedError) as e:
        coupling.pelagic_soil(pel, sed, T, params=coupling.default_params(mode=5))
    assert e.value.code == capi.SED_E_ARG
    fresh = pelagic.PelagicSolver(pcs)          # no state yet
    with pytest.raises(capi.SedError) as e:
        coupling.pelagic_soil(fresh, sed, T)
    assert e.value.code == capi.SED_E_STATE
    other = capi.Solver(small(ncol=32, K=10), precision=capi.SED_FP32)
    with pytest.raises(capi.SedError) as e:
        coupling.pelagic_soil(pel, other, np.full(32, 10.0))
    assert e.value.code == capi.SED_E_ARG
    coupling.pelagic_soil(pel, sed, T)           # the handles still work
    for s in (pel, sed, fresh, other):
        s.close()


def soil_fields_struct(d):
    return coupling.CplFields(*[int(d.get(n, -1)) for n in coupling.FIELD_NAMES])


@pytest.mark.gpu
@pytest.mark.parametrize("pel_precision", [capi.SED_FP64, capi.SED_FP32])
@pytest.mark.parametrize("fields", SOIL_FIELD_SETS)
def test_device_soil_to_pelagic_bit_exact(po, pel_precision, fields):
    ncol = 300
    pcs, cs, pel, sed = handles(ncol, pel_precision)
    sed.set_forcing()
    sed.step(1)
    fl = sed.fluxes()                       # the fluxes the soil exports
    p = coupling.soil_default_params(convertN=1.3, convertP=0.7, dinflux_const=2.5)
    st = coupling.CplStats()
    got, present = coupling.soil_pelagic(sed, pel, params=p, fields=soil_fields_struct(fields),
                                         stats=st)
    assert st.gpu_launches == 2 and st.columns == ncol
    pp = {n: getattr(p, n) for n in coupling.SOIL_PARAM_NAMES}
    ref, pres0 = po.cpl_soil_run(fl, fields, pp, pcs.bottom_flux)
    if pel_precision == capi.SED_FP32:   # the handle keeps its rows in FP32
        ref = ref.astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(present, pres0)
    np.testing.assert_array_equal(got, ref)
    pel.close()
    sed.close()


@pytest.mark.gpu
def test_two_way_coupled_loop_equals_host_route(po):
    """pel_step -> cpl_pelagic_soil -> sed_step -> cpl_soil_pelagic for a
    few coupling steps, all on the device, equals the loop that takes every
    exchanged field through the host, maps it with the oracles and sets it
    with sed_set_boundary and pel_set_forcing."""
    ncol = 128
    pcs, cs, pel, sed = handles(ncol, capi.SED_FP32, seed=8)
    _, _, pel2, sed2 = handles(ncol, capi.SED_FP32, seed=8)
    T = np.linspace(4.0, 16.0, ncol)
    depth = np.linspace(1.0, 50.0, ncol)
    bfl = pcs.bottom_flux.copy()
    for _ in range(3):
        pel.step(1)
        coupling.pelagic_soil(pel, sed, T, depth, read_back=False)
        sed.step(1)
        coupling.soil_pelagic(sed, pel, read_back=False)
        pel2.step(1)
        rc, S0, V0, P0 = po.cpl_run(pel2.get_state(), NPZD, po.cpl_defaults(), False, depth)
        sed2.set_boundary(T, S0, V0, P0)
        sed2.step(1)
        bfl, _ = po.cpl_soil_run(sed2.fluxes(), NPZD, None, bfl)
        pel2.set_forcing(bottom_flux=bfl)
    np.testing.assert_array_equal(pel.get_state(), pel2.get_state())
    np.testing.assert_array_equal(sed.get_state(), sed2.get_state())
    for s in (pel, sed, pel2, sed2):
        s.close()


@pytest.mark.gpu
def test_soil_coupling_errors():
    pcs, cs, pel, sed = handles(64, capi.SED_FP32)
    with pytest.raises(capi.SedError) as e:     # no forcing and no step yet
        coupling.soil_pelagic(sed, pel)
    assert e.value.code == capi.SED_E_STATE
    sed.set_forcing()
    with pytest.raises(capi.SedError) as e:
        coupling.soil_pelagic(sed, pel, fields=soil_fields_struct(dict(din=0, detN=0)))
    assert e.value.code == capi.SED_E_ARG
    coupling.soil_pelagic(sed, pel)
    pel.close()
    sed.close()
