"""The Fortran drop-in (fortran/sed_gpu.F90, fortran/type_sed_gpu.F90), read
as text: no Fortran compiler exists on either machine.

The driver's state has nvar tracers in FABM's order
(src/drivers/fabm_sediment_driver.F90:353); the shim must pass that count to
the library (which refuses any but 11) instead of assuming 11, map FABM's
state names onto the library's tracers, and take the rate constants from the
same namelist group FABM reads (examples/standalone/omexdia_p/fabm_sed.nml
:18-77, whose entries the golden fixture records)."""
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FORTRAN = os.path.join(ROOT, "mossco-code_gb300", "fortran")
BGC = ("rLabile", "rSemilabile", "NCrLdet", "NCrSdet", "PAds", "PAdsODU", "NH3Ads",
       "CprodMax", "rnit", "ksO2nitri", "rODUox", "ksO2oduox", "ksO2oxic", "ksNO3denit",
       "kinO2denit", "kinNO3anox", "kinO2anox")


def src(name):
    with open(os.path.join(FORTRAN, name)) as f:
        return f.read()


def code(text):
    """Fortran text without comments and with continuation lines joined."""
    lines = [re.sub(r"!.*$", "", l) for l in text.splitlines()]
    return re.sub(r"&\s*\n\s*", " ", "\n".join(lines))


def body(text, kind, name):
    m = re.search(rf"{kind}\s+{name}\s*\((.*?)\)(.*?)end\s+{kind}", code(text), re.S | re.I)
    assert m, name
    return m.group(1), m.group(2)


def test_sed_gpu_init_takes_and_passes_the_tracer_count():
    args, b = body(src("sed_gpu.F90"), "subroutine", "sed_gpu_init")
    names = [a.strip() for a in args.split(",")]
    assert names[:6] == ["gpu", "p", "inum", "jnum", "knum", "ntr"], names
    call = re.search(r"sed_create\((.*?)\)\s*\n", b, re.S).group(1)
    assert "int(ntr, c_int)" in call and "SED_NTR" not in call


def test_gpu_init_uses_nvar_and_the_name_map():
    text = src("type_sed_gpu.F90")
    _, init = body(text, "subroutine", "gpu_init")
    call = re.search(r"call sed_gpu_init\((.*?)\)\s*\n", init, re.S).group(1)
    args = [a.strip() for a in call.split(",")]
    assert args[5] == "self%nvar", args
    # the map comes first, and the minima follow it
    assert init.index("call gpu_tracer_map") < init.index("call sed_gpu_init")
    assert "state_variables(self%perm(n))%minimum" in init
    _, tmap = body(text, "subroutine", "gpu_tracer_map")
    assert "self%nvar /= SED_NTR" in tmap
    assert "state_variables(m)%name" in tmap and "SED_E_ARG" in tmap
    # every library tracer has a key, in sed_tracer_name() order
    keys = re.search(r"tracer_keys\(SED_NTR\)\s*=\s*\[.*?::(.*?)\]", code(text), re.S).group(1)
    keys = [k.strip().strip("'") for k in keys.split(",")]
    assert keys == ["ldetC", "sdetC", "ldetN", "sdetN", "ldetP", "adsP", "oxy", "no3", "nh3",
                    "odu", "po4"]


def test_step_permutes_when_the_orders_differ():
    _, step = body(src("type_sed_gpu.F90"), "subroutine", "gpu_ode_solver")
    assert "self%lconc(:,:,:,n) = self%conc(:,:,:,self%perm(n))" in step
    assert "self%conc(:,:,:,self%perm(n)) = self%lconc(:,:,:,n)" in step
    assert "self%lbdys(:,:,n + 1) = self%bdys(:,:,self%perm(n) + 1)" in step
    assert "self%fluxes(:,:,self%perm(n)) = self%lfluxes(:,:,n)" in step


def test_rate_constants_come_from_the_fabm_namelist():
    text = code(src("type_sed_gpu.F90"))
    fixture = json.load(open(os.path.join(ROOT, "tests", "golden", "omexdia_p_example.json")))
    for group in ("hzg_omexdia_cnp", "hzg_omexdia_p"):
        m = re.search(rf"namelist\s*/{group}/(.*?)\n", text, re.S)
        assert m, group
        declared = {v.strip() for v in m.group(1).split(",")}
        # every entry of the reference's group is declared (a namelist read
        # fails on an undeclared name), and every rate constant is read
        assert set(fixture[group]) <= declared, set(fixture[group]) - declared
        assert set(BGC) <= declared
    _, rb = body(src("type_sed_gpu.F90"), "subroutine", "gpu_read_bgc")
    for n in BGC:
        assert re.search(rf"p%{n}\s*=\s*{n}\b", rb), n
