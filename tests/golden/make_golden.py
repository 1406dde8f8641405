"""Writes omexdia_p_example.json and gotm_npzd_example.json next to this
script.

The fixture is the reference's standalone one-column OMEXDIA+P example
(examples/standalone/omexdia_p): the run and sediment namelists of
run_sed.nml and the hzg_omexdia_p parameters and initial values of
fabm_sed.nml, read as text from a checkout of the reference, and the FP64
oracle's state after 24 of the example's 360 s adaptive-Euler steps.  The
reference itself cannot be built (Fortran, FABM), so the state is the
oracle's: it pins regressions of the oracle and of the FP64 device path to
the reference's own example configuration.

    python tests/golden/make_golden.py <path-to-reference-checkout>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "mossco-code_gb300"), os.path.join(ROOT, "oracle"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

NSTEPS = 24


def namelist(text: str, block: str) -> dict:
    """name = value pairs of &block ... / (numbers only, comments dropped)."""
    m = re.search(r"&" + block + r"\b(.*?)\n\s*/", text, re.S)
    out = {}
    for line in m.group(1).splitlines():
        line = line.split("!")[0]
        for name, val in re.findall(r"(\w+)\s*=\s*([-+0-9.eEdD]+)", line):
            out[name] = float(val.replace("d", "e").replace("D", "e"))
    return out


def main(ref: str) -> None:
    ex = os.path.join(ref, "examples", "standalone", "omexdia_p")
    run_sed = open(os.path.join(ex, "run_sed.nml")).read()
    fabm = open(os.path.join(ex, "fabm_sed.nml")).read()
    fixture = {
        "source": "examples/standalone/omexdia_p: run_sed.nml (run_nml, sed_nml), "
                  "fabm_sed.nml (hzg_omexdia_p, hzg_omexdia_cnp N initial values)",
        "run_nml": namelist(run_sed, "run_nml"),
        "sed_nml": namelist(run_sed, "sed_nml"),
        "hzg_omexdia_p": namelist(fabm, "hzg_omexdia_p"),
        "hzg_omexdia_cnp": namelist(fabm, "hzg_omexdia_cnp"),
        "nsteps": NSTEPS,
    }
    import golden_case
    cs = golden_case.column_set(fixture)
    import oracle
    c = cs.conc.copy()
    rc, st, fl = oracle.OracleModel(cs).run(c, nsteps=NSTEPS, percol=True, nthreads=1)
    assert rc == 0
    fixture["state"] = c[:, :, 0].tolist()       # [tracer][layer] after NSTEPS
    fixture["fluxes"] = fl[:, 0].tolist()
    fixture["attempts"] = int(st["attempts"])
    with open(os.path.join(HERE, "omexdia_p_example.json"), "w") as f:
        json.dump(fixture, f, indent=1)
    # the pelagic set-ups' FABM model: &gotm_npzd of the fabm0d examples
    npzd = open(os.path.join(ref, "examples", "fabmsed_fabm0d", "fabm.nml")).read()
    with open(os.path.join(HERE, "gotm_npzd_example.json"), "w") as f:
        json.dump({"source": "examples/fabmsed_fabm0d/fabm.nml (gotm_npzd)",
                   "gotm_npzd": namelist(npzd, "gotm_npzd")}, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference source tree>")
    main(sys.argv[1])
