"""The ctypes mirrors of the C ABI's structs have the C layout.

A small C program, compiled here with gcc against include/*.h, prints the
size of every struct of the three headers and the offset of every member;
each must equal the ctypes Structure the Python host binds it with
(sedgpu/capi.py, pelagic.py, coupling.py).  A member added to a header and
not to its binding, or the other way round, fails here without a GPU."""
import ctypes
import os
import shutil
import subprocess

import pytest

from sedgpu import build, capi, coupling, pelagic

MIRRORS = {
    "sed_params": capi.SedParams,
    "sed_stats": capi.SedStats,
    "sed_tuning": capi.SedTuning,
    "pel_params": pelagic.PelParams,
    "pel_stats": pelagic.PelStats,
    "cpl_params": coupling.CplParams,
    "cpl_fields": coupling.CplFields,
    "cpl_stats": coupling.CplStats,
    "cpl_soil_params": coupling.CplSoilParams,
}


def c_layout(tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "mossco_cpl.h"',
             'int main(void) {']
    for cname, py in MIRRORS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", build.INCLUDE, str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        struct, what, value = line.split()
        table[(struct, what)] = int(value)
    return table


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_headers(tmp_path):
    table = c_layout(tmp_path)
    for cname, py in MIRRORS.items():
        assert ctypes.sizeof(py) == table[(cname, "sizeof")], cname
        for field, _ in py._fields_:
            assert getattr(py, field).offset == table[(cname, field)], (cname, field)


def test_every_struct_of_the_headers_has_a_mirror():
    import re
    structs = set()
    for h in ("mossco_sed.h", "mossco_pel.h", "mossco_cpl.h"):
        text = open(os.path.join(build.INCLUDE, h)).read()
        structs |= set(re.findall(r"typedef struct (\w+) \{", text))
    assert structs == set(MIRRORS)


FORTRAN = os.path.join(os.path.dirname(build.PKG_DIR), "fortran")
F_KINDS = {"real(c_double)": ctypes.c_double, "integer(c_int)": ctypes.c_int,
           "integer(c_long_long)": ctypes.c_longlong, "real(c_float)": ctypes.c_float}
F_PARAMS = {"sed_ntr": capi.NTR, "pel_ntr": pelagic.PEL_NTR}


def _split_names(text):
    out, depth, cur = [], 0, ""
    for ch in text:
        depth += ch == "("
        depth -= ch == ")"
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    out.append(cur.strip())
    return [n for n in out if n]


def fortran_types():
    """Every bind(C) derived type of the Fortran bindings as a list of
    (member, ctypes type, count) in declaration order."""
    import re
    types = {}
    for fn in sorted(os.listdir(FORTRAN)):
        lines = open(os.path.join(FORTRAN, fn)).read().splitlines()
        joined, cur = [], ""
        for line in lines:
            line = line.split("!")[0].rstrip()
            if line.endswith("&"):
                cur += line[:-1] + " "
                continue
            joined.append(cur + line)
            cur = ""
        name = None
        for line in joined:
            m = re.match(r"\s*type,\s*bind\(C\),\s*public\s*::\s*(\w+)", line, re.I)
            if m:
                name, types[m.group(1).lower()] = m.group(1).lower(), []
                continue
            if name and re.match(r"\s*end\s+type", line, re.I):
                name = None
                continue
            if name and "::" in line:
                kind, names = line.split("::")
                kind = re.sub(r"\s+", "", kind).lower()
                for n in _split_names(names):
                    m = re.match(r"(\w+)\s*(?:\((\w+)\))?", n)
                    count = m.group(2)
                    count = 1 if count is None else int(F_PARAMS.get(count.lower(), count))
                    types[name].append((m.group(1).lower(), F_KINDS[kind], count))
    return types


def test_fortran_bind_c_types_match_the_headers():
    """The Fortran modules cannot be compiled here: their bind(C) types are
    read as text and must list the C struct's members in order, with the
    same kinds and array lengths."""
    ftypes = fortran_types()
    assert set(ftypes) == {c + "_t" for c in MIRRORS}
    for cname, py in MIRRORS.items():
        members = []
        for field, ctype in py._fields_:
            if hasattr(ctype, "_length_"):
                members.append((field.lower(), ctype._type_, ctype._length_))
            else:
                members.append((field.lower(), ctype, 1))
        assert ftypes[cname + "_t"] == members, cname


def c_prototypes():
    """Argument counts of every function the three headers declare."""
    import re
    out = {}
    for h in ("mossco_sed.h", "mossco_pel.h", "mossco_cpl.h"):
        text = open(os.path.join(build.INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        for m in re.finditer(r"\b((?:sed|pel|cpl)_\w+)\s*\(([^()]*)\)\s*;", text):
            args = m.group(2).strip()
            out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def fortran_interfaces():
    """Argument counts of every bind(C) interface of the Fortran modules."""
    import re
    out = {}
    for fn in sorted(os.listdir(FORTRAN)):
        text = open(os.path.join(FORTRAN, fn)).read()
        text = re.sub(r"!.*", "", text)
        text = re.sub(r"&\s*\n\s*", " ", text)
        for m in re.finditer(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*"
                             r"name='(\w+)'\)", text, re.I):
            args = m.group(2).strip()
            out[m.group(3)] = 0 if not args else len(args.split(","))
    return out


LIBC = ("strlen",)


def test_fortran_interfaces_match_the_prototypes():
    """Every function of the three headers, the surrogate's included, has a
    bind(C) interface with the prototype's argument count."""
    c = c_prototypes()
    f = {k: v for k, v in fortran_interfaces().items() if k not in LIBC}
    for name, n in f.items():
        assert name in c, name
        assert n == c[name], (name, n, c[name])
    missing = sorted(k for k in c if k not in f)
    assert missing == [], missing
