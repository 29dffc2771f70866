"""The ctypes mirrors of the C structs, constants and signatures match their headers.

A small C program compiled with the host compiler against the header prints
sizeof and every field's offsetof; the Python structures must agree field by
field, so a field added on one side only fails here rather than as garbage
parameters: the C-ABI's (include/parmoon_cd.h: AssemblyParams, SolverParams,
SolveStats, Request, Result) and the oracle's (oracle/cd_oracle.h: Config,
SolverConfig).
"""
import ctypes
import os
import re
import shutil
import subprocess
import tempfile

import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "cdg_assembly_params": pg.AssemblyParams,
    "cdg_solver_params": pg.SolverParams,
    "cdg_solve_stats": pg.SolveStats,
    "cdg_request": pg.Request,
    "cdg_result": pg.Result,
}
ORACLE_STRUCTS = {
    "orc_config": po.Config,
    "orc_solver_config": po.SolverConfig,
}


def c_layout(header, include_dir, structs):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "%s"' % header,
             'int main(void) {']
    for cname, py in structs.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ['  return 0;', '}']
    d = tempfile.mkdtemp()
    try:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run(["gcc", "-std=c99", "-I", include_dir, src, "-o", exe],
                       check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    finally:
        shutil.rmtree(d, ignore_errors=True)
    table = {}
    for line in out.splitlines():
        s, f, v = line.split()
        table[(s, f)] = int(v)
    return table


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a host C compiler")
@pytest.mark.parametrize("which", ["library", "oracle"])
def test_ctypes_mirrors_match_the_header(which):
    if which == "library":
        header, inc, structs = "parmoon_cd.h", os.path.join(ROOT, "include"), STRUCTS
    else:
        header, inc, structs = "cd_oracle.h", os.path.join(ROOT, "oracle"), ORACLE_STRUCTS
    t = c_layout(header, inc, structs)
    for cname, py in structs.items():
        assert ctypes.sizeof(py) == t[(cname, "sizeof")], cname
        for fname, _ in py._fields_:
            assert getattr(py, fname).offset == t[(cname, fname)], (cname, fname)


def test_constants_match_the_headers():
    # the C-ABI's #defines against the package's constants
    hdr = open(os.path.join(ROOT, "include", "parmoon_cd.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in
            re.finditer(r"#define CDG_(\w+) \(?(-?\d+)\)?", hdr)}
    schemes = {"TIME_CRANK_NICOLSON": "crank_nicolson", "TIME_BACKWARD_EULER": "backward_euler",
               "TIME_BDF_TWO": "bdf_two"}
    seen = set()
    for name, value in defs.items():
        if name.startswith("EX_") or name.startswith("CELL_"):
            assert getattr(pg, name) == value, name
        elif name.startswith("ERR_"):
            assert pg.ERRORS[value] == "CDG_" + name, name
        elif name in schemes:
            assert pg.TIME_SCHEMES[schemes[name]] == value, name
        else:
            continue
        seen.add(name)
    assert len([n for n in seen if n.startswith("EX_")]) == 10
    assert len([n for n in seen if n.startswith("ERR_")]) == len(pg.ERRORS)
    # the oracle's enumerations against pyoracle
    ohdr = open(os.path.join(ROOT, "oracle", "cd_oracle.h")).read()
    for m in re.finditer(r"ORC_(EX_\w+) = (\d+)", ohdr):
        assert getattr(po, m.group(1)) == int(m.group(2)), m.group(1)
    for m in re.finditer(r"ORC_(TIME_\w+) = (\d+)", ohdr):
        assert po.TIME_SCHEMES[schemes[m.group(1)]] == int(m.group(2)), m.group(1)


def prototypes(path, prefix):
    hdr = open(path).read()
    hdr = re.sub(r"/\*.*?\*/", " ", hdr, flags=re.S)
    protos = {}
    pat = r"(?:const char \*|int|long long|void|orc_problem \*)\s*(%s\w+)\(([^)]*)\);" % prefix
    for m in re.finditer(pat, hdr, re.S):
        params = m.group(2).strip()
        protos[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return protos


def test_oracle_signatures_match_the_prototypes(built):
    L = po.lib()
    checked = 0
    for name, n in prototypes(os.path.join(ROOT, "oracle", "cd_oracle.h"), "orc_").items():
        at = getattr(L, name).argtypes
        if at is None:
            continue
        assert len(at) == n, (name, len(at), n)
        checked += 1
    assert checked >= 10


def test_ctypes_signatures_match_the_prototypes(built):
    # every function the package gives argtypes to takes as many parameters
    # as its prototype in the header declares
    protos = prototypes(os.path.join(ROOT, "include", "parmoon_cd.h"), "cdg_")
    L = pg.lib()
    checked = 0
    for name, n in protos.items():
        at = getattr(L, name).argtypes
        if at is None:
            continue
        assert len(at) == n, (name, len(at), n)
        checked += 1
    assert checked >= 40
