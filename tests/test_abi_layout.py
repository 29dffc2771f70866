"""The ctypes mirrors of the C structs match their headers.

A small C program compiled with the host compiler against the header prints
sizeof and every field's offsetof; the Python structures must agree field by
field, so a field added on one side only fails here rather than as garbage
parameters: the C-ABI's (include/parmoon_cd.h: AssemblyParams, SolverParams,
SolveStats, Request, Result) and the oracle's (oracle/cd_oracle.h: Config,
SolverConfig).
"""
import ctypes
import os
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
