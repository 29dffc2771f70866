"""Extract the golden values the reference's own tests hold for the CD path.

Reads (as text) test/cd2d_test.c++ (error norms of CD2D example 0 on the
4x4 UnitSquare for Q1..Q8, tolerance 1e-11), test/tcd2d_test.c++ (L2 / H1
errors of the Crank-Nicolson TCD2D example 0 after selected steps, Galerkin
and SUPG, tolerance 1e-10) and test/structure_test.c++ (pattern counts of
one-cell meshes), and writes reference_values.json next to this script.

    python tests/golden/make_reference_values.py <path of the ParMooN2022 source tree>

Runs where the reference tree is present; the JSON is committed so the tests
never need the reference itself.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_reference_values.py <ParMooN2022 source tree>")
REF = sys.argv[1]
HERE = os.path.dirname(os.path.abspath(__file__))


def cd2d_errors():
    src = open(os.path.join(REF, "test", "cd2d_test.c++")).read()
    quads = src[src.index("void tests_on_quads"):src.index("void tests_on_triangles")]
    out = {}
    for m in re.finditer(r'starting with (Q\d)"\);\s*errors = \{\{([^}]*)\}\};', quads):
        vals = [float(v) for v in m.group(2).replace("\n", " ").split(",")]
        out[m.group(1)] = dict(L2=vals[0], H1_semi=vals[1], SD=vals[2], L_inf=vals[3])
    tol = float(re.search(r"const double eps = ([0-9.e+-]+);", src).group(1))
    return out, tol


def tcd2d_errors():
    src = open(os.path.join(REF, "test", "tcd2d_test.c++")).read()

    def arr(name, conv):
        m = re.search(name + r"\[nb_test\] = \{([^}]*)\};", src)
        return [conv(v) for v in m.group(1).replace("\n", " ").split(",")]

    steps = arr("iter_m", int)
    tol = float(re.search(r"double eps = ([0-9.e+-]+);", src).group(1))
    out = {}
    for kind in ("galerkin", "supg"):
        out[kind] = dict(L2=arr("L2_" + kind, float), H1=arr("H1_" + kind, float))
    return steps, tol, out


def structure_counts():
    src = open(os.path.join(REF, "test", "structure_test.c++")).read()
    body = src[src.index("std::array<unsigned int, 4> get_reference_values("):]
    sq = body[body.index("case 0: // UnitSquare_quad.mesh"):body.index("case 1: // UnitSquareIrregular.GEO")]
    vals = re.findall(r"reference_values = \{(\d+), (\d+), (\d+), (\d+)\};", sq)
    # order 1/other 1 is the first entry, order 2/other 2 the sixth
    q1 = [int(v) for v in vals[0]]
    q2 = [int(v) for v in vals[5]]
    keys = ["n_rows", "n_columns", "n_entries", "n_entries_in_row_3"]
    return {"UnitSquare_quad_Q1": dict(zip(keys, q1)), "UnitSquare_quad_Q2": dict(zip(keys, q2))}


if __name__ == "__main__":
    errs, tol = cd2d_errors()
    tcd_steps, tcd_tol, tcd_errs = tcd2d_errors()
    data = {
        "cd2d_test": {
            "source": "test/cd2d_test.c++:42-145 (UnitSquare refined twice, example 0, "
                      "diffusion_coefficient 1, Neumann on boundary component 1)",
            "tolerance": tol,
            "errors": errs,
        },
        "tcd2d_test": {
            "source": "test/tcd2d_test.c++:24-137 (UnitSquare refined 5 times, Q1, example 0 "
                      "exp_sin_cos, diffusion 1, b = (1, -1), c = 1, Crank-Nicolson, "
                      "tau 0.05, direct solver)",
            "tolerance": tcd_tol,
            "steps": tcd_steps,
            "errors": tcd_errs,
        },
        "structure_test": {
            "source": "test/structure_test.c++:603-660 (one-cell UnitSquare_quad.mesh, no face integrals)",
            "counts": structure_counts(),
        },
    }
    with open(os.path.join(HERE, "reference_values.json"), "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print(json.dumps(data, indent=1))
