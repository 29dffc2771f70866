"""Pin the CPU oracle against the golden values of the reference's own tests.

test/cd2d_test.c++ asserts L2 / H1-semi / SD / L_inf errors of CD2D example 0
(sine Laplace, Neumann on boundary component 1) on the twice refined unit
square to 1e-11 for every solver it runs; the oracle must reproduce them with
a converged FGMRES+Jacobi solve and with FGMRES + 2-level W-cycle multigrid
(the test's multigrid configuration).  Known-answer cases: a linear exact
solution is reproduced exactly by Q1/Q2 in 2D and 3D (test/cd3d_solvers_test
zero-error examples), and the one-cell pattern counts of structure_test.
"""
import json
import os

import numpy as np
import pytest

import pyoracle as po

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_values.json")))


def _cd2d_problem(order):
    cfg = po.make_config(2, order, 2, po.EX_SINE_LAPLACE, eps=1.0, neumann_mask=1 << 1)
    p = po.Problem(cfg, 2)
    p.assemble()
    return p


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("solver", ["jacobi", "multigrid"])
def test_cd2d_golden_errors(built, order, solver):
    g = GOLD["cd2d_test"]["errors"]["Q%d" % order]
    tol = GOLD["cd2d_test"]["tolerance"]
    p = _cd2d_problem(order)
    if solver == "jacobi":
        s = po.make_solver("jacobi", max_it=1000, restart=100, tol_abs=1e-15, reduction=0.0)
    else:
        # cd2d_test.c++:256-266: fgmres + multigrid, 2 levels, W cycle, Jacobi
        # smoother, direct coarse solve, 2+2 smoothing steps
        s = po.make_solver("multigrid", max_it=1000, restart=20, tol_abs=1e-13, reduction=0.0,
                           mg_levels=2, mg_cycle="W", n_pre=2, n_post=2, correction_damp=1.0)
    p.solve(s)
    e = p.errors()
    assert abs(e[0] - g["L2"]) < tol
    assert abs(e[1] - g["H1_semi"]) < tol
    assert abs(e[2] - g["SD"]) < tol
    assert abs(e[4] - g["L_inf"]) < tol


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_linear_solution_reproduced(built, dim, order):
    cfg = po.make_config(dim, order, 2, po.EX_POLY1, eps=0.3, b=(1.0, -0.5, 0.25), c=0.7,
                         supg=True, sdfem_type=2)
    p = po.Problem(cfg, 1)
    p.assemble()
    p.solve(po.make_solver("jacobi", max_it=2000, restart=80, tol_abs=1e-14, reduction=0.0))
    e = p.errors()
    assert e[0] < 1e-11 and e[1] < 1e-10 and e[4] < 1e-11


@pytest.mark.parametrize("order", [1, 2])
def test_one_cell_pattern_counts(built, order):
    ref = GOLD["structure_test"]["counts"]["UnitSquare_quad_Q%d" % order]
    p = po.Problem(po.make_config(2, order, 0, po.EX_SINE), 1)
    rp, col = p.structure()
    assert len(rp) - 1 == ref["n_rows"]
    assert int(col.max()) + 1 == ref["n_columns"]
    assert len(col) == ref["n_entries"]
    assert rp[4] - rp[3] == ref["n_entries_in_row_3"]
