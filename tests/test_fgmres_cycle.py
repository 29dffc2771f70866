"""FGMRES restart cycles as one cooperative kernel (Jacobi preconditioner,
systems of at most 65,536 rows) against the graph-captured kernels and the
oracle: the same iteration counts (+-1), solutions to 1e-10 relative of each
other and to 1e-8 of the oracle, restarts inside a solve, divergence and
stopping at max_n_iterations reported as by the graph path.
"""
import os

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu


def solve(ctx, h, a, s, cycle):
    old = os.environ.get("CDG_FGMRES_CYCLE")
    os.environ["CDG_FGMRES_CYCLE"] = "1" if cycle else "0"
    try:
        cd = pg.ConvectionDiffusion(ctx, h)
        cd.set_solution(None)
        cd.assemble(a)
        st = cd.solve(s)
        launches = ctx.launches()
        return st, cd.solution()
    finally:
        if old is None:
            os.environ.pop("CDG_FGMRES_CYCLE", None)
        else:
            os.environ["CDG_FGMRES_CYCLE"] = old


CASES = {
    # name: (dim, order, nref, restart, example, eps, b, c)
    "q1_2d_64_m50": (2, 1, 6, 50, pg.EX_SINE, 1e-2, (1.0, 0.5), 1.0),
    "q2_2d_16_m20": (2, 2, 4, 20, pg.EX_SINE, 1e-2, (1.0, 0.5), 0.5),
    "q1_3d_16_m30": (3, 1, 4, 30, pg.EX_SINE, 0.1, (1.0, 0.3, -0.2), 1.0),
}


@pytest.mark.parametrize("name", list(CASES))
def test_cycle_equals_graph_and_oracle(ctx, name):
    dim, order, nref, m, ex, eps, b, c = CASES[name]
    h = pg.Hierarchy(dim, order, nref)
    a = pg.assembly_params(example=ex, eps=eps, b=b, c=c)
    s = pg.solver_params("jacobi", max_n_iterations=2000, gmres_restart=m,
                         residual_tolerance=0.0, residual_reduction=1e-10)
    st_c, x_c = solve(ctx, h, a, s, True)
    st_g, x_g = solve(ctx, h, a, s, False)
    assert abs(st_c.iterations - st_g.iterations) <= 1
    assert st_c.residual <= 1e-10 * st_c.initial_residual * 1.0001
    assert np.max(np.abs(x_c - x_g)) <= 1e-10 * np.max(np.abs(x_g))
    o = po.Problem(po.make_config(dim, order, nref, ex, eps=eps, b=b, c=c), 1)
    o.assemble()
    it_o, _, _ = o.solve(po.make_solver("jacobi", max_it=2000, restart=m, reduction=1e-10))
    assert abs(st_c.iterations - it_o) <= 1
    assert np.max(np.abs(x_c - o.solution())) <= 1e-8 * np.max(np.abs(o.solution()))


def test_cycle_stops_at_max_iterations_like_graph(ctx):
    h = pg.Hierarchy(2, 1, 6)
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1.0, 0.5), c=1.0)
    s = pg.solver_params("jacobi", max_n_iterations=37, gmres_restart=10,
                         residual_tolerance=0.0, residual_reduction=1e-14)
    st_c, x_c = solve(ctx, h, a, s, True)
    st_g, x_g = solve(ctx, h, a, s, False)
    assert st_c.iterations == st_g.iterations
    assert abs(st_c.residual - st_g.residual) <= 1e-9 * st_g.residual
    assert np.max(np.abs(x_c - x_g)) <= 1e-10 * np.max(np.abs(x_g))
