"""Classical Gram-Schmidt of FGMRES as one cooperative launch (an option).

With CDG_CGS_COOP=1, systems of at least 100,000 rows run the Arnoldi step of
each FGMRES iteration (Iteration_gmres.C:515-527: the inner products with the
basis, the update, the norm, the Givens rotation of the new Hessenberg column
and the new basis vector) as one cooperative kernel with grid-wide barriers,
in place of three kernels (the default, measured faster on GB300).  The two
forms sum the block partials in different orders, so the bars are those of
FP64 round-off in a Krylov method: the same residual reduction, iterations
within one, solutions to 1e-10 relative; the oracle's iteration count within
one for both.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def solve(ctx, h, a, s):
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.assemble(a)
    st = cd.solve(s)
    x = cd.solution()
    cd.close()
    return st, x


@pytest.mark.parametrize("precision,restart", [("fp64", 30), ("mixed", 30), ("mixed", 4)])
def test_cooperative_step_equals_three_kernels(ctx, monkeypatch, precision, restart):
    # 2D Q1 on 512^2 cells (263,169 rows), SUPG, multigrid V(2,2); a short
    # restart length runs the cycle-start path many times
    h = pg.Hierarchy(2, 1, 9, n_levels=5)
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-3, b=(1.0, 0.4), c=0.2,
                           space_discretization_type="supg", sdfem_type=2)
    s = pg.solver_params("multigrid", precision=precision, max_n_iterations=400,
                         gmres_restart=restart, residual_tolerance=0.0,
                         residual_reduction=1e-10, multigrid_n_levels=5,
                         multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.8)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("CDG_CGS_COOP", flag)
        st, x = solve(ctx, h, a, s)
        assert st.residual <= 1e-10 * st.initial_residual, (flag, st.iterations)
        out.append((st, x))
    (s1, x1), (s0, x0) = out
    assert abs(s1.iterations - s0.iterations) <= 1
    assert rel(x1, x0) < 1e-10


@pytest.mark.parametrize("flag", ["1", "0"])
def test_cooperative_step_against_the_oracle(ctx, monkeypatch, flag):
    # FP64 multigrid FGMRES(30) on 2D Q1 SUPG, 512^2 cells (263,169 rows),
    # against the oracle on the same hierarchy
    monkeypatch.setenv("CDG_CGS_COOP", flag)
    kw = dict(eps=1e-3, b=(1.0, 0.4), c=0.2)
    levels = 5
    o = po.Problem(po.make_config(2, 1, 9, po.EX_SINE, supg=True, sdfem_type=2, **kw), levels)
    o.assemble()
    it_o, res_o, ini_o = o.solve(po.make_solver("multigrid", max_it=400, restart=30,
                                                reduction=1e-10, mg_levels=levels, n_pre=2,
                                                n_post=2, jacobi_damp=0.8))
    assert res_o <= 1e-10 * ini_o
    h = pg.Hierarchy(2, 1, 9, n_levels=levels)
    assert h.info(0)["ndof"] >= 100000
    a = pg.assembly_params(example=pg.EX_SINE, space_discretization_type="supg",
                           sdfem_type=2, **kw)
    s = pg.solver_params("multigrid", precision="fp64", max_n_iterations=400,
                         gmres_restart=30, residual_tolerance=0.0, residual_reduction=1e-10,
                         multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                         multigrid_n_post_smooth=2, jacobi_damp=0.8)
    st, x = solve(ctx, h, a, s)
    assert st.residual <= 1e-10 * st.initial_residual
    assert abs(st.iterations - it_o) <= 1, (st.iterations, it_o)
    assert rel(x, o.solution()) < 1e-8
