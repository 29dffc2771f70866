"""Neumann data on hexahedron faces (Assemble3D.C:552-655): the oracle on its
own (CPU) and the CUDA path against it (GPU).

CPU: a solution linear in x lies in Q1 and Q2, so with consistent Neumann
data g = eps dn u the Galerkin solution is exact (L2/H1 errors at round-off)
for several Neumann parts of the boundary; for u = sin(pi x) sin(pi y)
sin(pi z) the L2 error falls at the element order + 1.  GPU: rhs, matrix and
solution parity against the oracle (1e-12 / 1e-8), tetrahedra rejected.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("mask", [4, 36, 47])
def test_oracle_neumann_faces_exact_for_linear(built, order, mask):
    cfg = po.make_config(3, order, 2, po.EX_POLY1, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0,
                         neumann_mask=mask)
    o = po.Problem(cfg, 1)
    o.assemble()
    it, res, ini = o.solve(po.make_solver("jacobi", max_it=2000, restart=50, reduction=1e-13))
    e = o.errors()
    assert e[0] < 1e-11 and e[1] < 1e-10


@pytest.mark.parametrize("order,rate", [(1, 1.9), (2, 2.8)])
def test_oracle_neumann_faces_convergence(built, order, rate):
    errs = []
    for nref in (1, 2, 3):
        cfg = po.make_config(3, order, nref, po.EX_SINE, eps=1.0, neumann_mask=36)
        o = po.Problem(cfg, 1)
        o.assemble()
        o.solve(po.make_solver("jacobi", max_it=4000, restart=50, reduction=1e-12))
        errs.append(o.errors()[0])
    assert np.log2(errs[1] / errs[2]) > rate


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_neumann_faces_solve_parity(ctx, order):
    mask = 36
    cfg = po.make_config(3, order, 3, po.EX_SINE, eps=0.05, b=(1.0, 0.3, -0.2), c=0.5,
                         neumann_mask=mask)
    o = po.Problem(cfg, 2)
    o.assemble()
    osol = po.make_solver("multigrid", max_it=200, restart=30, reduction=1e-10, mg_levels=2,
                          n_pre=2, n_post=2, jacobi_damp=0.6)
    it_o, _, _ = o.solve(osol)
    h = pg.Hierarchy(3, order, 3, n_levels=2, neumann_mask=mask)
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.set_solution(None)
    cd.assemble(pg.assembly_params(example=pg.EX_SINE, eps=0.05, b=(1.0, 0.3, -0.2), c=0.5,
                                   neumann_mask=mask))
    rel = lambda x, y: np.max(np.abs(x - y)) / np.max(np.abs(y))
    assert rel(cd.rhs(0), o.rhs(0)) < 1e-12
    st = cd.solve(pg.solver_params("multigrid", max_n_iterations=200, gmres_restart=30,
                                   residual_tolerance=0.0, residual_reduction=1e-10,
                                   multigrid_n_levels=2, multigrid_n_pre_smooth=2,
                                   multigrid_n_post_smooth=2, jacobi_damp=0.6, precision="fp64"))
    assert abs(st.iterations - it_o) <= 1
    assert rel(cd.solution(), o.solution()) < 1e-8


@pytest.mark.gpu
def test_neumann_on_tetrahedra_rejected(ctx):
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, 1, roots=1, tetra=True))
    with pytest.raises(pg.CdgError) as e:
        cd.assemble(pg.assembly_params(example=pg.EX_SINE, neumann_mask=4))
    assert e.value.code == -1
