"""Neumann data on hexahedron and tetrahedron faces (Assemble3D.C:552-655,
quadrilateral and triangular faces): the oracle on its own (CPU) and the CUDA
path against it (GPU).

CPU: a solution linear in x lies in Q1/Q2 and P1/P2, so with consistent
Neumann data g = eps dn u the Galerkin solution is exact (L2/H1 errors at
round-off) for several Neumann parts of the boundary; on tetrahedra the
Crank-Nicolson solution u = t^2 (x^2 + yz) is exact in P2 with Neumann faces
(g is linear in x, so the face rule is exact); for u = sin(pi x) sin(pi y)
sin(pi z) the L2 error falls at the element order + 1.  GPU: rhs and
solution parity against the oracle (1e-12 / 1e-8) on hexahedra and on
perturbed tetrahedra.
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


def tet_levels(h):
    out = []
    for lvl in range(h.n_levels):
        rp, col = h.pattern(lvl)
        i = h.info(lvl)
        out.append(dict(verts=h.mesh(lvl), gdof=h.dofs(lvl), ndof=i["ndof"],
                        nactive=i["nactive"], row_ptr=rp, col=col))
    return out


def test_tetra_neumann_dofs_are_active(built):
    # the DOFs on a Neumann face (and not on a Dirichlet one) join the actives
    for order in (1, 2):
        d = pg.Hierarchy(3, order, 2, tetra=True).info(0)
        n = pg.Hierarchy(3, order, 2, tetra=True, neumann_mask=1 << 2).info(0)
        m = order * 4
        assert d["ndof"] == n["ndof"] == (m + 1) ** 3
        assert d["nactive"] == (m - 1) ** 3 and n["nactive"] == (m - 1) ** 2 * m


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("mask", [4, 36, 47])
def test_oracle_tetra_neumann_exact_for_linear(built, order, mask):
    h = pg.Hierarchy(3, order, 2, tetra=True, neumann_mask=mask, perturb=0.2, seed=3)
    cfg = po.make_config(3, order, 0, po.EX_POLY1, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0,
                         neumann_mask=mask, tetra=True)
    o = po.Problem(cfg, arrays=tet_levels(h))
    o.assemble()
    o.solve(po.make_solver("jacobi", max_it=2000, restart=50, reduction=1e-13))
    e = o.errors()
    assert e[0] < 1e-11 and e[1] < 1e-10


def test_oracle_tetra_neumann_crank_nicolson_exact(built):
    h = pg.Hierarchy(3, 2, 2, tetra=True, neumann_mask=36)
    cfg = po.make_config(3, 2, 0, po.EX_QUAD_ST, eps=1.0, b=(4.0, 3.0, 2.0), c=1.0,
                         neumann_mask=36, tetra=True, time_step=0.1)
    o = po.Problem(cfg, arrays=tet_levels(h))
    o.tcd_initialize()
    s = po.make_solver("jacobi", max_it=5000, restart=100, tol_abs=1e-15, reduction=0.0)
    for k in range(1, 6):
        o.tcd_step(0.1 * k, 0.1, s)
        e = o.errors()
        assert e[0] < 1e-11 and e[1] < 1e-10, (k, e)


@pytest.mark.parametrize("order,nrefs,rate", [(1, (2, 3, 4), 1.85), (2, (1, 2, 3), 2.85)])
def test_oracle_tetra_neumann_convergence(built, order, nrefs, rate):
    errs = []
    for nref in nrefs:
        h = pg.Hierarchy(3, order, nref, tetra=True, neumann_mask=36)
        cfg = po.make_config(3, order, 0, po.EX_SINE, eps=1.0, neumann_mask=36, tetra=True)
        o = po.Problem(cfg, arrays=tet_levels(h))
        o.assemble()
        o.solve(po.make_solver("jacobi", max_it=4000, restart=50, reduction=1e-12))
        errs.append(o.errors()[0])
    assert np.log2(errs[1] / errs[2]) > rate


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_tetra_neumann_solve_parity(ctx, order):
    mask = 36
    h = pg.Hierarchy(3, order, 3, n_levels=2, tetra=True, neumann_mask=mask, perturb=0.2, seed=5)
    kw = dict(eps=0.05, b=(1.0, 0.3, -0.2), c=0.5, neumann_mask=mask)
    o = po.Problem(po.make_config(3, order, 0, po.EX_SINE, tetra=True, **kw), arrays=tet_levels(h))
    o.assemble()
    it_o, _, _ = o.solve(po.make_solver("multigrid", max_it=200, restart=30, reduction=1e-10,
                                        mg_levels=2, n_pre=2, n_post=2, jacobi_damp=0.5))
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.set_solution(None)
    cd.assemble(pg.assembly_params(example=pg.EX_SINE, **kw))
    rel = lambda x, y: np.max(np.abs(x - y)) / np.max(np.abs(y))
    assert rel(cd.rhs(0), o.rhs(0)) < 1e-12
    st = cd.solve(pg.solver_params("multigrid", max_n_iterations=200, gmres_restart=30,
                                   residual_tolerance=0.0, residual_reduction=1e-10,
                                   multigrid_n_levels=2, multigrid_n_pre_smooth=2,
                                   multigrid_n_post_smooth=2, jacobi_damp=0.5, precision="fp64"))
    assert abs(st.iterations - it_o) <= 1
    assert rel(cd.solution(), o.solution()) < 1e-8


@pytest.mark.gpu
def test_tetra_neumann_exact_on_gpu(ctx):
    h = pg.Hierarchy(3, 2, 2, tetra=True, neumann_mask=47, perturb=0.2, seed=3)
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.set_solution(None)
    a = pg.assembly_params(example=pg.EX_POLY1, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0,
                           neumann_mask=47)
    cd.assemble(a)
    cd.solve(pg.solver_params("jacobi", max_n_iterations=2000, gmres_restart=50,
                              residual_tolerance=0.0, residual_reduction=1e-13))
    e = cd.errors(a)
    assert e[0] < 1e-11 and e[1] < 1e-10
