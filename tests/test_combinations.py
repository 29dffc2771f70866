"""Features of the time-dependent path in combination: time scheme, SUPG
parameter type and cell measure, Neumann faces, element shape.

CPU: the space-time examples stay exact (errors at round-off) with Neumann
faces under BDF2 and backward Euler on hexahedra and perturbed tetrahedra --
the Neumann data g = eps n.grad u are polynomials the face rules integrate
exactly.  GPU: the CUDA path against the oracle step by step (stiffness,
mass and system matrices to 1e-12, solutions to 1e-9) for BDF2 + SUPG +
Neumann faces on perturbed P2 tetrahedra and backward Euler + SDFEM type 7 +
CELL_MEASURE 4 on Q2 hexahedra.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po


def levels_of(h):
    out = []
    for lvl in range(h.n_levels):
        rp, col = h.pattern(lvl)
        i = h.info(lvl)
        out.append(dict(verts=h.mesh(lvl), gdof=h.dofs(lvl), ndof=i["ndof"],
                        nactive=i["nactive"], row_ptr=rp, col=col))
    return out


def rel(x, y):
    return float(np.max(np.abs(x - y)) / np.max(np.abs(y)))


@pytest.mark.parametrize("tetra", [False, True], ids=["hexa", "tetra"])
@pytest.mark.parametrize("scheme,first,ex,order,b,c", [
    ("bdf_two", "crank_nicolson", po.EX_QUAD_ST, 2, (4.0, 3.0, 2.0), 1.0),
    ("backward_euler", "backward_euler", po.EX_LINEAR_ST, 1, (1.0, 2.0, 3.0), 0.0),
])
def test_oracle_space_time_exact_with_neumann(built, tetra, scheme, first, ex, order, b, c):
    mask = 36   # faces x = 1 and z = 1
    if tetra:
        h = pg.Hierarchy(3, order, 2, tetra=True, neumann_mask=mask, perturb=0.2, seed=2)
    else:
        h = pg.Hierarchy(3, order, 2, neumann_mask=mask)
    cfg = po.make_config(3, order, 0, ex, eps=1.0, b=b, c=c, tetra=tetra, neumann_mask=mask,
                         time_step=0.1, time_discretization=scheme, bdf_two_first_step=first)
    o = po.Problem(cfg, arrays=levels_of(h))
    o.tcd_initialize()
    s = po.make_solver("jacobi", max_it=5000, restart=100, tol_abs=1e-15, reduction=0.0)
    for k in range(1, 6):
        o.tcd_step(0.1 * k, 0.1, s)
        e = o.errors()
        assert e[0] < 1e-11 and e[1] < 1e-10, (k, e)


def run_pair(ctx, h, cfg_kw, gpu_kw, steps, tau):
    o = po.Problem(po.make_config(3, h.order, 0, **cfg_kw), arrays=levels_of(h))
    cd = pg.ConvectionDiffusion(ctx, h)
    a = lambda t: pg.assembly_params(t=t, **gpu_kw)
    o.tcd_initialize()
    cd.tcd_initialize(a(0.0))
    osv = po.make_solver("multigrid", max_it=100, restart=30, reduction=1e-12, mg_levels=2,
                         n_pre=2, n_post=2, jacobi_damp=0.45)
    gs = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                          residual_tolerance=0.0, residual_reduction=1e-12, multigrid_n_levels=2,
                          multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.45,
                          precision="fp64")
    for k in range(1, steps + 1):
        o.tcd_step(k * tau, tau, osv)
        cd.tcd_step(a(k * tau), tau, gs)
        for which in (0, 1, 2):
            assert rel(cd.tcd_matrix(which, 0), o.tcd_matrix(which, 0)) < 1e-12, (k, which)
        assert rel(cd.solution(), o.solution()) < 1e-9, k


@pytest.mark.gpu
def test_cuda_bdf2_supg_neumann_tetra(ctx):
    mask, tau, b = 36, 0.02, (0.8, 0.3, 0.2)
    h = pg.Hierarchy(3, 2, 3, n_levels=2, tetra=True, neumann_mask=mask, perturb=0.2, seed=6)
    common = dict(eps=1e-2, b=b, c=0.3, neumann_mask=mask, time_step=tau,
                  time_discretization="bdf_two", bdf_two_first_step="crank_nicolson")
    run_pair(ctx, h, dict(example=po.EX_EXP_SIN, tetra=True, supg=True, sdfem_type=2, **common),
             dict(example=pg.EX_EXP_SIN, space_discretization_type="supg", sdfem_type=2,
                  **common), steps=4, tau=tau)


@pytest.mark.gpu
def test_cuda_backward_euler_codina_convection_size_hexa(ctx):
    tau, b = 0.05, (0.9, 0.4, 0.2)
    h = pg.Hierarchy(3, 2, 3, n_levels=2)
    common = dict(eps=1e-3, b=b, c=0.5, cell_measure=4, time_step=tau,
                  time_discretization="backward_euler")
    run_pair(ctx, h, dict(example=po.EX_EXP_SIN, supg=True, sdfem_type=7, **common),
             dict(example=pg.EX_EXP_SIN, space_discretization_type="supg", sdfem_type=7,
                  **common), steps=3, tau=tau)
