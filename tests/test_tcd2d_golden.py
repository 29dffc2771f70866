"""Pin the Crank-Nicolson TCD path against the reference's test/tcd2d_test.c++.

The reference runs TCD2D example 0 (exp_sin_cos: u = e^{sin 2 pi t}
sin(2 pi x) sin(2 pi y), diffusion 1, b = (1, -1), c = 1) with Q1 on the unit
square refined five times (32 x 32 cells), Crank-Nicolson with tau = 0.05 up
to t = 1, a direct solver, Galerkin and SUPG (delta0 1, SDFEM_TYPE 2), and
asserts the L2 and H1-semi errors after steps 0, 1, 2, 3, 18, 19 and 20 to
1e-10 (test/tcd2d_test.c++:24-137).  Both the CPU oracle and the CUDA path
(through the C-ABI) must reproduce those numbers to the same tolerance; a
tight FGMRES solve (relative reduction 1e-14) stands in for the direct
solver.
"""
import json
import os

import numpy as np
import pytest

import pyoracle as po

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                   "reference_values.json")))["tcd2d_test"]
TAU = 0.05
N_STEPS = 20


def check(errs, kind):
    g = GOLD["errors"][kind]
    tol = GOLD["tolerance"]
    for i, k in enumerate(GOLD["steps"]):
        assert abs(errs[k][0] - g["L2"][i]) <= tol, (kind, k, errs[k][0], g["L2"][i])
        assert abs(errs[k][1] - g["H1"][i]) <= tol, (kind, k, errs[k][1], g["H1"][i])


@pytest.mark.parametrize("kind", ["galerkin", "supg"])
def test_oracle_tcd2d_golden_errors(built, kind):
    cfg = po.make_config(2, 1, 5, po.EX_EXP_SIN, eps=1.0, b=(1.0, -1.0), c=1.0,
                         supg=kind == "supg", sdfem_type=2, delta0=1.0, time_step=TAU, t=0.0)
    o = po.Problem(cfg, 1)
    o.tcd_initialize()
    errs = {0: o.errors()}
    s = po.make_solver("jacobi", max_it=5000, restart=100, reduction=1e-15)
    for k in range(1, N_STEPS + 1):
        o.tcd_step(k * TAU, TAU, s)
        errs[k] = o.errors()
    check(errs, kind)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,solver", [("galerkin", "jacobi"), ("supg", "jacobi"),
                                         ("galerkin", "multigrid"), ("supg", "multigrid")])
def test_cuda_tcd2d_golden_errors(ctx, kind, solver):
    import parmoon2022_gb300 as pg
    levels = 5 if solver == "multigrid" else 1
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 5, n_levels=levels))
    a = lambda t: pg.assembly_params(example=pg.EX_EXP_SIN, eps=1.0, b=(1.0, -1.0), c=1.0, t=t,
                                     space_discretization_type=kind, sdfem_type=2, delta0=1.0,
                                     time_step=TAU)
    if solver == "jacobi":
        s = pg.solver_params("jacobi", max_n_iterations=5000, gmres_restart=100,
                             residual_tolerance=0.0, residual_reduction=1e-14, precision="fp64")
    else:
        # FP32 multigrid inside the FP64 FGMRES
        s = pg.solver_params("multigrid", max_n_iterations=200, gmres_restart=30,
                             residual_tolerance=0.0, residual_reduction=1e-14,
                             multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                             multigrid_n_post_smooth=2, jacobi_damp=0.8, precision="mixed")
    cd.tcd_initialize(a(0.0))
    errs = {0: cd.errors(a(0.0))}
    for k in range(1, N_STEPS + 1):
        st = cd.tcd_step(a(k * TAU), TAU, s)
        assert st.residual <= 1e-14 * st.initial_residual * 1.0001 or st.residual < 1e-13
        errs[k] = cd.errors(a(k * TAU))
    check(errs, kind)
