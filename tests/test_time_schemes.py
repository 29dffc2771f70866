"""The TimeDiscretization schemes of the time-dependent path: backward Euler,
Crank-Nicolson and BDF2 (first step by backward Euler or Crank-Nicolson).

Pinned by test/tcd3d_solvers_test.c++:218-239: on the unit cube refined
twice, hexahedra and tetrahedra, tau = 0.1 up to t = 1, example -2 (u = 1 +
2x + 3ty + 4tz, linear in space and time; diffusion 1, b = (1, 2, 3), c = 0)
with Q1/P1 and backward Euler, and example -1 (u = t^2 (x^2 + yz); diffusion
1, b = (4, 3, 2), c = 1) with Q2/P2 and Crank-Nicolson lie in the discrete
space, and the reference asserts L2(0,t;L2) = L2(0,t;H1) = 0 to 1e-10 after
every step for each of its solvers.  The same holds for BDF2 where its first
step is exact (backward Euler for example -2, Crank-Nicolson for -1), and a
BDF2 run whose backward-Euler first step is not exact shows that the first
step takes the other scheme.  On the GPU the CUDA path meets the same bar
through the C-ABI, and matches the oracle's solutions and system matrices
step by step with SUPG for every scheme.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

TAU = 0.1
N_STEPS = 10
TOL = 1e-10          # tcd3d_solvers_test.c++ get_tolerance for the iterative solvers

# (example, order, scheme, first step, b, c)
LINEAR = (po.EX_LINEAR_ST, 1, "backward_euler", "backward_euler", (1.0, 2.0, 3.0), 0.0)
QUADRATIC = (po.EX_QUAD_ST, 2, "crank_nicolson", "backward_euler", (4.0, 3.0, 2.0), 1.0)
CASES = {
    "linear_backward_euler": LINEAR,
    "quadratic_crank_nicolson": QUADRATIC,
    "linear_bdf2_be_first": (po.EX_LINEAR_ST, 1, "bdf_two", "backward_euler", (1.0, 2.0, 3.0), 0.0),
    "quadratic_bdf2_cn_first": (po.EX_QUAD_ST, 2, "bdf_two", "crank_nicolson", (4.0, 3.0, 2.0), 1.0),
}


def hierarchy(order, tetra):
    return pg.Hierarchy(3, order, 2, n_levels=1, roots=1, tetra=tetra)


def levels_of(h):
    out = []
    for lvl in range(h.n_levels):
        rp, col = h.pattern(lvl)
        i = h.info(lvl)
        out.append(dict(verts=h.mesh(lvl), gdof=h.dofs(lvl), ndof=i["ndof"],
                        nactive=i["nactive"], row_ptr=rp, col=col))
    return out


def oracle_for(case, tetra, **kw):
    ex, order, scheme, first, b, c = CASES[case]
    scheme, first = kw.pop("scheme", scheme), kw.pop("first", first)
    h = hierarchy(order, tetra)
    cfg = po.make_config(3, order, 0, ex, eps=1.0, b=b, c=c, tetra=tetra,
                         time_discretization=scheme, bdf_two_first_step=first, time_step=TAU, **kw)
    return po.Problem(cfg, arrays=levels_of(h))


def run_oracle(o, supg=False):
    o.tcd_initialize()
    acc = pg.TimeErrors(supg)
    s = po.make_solver("jacobi", max_it=5000, restart=100, tol_abs=1e-15, reduction=0.0)
    out = []
    for k in range(1, N_STEPS + 1):
        o.tcd_step(k * TAU, TAU, s)
        acc.add(o.errors(), TAU, k * TAU)
        out.append(acc.get_errors())
    return out


@pytest.mark.parametrize("tetra", [False, True], ids=["hexa", "tetra"])
@pytest.mark.parametrize("case", list(CASES))
def test_oracle_zero_error_examples(built, case, tetra):
    for k, e in enumerate(run_oracle(oracle_for(case, tetra)), 1):
        assert e[0] <= TOL and e[1] <= TOL, (case, k, e)


def test_oracle_bdf2_first_step_scheme(built):
    # t^2 (x^2 + yz) is not exact under backward Euler: BDF2 begun by it keeps
    # an O(tau) error, BDF2 begun by Crank-Nicolson none
    o = oracle_for("quadratic_crank_nicolson", False, scheme="bdf_two", first="backward_euler")
    assert run_oracle(o)[-1][0] > 1e-5


def test_assembly_params_schemes():
    a = pg.assembly_params(time_discretization="bdf_two", bdf_two_first_step="crank_nicolson")
    assert (a.time_discretization, a.bdf_two_first_step) == (2, 1)
    assert pg.assembly_params().time_discretization == 0        # Crank-Nicolson
    with pytest.raises(ValueError):
        pg.assembly_params(time_discretization="fractional_step")


def test_time_errors_accumulation():
    acc = pg.TimeErrors()
    acc.add([2.0, 4.0, 0, 0, 1.0], 0.5, 0.5)
    acc.add([2.0, 4.0, 0, 0, 3.0], 0.5, 1.0)
    # trapezoids from a zero start: 0.25 * 4 + 0.25 * 8, 0.25 * 16 + 0.25 * 32
    assert acc.get_errors() == (np.sqrt(3.0), np.sqrt(12.0), 3.0)
    assert acc.t_linf == 1.0 and acc.t_l2 == 0.5


# ---------------------------------------------------------------------------
# CUDA path (GB300)
# ---------------------------------------------------------------------------
def gpu_params(case, t, supg=False, **kw):
    ex, order, scheme, first, b, c = CASES[case]
    return pg.assembly_params(example=ex, eps=kw.pop("eps", 1.0), b=kw.pop("b", b),
                              c=kw.pop("c", c), t=t, time_step=TAU,
                              space_discretization_type="supg" if supg else "galerkin",
                              sdfem_type=2, time_discretization=scheme,
                              bdf_two_first_step=first, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["jacobi", "multigrid"])
@pytest.mark.parametrize("tetra", [False, True], ids=["hexa", "tetra"])
@pytest.mark.parametrize("case", list(CASES))
def test_cuda_zero_error_examples(ctx, case, tetra, solver):
    order = CASES[case][1]
    levels = 2 if solver == "multigrid" else 1
    if tetra:
        h = pg.Hierarchy(3, order, 2, n_levels=levels, roots=1, tetra=True)
    else:
        h = pg.Hierarchy(3, order, 2 + (levels - 1), n_levels=levels)
    cd = pg.ConvectionDiffusion(ctx, h)
    if solver == "jacobi":
        s = pg.solver_params("jacobi", max_n_iterations=5000, gmres_restart=100,
                             residual_tolerance=1e-15, residual_reduction=0.0, precision="fp64")
    else:
        # tcd3d_solvers_test.c++:116-136: FGMRES + 2-level W-cycle multigrid,
        # 3+3 smoothing steps, damping 0.8 (the Jacobi smoother stands in for SOR)
        s = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                             residual_tolerance=1e-15, residual_reduction=0.0,
                             multigrid_n_levels=2, multigrid_cycle_type="W",
                             multigrid_n_pre_smooth=3, multigrid_n_post_smooth=3,
                             multigrid_correction_damp_factor=0.8, jacobi_damp=0.8,
                             precision="fp64")
    cd.tcd_initialize(gpu_params(case, 0.0))
    acc = pg.TimeErrors()
    for k in range(1, N_STEPS + 1):
        cd.tcd_step(gpu_params(case, k * TAU), TAU, s)
        acc.add(cd.errors(gpu_params(case, k * TAU)), TAU, k * TAU)
        e = acc.get_errors()
        assert e[0] <= TOL and e[1] <= TOL, (case, k, e)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,first", [("backward_euler", "backward_euler"),
                                          ("crank_nicolson", "backward_euler"),
                                          ("bdf_two", "backward_euler"),
                                          ("bdf_two", "crank_nicolson")])
def test_cuda_schemes_match_oracle_supg(ctx, scheme, first):
    # a solution outside the space, SUPG (the parameter takes theta1 * tau),
    # two multigrid levels: solutions and system matrices step by step
    h = pg.Hierarchy(2, 2, 4, n_levels=2)
    kw = dict(eps=1e-2, b=(1.0, -0.5), c=0.5)
    cfg = po.make_config(2, 2, 0, po.EX_EXP_SIN, supg=True, sdfem_type=2, time_step=0.05,
                         time_discretization=scheme, bdf_two_first_step=first, **kw)
    o = po.Problem(cfg, arrays=levels_of(h))
    cd = pg.ConvectionDiffusion(ctx, h)
    a = lambda t: pg.assembly_params(example=pg.EX_EXP_SIN, t=t, time_step=0.05,
                                     space_discretization_type="supg", sdfem_type=2,
                                     time_discretization=scheme, bdf_two_first_step=first, **kw)
    o.tcd_initialize()
    cd.tcd_initialize(a(0.0))
    gs = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                          residual_tolerance=0.0, residual_reduction=1e-12, multigrid_n_levels=2,
                          multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.8,
                          precision="fp64")
    osv = po.make_solver("multigrid", max_it=100, restart=30, reduction=1e-12, mg_levels=2,
                         n_pre=2, n_post=2, jacobi_damp=0.8)
    for k in range(1, 5):
        cd.tcd_step(a(k * 0.05), 0.05, gs)
        o.tcd_step(k * 0.05, 0.05, osv)
        S, So = cd.tcd_matrix(2, 0), o.tcd_matrix(2, 0)
        assert np.max(np.abs(S - So)) <= 1e-12 * np.max(np.abs(So)), k
        x, xo = cd.solution(), o.solution()
        assert np.max(np.abs(x - xo)) <= 1e-9 * np.max(np.abs(xo)), k
