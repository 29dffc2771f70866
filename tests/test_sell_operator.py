"""The sliced ELLPACK copy of the FP64 operator on levels of 32768 rows or
more (smaller levels keep CSR).

The layout is internal: the FGMRES operator, the restart residual and the
FP64 multigrid smoother and defect run on it, and it must give the oracle's
CSR products.  Bars: operator application 1e-12 relative to the largest
entry (another summation order than CSR, FP64 round-off only); FP64
multigrid cycle 1e-10; identity rows where the time-dependent system keeps
assembled Dirichlet rows; Crank-Nicolson solutions 1e-8 with the same
iteration count +-1.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


CASES = {
    # name: (dim, order, nref, example, eps, b, c, supg, sdfem, lanes)
    # 66,049 rows of ~25 entries: 2 lanes per row
    "q2_2d_n128": (2, 2, 7, po.EX_SINE, 1e-3, (1.0, 0.5), 0.5, True, 2, 2),
    # 263,169 rows of ~9 entries: 1 lane per row
    "q1_2d_n512": (2, 1, 9, po.EX_SINE, 1e-2, (1.0, 0.5), 1.0, False, 2, 1),
    # 35,937 rows of ~62 entries: 2 lanes give 2,246 warps, doubled to 4
    "q2_3d_n16": (3, 2, 4, po.EX_POLYEXP, 1e-3, (0.6, 0.64, 0.48), 0.0, True, 5, 4),
}


def make(name, n_levels=1):
    dim, order, nref, ex, eps, b, c, supg, sdfem, lanes = CASES[name]
    cfg = po.make_config(dim, order, nref, ex, eps=eps, b=b, c=c, supg=supg, sdfem_type=sdfem)
    a = pg.assembly_params(example=ex, eps=eps, b=b, c=c,
                           space_discretization_type="supg" if supg else "galerkin",
                           sdfem_type=sdfem)
    return po.Problem(cfg, n_levels), pg.Hierarchy(dim, order, nref, n_levels=n_levels), a, lanes


@pytest.mark.parametrize("name", list(CASES))
def test_sell_operator_equals_csr_product(ctx, name):
    o, h, a, lanes = make(name, n_levels=2)
    gpu = pg.ConvectionDiffusion(ctx, h)
    lay = gpu.operator_layout(0)
    assert lay["lanes"] == lanes
    nnz = gpu.info(0)["nnz"]
    # identity rows take one slot each, whatever their CSR pattern holds
    assert 0.8 * nnz <= lay["slots"] < 1.2 * nnz + 32 * 16
    assert (gpu.operator_layout(1)["lanes"] > 0) == (gpu.info(1)["ndof"] >= 32768)
    o.assemble()
    gpu.assemble(a)
    assert rel(gpu.matrix(0), o.matrix(0)) < 1e-12
    rng = np.random.default_rng(4)
    for _ in range(2):
        x = rng.standard_normal(gpu.info(0)["ndof"])
        assert rel(gpu.apply(x), o.apply(x)) < 1e-12
    # a second assembly with other coefficients refreshes the copy
    a2 = pg.assembly_params(example=a.example, eps=a.eps * 3, b=tuple(a.b), c=a.c + 0.25,
                            space_discretization_type="supg" if a.supg else "galerkin",
                            sdfem_type=a.sdfem_type)
    gpu.assemble(a2)
    o2 = po.Problem(po.make_config(*CASES[name][:4], eps=a.eps * 3, b=tuple(a.b)[:CASES[name][0]],
                                   c=a.c + 0.25, supg=bool(a.supg), sdfem_type=a.sdfem_type), 2)
    o2.assemble()
    x = rng.standard_normal(gpu.info(0)["ndof"])
    assert rel(gpu.apply(x), o2.apply(x)) < 1e-12


def test_fp64_multigrid_on_sell_levels(ctx):
    o, h, a, _ = make("q2_2d_n128", n_levels=3)
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.assemble()
    gpu.assemble(a)
    v = np.random.default_rng(5).standard_normal(gpu.info(0)["ndof"])
    so = po.make_solver("multigrid", mg_levels=3, n_pre=2, n_post=2, jacobi_damp=0.8)
    s = pg.solver_params("multigrid", multigrid_n_levels=3, multigrid_n_pre_smooth=2,
                         multigrid_n_post_smooth=2, jacobi_damp=0.8, precision="fp64")
    assert rel(gpu.precondition(s, v), o.mg_apply(so, v)) < 1e-10


def test_solve_on_sell_operator(ctx):
    o, h, a, _ = make("q2_3d_n16", n_levels=3)
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.assemble()
    gpu.assemble(a)
    gpu.set_solution(None)
    so = po.make_solver("multigrid", max_it=200, restart=30, reduction=1e-10, mg_levels=3,
                        n_pre=2, n_post=2, jacobi_damp=0.5)
    it_o, res_o, ini_o = o.solve(so)
    for prec in ("fp64", "mixed"):
        gpu.set_solution(None)
        st = gpu.solve(pg.solver_params("multigrid", max_n_iterations=200, gmres_restart=30,
                                        residual_tolerance=0.0, residual_reduction=1e-10,
                                        multigrid_n_levels=3, multigrid_n_pre_smooth=2,
                                        multigrid_n_post_smooth=2, jacobi_damp=0.5,
                                        precision=prec))
        assert st.residual <= 1e-10 * st.initial_residual * 1.0001
        if prec == "fp64":
            assert abs(st.iterations - it_o) <= 1
        assert rel(gpu.solution(), o.solution()) < 1e-8, prec


def test_tcd_system_on_sell_operator(ctx):
    # 33^3 P2 DOFs on tetrahedra: the Crank-Nicolson system keeps assembled
    # Dirichlet rows, which the operator treats as identity rows
    h = pg.Hierarchy(3, 2, 4, n_levels=3, roots=1, tetra=True, perturb=0.15, seed=8)
    levels = []
    for lvl in range(3):
        rp, col = h.pattern(lvl)
        i = h.info(lvl)
        levels.append(dict(verts=h.mesh(lvl), gdof=h.dofs(lvl), ndof=i["ndof"],
                           nactive=i["nactive"], row_ptr=rp, col=col))
    kw = dict(eps=1e-3, b=(0.8, 0.3, 0.2), supg=True, sdfem_type=2, time_step=1e-2,
              ic=(0.4, 0.5, 0.6, 0.15))
    o = po.Problem(po.make_config(3, 2, 0, po.EX_BUMP, tetra=True, **kw), arrays=levels)
    gpu = pg.ConvectionDiffusion(ctx, h)
    assert gpu.operator_layout(0)["lanes"] > 0
    ga = lambda t: pg.assembly_params(example=pg.EX_BUMP, eps=1e-3, b=(0.8, 0.3, 0.2), t=t,
                                      ic=(0.4, 0.5, 0.6, 0.15),
                                      space_discretization_type="supg", sdfem_type=2,
                                      time_step=1e-2)
    o.tcd_initialize()
    gpu.tcd_initialize(ga(0.0))
    gs = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                          residual_tolerance=0.0, residual_reduction=1e-10, multigrid_n_levels=3,
                          multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.45,
                          precision="fp64")
    osv = po.make_solver("multigrid", max_it=100, restart=30, reduction=1e-10, mg_levels=3,
                         n_pre=2, n_post=2, jacobi_damp=0.45)
    for k in (1, 2):
        st = gpu.tcd_step(ga(k * 1e-2), 1e-2, gs)
        it_o, res_o, ini_o = o.tcd_step(k * 1e-2, 1e-2, osv)
        assert abs(st.iterations - it_o) <= 1
        assert rel(gpu.solution(), o.solution()) < 1e-8
    rp, col = levels[0]["row_ptr"], levels[0]["col"]
    na = levels[0]["nactive"]
    S = gpu.tcd_matrix(2, 0)
    x = np.random.default_rng(6).standard_normal(len(rp) - 1)
    prod = np.add.reduceat(S * x[col], rp[:-1])
    prod[na:] = x[na:]
    assert rel(gpu.apply(x), prod) < 1e-12


@pytest.mark.parametrize("name", ["q1_2d_n512", "q2_3d_n16"])
def test_device_layout_equals_host_layout(ctx, name):
    import os
    out = []
    for host in (True, False):
        if host:
            os.environ["CDG_SELL_HOST"] = "1"
        try:
            o, h, a, lanes = make(name, n_levels=1)
            gpu = pg.ConvectionDiffusion(ctx, h)
        finally:
            os.environ.pop("CDG_SELL_HOST", None)
        gpu.assemble(a)
        x = np.random.default_rng(9).standard_normal(gpu.info(0)["ndof"])
        out.append((gpu.operator_layout(0), gpu.apply(x)))
    assert out[0][0] == out[1][0]
    assert rel(out[1][1], out[0][1]) < 1e-14
