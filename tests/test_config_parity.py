"""CUDA path against the oracle at the benchmark's own configurations.

The other parity tests use small meshes; these run the workloads that
bench.py times, through the C-ABI, against the oracle on the same inputs:

  * CD2D 64x64 Q1 (4,225 DOFs), eps=1e-2, b=(1,0.5), c=1, Galerkin,
    FGMRES(50)+Jacobi in FP64 to a 1e-10 relative residual;
  * CD3D 32^3 Q2 (274,625 DOFs, four levels), eps=1e-3, b=(1,1,1)/sqrt3,
    c=0, SUPG with SDFEM_TYPE 5 and CELL_MEASURE 2, 3x3x3 Gauss,
    FGMRES(30) + multigrid V(2,2), damped Jacobi 0.8, direct coarse solve,
    in FP64 and in mixed precision (FP32 multigrid);
  * TCD3D on 24^3 cubes x 6 tetrahedra with interior vertices perturbed by
    U(+-0.2h), P2, the Crank-Nicolson steps of the time-dependent workload
    (its 48^3 mesh refined once less, four levels).

Bars: DOF numbering, CSR pattern and the coupling -> CSR slot map bit-exact
on every level (host- and device-built hierarchies); FP64 matrices and rhs to
1e-12 relative to the largest entry; FP64 solves with the oracle's iteration
count +-1 and solutions to 1e-8 relative; mixed solves at the same 1e-10
residual reduction with solutions to 1e-8 and L2/H1 errors equal to the
oracle's to 3 significant digits.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu

S3 = 0.57735026918962573


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def slots_from_pattern(dofs, rp, col):
    """CSR position of every local coupling (row dof i, column dof j) of every
    cell: the row's offset plus the column's rank inside the sorted row."""
    ndof = len(rp) - 1
    row_of = np.repeat(np.arange(ndof, dtype=np.int64), np.diff(rp))
    keys = row_of * ndof + col.astype(np.int64)
    nloc = dofs.shape[1]
    r = np.repeat(dofs.astype(np.int64), nloc, axis=1)
    c = np.tile(dofs.astype(np.int64), (1, nloc))
    want = np.searchsorted(keys, r * ndof + c)
    assert np.array_equal(keys[want], r * ndof + c)
    return want.astype(np.int32)


def check_level_structure(h, o, lvl):
    assert h.info(lvl)["ndof"] == o.info(lvl)["ndof"]
    assert h.info(lvl)["nactive"] == o.info(lvl)["nactive"]
    assert np.array_equal(h.dofs(lvl), o.gdof(lvl))
    rp, col = h.pattern(lvl)
    rpo, colo = o.structure(lvl)
    assert np.array_equal(rp, rpo) and np.array_equal(col, colo)


# ---------------------------------------------------------------------------
# CD2D 64x64 Q1, FGMRES(50) + Jacobi
# ---------------------------------------------------------------------------
def test_cd2d_q1_64_full_solve(ctx):
    kw = dict(eps=1e-2, b=(1.0, 0.5), c=1.0)
    o = po.Problem(po.make_config(2, 1, 6, po.EX_SINE, **kw), 1)
    h = pg.Hierarchy(2, 1, 6)
    check_level_structure(h, o, 0)
    o.assemble()
    it_o, res_o, ini_o = o.solve(po.make_solver("jacobi", max_it=5000, restart=50,
                                                reduction=1e-10))
    gpu = pg.ConvectionDiffusion(ctx, h)
    a = pg.assembly_params(example=pg.EX_SINE, **kw)
    gpu.assemble(a)
    rp, col = h.pattern(0)
    assert np.array_equal(gpu.slots(0), slots_from_pattern(h.dofs(0), rp, col))
    assert rel(gpu.matrix(0), o.matrix(0)) < 1e-12
    assert rel(gpu.rhs(0), o.rhs(0)) < 1e-12
    st = gpu.solve(pg.solver_params("jacobi", max_n_iterations=5000, gmres_restart=50,
                                    residual_tolerance=0.0, residual_reduction=1e-10))
    assert st.residual <= 1e-10 * st.initial_residual
    assert abs(st.initial_residual - ini_o) <= 1e-12 * ini_o
    assert abs(st.iterations - it_o) <= 1, (st.iterations, it_o)
    assert rel(gpu.solution(), o.solution()) < 1e-8
    e, e_o = gpu.errors(a), o.errors()
    for k in (0, 1):
        assert abs(e[k] - e_o[k]) <= 5e-4 * e_o[k], (k, e[k], e_o[k])
    gpu.close()


# ---------------------------------------------------------------------------
# CD3D 32^3 Q2 SUPG, four multigrid levels
# ---------------------------------------------------------------------------
C2 = dict(eps=1e-3, b=(S3, S3, S3), c=0.0)
C2_LEVELS = 4


def c2_assembly():
    return pg.assembly_params(example=pg.EX_POLYEXP, space_discretization_type="supg",
                              sdfem_type=5, delta0=1.0, cell_measure=2, problem_linear=1,
                              **C2)


def c2_solver(precision):
    return pg.solver_params("multigrid", precision=precision, max_n_iterations=1000,
                            gmres_restart=30, residual_tolerance=0.0, residual_reduction=1e-10,
                            multigrid_n_levels=C2_LEVELS, multigrid_cycle_type="V",
                            multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                            jacobi_damp=0.8, multigrid_correction_damp_factor=1.0,
                            multigrid_smoother_coarse="direct_solve")


@pytest.fixture(scope="module")
def c2_oracle(built):
    cfg = po.make_config(3, 2, 5, po.EX_POLYEXP, supg=True, sdfem_type=5, delta0=1.0,
                         cell_measure=2, problem_linear=1, **C2)
    o = po.Problem(cfg, C2_LEVELS)
    o.assemble()
    mats = [o.matrix(l) for l in range(C2_LEVELS)]
    rhs = [o.rhs(l) for l in range(C2_LEVELS)]
    it, res, ini = o.solve(po.make_solver("multigrid", max_it=1000, restart=30,
                                          reduction=1e-10, mg_levels=C2_LEVELS, mg_cycle="V",
                                          n_pre=2, n_post=2, jacobi_damp=0.8,
                                          correction_damp=1.0))
    assert res <= 1e-10 * ini
    return dict(o=o, mats=mats, rhs=rhs, it=it, ini=ini, x=o.solution(), e=o.errors())


def test_cd3d_q2_32_setup_bit_exact(ctx, c2_oracle):
    o = c2_oracle["o"]
    for h in (pg.Hierarchy(3, 2, 5, n_levels=C2_LEVELS),
              pg.Hierarchy(3, 2, 5, n_levels=C2_LEVELS, ctx=ctx)):
        for lvl in range(C2_LEVELS):
            check_level_structure(h, o, lvl)
            assert np.array_equal(h.mesh(lvl), o.mesh(lvl))


def test_cd3d_q2_32_assembly_all_levels(ctx, c2_oracle):
    h = pg.Hierarchy(3, 2, 5, n_levels=C2_LEVELS, ctx=ctx)
    gpu = pg.ConvectionDiffusion(ctx, h)
    gpu.assemble(c2_assembly())
    for lvl in range(C2_LEVELS):
        rp, col = h.pattern(lvl)
        assert np.array_equal(gpu.slots(lvl), slots_from_pattern(h.dofs(lvl), rp, col)), lvl
        assert rel(gpu.matrix(lvl), c2_oracle["mats"][lvl]) < 1e-12, lvl
        assert rel(gpu.rhs(lvl), c2_oracle["rhs"][lvl]) < 1e-12, lvl
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cd3d_q2_32_solve(ctx, c2_oracle, precision):
    h = pg.Hierarchy(3, 2, 5, n_levels=C2_LEVELS, ctx=ctx)
    gpu = pg.ConvectionDiffusion(ctx, h)
    a = c2_assembly()
    gpu.assemble(a)
    st = gpu.solve(c2_solver(precision))
    assert st.residual <= 1e-10 * st.initial_residual
    assert abs(st.initial_residual - c2_oracle["ini"]) <= 1e-12 * c2_oracle["ini"]
    if precision == "fp64":
        assert abs(st.iterations - c2_oracle["it"]) <= 1, (st.iterations, c2_oracle["it"])
    else:
        assert abs(st.iterations - c2_oracle["it"]) <= 3, (st.iterations, c2_oracle["it"])
    x = gpu.solution()
    assert rel(x, c2_oracle["x"]) < 1e-8
    e, e_o = gpu.errors(a), c2_oracle["e"]
    for k in (0, 1):
        assert abs(e[k] - e_o[k]) <= 5e-4 * e_o[k], (precision, k, e[k], e_o[k])
    gpu.close()


# ---------------------------------------------------------------------------
# TCD3D on 24^3 x 6 perturbed P2 tetrahedra, Crank-Nicolson
# ---------------------------------------------------------------------------
TCD = dict(roots=3, nref=3, levels=4, perturb=0.2, seed=2024, eps=1e-4, b=(0.5, -0.5, 0.2),
           b_grad=((0.0, -1.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
           ic=(0.3, 0.5, 0.5, 0.1), tau=1e-3, damp=0.45)


def tcd_levels(h):
    out = []
    for l in range(h.n_levels):
        rp, col = h.pattern(l)
        i = h.info(l)
        out.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"], nactive=i["nactive"],
                        row_ptr=rp, col=col))
    return out


def tcd_gpu_params(t):
    return pg.assembly_params(example=pg.EX_BUMP, eps=TCD["eps"], b=TCD["b"],
                              b_grad=TCD["b_grad"], t=t, ic=TCD["ic"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tcd3d_p2_24_crank_nicolson_steps(ctx, precision):
    L = TCD["levels"]
    h = pg.Hierarchy(3, 2, TCD["nref"], n_levels=L, roots=TCD["roots"], tetra=True,
                     perturb=TCD["perturb"], seed=TCD["seed"], ctx=ctx)
    cfg = po.make_config(3, 2, 0, po.EX_BUMP, eps=TCD["eps"], b=TCD["b"], b_grad=TCD["b_grad"],
                         tetra=True, ic=TCD["ic"])
    o = po.Problem(cfg, arrays=tcd_levels(h))
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.tcd_initialize()
    gpu.tcd_initialize(tcd_gpu_params(0.0))
    if precision == "fp64":
        for lvl in range(L):
            assert rel(gpu.tcd_matrix(0, lvl), o.tcd_matrix(0, lvl)) < 1e-12, lvl
            assert rel(gpu.tcd_matrix(1, lvl), o.tcd_matrix(1, lvl)) < 1e-12, lvl
    assert rel(gpu.solution(), o.solution()) < 1e-14
    gs = pg.solver_params("multigrid", precision=precision, max_n_iterations=1000,
                          gmres_restart=30, residual_tolerance=0.0, residual_reduction=1e-10,
                          multigrid_n_levels=L, multigrid_cycle_type="V",
                          multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                          jacobi_damp=TCD["damp"], multigrid_correction_damp_factor=1.0,
                          multigrid_smoother_coarse="direct_solve")
    so = po.make_solver("multigrid", max_it=1000, restart=30, reduction=1e-10, mg_levels=L,
                        n_pre=2, n_post=2, jacobi_damp=TCD["damp"], correction_damp=1.0)
    tau = TCD["tau"]
    for k in range(1, 3):
        st = gpu.tcd_step(tcd_gpu_params(k * tau), tau, gs)
        it_o, res_o, ini_o = o.tcd_step(k * tau, tau, so)
        assert res_o <= 1e-10 * ini_o
        assert st.residual <= 1e-10 * st.initial_residual
        assert abs(st.iterations - it_o) <= (1 if precision == "fp64" else 3), \
            (st.iterations, it_o)
        assert rel(gpu.rhs(0), o.rhs(0)) < 1e-11
        assert rel(gpu.solution(), o.solution()) < 1e-8
    if precision == "fp64":
        assert rel(gpu.tcd_matrix(2, 0), o.tcd_matrix(2, 0)) < 1e-12
    gpu.close()
