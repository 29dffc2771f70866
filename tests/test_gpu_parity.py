"""GPU parity of the CUDA path against the CPU oracle, through the C-ABI.

Bars (from the scope of the path):
  * coupling->CSR slot map, DOF numbering, pattern: bit-exact;
  * FP64 matrix entries, rhs, operator application: 1e-12 relative to the
    largest entry;
  * FP64 solutions: same iteration count (+-1) and 1e-8 relative difference
    at a 1e-10 residual reduction; L2/H1 errors against the manufactured
    solution equal to 3 significant digits; the reference's own cd2d_test
    golden errors to its 1e-11 tolerance;
  * mixed precision (FP32 multigrid inside FP64 FGMRES): the same 1e-10
    residual reduction and FP64-equal L2/H1 errors (3 significant digits).
"""
import json
import os

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_values.json")))

CASES = {
    # name: (dim, order, nref, example, eps, b, c, supg, sdfem, nmask)
    "q1_2d_cd": (2, 1, 4, po.EX_SINE, 1e-2, (1.0, 0.5), 1.0, False, 2, 0),
    "q2_2d_supg": (2, 2, 3, po.EX_SINE, 1e-3, (1.0, 0.5), 0.5, True, 2, 0),
    "q2_2d_supg_r4": (2, 2, 4, po.EX_SINE, 1e-3, (1.0, 0.5), 0.5, True, 2, 0),
    # coarse block of 961 active DOFs: beyond a cluster's shared memory, the
    # grid-wide Gauss-Jordan; smaller blocks take the cluster kernel
    "q2_2d_supg_r5": (2, 2, 5, po.EX_SINE, 1e-3, (1.0, 0.5), 0.5, True, 2, 0),
    "q1_2d_neumann": (2, 1, 3, po.EX_SINE_LAPLACE, 1.0, (0.0, 0.0), 0.0, False, 2, 2),
    "q2_2d_neumann": (2, 2, 2, po.EX_SINE_LAPLACE, 1.0, (0.0, 0.0), 0.0, False, 2, 2),
    "q1_3d_cd": (3, 1, 3, po.EX_SINE, 0.1, (1.0, 0.3, -0.2), 1.0, False, 2, 0),
    "q2_3d_supg": (3, 2, 2, po.EX_POLYEXP, 1e-3, (0.57735026918962573, 0.57735026918962573,
                                                     0.57735026918962573), 0.0, True, 5, 0),
    "q2_3d_galerkin": (3, 2, 2, po.EX_SINE, 1.0, (0.0, 0.0, 0.0), 0.0, False, 2, 0),
    # Neumann faces on hexahedra (x = 1 and z = 1; y = 0 alone)
    "q1_3d_neumann": (3, 1, 3, po.EX_SINE, 0.1, (1.0, 0.3, -0.2), 1.0, False, 2, 36),
    "q2_3d_neumann_supg": (3, 2, 2, po.EX_POLYEXP, 1e-3, (0.6, 0.64, 0.48), 0.0, True, 5, 2),
}


def make_pair(name, n_levels=1, problem_linear=0):
    dim, order, nref, ex, eps, b, c, supg, sdfem, nmask = CASES[name]
    cfg = po.make_config(dim, order, nref, ex, eps=eps, b=b, c=c, supg=supg, sdfem_type=sdfem,
                         problem_linear=problem_linear, neumann_mask=nmask)
    a = pg.assembly_params(example=ex, eps=eps, b=b, c=c,
                           space_discretization_type="supg" if supg else "galerkin",
                           sdfem_type=sdfem, problem_linear=problem_linear, neumann_mask=nmask)
    o = po.Problem(cfg, n_levels)
    h = pg.Hierarchy(dim, order, nref, n_levels=n_levels, neumann_mask=nmask)
    return o, h, a


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.mark.parametrize("name", list(CASES))
def test_assembly_parity(ctx, name):
    o, h, a = make_pair(name, n_levels=2)
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.assemble()
    gpu.assemble(a)
    for lvl in range(2):
        # slots: position of every local coupling in the sorted CSR row
        rp, col = h.pattern(lvl)
        dofs = h.dofs(lvl)
        nloc = dofs.shape[1]
        rows = np.repeat(dofs, nloc, axis=1)
        cols = np.tile(dofs, (1, nloc))
        want = np.empty_like(rows)
        for r in np.unique(rows):
            m = rows == r
            want[m] = rp[r] + np.searchsorted(col[rp[r]:rp[r + 1]], cols[m])
        assert np.array_equal(gpu.slots(lvl), want)
        assert rel(gpu.matrix(lvl), o.matrix(lvl)) < 1e-12
        assert rel(gpu.rhs(lvl), o.rhs(lvl)) < 1e-12
    x = np.random.default_rng(1).standard_normal(o.info()["ndof"])
    assert rel(gpu.apply(x), o.apply(x)) < 1e-12


@pytest.mark.parametrize("name", ["q1_2d_cd", "q2_2d_supg", "q2_3d_supg"])
def test_transfer_parity(ctx, name):
    o, h, a = make_pair(name, n_levels=3)
    gpu = pg.ConvectionDiffusion(ctx, h)
    rng = np.random.default_rng(2)
    for fine in range(2):
        xc = rng.standard_normal(o.info(fine + 1)["ndof"])
        df = rng.standard_normal(o.info(fine)["ndof"])
        assert rel(gpu.prolongate(xc, fine), o.prolongate(xc, fine)) < 1e-13
        assert rel(gpu.restrict(df, fine), o.restrict(df, fine)) < 1e-13


@pytest.mark.parametrize("cycle", ["V", "W", "F"])
def test_multigrid_cycle_parity(ctx, cycle):
    o, h, a = make_pair("q2_2d_supg", n_levels=3)
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.assemble()
    gpu.assemble(a)
    v = np.random.default_rng(3).standard_normal(o.info()["ndof"])
    so = po.make_solver("multigrid", mg_levels=3, mg_cycle=cycle, n_pre=2, n_post=2,
                        jacobi_damp=0.8, correction_damp=1.0)
    z_ref = o.mg_apply(so, v)
    for prec, tol in [("fp64", 1e-10), ("mixed", 2e-5)]:
        s = pg.solver_params("multigrid", multigrid_n_levels=3, multigrid_cycle_type=cycle,
                             multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                             jacobi_damp=0.8, precision=prec)
        assert rel(gpu.precondition(s, v), z_ref) < tol, prec


@pytest.mark.parametrize("solver", ["jacobi", "multigrid"])
@pytest.mark.parametrize("order", [1, 2])
def test_cd2d_reference_golden_errors_on_gpu(ctx, solver, order):
    g = GOLD["cd2d_test"]["errors"]["Q%d" % order]
    tol = GOLD["cd2d_test"]["tolerance"]
    h = pg.Hierarchy(2, order, 2, n_levels=2, neumann_mask=2)
    a = pg.assembly_params(example=pg.EX_SINE_LAPLACE, eps=1.0, neumann_mask=2)
    gpu = pg.ConvectionDiffusion(ctx, h)
    gpu.assemble(a)
    if solver == "jacobi":
        s = pg.solver_params("jacobi", max_n_iterations=1000, gmres_restart=100,
                             residual_tolerance=1e-15)
    else:
        s = pg.solver_params("multigrid", max_n_iterations=1000, gmres_restart=20,
                             residual_tolerance=1e-13, multigrid_n_levels=2,
                             multigrid_cycle_type="W", multigrid_n_pre_smooth=2,
                             multigrid_n_post_smooth=2)
    gpu.solve(s)
    e = gpu.errors(a)
    for k, key in [(0, "L2"), (1, "H1_semi"), (2, "SD"), (4, "L_inf")]:
        assert abs(e[k] - g[key]) < tol, (key, e[k], g[key])


@pytest.mark.parametrize("name,prec_name,levels,restart", [
    ("q1_2d_cd", "jacobi", 1, 50),
    ("q2_2d_supg", "multigrid", 3, 30),
    ("q1_3d_cd", "multigrid", 3, 30),
    ("q2_3d_supg", "multigrid", 2, 30),
    ("q2_2d_supg_r4", "multigrid", 2, 30),
    ("q2_2d_supg_r5", "multigrid", 2, 30),
])
def test_solve_parity(ctx, name, prec_name, levels, restart):
    o, h, a = make_pair(name, n_levels=levels)
    o.assemble()
    so = po.make_solver(prec_name, max_it=2000, restart=restart, tol_abs=0.0, reduction=1e-10,
                        mg_levels=levels, mg_cycle="V", n_pre=2, n_post=2, jacobi_damp=0.8)
    it_o, res_o, ini_o = o.solve(so)
    x_o = o.solution()
    e_o = o.errors()
    for prec in ["fp64", "mixed"] if prec_name == "multigrid" else ["fp64"]:
        gpu = pg.ConvectionDiffusion(ctx, h)
        gpu.assemble(a)
        s = pg.solver_params(prec_name, max_n_iterations=2000, gmres_restart=restart,
                             residual_tolerance=0.0, residual_reduction=1e-10,
                             multigrid_n_levels=levels, multigrid_cycle_type="V",
                             multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                             jacobi_damp=0.8, precision=prec)
        st = gpu.solve(s)
        assert st.residual < 1e-10 * st.initial_residual
        assert abs(st.initial_residual - ini_o) < 1e-12 * ini_o
        x = gpu.solution()
        e = gpu.errors(a)
        if prec == "fp64":
            assert abs(st.iterations - it_o) <= 1, (st.iterations, it_o)
            assert rel(x, x_o) < 1e-8
        else:
            assert st.iterations <= 2 * it_o + 2, (st.iterations, it_o)
        # L2 and H1 errors to 3 significant digits
        for k in (0, 1):
            assert abs(e[k] - e_o[k]) <= 5e-4 * e_o[k], (prec, k, e[k], e_o[k])
        # device error norms equal the oracle's norms of the same vector
        o.set_solution(x)
        e_same = o.errors()
        assert np.allclose(e, e_same, rtol=1e-10, atol=1e-15)
        gpu.close()


@pytest.mark.parametrize("gs", ["classical", "modified"])
def test_gram_schmidt_variants(ctx, gs):
    # both Arnoldi branches of Iteration_gmres::flexible_gmres (:515-534)
    o, h, a = make_pair("q1_2d_cd", n_levels=1)
    o.assemble()
    it_o, res_o, ini_o = o.solve(po.make_solver("jacobi", max_it=2000, restart=50,
                                                reduction=1e-10, gram_schmidt=gs))
    gpu = pg.ConvectionDiffusion(ctx, h)
    gpu.assemble(a)
    st = gpu.solve(pg.solver_params("jacobi", max_n_iterations=2000, gmres_restart=50,
                                    residual_tolerance=0.0, residual_reduction=1e-10,
                                    gram_schmidt=gs))
    assert abs(st.iterations - it_o) <= 1
    assert rel(gpu.solution(), o.solution()) < 1e-8


def test_from_arrays_equals_hierarchy(ctx):
    o, h, a = make_pair("q2_2d_supg", n_levels=2)
    levels = []
    for l in range(2):
        rp, col = o.structure(l)
        i = o.info(l)
        levels.append(dict(verts=o.mesh(l), dofs=o.gdof(l), ndof=i["ndof"], nactive=i["nactive"],
                           row_ptr=rp, col=col))
    g1 = pg.ConvectionDiffusion.from_arrays(ctx, 2, 2, levels)
    g2 = pg.ConvectionDiffusion(ctx, h)
    g1.assemble(a)
    g2.assemble(a)
    assert np.array_equal(g1.matrix(0), g2.matrix(0)) or rel(g1.matrix(0), g2.matrix(0)) < 1e-14
    s = pg.solver_params("multigrid", max_n_iterations=200, gmres_restart=30,
                         residual_tolerance=0.0, residual_reduction=1e-10, multigrid_n_levels=2,
                         multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.8)
    st1 = g1.solve(s)
    st2 = g2.solve(s)
    assert st1.iterations == st2.iterations
    assert rel(g1.solution(), g2.solution()) < 1e-12


@pytest.mark.parametrize("dim", [2, 3])
def test_from_arrays_maps_non_affine_cells_multilinearly(ctx, dim):
    # a cell off the parallelogram (parallelepiped) is mapped as the
    # reference maps it, by TQuadBilinear / THexaTrilinear: the level is
    # assembled per point through the cells' multilinear maps and equals the
    # oracle's matrix and rhs; sheared (still affine) meshes keep the
    # contraction
    h = pg.Hierarchy(dim, 1, 2)
    rp, col = h.pattern(0)
    i = h.info(0)
    v = h.mesh(0).copy()
    lv = dict(verts=v, dofs=h.dofs(0), gdof=h.dofs(0), ndof=i["ndof"], nactive=i["nactive"],
              row_ptr=rp, col=col)
    ct = pg.CELL_QUAD if dim == 2 else pg.CELL_HEXA
    a = pg.assembly_params(example=pg.EX_SINE, eps=0.05, b=(1.0, 0.4, -0.3)[:dim], c=0.5)
    cfg = po.make_config(dim, 1, 0, po.EX_SINE, eps=0.05, b=(1.0, 0.4, -0.3)[:dim], c=0.5)
    bad = v.copy()
    bad[5, 2, 0] += 0.01 * (1.0 / 4)     # vertex 2 of cell 5 off the parallelogram
    for verts in (v + 0.0, bad):
        if verts is not bad:
            verts[..., 0] += 0.3 * verts[..., 1]
        gpu = pg.ConvectionDiffusion.from_arrays(ctx, ct, 1, [dict(lv, verts=verts)])
        gpu.assemble(a)
        o = po.Problem(cfg, arrays=[dict(lv, verts=verts)])
        o.assemble()
        assert rel(gpu.matrix(0), o.matrix(0)) < 1e-12
        # active rows (the sheared mesh's boundary nodes lie off the unit
        # square, where the oracle finds no boundary part to take values from)
        na = i["nactive"]
        assert rel(gpu.rhs(0)[:na], o.rhs(0)[:na]) < 1e-12
        gpu.close()


def test_errors_are_reported(ctx):
    # zero matrix (eps=b=c=0): Jacobi finds a zero diagonal, the reference
    # throws "zero entry on the diagonal"; here a status code comes back
    h = pg.Hierarchy(2, 1, 2)
    gpu = pg.ConvectionDiffusion(ctx, h)
    gpu.assemble(pg.assembly_params(example=pg.EX_CONST_F, eps=0.0))
    with pytest.raises(pg.CdgError) as e:
        gpu.solve(pg.solver_params("jacobi"))
    assert e.value.code == -6
    with pytest.raises(pg.CdgError) as e:
        gpu.solve(pg.solver_params("jacobi", gmres_restart=0))
    assert e.value.code == -1
    # the context stays usable
    gpu.assemble(pg.assembly_params(example=pg.EX_SINE, eps=1.0))
    st = gpu.solve(pg.solver_params("jacobi", residual_tolerance=0.0, residual_reduction=1e-8))
    assert st.residual < 1e-8 * st.initial_residual


def test_assembly_reproducible_to_roundoff(ctx):
    # the element scatter adds FP64 entries with atomics: two assemblies of
    # the same problem agree to round-off (not necessarily bit for bit); the
    # rhs is gathered in a fixed order and is bit-identical
    h = pg.Hierarchy(3, 2, 3, n_levels=2)
    a = pg.assembly_params(example=pg.EX_POLYEXP, eps=1e-3, b=(0.577, 0.577, 0.577),
                           space_discretization_type="supg", sdfem_type=5, cell_measure=2)
    m = []
    for _ in range(2):
        cd = pg.ConvectionDiffusion(ctx, h)
        cd.assemble(a)
        m.append((cd.matrix(0), cd.rhs(0)))
        cd.close()
    assert rel(m[0][0], m[1][0]) <= 1e-14
    assert np.array_equal(m[0][1], m[1][1])
