"""Matrix-free FP32 operator of the Q2 hexahedral multigrid levels.

The mixed-precision multigrid smooths with an FP32 copy of each level's
operator (JacobiSmoother::smooth, src/Multigrid/JacobiSmoother.C:21-29).  On
Q2 hexahedra that operator can also be applied without the CSR matrix: by sum
factorisation from per-cell factors, or, where all cells are translates of
one cell and the coefficients are constant, from one shared element matrix.
Bars:

  * the matrix-free product equals the FP32 CSR product and the oracle's FP64
    product (BlockFEMatrix::apply) to FP32 rounding (2e-5 relative to the
    largest entry of the active rows; identity on the non-active rows), on
    every level, for SUPG, Galerkin and a convection field linear in x, on
    uniform and sheared (still affine) meshes;
  * a mixed-precision solve with the matrix-free smoother reaches the same
    1e-10 residual reduction as with the CSR smoother, within two FGMRES
    iterations of it, with the solution equal to the oracle's to 1e-8 and
    L2/H1 errors equal to 3 significant digits;
  * the per-level kernel choice of the tuner is reported and gives the same
    solve within those bars;
  * on a uniform lattice with Dirichlet data on the whole boundary the
    stencil sweep (eight 125-point stencils summed from the element matrix)
    equals the CSR and the oracle's products to FP32 rounding and solves
    within one iteration of the tile sweep; other levels refuse it.
"""
import os

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu

S3 = 0.57735026918962573
ROT = ((0.0, -1.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0))

CASES = {
    # name: (nref, levels, kwargs shared by the oracle config and the assembly)
    "supg_polyexp": (3, 2, dict(example=po.EX_POLYEXP, eps=1e-3, b=(S3, S3, S3), c=0.0,
                                supg=True, sdfem_type=5, cell_measure=2, problem_linear=1)),
    "supg_sine_sdfem2": (3, 2, dict(example=po.EX_SINE, eps=1e-4, b=(1.0, 0.25, 0.1), c=0.2,
                                    supg=True, sdfem_type=2)),
    "galerkin_sine": (3, 2, dict(example=po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=0.5)),
    "galerkin_linear_b": (2, 2, dict(example=po.EX_SINE, eps=1e-2, b=(0.5, -0.5, 0.2),
                                     b_grad=ROT, c=0.3)),
}


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def gpu_params(kw):
    return pg.assembly_params(
        example=kw["example"], eps=kw["eps"], b=kw["b"], c=kw["c"], b_grad=kw.get("b_grad"),
        space_discretization_type="supg" if kw.get("supg") else "galerkin",
        sdfem_type=kw.get("sdfem_type", 2), cell_measure=kw.get("cell_measure", 0),
        problem_linear=kw.get("problem_linear", 0))


def oracle_cfg(nref, kw):
    ok = {k: v for k, v in kw.items() if k != "example"}
    return po.make_config(3, 2, nref, kw["example"], **ok)


def sheared_pair(ctx, nref, levels, kw):
    """the unit-cube hierarchy with x += 0.3 y: parallelepiped (affine) cells"""
    h = pg.Hierarchy(3, 2, nref, n_levels=levels)
    lv = []
    for l in range(levels):
        rp, col = h.pattern(l)
        i = h.info(l)
        v = h.mesh(l).copy()
        v[..., 0] += 0.3 * v[..., 1]
        lv.append(dict(verts=v, dofs=h.dofs(l), gdof=h.dofs(l), ndof=i["ndof"],
                       nactive=i["nactive"], row_ptr=rp, col=col))
    gpu = pg.ConvectionDiffusion.from_arrays(ctx, pg.CELL_HEXA, 2, lv)
    o = po.Problem(oracle_cfg(0, kw), arrays=lv)
    return gpu, o


@pytest.mark.parametrize("sheared", [False, True])
@pytest.mark.parametrize("name", list(CASES))
def test_matrix_free_operator_parity(ctx, name, sheared):
    nref, levels, kw = CASES[name]
    if sheared:
        gpu, o = sheared_pair(ctx, nref, levels, kw)
    else:
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        o = po.Problem(oracle_cfg(nref, kw), levels)
    gpu.assemble(gpu_params(kw))
    o.assemble()
    rng = np.random.default_rng(5)
    for lvl in range(levels):
        na = gpu.info(lvl)["nactive"]
        x = rng.standard_normal(gpu.info(lvl)["ndof"]).astype(np.float32)
        y_csr = gpu.apply32(x, lvl, 0)
        y_mf = gpu.apply32(x, lvl, 1)
        y_ref = o.apply(x.astype(np.float64), lvl)
        # active rows (the operator proper), relative to their largest entry
        assert rel(y_mf[:na], y_csr[:na]) < 2e-5, (lvl, rel(y_mf[:na], y_csr[:na]))
        assert rel(y_mf[:na], y_ref[:na]) < 2e-5, (lvl, rel(y_mf[:na], y_ref[:na]))
        # non-active rows are identity rows
        assert np.array_equal(y_mf[na:], x[na:])
    gpu.close()


def test_matrix_free_needs_a_stationary_hexahedral_assembly(ctx):
    h = pg.Hierarchy(2, 2, 3)
    gpu = pg.ConvectionDiffusion(ctx, h)
    gpu.assemble(pg.assembly_params(example=pg.EX_SINE, eps=1.0))
    with pytest.raises(pg.CdgError) as e:
        gpu.apply32(np.zeros(h.info(0)["ndof"], np.float32), 0, 1)
    assert e.value.code == -1
    gpu.close()


def mixed_solver(levels):
    return pg.solver_params("multigrid", precision="mixed", max_n_iterations=500,
                            gmres_restart=30, residual_tolerance=0.0, residual_reduction=1e-10,
                            multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                            multigrid_n_post_smooth=2, jacobi_damp=0.8)


def solve_with(ctx, nref, levels, kw, env):
    old = os.environ.get("CDG_MATFREE")
    if env is None:
        os.environ.pop("CDG_MATFREE", None)
    else:
        os.environ["CDG_MATFREE"] = env
    try:
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        a = gpu_params(kw)
        gpu.assemble(a)
        st = gpu.solve(mixed_solver(levels))
        out = dict(st=st, x=gpu.solution(), e=gpu.errors(a),
                   choice=[gpu.tuning(l)[0] for l in range(levels)])
        gpu.close()
        return out
    finally:
        if old is None:
            os.environ.pop("CDG_MATFREE", None)
        else:
            os.environ["CDG_MATFREE"] = old


@pytest.mark.parametrize("name", ["supg_polyexp", "galerkin_sine"])
def test_mixed_solve_with_matrix_free_smoother(ctx, name):
    nref, _, kw = CASES[name]
    levels = 3
    o = po.Problem(oracle_cfg(nref, kw), levels)
    o.assemble()
    it_o, res_o, ini_o = o.solve(po.make_solver("multigrid", max_it=500, restart=30,
                                                reduction=1e-10, mg_levels=levels, n_pre=2,
                                                n_post=2, jacobi_damp=0.8))
    assert res_o <= 1e-10 * ini_o
    x_o, e_o = o.solution(), o.errors()
    csr = solve_with(ctx, nref, levels, kw, "0")
    mf = solve_with(ctx, nref, levels, kw, "1")
    tuned = solve_with(ctx, nref, levels, kw, None)
    assert csr["choice"][:2] == [0, 0] and mf["choice"][:2] == [1, 1]
    assert all(c in (0, 1) for c in tuned["choice"][:levels - 1])
    for r in (csr, mf, tuned):
        st = r["st"]
        assert st.residual <= 1e-10 * st.initial_residual
        assert abs(st.iterations - csr["st"].iterations) <= 2
        assert abs(st.iterations - it_o) <= 3
        assert rel(r["x"], x_o) < 1e-8
        for k in (0, 1):
            assert abs(r["e"][k] - e_o[k]) <= 5e-4 * e_o[k]


def test_tuned_schedule_reproduced_by_its_settings(ctx, monkeypatch):
    # the tuner's choices (kernel, lanes per row, matrix-free grid) fixed
    # through the environment reproduce the tuned schedule and solve (the
    # FP64 element scatter adds with atomics, so two assemblies agree to
    # round-off, not bit for bit); the untuned defaults give the same solve
    # within the mixed-precision bars
    nref, _, kw = CASES["supg_polyexp"]
    levels = 3
    for name in ("CDG_MATFREE", "CDG_TPR32", "CDG_MF_CAP", "CDG_MF_MINB", "CDG_MF_STENCIL",
                 "CDG_TUNE"):
        monkeypatch.delenv(name, raising=False)

    def run():
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        a = gpu_params(kw)
        gpu.assemble(a)
        st = gpu.solve(mixed_solver(levels))
        det = [gpu.tuning_detail(l) for l in range(levels - 1)]
        x = gpu.solution()
        gpu.close()
        return st, x, det

    st_t, x_t, det = run()
    assert all(d[0] in (0, 1) for d in det)
    monkeypatch.setenv("CDG_MATFREE", ",".join(str(d[0]) for d in det))
    monkeypatch.setenv("CDG_TPR32", ",".join(str(d[2][0]) for d in det))
    # grid cap (two-launch sweep), register budget (one-launch sweep, -blocks)
    # or points per thread (stencil sweep, -100 - points)
    monkeypatch.setenv("CDG_MF_CAP", ",".join(str(max(d[2][1], 0)) for d in det))
    monkeypatch.setenv("CDG_MF_MINB", ",".join(str(-d[2][1] if -6 <= d[2][1] <= -4 else 4)
                                               for d in det))
    monkeypatch.setenv("CDG_MF_STENCIL", ",".join(str(-100 - d[2][1] if d[2][1] <= -100 else 0)
                                                  for d in det))
    st_f, x_f, det_f = run()
    assert [d[0] for d in det_f] == [d[0] for d in det]
    assert [d[2] for d in det_f] == [d[2] for d in det]
    assert st_f.iterations == st_t.iterations
    assert rel(x_f, x_t) < 1e-10
    for name in ("CDG_MATFREE", "CDG_TPR32", "CDG_MF_CAP", "CDG_MF_MINB", "CDG_MF_STENCIL"):
        monkeypatch.delenv(name)
    monkeypatch.setenv("CDG_TUNE", "0")
    st_d, x_d, det_d = run()
    assert all(d[0] == 0 for d in det_d)
    assert abs(st_d.iterations - st_t.iterations) <= 2
    assert rel(x_d, x_t) < 1e-8


def test_matrix_free_grid_does_not_change_results(ctx, monkeypatch):
    # two-kernel sweep with one cell per warp or 4 / 8 blocks per SM walking
    # the cells: the same matrix-free products, bit for bit (the operator of a
    # uniform level comes from cell 0's factors and is summed per row in a
    # fixed order)
    nref, levels, kw = CASES["supg_polyexp"]
    x = None
    outs = []
    monkeypatch.setenv("CDG_MF_FUSED", "0")
    monkeypatch.setenv("CDG_MF_STENCIL", "0")
    for cap in ("0", "4", "8"):
        monkeypatch.setenv("CDG_MATFREE", "1")
        monkeypatch.setenv("CDG_MF_CAP", cap)
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        gpu.assemble(gpu_params(kw))
        if x is None:
            x = np.random.default_rng(8).standard_normal(gpu.info(0)["ndof"]).astype(np.float32)
        gpu.precondition(mixed_solver(levels), x.astype(np.float64))   # runs the tuner
        assert gpu.tuning_detail(0)[0] == 1 and gpu.tuning_detail(0)[2][1] == int(cap)
        outs.append(gpu.apply32(x, 0, 1))
        gpu.close()
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("sheared", [False, True])
@pytest.mark.parametrize("name", ["supg_polyexp", "supg_sine_sdfem2", "galerkin_sine"])
def test_one_launch_sweep_equals_two_kernel_product(ctx, name, sheared):
    # uniform levels apply the shared element matrix in one launch per sweep
    # (row tiles recomputing their cells in shared memory); the product
    # equals the two-launch form (cell products to memory, then row sums)
    # bit for bit, and the oracle's FP64 product to FP32 rounding
    nref, levels, kw = CASES[name]
    if sheared:
        gpu, o = sheared_pair(ctx, nref, levels, kw)
    else:
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        o = po.Problem(oracle_cfg(nref, kw), levels)
    gpu.assemble(gpu_params(kw))
    o.assemble()
    rng = np.random.default_rng(11)
    for lvl in range(levels):
        na = gpu.info(lvl)["nactive"]
        x = rng.standard_normal(gpu.info(lvl)["ndof"]).astype(np.float32)
        y1 = gpu.apply32(x, lvl, 1)
        y2 = gpu.apply32(x, lvl, 2)
        assert np.array_equal(y1, y2), lvl
        assert rel(y1[:na], o.apply(x.astype(np.float64), lvl)[:na]) < 2e-5
    gpu.close()


def test_one_launch_sweep_in_solves(ctx, monkeypatch):
    # the mixed solve with the one-launch sweep against the two-kernel sweep
    # (CDG_MF_FUSED=0): the same iterations and solution (the FP64 finest
    # operators of two assemblies differ in round-off only)
    nref, _, kw = CASES["supg_polyexp"]
    levels = 3
    monkeypatch.setenv("CDG_MATFREE", "1")
    monkeypatch.setenv("CDG_MF_STENCIL", "0")
    out = []
    for fused in ("1", "0"):
        monkeypatch.setenv("CDG_MF_FUSED", fused)
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        a = gpu_params(kw)
        gpu.assemble(a)
        st = gpu.solve(mixed_solver(levels))
        assert st.residual <= 1e-10 * st.initial_residual
        out.append((st.iterations, gpu.solution(), gpu.tuning_detail(0)))
        gpu.close()
    assert out[0][2][2][1] in (-4, -5, -6) and out[1][2][2][1] >= 0
    assert abs(out[0][0] - out[1][0]) <= 1
    assert rel(out[0][1], out[1][1]) < 1e-10


@pytest.mark.parametrize("name", ["supg_polyexp", "supg_sine_sdfem2", "galerkin_sine"])
def test_uniform_fp64_matrix_equals_the_contraction(ctx, monkeypatch, name):
    # on a uniform level the FP64 matrix is one element matrix scattered
    # through the cells' frames; it equals the per-cell contraction
    # (CDG_UNIFORM_FP64=0) to round-off and the oracle to 1e-12
    nref, levels, kw = CASES[name]
    o = po.Problem(oracle_cfg(nref, kw), levels)
    o.assemble()
    mats = []
    for flag in ("1", "0"):
        monkeypatch.setenv("CDG_UNIFORM_FP64", flag)
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        gpu.assemble(gpu_params(kw))
        mats.append([gpu.matrix(l) for l in range(levels)])
        gpu.close()
    for l in range(levels):
        assert rel(mats[0][l], mats[1][l]) < 1e-14
        assert rel(mats[0][l], o.matrix(l)) < 1e-12


@pytest.mark.parametrize("sheared", [False, True])
@pytest.mark.parametrize("name", ["supg_polyexp", "supg_sine_sdfem2", "galerkin_sine"])
def test_stencil_sweep_operator(ctx, name, sheared):
    # every active row of a uniform lattice is one of eight 125-point
    # stencils (by the parities of its lattice point) summed from the element
    # matrix: the stencil product equals the CSR product and the oracle's
    # FP64 product to FP32 rounding on every level, identity on non-active rows
    nref, levels, kw = CASES[name]
    if sheared:
        gpu, o = sheared_pair(ctx, nref, levels, kw)
    else:
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        o = po.Problem(oracle_cfg(nref, kw), levels)
    gpu.assemble(gpu_params(kw))
    o.assemble()
    rng = np.random.default_rng(13)
    for lvl in range(levels):
        na = gpu.info(lvl)["nactive"]
        x = rng.standard_normal(gpu.info(lvl)["ndof"]).astype(np.float32)
        y3 = gpu.apply32(x, lvl, 3)
        y0 = gpu.apply32(x, lvl, 0)
        assert rel(y3[:na], y0[:na]) < 2e-5, (lvl, rel(y3[:na], y0[:na]))
        assert rel(y3[:na], o.apply(x.astype(np.float64), lvl)[:na]) < 2e-5
        assert np.array_equal(y3[na:], x[na:])
    gpu.close()


@pytest.mark.parametrize("sheared", [False, True])
def test_stencil_sweep_on_several_tiles(ctx, sheared):
    # a 32^3 Q2 lattice (65^3 points: two tiles along x, the last one partly
    # outside, z tiles ending at the boundary) against the CSR product
    kw = CASES["supg_polyexp"][2]
    if sheared:
        gpu, _ = sheared_pair(ctx, 5, 1, kw)
    else:
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, 5, n_levels=1))
    gpu.assemble(gpu_params(kw))
    na, n = gpu.info(0)["nactive"], gpu.info(0)["ndof"]
    x = np.random.default_rng(17).standard_normal(n).astype(np.float32)
    y3, y0 = gpu.apply32(x, 0, 3), gpu.apply32(x, 0, 0)
    assert rel(y3[:na], y0[:na]) < 2e-5
    assert np.array_equal(y3[na:], x[na:])
    # deterministic: the same product twice
    assert np.array_equal(gpu.apply32(x, 0, 3), y3)
    gpu.close()


def test_stencil_sweep_needs_a_dirichlet_lattice(ctx):
    # active DOFs on the boundary (Neumann faces) break the interior-stencil
    # rows; moved vertices leave no matrix-free operator: both refuse
    kw = CASES["galerkin_sine"][2]
    for h, a in ((pg.Hierarchy(3, 2, 2, neumann_mask=36),
                  pg.assembly_params(example=pg.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=0.5,
                                     neumann_mask=36)),
                 (pg.Hierarchy(3, 2, 2, perturb=0.2, seed=3), gpu_params(kw))):
        gpu = pg.ConvectionDiffusion(ctx, h)
        gpu.assemble(a)
        x = np.ones(gpu.info(0)["ndof"], np.float32)
        if a.neumann_mask:
            gpu.apply32(x, 0, 1)   # the tile sweep takes the level
        with pytest.raises(pg.CdgError) as e:
            gpu.apply32(x, 0, 3)
        assert e.value.code == -1
        gpu.close()


def test_stencil_sweep_in_solves(ctx, monkeypatch):
    # mixed solves with the stencil sweep on the finest level (8 and 4 lattice
    # points per thread) against the one-launch tile sweep: within one
    # iteration, the solutions to 1e-8 (the sweeps differ in FP32 rounding)
    nref, _, kw = CASES["supg_polyexp"]
    nref, levels = 4, 3
    monkeypatch.setenv("CDG_MATFREE", "1,0,0")
    out = []
    for st_env in ("8", "4", "0"):
        monkeypatch.setenv("CDG_MF_STENCIL", st_env)
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, nref, n_levels=levels))
        a = gpu_params(kw)
        gpu.assemble(a)
        st = gpu.solve(mixed_solver(levels))
        assert st.residual <= 1e-10 * st.initial_residual
        out.append((st.iterations, gpu.solution(), gpu.tuning_detail(0), gpu.errors(a)))
        gpu.close()
    assert out[0][2][2][1] == -108 and out[1][2][2][1] == -104
    assert out[2][2][2][1] in (-4, -5, -6)
    for it, x, _, e in out[:2]:
        assert abs(it - out[2][0]) <= 1
        assert rel(x, out[2][1]) < 1e-8
        for k in (0, 1):
            assert abs(e[k] - out[2][3][k]) <= 5e-4 * out[2][3][k]
