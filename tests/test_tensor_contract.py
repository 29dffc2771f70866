"""FP32-only multigrid operators from the tensor-core contraction.

With cdg_problem_set_fp32_tensor_levels, the levels between the finest and the
coarsest -- which the mixed-precision multigrid uses only as FP32 copies --
are assembled by a tcgen05 GEMM of the cell factors with the reference
tensors (split TF32, FP32 accumulation) instead of the FP64 contraction
(src/AssembleRoutines/ConvDiff.C:1776-1999 forms the same element matrices
per quadrature point).  Bars: those FP32 values equal the oracle's FP64
matrices to FP32-level accuracy (2e-6 of the largest entry); their FP64
values, formed on demand, equal the oracle's to 1e-12; mixed-precision solves
keep their iteration count within one and their solution to 1e-8; FP64 solves
on such a problem equal the plain problem's.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu

S3 = 0.57735026918962573

CASES = {
    # name: (dim, order, nref, levels, tetra, kwargs)
    "q2_hex_supg": (3, 2, 3, 3, False, dict(example=po.EX_POLYEXP, eps=1e-3, b=(S3, S3, S3),
                                             c=0.0, supg=True, sdfem_type=5, cell_measure=2,
                                             problem_linear=1)),
    "q1_hex_galerkin": (3, 1, 4, 3, False, dict(example=po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2),
                                                 c=0.5)),
    "q2_quad_supg": (2, 2, 5, 3, False, dict(example=po.EX_SINE, eps=1e-3, b=(1.0, 0.5), c=0.5,
                                              supg=True, sdfem_type=2)),
    "p2_tet_galerkin": (3, 2, 2, 3, True, dict(example=po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2),
                                                c=1.0)),
}


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def params(kw):
    return pg.assembly_params(
        example=kw["example"], eps=kw["eps"], b=kw["b"], c=kw["c"],
        space_discretization_type="supg" if kw.get("supg") else "galerkin",
        sdfem_type=kw.get("sdfem_type", 2), cell_measure=kw.get("cell_measure", 0),
        problem_linear=kw.get("problem_linear", 0))


def build(ctx, name):
    dim, order, nref, levels, tetra, kw = CASES[name]
    ok = {k: v for k, v in kw.items() if k != "example"}
    if tetra:
        h = pg.Hierarchy(3, order, nref, n_levels=levels, roots=1, tetra=True, perturb=0.15,
                         seed=6)
        lv = []
        for l in range(levels):
            rp, col = h.pattern(l)
            i = h.info(l)
            lv.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"], nactive=i["nactive"],
                           row_ptr=rp, col=col))
        o = po.Problem(po.make_config(3, order, 0, kw["example"], tetra=True, **ok), arrays=lv)
    else:
        h = pg.Hierarchy(dim, order, nref, n_levels=levels)
        o = po.Problem(po.make_config(dim, order, nref, kw["example"], **ok), levels)
    return h, o, params(kw), levels


def mixed(levels, precision="mixed"):
    return pg.solver_params("multigrid", precision=precision, max_n_iterations=500,
                            gmres_restart=30, residual_tolerance=0.0, residual_reduction=1e-10,
                            multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                            multigrid_n_post_smooth=2, jacobi_damp=0.8)


@pytest.mark.parametrize("name", list(CASES))
def test_tensor_core_operators_against_oracle(ctx, name):
    h, o, a, levels = build(ctx, name)
    o.assemble()
    tc = pg.ConvectionDiffusion(ctx, h)
    tc.set_fp32_tensor_levels(True)
    tc.assemble(a)
    for lvl in range(1, levels - 1):
        ref = o.matrix(lvl)
        got = tc.matrix32(lvl).astype(np.float64)
        assert rel(got, ref) < 2e-6, (lvl, rel(got, ref))
    # the finest and the coarsest level keep the FP64 contraction
    for lvl in (0, levels - 1):
        assert rel(tc.matrix32(lvl).astype(np.float64), o.matrix(lvl)) < 1e-7
    # FP64 values of a tensor-core level are formed when asked for
    for lvl in range(1, levels - 1):
        assert rel(tc.matrix(lvl), o.matrix(lvl)) < 1e-12
    tc.close()


@pytest.mark.parametrize("name", ["q2_hex_supg", "p2_tet_galerkin"])
def test_tensor_core_levels_in_solves(ctx, name):
    h, o, a, levels = build(ctx, name)
    out = {}
    for enable in (False, True):
        for prec in ("mixed", "fp64"):
            cd = pg.ConvectionDiffusion(ctx, h)
            cd.set_fp32_tensor_levels(enable)
            cd.assemble(a)
            st = cd.solve(mixed(levels, prec))
            assert st.residual <= 1e-10 * st.initial_residual
            out[(enable, prec)] = (st.iterations, cd.solution(), cd.errors(a))
            cd.close()
    for prec in ("mixed", "fp64"):
        it0, x0, e0 = out[(False, prec)]
        it1, x1, e1 = out[(True, prec)]
        assert abs(it1 - it0) <= 1, (prec, it0, it1)
        assert rel(x1, x0) < 1e-8
        for k in (0, 1):
            assert abs(e1[k] - e0[k]) <= 5e-4 * e0[k]
