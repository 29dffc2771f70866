"""General quadrilaterals and hexahedra: the reference's bilinear / trilinear
reference maps.

The reference maps a quadrilateral that is not a parallelogram by
TQuadBilinear and a hexahedron that is not a parallelepiped by THexaTrilinear
(the shape tests TQuadrangle::CheckQuad, Quadrangle.C:119-128, and
THexahedron::CheckHexa, Hexahedron.C:196-235; QuadBilinear.C:87-263,
HexaTrilinear.C:14-270): the Jacobian changes over the cell, and SUPG's
second derivatives on a bilinear cell go through the 5 x 5 system of
GetOrigAllDerivatives (QuadBilinear.C:131-205); on trilinear cells the
reference does not transform second derivatives (it throws), so SUPG there is
refused.  Meshes: the unit square / cube hierarchies with the finest level's
interior vertices moved (cdg_hierarchy_perturb).

CPU (oracle): a vanishing perturbation gives the affine matrices; the L2 and
H1 errors on moved meshes fall at the element's rates.  GPU, against the
oracle on the same meshes: matrices and rhs to 1e-12 relative, solves with
the oracle's iteration count +-1 and solutions to 1e-8, errors to 3
significant digits; unsupported combinations refused with CDG_ERR_ARG.
"""
import ctypes

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

S3 = 0.57735026918962573


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def arrays(h, levels):
    lv = []
    for l in range(levels):
        rp, col = h.pattern(l)
        i = h.info(l)
        lv.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"], nactive=i["nactive"],
                       row_ptr=rp, col=col))
    return lv


def oracle_on(h, levels, dim, order, example, **kw):
    return po.Problem(po.make_config(dim, order, 0, example, **kw), arrays=arrays(h, levels))


def test_vanishing_perturbation_gives_the_affine_matrices(built):
    # a 1e-6 h move makes every interior cell multilinear (the shape test's
    # threshold is 1e-8); its matrices differ from the affine mesh's by O(1e-6)
    for dim, order, nref, supg in [(2, 1, 3, True), (2, 2, 2, True), (3, 1, 2, False),
                                   (3, 2, 1, False)]:
        kw = dict(eps=0.05, b=(1.0, 0.4, -0.3)[:dim], c=0.5, supg=supg, sdfem_type=2)
        h0 = pg.Hierarchy(dim, order, nref)
        h1 = pg.Hierarchy(dim, order, nref, perturb=1e-6, seed=3)
        o0 = oracle_on(h0, 1, dim, order, po.EX_SINE, **kw)
        o1 = oracle_on(h1, 1, dim, order, po.EX_SINE, **kw)
        o0.assemble()
        o1.assemble()
        d = rel(o1.matrix(0), o0.matrix(0))
        assert 1e-12 < d < 1e-4, (dim, order, d)
        assert rel(o1.rhs(0), o0.rhs(0)) < 1e-4


@pytest.mark.parametrize("dim,order,supg,rates", [
    (2, 1, False, (4.0, 2.0)), (2, 2, False, (8.0, 4.0)), (2, 2, True, (8.0, 4.0)),
    (3, 1, False, (4.0, 2.0))])
def test_errors_fall_at_the_element_rates_on_moved_meshes(built, dim, order, supg, rates):
    kw = dict(eps=0.1, b=(1.0, 0.5, 0.2)[:dim], c=1.0, supg=supg, sdfem_type=2)
    errs = []
    nrefs = (2, 3) if dim == 3 else (3, 4)
    for nref in nrefs:
        h = pg.Hierarchy(dim, order, nref, perturb=0.2, seed=7)
        o = oracle_on(h, 1, dim, order, po.EX_SINE, **kw)
        o.assemble()
        it, res, ini = o.solve(po.make_solver("jacobi", max_it=5000, restart=50,
                                              reduction=1e-12))
        assert res <= 1e-12 * ini
        errs.append(o.errors())
    for k, expected in ((0, rates[0]), (1, rates[1])):
        ratio = errs[0][k] / errs[1][k]
        assert 0.7 * expected < ratio < 1.35 * expected, (k, ratio, expected)


CASES = {
    # name: (dim, order, nref, levels, kwargs)
    "q1_quad_supg": (2, 1, 5, 3, dict(example=po.EX_SINE, eps=1e-2, b=(1.0, 0.5), c=0.5,
                                      supg=True, sdfem_type=2)),
    "q2_quad_supg_measure": (2, 2, 4, 3, dict(example=po.EX_SINE, eps=1e-3, b=(1.0, 0.25),
                                              c=0.0, supg=True, sdfem_type=2,
                                              cell_measure=1)),
    "q2_quad_galerkin": (2, 2, 4, 3, dict(example=po.EX_SINE, eps=0.05, b=(0.3, -0.7), c=1.0)),
    "q1_hex_galerkin": (3, 1, 3, 2, dict(example=po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2),
                                         c=0.5)),
    "q2_hex_galerkin": (3, 2, 2, 2, dict(example=po.EX_POLYEXP, eps=0.05, b=(S3, S3, S3),
                                         c=0.0)),
}


def params(kw):
    return pg.assembly_params(
        example=kw["example"], eps=kw["eps"], b=kw["b"], c=kw["c"],
        space_discretization_type="supg" if kw.get("supg") else "galerkin",
        sdfem_type=kw.get("sdfem_type", 2), cell_measure=kw.get("cell_measure", 0))


def build(name):
    dim, order, nref, levels, kw = CASES[name]
    h = pg.Hierarchy(dim, order, nref, n_levels=levels, perturb=0.2, seed=11)
    ok = {k: v for k, v in kw.items() if k != "example"}
    o = oracle_on(h, levels, dim, order, kw["example"], **ok)
    return h, o, levels, kw


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_multilinear_cells_against_oracle(ctx, name):
    h, o, levels, kw = build(name)
    o.assemble()
    gpu = pg.ConvectionDiffusion(ctx, h)
    a = params(kw)
    gpu.assemble(a)
    for lvl in range(levels):
        assert rel(gpu.matrix(lvl), o.matrix(lvl)) < 1e-12, lvl
        assert rel(gpu.rhs(lvl), o.rhs(lvl)) < 1e-12, lvl
    it_o, res_o, ini_o = o.solve(po.make_solver("multigrid", max_it=500, restart=30,
                                                reduction=1e-10, mg_levels=levels, n_pre=2,
                                                n_post=2, jacobi_damp=0.5))
    assert res_o <= 1e-10 * ini_o
    for prec in ("fp64", "mixed"):
        cd = pg.ConvectionDiffusion(ctx, h)
        cd.assemble(a)
        st = cd.solve(pg.solver_params("multigrid", precision=prec, max_n_iterations=500,
                                       gmres_restart=30, residual_tolerance=0.0,
                                       residual_reduction=1e-10, multigrid_n_levels=levels,
                                       multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                                       jacobi_damp=0.5))
        assert st.residual <= 1e-10 * st.initial_residual
        if prec == "fp64":
            assert abs(st.iterations - it_o) <= 1, (st.iterations, it_o)
        assert rel(cd.solution(), o.solution()) < 1e-8
        e, e_o = cd.errors(a), o.errors()
        for k in (0, 1):
            assert abs(e[k] - e_o[k]) <= 5e-4 * e_o[k]
        cd.close()
    gpu.close()


@pytest.mark.gpu
def test_multilinear_refusals(ctx):
    h = pg.Hierarchy(3, 1, 2, perturb=0.2, seed=1)
    cd = pg.ConvectionDiffusion(ctx, h)
    # SUPG on trilinear hexahedra needs second derivatives the reference
    # does not transform
    with pytest.raises(pg.CdgError) as e:
        cd.assemble(pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1, 0, 0),
                                       space_discretization_type="supg"))
    assert e.value.code == -1
    # the allocation-free norms map cells affinely
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1, 0, 0))
    cd.assemble(a)
    out = np.zeros(5)
    rc = pg.lib().cdg_problem_errors_noalloc(cd.p, ctypes.byref(a),
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == -1
    cd.close()
