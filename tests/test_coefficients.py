"""Coefficients supplied by the caller, the reference's CoeffFct contract.

ParMooN examples built from callbacks (Example_CD2D/3D(exact, bc, bd, coeffs,
nu), include/Examples/Example_CD2D.h:67-71) hand LocalAssembling a
CoeffFct2D/3D(n_points, x, y[, z], params, coeffs)
(include/General/Constants.h:43-47) that fills eps, b, c, f at the quadrature
points of a cell.  Through the C-ABI the caller asks for the quadrature
points of a level (cdg_problem_quadrature_points), evaluates its function
there and passes the values (cdg_problem_assemble_coefficients).

CPU: the oracle's per-point assembly from caller values equals its assembly
from the example's own coefficients.  GPU, against the oracle on the same
field (each side evaluates it on its own points): matrices and rhs to 1e-12
relative, FP64 solves with the oracle's iteration count +-1 and solutions to
1e-8, mixed-precision multigrid solves to the same residual reduction, and
L2/H1 errors against the manufactured solution to 3 significant digits; the
per-point path with the built-in example's coefficients equals the
contraction path to 1e-12.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def variable_field(x):
    """eps, b, c varying in space; f from u = prod sin(pi x_i) for the form
    (eps grad u, grad v) + (b . grad u + c u, v) = (f, v)"""
    dim = x.shape[-1]
    s = np.sin(np.pi * x)
    cs = np.cos(np.pi * x)
    u = np.prod(s, axis=-1)
    grad = np.stack([np.pi * cs[..., a] * np.prod(np.delete(s, a, axis=-1), axis=-1)
                     for a in range(dim)], axis=-1)
    lap = -dim * np.pi ** 2 * u
    x0, x1 = x[..., 0], x[..., 1]
    z = x[..., 2] if dim == 3 else 0.0 * x0
    eps = 0.02 * (1 + x0 * x1) * (1 + 0.5 * z)
    deps = np.stack([0.02 * x1 * (1 + 0.5 * z), 0.02 * x0 * (1 + 0.5 * z)]
                    + ([0.01 * (1 + x0 * x1)] if dim == 3 else []), axis=-1)
    b = np.stack([1.0 + x[..., dim - 1], -0.5 + x0 ** 2] + ([0.3 + 0 * x0] if dim == 3 else []),
                 axis=-1)
    c = 0.5 + x0
    f = -(eps * lap + np.sum(deps * grad, axis=-1)) + np.sum(b * grad, axis=-1) + c * u
    return np.concatenate([eps[..., None], b, c[..., None], f[..., None]], axis=-1)


def example_field(x, eps, b, c, freq=1.0):
    """the built-in EX_SINE coefficients: constant eps, b, c and its f"""
    dim = x.shape[-1]
    k = freq * np.pi
    s, cs = np.sin(k * x), np.cos(k * x)
    u = np.prod(s, axis=-1)
    grad = np.stack([k * cs[..., a] * np.prod(np.delete(s, a, axis=-1), axis=-1)
                     for a in range(dim)], axis=-1)
    f = -eps * (-dim * k ** 2 * u) + np.sum(np.asarray(b[:dim]) * grad, axis=-1) + c * u
    ones = np.ones(x.shape[:-1])
    return np.concatenate([eps * ones[..., None],
                           np.broadcast_to(np.asarray(b[:dim]), x.shape[:-1] + (dim,)),
                           c * ones[..., None], f[..., None]], axis=-1)


@pytest.mark.parametrize("dim,order,nref,supg", [(2, 1, 3, False), (3, 2, 2, True)])
def test_oracle_coefficients_equal_example_assembly(built, dim, order, nref, supg):
    eps, b, c = 1e-2, (1.0, 0.5, -0.25), 0.5
    cfg = po.make_config(dim, order, nref, po.EX_SINE, eps=eps, b=b, c=c, supg=supg,
                         sdfem_type=2)
    o1 = po.Problem(cfg, 2)
    o1.assemble()
    o2 = po.Problem(cfg, 2)
    for lvl in range(2):
        o2.assemble_coefficients(lvl, example_field(o2.quadrature_points(lvl), eps, b, c))
        assert rel(o2.matrix(lvl), o1.matrix(lvl)) < 1e-13
        assert rel(o2.rhs(lvl), o1.rhs(lvl)) < 1e-13


CASES = {
    # name: (dim, order, nref, levels, tetra, supg)
    "q2_2d_galerkin": (2, 2, 4, 3, False, False),
    "q2_3d_supg": (3, 2, 2, 2, False, True),
    "p2_tet_galerkin": (3, 2, 2, 2, True, False),
}


def pair(ctx, name):
    dim, order, nref, levels, tetra, supg = CASES[name]
    kw = dict(supg=supg, sdfem_type=2)
    if tetra:
        h = pg.Hierarchy(3, order, nref, n_levels=levels, roots=1, tetra=True, perturb=0.15,
                         seed=3)
        lv = []
        for l in range(levels):
            rp, col = h.pattern(l)
            i = h.info(l)
            lv.append(dict(verts=h.mesh(l), gdof=h.dofs(l), ndof=i["ndof"], nactive=i["nactive"],
                           row_ptr=rp, col=col))
        o = po.Problem(po.make_config(3, order, 0, po.EX_SINE, tetra=True, **kw), arrays=lv)
    else:
        h = pg.Hierarchy(dim, order, nref, n_levels=levels)
        o = po.Problem(po.make_config(dim, order, nref, po.EX_SINE, **kw), levels)
    gpu = pg.ConvectionDiffusion(ctx, h)
    a = pg.assembly_params(example=pg.EX_SINE, space_discretization_type="supg" if supg
                           else "galerkin", sdfem_type=2)
    return gpu, o, a, levels


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_variable_coefficients_against_oracle(ctx, name):
    gpu, o, a, levels = pair(ctx, name)
    for lvl in range(levels):
        xg = gpu.quadrature_points(a, lvl)
        xo = o.quadrature_points(lvl)
        assert xg.shape == xo.shape
        gpu.assemble_coefficients(a, lvl, variable_field(xg))
        o.assemble_coefficients(lvl, variable_field(xo))
        assert rel(gpu.matrix(lvl), o.matrix(lvl)) < 1e-12, lvl
        assert rel(gpu.rhs(lvl), o.rhs(lvl)) < 1e-12, lvl
    it_o, res_o, ini_o = o.solve(po.make_solver("multigrid", max_it=500, restart=30,
                                                reduction=1e-10, mg_levels=levels, n_pre=2,
                                                n_post=2, jacobi_damp=0.8))
    assert res_o <= 1e-10 * ini_o
    x_o, e_o = o.solution(), o.errors()
    for prec in ("fp64", "mixed"):
        gpu.set_solution(np.where(np.arange(gpu.info(0)["ndof"]) < gpu.info(0)["nactive"], 0.0,
                                  gpu.rhs(0)))
        st = gpu.solve(pg.solver_params("multigrid", precision=prec, max_n_iterations=500,
                                        gmres_restart=30, residual_tolerance=0.0,
                                        residual_reduction=1e-10, multigrid_n_levels=levels,
                                        multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                                        jacobi_damp=0.8))
        assert st.residual <= 1e-10 * st.initial_residual
        if prec == "fp64":
            assert abs(st.iterations - it_o) <= 1, (st.iterations, it_o)
        assert rel(gpu.solution(), x_o) < 1e-8
        e = gpu.errors(a)
        for k in (0, 1):
            assert abs(e[k] - e_o[k]) <= 5e-4 * e_o[k], (prec, k, e[k], e_o[k])
    gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dim,order,nref,supg", [(2, 1, 4, False), (3, 2, 2, True)])
def test_per_point_path_equals_contraction(ctx, dim, order, nref, supg):
    eps, b, c = 1e-2, (1.0, 0.5, -0.25), 0.5
    a = pg.assembly_params(example=pg.EX_SINE, eps=eps, b=b[:dim], c=c,
                           space_discretization_type="supg" if supg else "galerkin",
                           sdfem_type=2)
    h = pg.Hierarchy(dim, order, nref, n_levels=1)
    g1 = pg.ConvectionDiffusion(ctx, h)
    g1.assemble(a)
    g2 = pg.ConvectionDiffusion(ctx, h)
    g2.assemble_coefficients(a, 0, example_field(g2.quadrature_points(a, 0), eps, b, c))
    assert rel(g2.matrix(0), g1.matrix(0)) < 1e-12
    assert rel(g2.rhs(0), g1.rhs(0)) < 1e-12
    g1.close()
    g2.close()


@pytest.mark.gpu
def test_coefficient_path_rejects_neumann_parts(ctx):
    h = pg.Hierarchy(2, 1, 3, neumann_mask=2)
    gpu = pg.ConvectionDiffusion(ctx, h)
    a = pg.assembly_params(example=pg.EX_SINE_LAPLACE, neumann_mask=2)
    x = gpu.quadrature_points(a, 0)
    with pytest.raises(pg.CdgError) as e:
        gpu.assemble_coefficients(a, 0, np.ones(x.shape[:-1] + (5,)))
    assert e.value.code == -1
    gpu.close()
