"""The SUPG parameter types of Compute_SDFEM_delta (ConvDiff.C:269-495)
beyond the steady ones: 6 (Franca/Valentin), 9-11 (John/Novo, time step
dependent) and 12, the rejection of the types the reference throws on, and
CELL_MEASURE 4 (Mesh_size_in_convection_direction, ConvDiff.C:26-254).

CPU: on the unit cube of 4^3 equal cubes every cell has h_K = sqrt(3)/4
(CELL_MEASURE 0), so each type gives one delta for all cells.  A Python
restatement of the type's formula (with the time-dependent routines' rule:
coefficients unscaled in 3D, delta *= theta1 tau except for 2 and 9-12)
gives that delta, and a run with type 9 (delta = delta0 tau) and delta0 =
delta / tau must produce the same Crank-Nicolson system and mass matrices.
GPU: the CUDA path against the oracle for each type, stationary and
time-dependent, 2D and 3D; unknown types and the time-step types in the
stationary problem are rejected.
"""
import math

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

EPS, B, C, TAU, THETA1, D0 = 1e-2, (1.0, 0.5, 0.25), 0.5, 0.05, 0.5, 0.7


def expected_delta(ty, h):
    nb = math.sqrt(sum(b * b for b in B))
    if ty == 6:
        r = C if C >= 1e-20 else 1e20
        a1 = max(1.0, 6 * EPS / (h * h * r))
        a2 = max(1.0, h * nb / (3 * EPS))
        return D0 * h * h / (r * h * h * a1 + 6 * EPS * a2) * THETA1 * TAU
    if ty == 7:
        return D0 * h * h / (4 * EPS + 2 * h * nb + h * h * C) * THETA1 * TAU
    if ty == 10:
        eu = EPS / (THETA1 * TAU)
        return D0 * h if eu <= h else D0 * h * h / eu
    if ty == 11:
        return D0 * h * math.sqrt(TAU) / (nb / TAU)
    if ty == 12:
        return 100 * min(h / (2 * math.sqrt(3) * D0) * min(0.25, math.sqrt(3) * h / (8 * EPS * D0)),
                         1.0)
    raise ValueError(ty)


def oracle_tcd(ty, delta0):
    cfg = po.make_config(3, 1, 2, po.EX_SINE, eps=EPS, b=B, c=C, supg=True, sdfem_type=ty,
                         delta0=delta0, time_step=TAU)
    o = po.Problem(cfg, 1)
    o.tcd_initialize()
    o.tcd_step(TAU, TAU, po.make_solver("jacobi", max_it=500, restart=50, reduction=1e-10))
    return o.tcd_matrix(2, 0), o.tcd_matrix(1, 0)


@pytest.mark.parametrize("ty", [6, 7, 10, 11, 12])
def test_oracle_delta_formula(built, ty):
    d = expected_delta(ty, math.sqrt(3) / 4)
    S, M = oracle_tcd(ty, D0)
    S9, M9 = oracle_tcd(9, d / TAU)
    assert np.max(np.abs(S - S9)) <= 1e-13 * np.max(np.abs(S))
    assert np.max(np.abs(M - M9)) <= 1e-13 * np.max(np.abs(M))
    # and the stabilisation is on: type 9 with a tenth of the delta differs
    S9b, _ = oracle_tcd(9, 0.1 * d / TAU)
    assert np.max(np.abs(S - S9b)) > 1e-8 * np.max(np.abs(S))


@pytest.mark.parametrize("ty", [3, 13, 100])
def test_oracle_rejects_unknown_types(built, ty):
    o = po.Problem(po.make_config(2, 1, 2, po.EX_SINE, eps=EPS, b=B[:2], supg=True,
                                  sdfem_type=ty), 1)
    with pytest.raises(RuntimeError):
        o.assemble()


def test_oracle_time_step_types_need_the_time_dependent_problem(built):
    o = po.Problem(po.make_config(2, 1, 2, po.EX_SINE, eps=EPS, b=B[:2], supg=True,
                                  sdfem_type=10), 1)
    with pytest.raises(RuntimeError):
        o.assemble()


def rel(x, y):
    return float(np.max(np.abs(x - y)) / np.max(np.abs(y)))


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("ty", [6, 9, 10, 11, 12])
def test_cuda_tcd_types_match_oracle(ctx, dim, ty):
    b = B[:dim]
    cfg = po.make_config(dim, 2, 3 if dim == 2 else 2, po.EX_EXP_SIN, eps=EPS, b=b, c=C,
                         supg=True, sdfem_type=ty, delta0=D0, time_step=TAU)
    o = po.Problem(cfg, 2)
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(dim, 2, 3 if dim == 2 else 2, n_levels=2))
    a = lambda t: pg.assembly_params(example=pg.EX_EXP_SIN, eps=EPS, b=b, c=C, t=t,
                                     space_discretization_type="supg", sdfem_type=ty,
                                     delta0=D0, time_step=TAU)
    o.tcd_initialize()
    cd.tcd_initialize(a(0.0))
    osv = po.make_solver("multigrid", max_it=100, restart=30, reduction=1e-12, mg_levels=2,
                         n_pre=2, n_post=2, jacobi_damp=0.6)
    gs = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                          residual_tolerance=0.0, residual_reduction=1e-12, multigrid_n_levels=2,
                          multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.6,
                          precision="fp64")
    for k in (1, 2):
        o.tcd_step(k * TAU, TAU, osv)
        cd.tcd_step(a(k * TAU), TAU, gs)
        for which in (0, 1, 2):
            assert rel(cd.tcd_matrix(which, 0), o.tcd_matrix(which, 0)) < 1e-12, (k, which)
        assert rel(cd.solution(), o.solution()) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("ty", [6, 12])
def test_cuda_stationary_types_match_oracle(ctx, dim, ty):
    b = B[:dim]
    nref = 3 if dim == 2 else 2
    o = po.Problem(po.make_config(dim, 2, nref, po.EX_SINE, eps=EPS, b=b, c=C, supg=True,
                                  sdfem_type=ty, delta0=D0), 1)
    o.assemble()
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(dim, 2, nref))
    cd.assemble(pg.assembly_params(example=pg.EX_SINE, eps=EPS, b=b, c=C,
                                   space_discretization_type="supg", sdfem_type=ty, delta0=D0))
    assert rel(cd.matrix(0), o.matrix(0)) < 1e-12
    assert rel(cd.rhs(0), o.rhs(0)) < 1e-12


@pytest.mark.gpu
def test_cuda_rejects_unknown_and_stationary_time_step_types(ctx):
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 2))
    for ty in (3, 13, 100, 9, 10, 11):
        with pytest.raises(pg.CdgError) as e:
            cd.assemble(pg.assembly_params(example=pg.EX_SINE, eps=EPS, b=B[:2],
                                           space_discretization_type="supg", sdfem_type=ty))
        assert e.value.code == -1
    # Galerkin ignores the type
    cd.assemble(pg.assembly_params(example=pg.EX_SINE, eps=EPS, b=B[:2], sdfem_type=3))


# ---------------------------------------------------------------------------
# CELL_MEASURE 4: mesh size in convection direction (ConvDiff.C:26-254)
# ---------------------------------------------------------------------------
def stationary_matrix(dim, order, measure, b, ty=2, delta0=1.0):
    o = po.Problem(po.make_config(dim, order, 2, po.EX_SINE, eps=EPS, b=b, c=C, supg=True,
                                  sdfem_type=ty, cell_measure=measure, delta0=delta0), 1)
    o.assemble()
    return o.matrix(0)


def same(A, B):
    return np.max(np.abs(A - B)) <= 1e-13 * np.max(np.abs(B))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("ty", [2, 7])
def test_oracle_convection_size_known_answers(built, dim, ty):
    # cells of side s: for b along x the size in convection direction is the
    # edge s (CELL_MEASURE 2); for b along the diagonal it is the diameter
    # sqrt(2) s in 2D (CELL_MEASURE 0), and 2 s / sqrt(3) = 2/3 of the diameter
    # in 3D, which SDFEM type 0 (delta = delta0 h / |b| here) turns into a
    # factor 2/3 on delta0
    axis = tuple([0.9] + [0.0] * (dim - 1))
    assert same(stationary_matrix(dim, 1, 4, axis, ty), stationary_matrix(dim, 1, 2, axis, ty))
    diag = tuple([0.6] * dim)
    if dim == 2:
        assert same(stationary_matrix(2, 1, 4, diag, ty), stationary_matrix(2, 1, 0, diag, ty))
    else:
        assert same(stationary_matrix(3, 1, 4, diag, 0, 0.9),
                    stationary_matrix(3, 1, 0, diag, 0, 0.9 * 2 / 3))
    # and differs from both for another direction
    b = (0.9, 0.4, 0.2)[:dim]
    A4 = stationary_matrix(dim, 1, 4, b, ty)
    assert np.max(np.abs(A4 - stationary_matrix(dim, 1, 0, b, ty))) > 1e-10
    assert np.max(np.abs(A4 - stationary_matrix(dim, 1, 2, b, ty))) > 1e-10


@pytest.mark.gpu
def test_cuda_convection_size_matches_oracle(ctx):
    b3 = (0.9, 0.4, 0.2)
    # perturbed P2 tetrahedra (irregular cells), stationary
    h = pg.Hierarchy(3, 2, 2, tetra=True, perturb=0.2, seed=9)
    lv = []
    for lvl in range(h.n_levels):
        rp, col = h.pattern(lvl)
        i = h.info(lvl)
        lv.append(dict(verts=h.mesh(lvl), gdof=h.dofs(lvl), ndof=i["ndof"],
                       nactive=i["nactive"], row_ptr=rp, col=col))
    o = po.Problem(po.make_config(3, 2, 0, po.EX_SINE, eps=EPS, b=b3, c=C, supg=True,
                                  sdfem_type=2, cell_measure=4, tetra=True), arrays=lv)
    o.assemble()
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.assemble(pg.assembly_params(example=pg.EX_SINE, eps=EPS, b=b3, c=C,
                                   space_discretization_type="supg", sdfem_type=2,
                                   cell_measure=4))
    assert rel(cd.matrix(0), o.matrix(0)) < 1e-12
    assert rel(cd.rhs(0), o.rhs(0)) < 1e-12
    # quadrilaterals, time-dependent (type 5, coefficients scaled by theta1 tau)
    cfg = po.make_config(2, 2, 3, po.EX_EXP_SIN, eps=EPS, b=b3[:2], c=C, supg=True,
                         sdfem_type=5, cell_measure=4, time_step=TAU)
    o2 = po.Problem(cfg, 1)
    cd2 = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 2, 3))
    a = lambda t: pg.assembly_params(example=pg.EX_EXP_SIN, eps=EPS, b=b3[:2], c=C, t=t,
                                     space_discretization_type="supg", sdfem_type=5,
                                     cell_measure=4, time_step=TAU)
    o2.tcd_initialize()
    cd2.tcd_initialize(a(0.0))
    o2.tcd_step(TAU, TAU, po.make_solver("jacobi", max_it=500, restart=50, reduction=1e-12))
    cd2.tcd_step(a(TAU), TAU, pg.solver_params("jacobi", max_n_iterations=500, gmres_restart=50,
                                               residual_tolerance=0.0, residual_reduction=1e-12))
    for which in (0, 1, 2):
        assert rel(cd2.tcd_matrix(which, 0), o2.tcd_matrix(which, 0)) < 1e-12


def test_oracle_convection_size_kuhn_tetrahedra(built):
    # on unperturbed Kuhn tetrahedra (cube side s) the P1 vertex gradients
    # give h = s for b along x (the shortest edge, CELL_MEASURE 2) and
    # h = sqrt(3) s for b along the cube diagonal (the longest edge, the
    # diameter, CELL_MEASURE 0) in every one of the six orientations
    h = pg.Hierarchy(3, 1, 2, tetra=True)
    lv = []
    for lvl in range(h.n_levels):
        rp, col = h.pattern(lvl)
        i = h.info(lvl)
        lv.append(dict(verts=h.mesh(lvl), gdof=h.dofs(lvl), ndof=i["ndof"],
                       nactive=i["nactive"], row_ptr=rp, col=col))

    def mat(measure, b):
        o = po.Problem(po.make_config(3, 1, 0, po.EX_SINE, eps=EPS, b=b, c=C, supg=True,
                                      sdfem_type=2, cell_measure=measure, tetra=True), arrays=lv)
        o.assemble()
        return o.matrix(0)

    assert same(mat(4, (0.9, 0.0, 0.0)), mat(2, (0.9, 0.0, 0.0)))
    assert same(mat(4, (0.6, 0.6, 0.6)), mat(0, (0.6, 0.6, 0.6)))
    assert np.max(np.abs(mat(4, (0.9, 0.4, 0.2)) - mat(0, (0.9, 0.4, 0.2)))) > 1e-10


def expected_delta_2d(ty, h):
    # the 2D time-dependent routines scale the coefficients by theta1 tau
    # first (reaction 1 + theta1 tau c), except for types 2 and 12
    b = B[:2]
    tt = THETA1 * TAU
    nb = math.sqrt(sum(x * x for x in b))
    es, nbs, rs = tt * EPS, tt * nb, 1.0 + tt * C
    if ty == 6:
        a1 = max(1.0, 6 * es / (h * h * rs))
        a2 = max(1.0, h * nbs / (3 * es))
        return D0 * h * h / (rs * h * h * a1 + 6 * es * a2) * tt
    if ty == 7:
        return D0 * h * h / (4 * es + 2 * h * nbs + h * h * rs) * tt
    if ty == 10:
        eu = es / tt
        return D0 * h if eu <= h else D0 * h * h / eu
    if ty == 11:
        return D0 * h * math.sqrt(TAU) / (nbs / TAU)
    if ty == 12:
        return 100 * min(h / (2 * math.sqrt(3) * D0) * min(0.25, math.sqrt(3) * h / (8 * EPS * D0)),
                         1.0)
    raise ValueError(ty)


def oracle_tcd_2d(ty, delta0):
    cfg = po.make_config(2, 1, 2, po.EX_SINE, eps=EPS, b=B[:2], c=C, supg=True, sdfem_type=ty,
                         delta0=delta0, time_step=TAU)
    o = po.Problem(cfg, 1)
    o.tcd_initialize()
    o.tcd_step(TAU, TAU, po.make_solver("jacobi", max_it=500, restart=50, reduction=1e-10))
    return o.tcd_matrix(2, 0), o.tcd_matrix(1, 0)


@pytest.mark.parametrize("ty", [6, 7, 10, 11, 12])
def test_oracle_delta_formula_2d_scaled_coefficients(built, ty):
    d = expected_delta_2d(ty, math.sqrt(2) / 4)
    S, M = oracle_tcd_2d(ty, D0)
    S9, M9 = oracle_tcd_2d(9, d / TAU)
    assert np.max(np.abs(S - S9)) <= 1e-13 * np.max(np.abs(S))
    assert np.max(np.abs(M - M9)) <= 1e-13 * np.max(np.abs(M))
