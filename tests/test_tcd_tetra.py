"""P2/P1 tetrahedra and the time-dependent problem (Crank-Nicolson).

CPU tests check the oracle on its own: quadrature on tetrahedra (the mass
matrix sums to the volume), known answers (a solution inside the FE space is
reproduced exactly, also through Crank-Nicolson steps, which are exact for a
solution linear in time), and the arrays constructor against the structured
one.  GPU tests compare the CUDA path with the oracle through the C-ABI:
matrices and rhs to 1e-12 relative, transfers to 1e-13, Crank-Nicolson
solutions to 1e-8 relative (same iteration count +-1).
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

B_ROT = (0.5, -0.5, 0.2)                      # b(x) = (-(y-1/2), x-1/2, 0.2)
B_ROT_GRAD = ((0.0, -1.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0))


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def hierarchy_levels(h):
    out = []
    for l in range(h.n_levels):
        rp, col = h.pattern(l)
        i = h.info(l)
        out.append(dict(verts=h.mesh(l), gdof=h.dofs(l), dofs=h.dofs(l), ndof=i["ndof"],
                        nactive=i["nactive"], row_ptr=rp, col=col))
    return out


def tet_oracle(h, order, example, **kw):
    cfg = po.make_config(3, order, 0, example, tetra=True, **kw)
    return po.Problem(cfg, arrays=hierarchy_levels(h))


def fgmres_jacobi(red=1e-12):
    return po.make_solver("jacobi", max_it=2000, restart=50, reduction=red)


# ---------------------------------------------------------------------------
# oracle on its own (CPU)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("order", [1, 2])
def test_oracle_tet_mass_sums_to_volume(built, order):
    h = pg.Hierarchy(3, order, 1, roots=2, tetra=True, perturb=0.2, seed=3)
    o = tet_oracle(h, order, po.EX_POLY1)
    o.tcd_initialize()
    assert abs(o.tcd_matrix(1).sum() - 1.0) < 1e-12


# the reference's tetrahedral rules by degree (QuadratureFormulaDatabase.C:30-37;
# QuadFormula.C:1693 P4Tetra, :1739 P5Tetra): Keast's symmetric rules, as
# orbits in barycentric coordinates (kind, a, b, weight per point)
KEAST = {
    2: [(4, 0.585410196624968454461376050311, 0.138196601125010515179541316563, 1 / 24)],
    4: [(1, 0.25, 0.25, -74 / 5625), (4, 11 / 14, 1 / 14, 343 / 45000),
        (6, 0.399403576166799204996102147462, 0.100596423833200795003897852538, 56 / 2250)],
    5: [(4, 0.0, 1 / 3, 0.602678571428571428571428571428571e-2),
        (1, 0.25, 0.25, 0.302836780970891758063769725577305e-1),
        (4, 8 / 11, 1 / 11, 0.116452490860289694108936091443380e-1),
        (6, 0.665501535736642982398804642263025e-1, 0.433449846426335701760119535773697,
         0.109491415613864593456430191124068e-1)],
}


def keast_points(deg):
    pts = []
    for kind, a, b, w in KEAST[deg]:
        if kind == 1:
            pts.append(((0.25,) * 4, w))
        for i in range(4):
            for j in range(i, 4):
                if (kind == 4 and j == i) or (kind == 6 and j > i):
                    l = [b] * 4
                    l[i] = l[j] = a
                    pts.append((tuple(l), w))
    return pts


@pytest.mark.parametrize("deg", [2, 4, 5])
def test_keast_rules_exact_to_their_degree(deg):
    from math import factorial
    pts = keast_points(deg)
    assert len(pts) == {2: 4, 4: 11, 5: 15}[deg]
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            for c in range(deg + 1 - a - b):
                q = sum(w * l[1] ** a * l[2] ** b * l[3] ** c for l, w in pts)
                exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 3)
                assert abs(q - exact) < 1e-15


@pytest.mark.parametrize("order,linear,deg", [(1, 1, 2), (1, 0, 4), (2, 1, 4), (2, 0, 5)])
def test_oracle_uses_the_reference_tet_rules(built, order, linear, deg):
    # one reference-shaped tetrahedron: physical = reference coordinates
    nl = 4 if order == 1 else 10
    lv = [dict(verts=np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]], dtype=float),
               gdof=np.arange(nl, dtype=np.int32)[None, :], ndof=nl, nactive=nl,
               row_ptr=np.arange(0, nl * nl + 1, nl, dtype=np.int32),
               col=np.tile(np.arange(nl, dtype=np.int32), nl))]
    o = po.Problem(po.make_config(3, order, 0, po.EX_SINE, tetra=True, problem_linear=linear),
                   arrays=lv)
    x = o.quadrature_points(0)[0]
    want = sorted(tuple(round(v, 12) for v in l[1:]) for l, _ in keast_points(deg))
    got = sorted(tuple(round(v, 12) for v in p) for p in x)
    assert got == want


def test_oracle_tet_p2_reproduces_linear_solution(built):
    # u = 1 + x + 2y + 3z lies in P2: Galerkin gives the interpolant
    h = pg.Hierarchy(3, 2, 1, roots=2, tetra=True, perturb=0.2, seed=5)
    o = tet_oracle(h, 2, po.EX_POLY1, eps=0.1, b=B_ROT, b_grad=B_ROT_GRAD, c=0.5)
    o.assemble()
    it, res, ini = o.solve(fgmres_jacobi())
    assert res <= 1e-12 * ini
    e = o.errors()
    assert e[0] < 1e-10 and e[1] < 1e-9


def test_oracle_crank_nicolson_exact_for_linear_in_time(built):
    # u = (1+t)(1 + x + 2y + 3z): in space inside P2, linear in time, so the
    # trapezoidal rule has no time error either
    h = pg.Hierarchy(3, 2, 1, roots=1, tetra=True, perturb=0.15, seed=1)
    o = tet_oracle(h, 2, po.EX_POLY1_T, eps=0.05, b=B_ROT, b_grad=B_ROT_GRAD, c=0.3)
    o.tcd_initialize()
    tau = 0.05
    for k in range(1, 4):
        it, res, ini = o.tcd_step(k * tau, tau, fgmres_jacobi())
        assert res <= 1e-12 * max(ini, 1e-300) or res < 1e-13
    e = o.errors()
    assert e[0] < 1e-10 and e[1] < 1e-9


@pytest.mark.parametrize("dim,order,sdfem_type", [(3, 2, 2), (3, 1, 5), (2, 2, 5), (2, 1, 0)])
def test_oracle_crank_nicolson_supg_exact_for_linear_in_time(built, dim, order, sdfem_type):
    # SUPG in time is consistent: with the same delta in the stiffness, mass
    # and rhs terms, a solution linear in space and time is reproduced
    tau = 0.05
    kw = dict(eps=1e-3, b=(1.0, -0.5, 0.3)[:dim], c=0.4, supg=True, sdfem_type=sdfem_type,
              time_step=tau)
    if dim == 3:
        h = pg.Hierarchy(3, order, 3 - order, roots=1, tetra=True, perturb=0.15, seed=2)
        o = tet_oracle(h, order, po.EX_POLY1_T, **kw)
    else:
        o = po.Problem(po.make_config(2, order, 3, po.EX_POLY1_T, **kw), 1)
    o.tcd_initialize()
    for k in range(1, 4):
        it, res, ini = o.tcd_step(k * tau, tau, fgmres_jacobi())
        assert res <= 1e-12 * max(ini, 1e-300) or res < 1e-13
    e = o.errors()
    assert e[0] < 1e-10 and e[1] < 1e-9


def test_oracle_tcd_supg_terms(built):
    # the SUPG mass term integrates delta (b . grad phi_i) phi_j: summed over
    # j (sum phi_j = 1) every row holds delta * int b . grad phi_i, and those
    # sum to zero over all i; SDFEM_TYPE 5 delta scales with theta1*tau
    cfg = dict(eps=1e-3, b=(1.0, 0.5), supg=True, sdfem_type=5)
    mats = []
    for tau in (0.01, 0.02):
        o = po.Problem(po.make_config(2, 1, 3, po.EX_SINE, time_step=tau, **cfg), 1)
        o.tcd_initialize()
        mats.append(o.tcd_matrix(1))
    g = po.Problem(po.make_config(2, 1, 3, po.EX_SINE, **dict(cfg, supg=False)), 1)
    g.tcd_initialize()
    m0 = g.tcd_matrix(1)
    s1, s2 = mats[0] - m0, mats[1] - m0
    assert np.max(np.abs(s1)) > 1e-8
    assert abs(s1.sum()) < 1e-14
    # h/(2|b|) >> the scaled eps: delta ~ (theta1 tau)^2 h/(2 theta1 tau |b|)
    # = theta1 tau h/(2|b|) up to the reaction term 1 in the scaled
    # reaction, so doubling tau doubles it up to that correction
    r = np.max(np.abs(s2)) / np.max(np.abs(s1))
    assert 1.5 < r < 2.05


def test_oracle_crank_nicolson_multigrid_converges(built):
    h = pg.Hierarchy(3, 2, 2, n_levels=3, roots=1, tetra=True, perturb=0.2, seed=4)
    o = tet_oracle(h, 2, po.EX_BUMP, eps=1e-4, b=B_ROT, b_grad=B_ROT_GRAD,
                   ic=(0.3, 0.5, 0.5, 0.1))
    o.tcd_initialize()
    _, s = mg_solver(3)
    for k in range(1, 3):
        it, res, ini = o.tcd_step(k * 1e-3, 1e-3, s)
        assert it < 40 and res <= 1e-10 * ini


def test_oracle_arrays_equal_structured(built):
    cfg = po.make_config(3, 2, 2, po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0)
    o1 = po.Problem(cfg, 2)
    levels = []
    for l in range(2):
        rp, col = o1.structure(l)
        i = o1.info(l)
        levels.append(dict(verts=o1.mesh(l), gdof=o1.gdof(l), ndof=i["ndof"],
                           nactive=i["nactive"], row_ptr=rp, col=col))
    o2 = po.Problem(cfg, arrays=levels)
    o1.assemble()
    o2.assemble()
    for l in range(2):
        assert np.array_equal(o1.matrix(l), o2.matrix(l))
        assert np.array_equal(o1.rhs(l), o2.rhs(l))
    xc = np.random.default_rng(0).standard_normal(o1.info(1)["ndof"])
    assert np.array_equal(o1.prolongate(xc), o2.prolongate(xc))


# ---------------------------------------------------------------------------
# CUDA path against the oracle (GPU)
# ---------------------------------------------------------------------------
TET_CASES = {
    # name: (order, nref, roots, perturb, kwargs)
    "p2_galerkin_linear_b": (2, 1, 2, 0.2, dict(example=po.EX_SINE, eps=1e-2, b=B_ROT,
                                                b_grad=B_ROT_GRAD, c=0.5)),
    "p2_supg": (2, 1, 2, 0.2, dict(example=po.EX_POLYEXP, eps=1e-4, b=(0.577, 0.577, 0.577),
                                   supg=True, sdfem_type=2, cell_measure=2)),
    "p1_galerkin": (1, 2, 1, 0.2, dict(example=po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0)),
}


def gpu_params(kw, t=0.0, ic=(0.5, 0.5, 0.5, 0.1)):
    return pg.assembly_params(
        example=kw["example"], eps=kw.get("eps", 1.0), b=kw.get("b", (0, 0, 0)),
        c=kw.get("c", 0.0), b_grad=kw.get("b_grad"), t=t, ic=ic,
        space_discretization_type="supg" if kw.get("supg") else "galerkin",
        sdfem_type=kw.get("sdfem_type", 2), cell_measure=kw.get("cell_measure", 0),
        time_step=kw.get("time_step", 0.0))


def oracle_kw(kw):
    return {k: v for k, v in kw.items() if k != "example"}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(TET_CASES))
def test_tet_assembly_parity(ctx, name):
    order, nref, roots, perturb, kw = TET_CASES[name]
    h = pg.Hierarchy(3, order, nref, n_levels=2, roots=roots, tetra=True, perturb=perturb,
                     seed=7)
    o = tet_oracle(h, order, kw["example"], **oracle_kw(kw))
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.assemble()
    gpu.assemble(gpu_params(kw))
    for l in range(2):
        assert rel(gpu.matrix(l), o.matrix(l)) < 1e-12, l
        assert rel(gpu.rhs(l), o.rhs(l)) < 1e-12, l


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_tet_transfer_parity(ctx, order):
    h = pg.Hierarchy(3, order, 2, n_levels=3, roots=1, tetra=True)
    o = tet_oracle(h, order, po.EX_SINE)
    gpu = pg.ConvectionDiffusion(ctx, h)
    rng = np.random.default_rng(11)
    for fine in range(2):
        xc = rng.standard_normal(h.info(fine + 1)["ndof"])
        df = rng.standard_normal(h.info(fine)["ndof"])
        assert rel(gpu.prolongate(xc, fine), o.prolongate(xc, fine)) < 1e-13
        assert rel(gpu.restrict(df, fine), o.restrict(df, fine)) < 1e-13


def mg_solver(levels, precision="fp64", damp=0.45):
    # omega 0.45: the Jacobi-scaled Crank-Nicolson system of P2 tetrahedra has
    # eigenvalues up to ~4.2 (mass dominated), damped Jacobi needs omega < 0.48
    g = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                         residual_tolerance=0.0, residual_reduction=1e-10,
                         multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                         multigrid_n_post_smooth=2, jacobi_damp=damp, precision=precision)
    o = po.make_solver("multigrid", max_it=100, restart=30, reduction=1e-10, mg_levels=levels,
                       n_pre=2, n_post=2, jacobi_damp=damp)
    return g, o


TAU = 1e-2
TCD_CASES = {
    # name: (dim, tetra, order, nref, levels, kwargs)
    "p2_tet_bump": (3, True, 2, 2, 3, dict(example=po.EX_BUMP, eps=1e-3, b=B_ROT,
                                           b_grad=B_ROT_GRAD)),
    "q2_hex_sine": (3, False, 2, 2, 2, dict(example=po.EX_SINE, eps=1e-2, b=(1.0, 0.3, -0.2),
                                            c=0.5)),
    # SUPG (TCDStiffSUPG, TCDMassSUPG, TCDRhsSUPG): SDFEM_TYPE 2 keeps the
    # unscaled delta, 5 and 0 take the theta1*tau-scaled coefficients in 2D
    # and delta *= theta1*tau
    "p2_tet_supg_t2": (3, True, 2, 2, 3, dict(example=po.EX_BUMP, eps=1e-4, b=(0.8, 0.3, 0.2),
                                              supg=True, sdfem_type=2, time_step=TAU)),
    "q2_hex_supg_t5": (3, False, 2, 2, 2, dict(example=po.EX_SINE, eps=1e-3, b=(1.0, 0.3, -0.2),
                                               c=0.5, supg=True, sdfem_type=5,
                                               time_step=TAU)),
    "q2_quad_supg_t5": (2, False, 2, 4, 3, dict(example=po.EX_POLY1_T, eps=1e-3, b=(1.0, 0.5),
                                                c=0.5, supg=True, sdfem_type=5,
                                                time_step=TAU)),
    "q1_quad_supg_t0": (2, False, 1, 5, 3, dict(example=po.EX_SINE, eps=1e-4, b=(-0.6, 0.8),
                                                supg=True, sdfem_type=0, time_step=TAU)),
}


def tcd_pair(ctx, name):
    dim, tetra, order, nref, levels, kw = TCD_CASES[name]
    ic = (0.4, 0.5, 0.6, 0.15)
    if tetra:
        h = pg.Hierarchy(3, order, nref, n_levels=levels, roots=1, tetra=True)
        o = tet_oracle(h, order, kw["example"], ic=ic, **oracle_kw(kw))
    else:
        h = pg.Hierarchy(dim, order, nref, n_levels=levels)
        cfg = po.make_config(dim, order, nref, kw["example"], ic=ic, **oracle_kw(kw))
        o = po.Problem(cfg, levels)
    gpu = pg.ConvectionDiffusion(ctx, h)
    return o, gpu, levels, kw, ic


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(TCD_CASES))
def test_tcd_matrices_and_steps_parity(ctx, name):
    o, gpu, levels, kw, ic = tcd_pair(ctx, name)
    tau = TAU
    o.tcd_initialize()
    gpu.tcd_initialize(gpu_params(kw, t=0.0, ic=ic))
    for l in range(levels):
        assert rel(gpu.tcd_matrix(0, l), o.tcd_matrix(0, l)) < 1e-12
        assert rel(gpu.tcd_matrix(1, l), o.tcd_matrix(1, l)) < 1e-12
    assert rel(gpu.solution(), o.solution()) < 1e-14
    gs, osv = mg_solver(levels)
    for k in range(1, 4):
        st = gpu.tcd_step(gpu_params(kw, t=k * tau, ic=ic), tau, gs)
        it_o, res_o, ini_o = o.tcd_step(k * tau, tau, osv)
        assert it_o < 100 and res_o <= 1e-10 * ini_o
        assert abs(st.iterations - it_o) <= 1
        assert rel(gpu.rhs(0), o.rhs(0)) < 1e-11
        assert rel(gpu.solution(), o.solution()) < 1e-8
    for l in range(levels):
        assert rel(gpu.tcd_matrix(1, l), o.tcd_matrix(1, l)) < 1e-12
        assert rel(gpu.tcd_matrix(2, l), o.tcd_matrix(2, l)) < 1e-12
    # the operator of the solver (sliced ELLPACK copy on the finest level):
    # the system matrix on active rows, identity rows where Dirichlet rows
    # hold assembled values
    rp, col = o.structure(0)
    na = o.info(0)["nactive"]
    S = gpu.tcd_matrix(2, 0)
    x = np.random.default_rng(2).standard_normal(len(rp) - 1)
    want = np.array([S[rp[r]:rp[r + 1]] @ x[col[rp[r]:rp[r + 1]]] for r in range(len(rp) - 1)])
    want[na:] = x[na:]
    assert rel(gpu.apply(x), want) < 1e-13


@pytest.mark.gpu
def test_tcd_supg_needs_time_step(ctx):
    o, gpu, levels, kw, ic = tcd_pair(ctx, "q1_quad_supg_t0")
    with pytest.raises(pg.CdgError) as e:
        gpu.tcd_initialize(gpu_params(dict(kw, time_step=0.0), ic=ic))
    assert e.value.code == -1


@pytest.mark.gpu
def test_tcd_mixed_precision_matches_fp64(ctx):
    o, gpu, levels, kw, ic = tcd_pair(ctx, "p2_tet_bump")
    tau = 1e-2
    o.tcd_initialize()
    gpu.tcd_initialize(gpu_params(kw, t=0.0, ic=ic))
    gs, osv = mg_solver(levels, precision="mixed")
    for k in range(1, 3):
        st = gpu.tcd_step(gpu_params(kw, t=k * tau, ic=ic), tau, gs)
        o.tcd_step(k * tau, tau, osv)
        assert st.iterations < 100
        assert st.residual <= 1e-10 * st.initial_residual * 1.0001
        assert rel(gpu.solution(), o.solution()) < 1e-7


@pytest.mark.gpu
def test_tcd_known_answer_on_perturbed_tets(ctx):
    h = pg.Hierarchy(3, 2, 2, n_levels=2, roots=1, tetra=True, perturb=0.2, seed=9)
    gpu = pg.ConvectionDiffusion(ctx, h)
    kw = dict(example=po.EX_POLY1_T, eps=0.05, b=B_ROT, b_grad=B_ROT_GRAD, c=0.3)
    gpu.tcd_initialize(gpu_params(kw))
    s = pg.solver_params("jacobi", max_n_iterations=1000, gmres_restart=50,
                         residual_tolerance=0.0, residual_reduction=1e-13)
    tau = 0.05
    for k in range(1, 4):
        gpu.tcd_step(gpu_params(kw, t=k * tau), tau, s)
    e = gpu.errors(gpu_params(kw, t=3 * tau))
    assert e[0] < 1e-10 and e[1] < 1e-9


@pytest.mark.gpu
def test_single_level_multigrid_is_the_coarse_solve(ctx):
    # multigrid_n_levels = 1: the cycle is the direct coarse solve on the
    # finest level, so FGMRES converges in one iteration on both sides
    h = pg.Hierarchy(3, 2, 1, n_levels=1, roots=1, tetra=True, perturb=0.1, seed=2)
    kw = dict(example=po.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0)
    o = tet_oracle(h, 2, kw["example"], **oracle_kw(kw))
    gpu = pg.ConvectionDiffusion(ctx, h)
    o.assemble()
    gpu.assemble(gpu_params(kw))
    gs, osv = mg_solver(1, damp=0.8)
    st = gpu.solve(gs)
    it_o, _, _ = o.solve(osv)
    assert st.iterations == it_o == 1
    assert rel(gpu.solution(), o.solution()) < 1e-10
