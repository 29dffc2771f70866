"""FE space numbering and TStructure built on the GPU.

Bar: bit-exact with the host setup layer (itself bit-exact with the oracle's
numbering and pattern): the same global DOF of every (cell, local DOF), the
same n_dof / n_active, the same row offsets and columns, on every level of
quadrilateral, hexahedral and tetrahedral hierarchies, with Neumann boundary
parts; a problem on a GPU-built hierarchy gives the same solution (same
iteration count, 1e-12 relative: the FP64 assembly's atomics sum entries in a
run-dependent order).
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg

pytestmark = pytest.mark.gpu

CASES = {
    # name: (dim, order, nref, n_levels, roots, neumann_mask, tetra, perturb)
    "q1_2d": (2, 1, 4, 3, 1, 0, False, 0.0),
    "q1_2d_neumann": (2, 1, 3, 2, 3, 2, False, 0.0),
    "q2_2d_neumann": (2, 2, 3, 2, 1, 5, False, 0.0),
    "q1_3d": (3, 1, 3, 2, 1, 0, False, 0.0),
    "q2_3d_roots3": (3, 2, 2, 2, 3, 0, False, 0.0),
    "q2_3d_neumann": (3, 2, 2, 2, 1, 33, False, 0.0),
    "p1_tet": (3, 1, 2, 2, 2, 0, True, 0.0),
    "p2_tet_perturbed": (3, 2, 2, 2, 1, 0, True, 0.2),
    "p1_tet_neumann": (3, 1, 2, 2, 2, 47, True, 0.0),
    "p2_tet_neumann_perturbed": (3, 2, 2, 2, 1, 36, True, 0.2),
}


def build(name, ctx=None):
    dim, order, nref, nl, roots, nmask, tetra, perturb = CASES[name]
    return pg.Hierarchy(dim, order, nref, n_levels=nl, roots=roots, neumann_mask=nmask,
                        tetra=tetra, perturb=perturb, seed=4, ctx=ctx)


def same_hierarchy(a, b, n_levels):
    for lvl in range(n_levels):
        assert a.info(lvl) == b.info(lvl), lvl
        assert np.array_equal(a.dofs(lvl), b.dofs(lvl)), lvl
        ra, ca = a.pattern(lvl)
        rb, cb = b.pattern(lvl)
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb), lvl
        assert np.array_equal(a.mesh(lvl), b.mesh(lvl)), lvl


@pytest.mark.parametrize("name", list(CASES))
def test_device_hierarchy_equals_host(ctx, name):
    same_hierarchy(build(name), build(name, ctx), CASES[name][3])


def test_device_entry_points(ctx):
    h = build("q2_3d_roots3")
    i = h.info(0)
    g, ndof, nactive = pg.space_number_device(ctx, pg.CELL_HEXA, 2, h.mesh(0))
    assert (ndof, nactive) == (i["ndof"], i["nactive"])
    assert np.array_equal(g, h.dofs(0))
    rp, col = pg.structure_build_device(ctx, h.dofs(0), ndof)
    rp_h, col_h = h.pattern(0)
    assert np.array_equal(rp, rp_h) and np.array_equal(col, col_h)
    # too small a column buffer: the offsets and the count, then CDG_ERR_LIMIT
    gd = np.ascontiguousarray(h.dofs(0), dtype=np.int32)
    rp2 = np.zeros(ndof + 1, dtype=np.int32)
    small = np.zeros(16, dtype=np.int32)
    nnz = pg.ctypes.c_longlong(0)
    rc = pg.lib().cdg_structure_build_device(ctx.c, gd.shape[0], gd.shape[1], ndof, pg._ip(gd),
                                             pg._ip(rp2), pg._ip(small), 16,
                                             pg.ctypes.byref(nnz))
    assert rc == -10 and nnz.value == len(col_h) and np.array_equal(rp2, rp_h)


def test_device_numbering_rejects_points_off_the_lattice(ctx):
    h = build("q1_2d")
    v = h.mesh(0).copy()
    v[5, 1, 0] = 1.5          # a vertex of the affine map outside the unit square
    with pytest.raises(pg.CdgError) as e:
        pg.space_number_device(ctx, pg.CELL_QUAD, 1, v)
    assert e.value.code == -1
    with pytest.raises(pg.CdgError) as e:
        g = h.dofs(0).copy()
        g[0, 0] = h.info(0)["ndof"]
        pg.structure_build_device(ctx, g, h.info(0)["ndof"])
    assert e.value.code == -1


def test_problem_on_device_hierarchy_solves_identically(ctx):
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1.0, 0.5, 0.25), c=1.0)
    s = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                         residual_tolerance=0.0, residual_reduction=1e-10, multigrid_n_levels=2,
                         multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.8,
                         precision="fp64")
    out = []
    for c in (None, ctx):
        cd = pg.ConvectionDiffusion(ctx, build("q1_3d", c))
        cd.set_solution(None)
        cd.assemble(a)
        st = cd.solve(s)
        out.append((st.iterations, cd.solution()))
    assert out[0][0] == out[1][0]
    assert np.max(np.abs(out[0][1] - out[1][1])) <= 1e-12 * np.max(np.abs(out[0][1]))


def test_large_hierarchy_bit_exact(ctx):
    # 32^3 Q2 hexahedra, four levels (274,625 DOFs, 16,974,593 entries) and
    # 663,552 P2 tetrahedra (912,673 DOFs)
    same_hierarchy(pg.Hierarchy(3, 2, 5, n_levels=4),
                   pg.Hierarchy(3, 2, 5, n_levels=4, ctx=ctx), 4)
    same_hierarchy(pg.Hierarchy(3, 2, 3, n_levels=2, roots=6, tetra=True, perturb=0.2, seed=1),
                   pg.Hierarchy(3, 2, 3, n_levels=2, roots=6, tetra=True, perturb=0.2, seed=1,
                                ctx=ctx), 2)
