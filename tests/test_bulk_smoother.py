"""FP32 smoothing and defect with the CSR stream staged through shared memory
(cp.async.bulk into per-warp double buffers) on levels of 65,536 active rows
or more.

The staged kernel gives every lane the same entries in the same order as the
register-streaming CSR kernel, so a multigrid cycle is bit-identical with
either kernel, for every chunk size; the mixed solve on a staged level reaches
the oracle's solution.
"""
import os

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu

CASES = {
    # name: (dim, order, nref, levels, tetra, roots) -- lanes per row 2, 4, 4, 8
    "q1_2d_n512": (2, 1, 9, 6, False, 1),
    "q2_2d_n256": (2, 2, 8, 5, False, 1),
    "p2_tet_24": (3, 2, 3, 4, True, 3),
    "q2_3d_n32": (3, 2, 5, 4, False, 1),
}


def problem(ctx, name, chunk):
    dim, order, nref, levels, tetra, roots = CASES[name]
    old = os.environ.get("CDG_BULK_CHUNK")
    os.environ["CDG_BULK_CHUNK"] = str(chunk)
    try:
        h = pg.Hierarchy(dim, order, nref, n_levels=levels, roots=roots, tetra=tetra)
        cd = pg.ConvectionDiffusion(ctx, h)
    finally:
        if old is None:
            del os.environ["CDG_BULK_CHUNK"]
        else:
            os.environ["CDG_BULK_CHUNK"] = old
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1.0, 0.5, 0.25)[:dim], c=0.5,
                           space_discretization_type="supg", sdfem_type=2)
    cd.assemble(a)
    return cd, levels


@pytest.mark.parametrize("name", list(CASES))
def test_staged_cycle_bit_identical(ctx, name, monkeypatch):
    # both kernels stream the CSR matrix with the default lanes per row: the
    # tuner (matrix-free operator, other lane counts) stays off
    monkeypatch.setenv("CDG_TUNE", "0")
    outs = []
    for chunk in (0, 256, 512, 1024):
        cd, levels = problem(ctx, name, chunk)
        v = np.random.default_rng(7).standard_normal(cd.info(0)["ndof"])
        s = pg.solver_params("multigrid", multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                             multigrid_n_post_smooth=2, jacobi_damp=0.5, precision="mixed")
        outs.append(cd.precondition(s, v))
    for z in outs[1:]:
        assert np.array_equal(z, outs[0])


def test_staged_mixed_solve_matches_oracle(ctx):
    cfg = po.make_config(2, 1, 9, po.EX_SINE, eps=1e-2, b=(1.0, 0.5), c=1.0)
    o = po.Problem(cfg, 6)
    o.assemble()
    it_o, res_o, ini_o = o.solve(po.make_solver("multigrid", max_it=300, restart=30,
                                                reduction=1e-10, mg_levels=6, n_pre=2, n_post=2,
                                                jacobi_damp=0.8))
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 9, n_levels=6))
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1.0, 0.5), c=1.0)
    cd.set_solution(None)
    cd.assemble(a)
    st = cd.solve(pg.solver_params("multigrid", max_n_iterations=300, gmres_restart=30,
                                   residual_tolerance=0.0, residual_reduction=1e-10,
                                   multigrid_n_levels=6, multigrid_n_pre_smooth=2,
                                   multigrid_n_post_smooth=2, jacobi_damp=0.8,
                                   precision="mixed"))
    assert st.residual <= 1e-10 * st.initial_residual * 1.0001
    x, xo = cd.solution(), o.solution()
    assert np.max(np.abs(x - xo)) <= 1e-8 * np.max(np.abs(xo))
