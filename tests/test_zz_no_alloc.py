"""The allocation-free error-norm entry point, through the C-ABI.

cdg_problem_errors_noalloc serves callers that may not allocate device
memory when they ask for the error norms (an application whose GPU memory
is handed out by its own pool, or a loop that must not call cudaMalloc /
cudaFree because they can synchronise the device).  It keeps its scratch in
a fixed device array instead.  This file is collected last so that a run
stopping at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

import parmoon2022_gb300 as pg

pytestmark = pytest.mark.gpu


def _noalloc(cd, a):
    e = np.zeros(5)
    rc = pg.lib().cdg_problem_errors_noalloc(cd.p, ctypes.byref(a),
                                             e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return rc, e


@pytest.mark.parametrize("dim,order,nref,example,eps,b,c,supg", [
    (2, 1, 6, pg.EX_SINE, 1e-2, (1.0, 0.5), 1.0, False),
    (2, 2, 4, pg.EX_SINE, 1e-3, (1.0, 0.5), 0.5, True),
    (3, 2, 3, pg.EX_POLYEXP, 1e-3, (0.57735, 0.57735, 0.57735), 0.0, True),
])
def test_noalloc_errors_match_allocating_entry(ctx, dim, order, nref, example, eps, b, c, supg):
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(dim, order, nref, n_levels=1))
    a = pg.assembly_params(example=example, eps=eps, b=b, c=c,
                           space_discretization_type="supg" if supg else "galerkin",
                           sdfem_type=2)
    cd.assemble(a)
    cd.solve(pg.solver_params("jacobi", max_n_iterations=300, gmres_restart=50,
                              residual_tolerance=0.0, residual_reduction=1e-8))
    want = cd.errors(a)
    for _ in range(2):   # two calls in a row share and reuse the scratch array
        rc, got = _noalloc(cd, a)
        assert rc == 0, pg.lib().cdg_last_error().decode()
        assert np.allclose(got, want, rtol=1e-12, atol=0.0), (got, want)
    cd.close()


def test_noalloc_rejects_levels_beyond_its_scratch(ctx):
    # 512 x 512 quadrilaterals = 262,144 cells > 131,072
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 9, n_levels=1))
    a = pg.assembly_params(example=pg.EX_SINE, eps=1.0)
    rc, _ = _noalloc(cd, a)
    assert rc == -10
    assert "131072" in pg.lib().cdg_last_error().decode()
    cd.close()
