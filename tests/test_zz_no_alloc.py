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

ROT = ((0.0, -1.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0))


def _noalloc(cd, a):
    e = np.zeros(5)
    rc = pg.lib().cdg_problem_errors_noalloc(cd.p, ctypes.byref(a),
                                             e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return rc, e


@pytest.mark.parametrize("dim,order,nref,kw", [
    (2, 1, 6, dict(example=pg.EX_SINE, eps=1e-2, b=(1.0, 0.5), c=1.0)),
    (2, 2, 4, dict(example=pg.EX_SINE, eps=1e-3, b=(1.0, 0.5), c=0.5,
                   space_discretization_type="supg", sdfem_type=2)),
    (3, 2, 3, dict(example=pg.EX_POLYEXP, eps=1e-3, b=(0.57735, 0.57735, 0.57735),
                   space_discretization_type="supg", sdfem_type=5, cell_measure=2,
                   problem_linear=1)),
    # a convection field linear in x: b and delta change from point to point
    (2, 2, 4, dict(example=pg.EX_SINE, eps=1e-2, b=(0.5, -0.5), b_grad=ROT, c=0.5)),
    (3, 1, 3, dict(example=pg.EX_SINE, eps=1e-2, b=(0.5, -0.5, 0.2), b_grad=ROT, c=0.3)),
    # a time-dependent example at t = 0.3 (its exact solution depends on t)
    (2, 2, 4, dict(example=pg.EX_EXP_SIN, eps=1.0, b=(1.0, -1.0), c=1.0, t=0.3)),
])
def test_noalloc_errors_match_allocating_entry(ctx, dim, order, nref, kw):
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(dim, order, nref, n_levels=1))
    a = pg.assembly_params(**kw)
    cd.assemble(a)
    cd.solve(pg.solver_params("jacobi", max_n_iterations=300, gmres_restart=50,
                              residual_tolerance=0.0, residual_reduction=1e-8))
    want = cd.errors(a)
    for _ in range(2):   # two calls in a row share and reuse the scratch array
        rc, got = _noalloc(cd, a)
        assert rc == 0, pg.lib().cdg_last_error().decode()
        assert np.allclose(got, want, rtol=1e-12, atol=0.0), (got, want)
    cd.close()


def test_noalloc_leaves_device_memory_unchanged(ctx):
    torch = pytest.importorskip("torch")
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, 3, n_levels=1))
    a = pg.assembly_params(example=pg.EX_SINE, eps=1e-2, b=(1.0, 0.3, -0.2), c=0.5)
    cd.assemble(a)
    rc, _ = _noalloc(cd, a)        # first call on the device: the array's address
    assert rc == 0
    ctx.synchronize()
    free0 = torch.cuda.mem_get_info(ctx.device)[0]
    for _ in range(3):
        rc, _ = _noalloc(cd, a)
        assert rc == 0
    ctx.synchronize()
    assert torch.cuda.mem_get_info(ctx.device)[0] == free0
    cd.close()


def test_noalloc_rejects_what_the_allocating_entry_rejects(ctx):
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 3, n_levels=1))
    for bad in (dict(example=pg.EX_POLYEXP),             # a 3D example on a 2D problem
                dict(example=42),
                dict(example=pg.EX_SINE, time_discretization="crank_nicolson")):
        a = pg.assembly_params(**bad)
        if bad.get("time_discretization"):
            a.time_discretization = 7
        rc, _ = _noalloc(cd, a)
        e = np.zeros(5)
        rc_alloc = pg.lib().cdg_problem_errors(cd.p, ctypes.byref(a),
                                               e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert rc == rc_alloc == -1, (bad, rc, rc_alloc)
    cd.close()


def test_noalloc_rejects_levels_beyond_its_scratch(ctx):
    # 512 x 512 quadrilaterals = 262,144 cells > 131,072
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 9, n_levels=1))
    a = pg.assembly_params(example=pg.EX_SINE, eps=1.0)
    rc, _ = _noalloc(cd, a)
    assert rc == -10
    assert "131072" in pg.lib().cdg_last_error().decode()
    cd.close()
