"""Many small solves in one launch (cdg_solve_batched): one block per request.

The batched solver runs the same FGMRES(m) + FP32 multigrid V-cycle as
cdg_problem_solve (Iteration_gmres.C:430-620 around Multigrid.C:157-410), with
every operation of a request inside one block.  Bars:

  * against the same request solved alone by the stream-level solver: the
    same 1e-10 residual reduction, iterations within one, the solution to
    1e-8 relative and the errors to 3 significant digits;
  * a request's result is the same, bit for bit, alone in a batch and in a
    mix of other requests (each block works only on its own instance);
  * ineligible parameters are rejected before anything runs.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg

pytestmark = pytest.mark.gpu

# (dim, order, nref, levels, eps, b, c)
REQS = [
    (2, 1, 4, 3, 1e-2, (0.6, 0.8), 0.5),
    (2, 2, 4, 3, 1e-3, (1.0, 0.2), 0.0),
    (3, 1, 3, 2, 1e-2, (0.5, -0.5, 0.7), 1.0),
    (2, 1, 5, 4, 1e-4, (-0.3, 0.9), 0.2),
    (3, 1, 4, 3, 0.5, (0.0, 0.0, 1.0), 0.0),
    (2, 2, 5, 4, 1e-2, (0.7, 0.7), 0.3),
]


def params(levels, precision="mixed", restart=30):
    return pg.solver_params("multigrid", precision=precision, max_n_iterations=500,
                            gmres_restart=restart, residual_tolerance=0.0,
                            residual_reduction=1e-10, multigrid_n_levels=levels,
                            multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2,
                            jacobi_damp=0.5)


def assembly(q):
    dim, order, nref, levels, eps, b, c = q
    return pg.assembly_params(example=pg.EX_CONST_F, eps=eps, b=b, c=c,
                              space_discretization_type="supg", sdfem_type=2)


def make(ctx, q):
    dim, order, nref, levels, *_ = q
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(dim, order, nref, n_levels=levels))
    cd.assemble(assembly(q))
    return cd


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def test_batched_equals_stream_solver(ctx):
    alone = []
    for q in REQS:
        cd = make(ctx, q)
        st = cd.solve(params(q[3]))
        alone.append((st.iterations, cd.solution(), cd.errors(assembly(q))))
        cd.close()
    probs = [make(ctx, q) for q in REQS]
    out = pg.solve_batched(ctx, probs, [params(q[3]) for q in REQS])
    for q, cd, (status, st), (it0, x0, e0) in zip(REQS, probs, out, alone):
        assert status == 0
        assert st.residual <= 1e-10 * st.initial_residual, q
        assert abs(st.iterations - it0) <= 1, (q, st.iterations, it0)
        x = cd.solution()
        assert rel(x, x0) < 1e-8, (q, rel(x, x0))
        e = cd.errors(assembly(q))
        for k in (0, 1):
            assert abs(e[k] - e0[k]) <= 5e-4 * e0[k]
    for cd in probs:
        cd.close()


def test_result_same_alone_and_in_the_mix(ctx):
    # the same assembled instances (two assemblies differ in round-off: the
    # FP64 element scatter adds with atomics), each restarted from its start
    # iterate
    probs = [make(ctx, q) for q in REQS]
    x0 = [p.solution() for p in probs]
    (s1, st1), = pg.solve_batched(ctx, [probs[1]], [params(REQS[1][3])])
    x_alone = probs[1].solution()
    for p, x in zip(probs, x0):
        p.set_solution(x)
    out = pg.solve_batched(ctx, probs, [params(q[3]) for q in REQS])
    s2, st2 = out[1]
    assert s1 == s2 == 0
    assert st1.iterations == st2.iterations
    assert st1.residual == st2.residual
    assert np.array_equal(probs[1].solution(), x_alone)
    for p in probs:
        p.close()


def test_restarts_in_the_batch(ctx):
    # a short restart length: the restart path (true residual, test on the
    # last estimate) against the stream solver
    q = REQS[3]
    cd = make(ctx, q)
    st = cd.solve(params(q[3], restart=5))
    x0 = cd.solution()
    cd.close()
    cd = make(ctx, q)
    (status, sb), = pg.solve_batched(ctx, [cd], [params(q[3], restart=5)])
    assert status == 0 and sb.residual <= 1e-10 * sb.initial_residual
    assert abs(sb.iterations - st.iterations) <= 1
    assert rel(cd.solution(), x0) < 1e-8
    cd.close()


def test_ineligible_requests_are_rejected(ctx):
    q = REQS[0]
    cd = make(ctx, q)
    with pytest.raises(pg.CdgError) as e:
        pg.solve_batched(ctx, [cd], [params(q[3], precision="fp64")])
    assert e.value.code == -1
    with pytest.raises(pg.CdgError) as e:
        pg.solve_batched(ctx, [cd, cd], [params(q[3])] * 2)
    assert e.value.code == -1
    cd.close()


def test_statuses_per_request(ctx):
    # a zero diagonal (eps = b = c = 0: the reference's Jacobi throws "zero
    # entry on the diagonal") ends that request with its status; the others
    # in the launch still solve
    good = make(ctx, REQS[0])
    zero = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 1, 4, n_levels=3))
    zero.assemble(pg.assembly_params(example=pg.EX_CONST_F, eps=0.0))
    out = pg.solve_batched(ctx, [good, zero], [params(3), params(3)])
    assert out[0][0] == 0 and out[0][1].residual <= 1e-10 * out[0][1].initial_residual
    assert out[1][0] == -6 and out[1][1].iterations == 0
    good.close()
    zero.close()


def test_batched_tetrahedra(ctx):
    # the batched solver is element-agnostic (CSR levels, transfers, coarse
    # inverse): P2 tetrahedra with moved vertices against the stream solver
    a = pg.assembly_params(example=pg.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=1.0)
    h = pg.Hierarchy(3, 2, 2, n_levels=2, tetra=True, perturb=0.15, seed=4)
    s = params(2)
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.assemble(a)
    st = cd.solve(s)
    x0 = cd.solution()
    cd.close()
    cd = pg.ConvectionDiffusion(ctx, h)
    cd.assemble(a)
    (status, sb), = pg.solve_batched(ctx, [cd], [s])
    assert status == 0 and sb.residual <= 1e-10 * sb.initial_residual
    assert abs(sb.iterations - st.iterations) <= 1
    assert rel(cd.solution(), x0) < 1e-8
    cd.close()
