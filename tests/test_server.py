"""Request server (served form): admission, concurrency, eviction, and the
same result alone and in the mix.

Bars: each request's solution in a mix of concurrent requests equals its
solution when it runs alone to 1e-9 relative (FP64 atomics in the assembly
order entries differently between runs at round-off), with the same
iteration count +-1; a served solve equals the direct C-ABI solve of the same
problem and, for a small request, the oracle's solution to 1e-8.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po


def served_solver(levels=0):
    return pg.solver_params("multigrid", max_n_iterations=500, gmres_restart=30,
                            residual_tolerance=0.0, residual_reduction=1e-10,
                            multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                            multigrid_n_post_smooth=2, jacobi_damp=0.5, precision="mixed")


def coefficients(rng, dim):
    d = rng.standard_normal(dim)
    d /= np.linalg.norm(d)
    b = tuple(d * rng.uniform(0, 1))
    return pg.assembly_params(example=pg.EX_CONST_F, eps=10 ** rng.uniform(-4, 0), b=b,
                              c=rng.uniform(0, 1), space_discretization_type="supg",
                              sdfem_type=2)


MIX = [(2, 1, 16), (2, 2, 16), (2, 1, 32), (3, 1, 8), (3, 1, 12), (2, 2, 32), (2, 1, 48),
       (3, 1, 16), (2, 1, 16), (3, 1, 8), (2, 2, 16), (2, 1, 64)]


def mix_requests(seed=0):
    rng = np.random.default_rng(seed)
    return [pg.request(d, o, n, coefficients(rng, d), served_solver()) for d, o, n in MIX]


def test_request_ndof(built):
    a = pg.assembly_params()
    s = served_solver()
    assert pg.request_ndof(pg.request(2, 1, 16, a, s)) == 17 ** 2
    assert pg.request_ndof(pg.request(2, 2, 256, a, s)) == 513 ** 2
    assert pg.request_ndof(pg.request(3, 1, 48, a, s)) == 49 ** 3
    for bad in [(2, 1, 10), (2, 1, 5), (4, 1, 16), (2, 3, 16), (2, 1, 1)]:
        with pytest.raises(pg.CdgError) as e:
            pg.request_ndof(pg.request(*bad, a, s))
        assert e.value.code == -1


def test_server_needs_a_device(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pg.CdgError) as e:
        pg.Server(0, 2)
    assert e.value.code == -9


@pytest.mark.gpu
def test_same_result_alone_and_in_the_mix(ctx):
    reqs = mix_requests(0)
    # alone: one slot, one request at a time
    alone = pg.Server(0, n_slots=1)
    ref = []
    for r in reqs:
        res, x = alone.wait(alone.submit(r))
        assert res.status == 0
        assert res.stats.residual <= 1e-10 * res.stats.initial_residual * 1.0001
        ref.append((res.stats.iterations, x))
    alone.close()
    # in the mix: all submitted at once to four slots
    srv = pg.Server(0, n_slots=4)
    tickets = [srv.submit(r) for r in reqs]
    for t, (it, x_ref) in zip(tickets, ref):
        res, x = srv.wait(t)
        assert res.status == 0
        assert abs(res.stats.iterations - it) <= 1
        assert np.max(np.abs(x - x_ref)) <= 1e-9 * np.max(np.abs(x_ref))
    c = srv.counters()
    assert c["completed"] == len(reqs) and c["failed"] == 0
    assert c["peak_running"] >= 2          # work overlapped on the device
    srv.close()


@pytest.mark.gpu
def test_served_equals_direct_and_oracle(ctx):
    rng = np.random.default_rng(5)
    a = coefficients(rng, 2)
    s = served_solver(levels=3)
    srv = pg.Server(0, n_slots=2)
    res, x = srv.wait(srv.submit(pg.request(2, 2, 16, a, s)))
    srv.close()
    assert res.status == 0
    # direct C-ABI solve of the same problem
    cd = pg.ConvectionDiffusion(ctx, pg.Hierarchy(2, 2, 4, n_levels=3))
    cd.set_solution(None)
    cd.assemble(a)
    st = cd.solve(s)
    assert abs(st.iterations - res.stats.iterations) <= 1
    assert np.max(np.abs(cd.solution() - x)) <= 1e-9 * np.max(np.abs(x))
    # the oracle (FP64 multigrid) to the solver tolerance
    cfg = po.make_config(2, 2, 4, po.EX_CONST_F, eps=a.eps, b=tuple(a.b), c=a.c, supg=True,
                         sdfem_type=2)
    o = po.Problem(cfg, 3)
    o.assemble()
    o.solve(po.make_solver("multigrid", max_it=500, restart=30, reduction=1e-10, mg_levels=3,
                           n_pre=2, n_post=2, jacobi_damp=0.5))
    assert np.max(np.abs(o.solution() - x)) <= 1e-8 * np.max(np.abs(x))


@pytest.mark.gpu
def test_budget_admission_and_eviction(ctx):
    # a budget that holds about two of these instances: requests of four mesh
    # classes still all complete, by evicting idle instances
    reqs = []
    rng = np.random.default_rng(3)
    for rep in range(3):
        for d, o, n in [(2, 1, 64), (2, 2, 32), (3, 1, 16), (2, 1, 48)]:
            reqs.append(pg.request(d, o, n, coefficients(rng, d), served_solver()))
    alone = pg.Server(0, n_slots=1)
    ref = [alone.wait(alone.submit(r))[1] for r in reqs]
    alone.close()
    srv = pg.Server(0, n_slots=3, hbm_budget=24 << 20)
    tickets = [srv.submit(r) for r in reqs]
    for t, x_ref in zip(tickets, ref):
        res, x = srv.wait(t, timeout=120.0)
        assert res.status == 0
        assert np.max(np.abs(x - x_ref)) <= 1e-9 * np.max(np.abs(x_ref))
    c = srv.counters()
    assert c["completed"] == len(reqs) and c["failed"] == 0
    assert c["evictions"] > 0
    assert c["resident_bytes"] <= c["budget_bytes"]
    srv.close()


@pytest.mark.gpu
def test_small_requests_are_batched_per_launch(ctx, monkeypatch):
    # every request of the mix is small enough for the batched solver (cap
    # raised to its limit): with batching on they are solved in launches of
    # one block per request (the result's slot is n_slots), and each result
    # equals the same request served with batching off (every request on its
    # slot's stream)
    reqs = mix_requests(1)
    monkeypatch.setenv("CDG_SERVER_BATCH_DOFS", "20000")
    monkeypatch.setenv("CDG_SERVER_BATCH", "0")
    plain = pg.Server(0, n_slots=4)
    ref = [plain.wait(t) for t in [plain.submit(r) for r in reqs]]
    c = plain.counters()
    assert c["batching"] == 0 and c["batched"] == 0
    plain.close()
    monkeypatch.delenv("CDG_SERVER_BATCH")
    srv = pg.Server(0, n_slots=4)
    out = [srv.wait(t) for t in [srv.submit(r) for r in reqs]]
    c = srv.counters()
    assert c["batching"] == 1 and c["batched"] == len(reqs)
    assert 1 <= c["batch_launches"] <= len(reqs)
    assert c["completed"] == len(reqs) and c["failed"] == 0
    for (r0, x0), (r1, x1) in zip(ref, out):
        assert r0.status == 0 and r1.status == 0
        assert r1.slot == 4
        assert r1.stats.residual <= 1e-10 * r1.stats.initial_residual * 1.0001
        assert abs(r1.stats.iterations - r0.stats.iterations) <= 1
        assert np.max(np.abs(x1 - x0)) <= 1e-8 * np.max(np.abs(x0))
    srv.close()
