"""Checkpoints in the reference's format (BlockVector::write_to_stream /
read_from_stream, CheckpointIO).

CPU: the file bytes are exactly a line with the entry count followed by the
raw doubles; reading accepts that and rejects what the reference rejects
(extra tokens on the count line, a count other than the expected one); the
CheckpointIO file name and step rules.  GPU: a Crank-Nicolson run restarted
from a checkpoint continues as the uninterrupted run (1e-12 relative).
"""
import os

import numpy as np
import pytest

import parmoon2022_gb300 as pg


def test_write_format_bytes(built, tmp_path):
    v = np.array([1.5, -2.25, 3e-300, np.pi])
    f = tmp_path / "sol"
    pg.write_vector(str(f), v)
    assert f.read_bytes() == b"4\n" + v.astype("<f8").tobytes()


def test_read_round_trip_and_reference_files(built, tmp_path):
    rng = np.random.default_rng(0)
    v = rng.standard_normal(1000)
    f = tmp_path / "a"
    pg.write_vector(str(f), v)
    assert np.array_equal(pg.read_vector(str(f), n=1000), v)
    assert np.array_equal(pg.read_vector(str(f)), v)          # empty target: any count
    # a file as the reference writes it, count line with trailing blanks too
    g = tmp_path / "b"
    g.write_bytes(b"3  \n" + np.array([7.0, 8.0, 9.0]).tobytes())
    assert np.array_equal(pg.read_vector(str(g), n=3), [7.0, 8.0, 9.0])
    z = tmp_path / "z"
    pg.write_vector(str(z), np.zeros(0))
    assert z.read_bytes() == b"0\n"
    assert pg.read_vector(str(z), capacity=4).size == 0


@pytest.mark.parametrize("content,n,code,msg", [
    (b"3 4\n" + bytes(24), 0, -1, "formatting error"),
    (b"5\n" + bytes(40), 3, -1, "unexpected size"),
    (b"abc\n", 3, -1, "unexpected size"),         # parses as 0 entries
    (b"4\n" + bytes(16), 4, -1, "ends after"),
])
def test_read_rejects(built, tmp_path, content, n, code, msg):
    f = tmp_path / "bad"
    f.write_bytes(content)
    with pytest.raises(pg.CdgError) as e:
        pg.read_vector(str(f), n=n, capacity=8)
    assert e.value.code == code and msg in str(e.value)


def test_read_limits_and_missing_file(built, tmp_path):
    f = tmp_path / "big"
    pg.write_vector(str(f), np.ones(10))
    with pytest.raises(pg.CdgError) as e:
        pg.read_vector(str(f), capacity=4)
    assert e.value.code == -10
    with pytest.raises(pg.CdgError) as e:
        pg.read_vector(str(tmp_path / "nope"), n=3)
    assert e.value.code == -1
    with pytest.raises(pg.CdgError) as e:
        pg.write_vector(str(tmp_path / "no_dir" / "x"), np.ones(2))
    assert e.value.code == -1


def test_checkpoint_file_names(built):
    assert pg.checkpoint_file_name("run/sol", 0.01) == "run/sol.0.010000"
    assert pg.checkpoint_file_name("sol", 1.5) == "sol.1.500000"
    assert pg.checkpoint_file_name("sol", 0.01, overwrite=True) == "sol"


@pytest.mark.gpu
def test_restart_from_checkpoint_continues_the_run(ctx, tmp_path):
    h = pg.Hierarchy(3, 2, 2, n_levels=2, roots=1, tetra=True, perturb=0.1, seed=3)
    a = lambda t: pg.assembly_params(example=pg.EX_POLY1_T, eps=1e-2, b=(0.6, -0.3, 0.2), c=0.5,
                                     t=t, space_discretization_type="supg", sdfem_type=2,
                                     time_step=0.05)
    s = pg.solver_params("multigrid", max_n_iterations=100, gmres_restart=30,
                         residual_tolerance=0.0, residual_reduction=1e-12, multigrid_n_levels=2,
                         multigrid_n_pre_smooth=2, multigrid_n_post_smooth=2, jacobi_damp=0.45,
                         precision="fp64")
    tau = 0.05
    base = str(tmp_path / "tcd")
    run = pg.ConvectionDiffusion(ctx, h)
    run.tcd_initialize(a(0.0))
    written = []
    for k in range(1, 5):
        run.tcd_step(a(k * tau), tau, s)
        if run.checkpoint(base, k, k * tau, every_n_steps=2):
            written.append(k)
    assert written == [2, 4]
    assert not run.checkpoint(base, 0, 0.0)              # never at the initial time
    final = run.solution()
    # restart at t = 2 tau from the step-2 checkpoint
    name = pg.checkpoint_file_name(base, 2 * tau)
    assert os.path.exists(name)
    again = pg.ConvectionDiffusion(ctx, h)
    again.tcd_initialize(a(2 * tau))
    again.read_solution(name)
    for k in (3, 4):
        again.tcd_step(a(k * tau), tau, s)
    assert np.max(np.abs(again.solution() - final)) <= 1e-12 * np.max(np.abs(final))
    # the step-4 file holds the final solution bit for bit
    assert np.array_equal(pg.read_vector(pg.checkpoint_file_name(base, 4 * tau),
                                         n=final.size), final)
