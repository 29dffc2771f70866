"""Host setup layer of the library (no GPU): meshes, DOF numbering and CSR
patterns must equal the oracle's restatement of the reference's
ConstructSpace marker algorithm (src/FE/FESpace2D.C:83-312,
FESpace3D.C:186-420 for tetrahedra, FEMapper.C:456-600, FESpace.C:1863-2099)
and TStructure (src/Matrix/Structure.C:226-618) bit for bit, up to the
workloads' finest levels; the C-ABI library must load without a GPU and
export every symbol include/parmoon_cd.h declares."""
import ctypes
import os
import re

import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("dim,order,nref,nmask", [
    (2, 1, 3, 0), (2, 2, 3, 0), (2, 1, 2, 2), (2, 2, 3, 2), (2, 2, 4, 0b1010),
    (3, 1, 2, 0), (3, 2, 2, 0), (3, 2, 3, 0), (3, 1, 2, 4), (3, 2, 2, 0b100001),
])
def test_mesh_dofs_pattern_bit_exact(built, dim, order, nref, nmask):
    h = pg.Hierarchy(dim, order, nref, n_levels=2, neumann_mask=nmask)
    o = po.Problem(po.make_config(dim, order, nref, po.EX_SINE, neumann_mask=nmask), 2)
    for lvl in range(2):
        assert h.info(lvl)["ndof"] == o.info(lvl)["ndof"]
        assert h.info(lvl)["nactive"] == o.info(lvl)["nactive"]
        assert np.array_equal(h.mesh(lvl), o.mesh(lvl))
        assert np.array_equal(h.dofs(lvl), o.dofs(lvl) if hasattr(o, "dofs") else o.gdof(lvl))
        rp1, c1 = h.pattern(lvl)
        rp2, c2 = o.structure(lvl)
        assert np.array_equal(rp1, rp2) and np.array_equal(c1, c2)


@pytest.mark.parametrize("dim,order,nref", [(2, 1, 6), (3, 2, 5)])
def test_config_size_numbering_bit_exact(built, dim, order, nref):
    # the workloads' finest levels (64^2 Q1: 4,225 DOFs; 32^3 Q2: 274,625
    # DOFs, 16,974,593 entries) against the oracle's marker algorithm
    h = pg.Hierarchy(dim, order, nref, n_levels=1)
    o = po.Problem(po.make_config(dim, order, nref, po.EX_SINE), 1)
    assert h.info(0)["ndof"] == o.info(0)["ndof"]
    assert h.info(0)["nactive"] == o.info(0)["nactive"]
    assert np.array_equal(h.mesh(0), o.mesh(0))
    assert np.array_equal(h.dofs(0), o.dofs(0) if hasattr(o, "dofs") else o.gdof(0))
    rp1, c1 = h.pattern(0)
    rp2, c2 = o.structure(0)
    assert np.array_equal(rp1, rp2) and np.array_equal(c1, c2)


def _pattern(g, n):
    # TStructure: the union of the cells' couplings, full rows, sorted columns
    nl = g.shape[1]
    key = np.unique(np.repeat(g, nl, axis=1).ravel().astype(np.int64) * n +
                    np.tile(g, (1, nl)).ravel())
    rows = key // n
    rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int32)
    return rp, (key % n).astype(np.int32)


@pytest.mark.parametrize("order,nref,roots,mask,check_pattern", [
    (1, 3, 2, 0b100001, True), (2, 3, 3, 0, True), (2, 3, 1, 36, True),
    (2, 4, 3, 0, False)])
def test_tetrahedral_numbering_against_the_marker_algorithm(built, order, nref, roots, mask,
                                                             check_pattern):
    # Kuhn tetrahedra with the finest interior vertices moved; the last case
    # is the time-dependent workload's finest level (48^3 x 6 P2, 663,552
    # cells, 912,673 DOFs); the oracle numbers the product's mesh itself
    h = pg.Hierarchy(3, order, nref, n_levels=1, roots=roots, tetra=True, neumann_mask=mask,
                     perturb=0.2, seed=2024)
    cfg = po.make_config(3, order, 0, po.EX_SINE, tetra=True, neumann_mask=mask)
    g, nd, na = po.marker_numbering(cfg, h.mesh(0))
    assert (nd, na) == (h.info(0)["ndof"], h.info(0)["nactive"])
    assert np.array_equal(g, h.dofs(0))
    if check_pattern:
        rp, col = _pattern(g, nd)
        rp2, col2 = h.pattern(0)
        assert np.array_equal(rp, rp2) and np.array_equal(col, col2)


def test_config_sizes(built):
    # 64x64 Q1: 4225 DOFs, 3969 active, nnz (3N+1)^2 (configs' CD2D case)
    h = pg.Hierarchy(2, 1, 6)
    i = h.info()
    assert (i["ndof"], i["nactive"], i["nnz"]) == (4225, 3969, 193 ** 2)
    # 32^3 Q2: 274625 DOFs, nnz (8N+1)^3
    h = pg.Hierarchy(3, 2, 5)
    i = h.info()
    assert (i["ndof"], i["nnz"]) == (274625, 257 ** 3)


def test_root_grid_hierarchy(built):
    # 3 roots per direction refined twice: 12^3 cells, parent(f) = f // 8
    h = pg.Hierarchy(3, 1, 2, n_levels=3, roots=3)
    assert h.info(0)["ncells"] == 12 ** 3 and h.info(2)["ncells"] == 27
    fine, coarse = h.mesh(0), h.mesh(1)
    ctr_f = fine.mean(axis=1)
    lo, hi = coarse.min(axis=1), coarse.max(axis=1)
    par = np.arange(len(fine)) // 8
    assert np.all((ctr_f >= lo[par]) & (ctr_f <= hi[par]))


def test_abi_exports_every_declared_symbol(built):
    L = ctypes.CDLL(pg.LIB_PATH)
    hdr = open(os.path.join(ROOT, "include", "parmoon_cd.h")).read()
    declared = set(re.findall(r"^\s*(?:const char \*|int|long long)\s*(cdg_\w+)\(", hdr, re.M))
    assert declared == set(pg.EXPORTED)
    for name in declared:
        assert hasattr(L, name), name


def test_no_device_is_reported_not_faked(built):
    # without a GPU the library reports CDG_ERR_NO_DEVICE instead of running
    # anything on the CPU
    import subprocess
    code = ("import parmoon2022_gb300 as pg\n"
            "try:\n pg.Context(0)\nexcept pg.CdgError as e:\n print('ERR', e.code)\n"
            "else:\n print('OK')\n")
    out = subprocess.run(["python", "-c", code], capture_output=True, text=True, cwd=ROOT,
                         env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert "ERR -9" in out.stdout, out.stdout + out.stderr
