"""Grid transfers on nested uniform Q2 lattices.

GridTransfer::Prolongate / DefectRestriction (src/Multigrid/GridTransfer.C:
29-410) on a refined uniform Q2 hexahedral mesh is a tensor product of 1D
interpolations (a fine point takes the coarse node it sits on, or the Q2
basis at the quarter points of its coarse cell: 3/8, 3/4, -1/8), and the
restriction is its transpose.  Where both levels are such lattices (Dirichlet
data on the whole boundary), the multigrid and the transfer calls can gather
through the lattice maps instead of streaming the P and R matrices (an
option, CDG_LAT_TRANSFER=1: slower than the CSR kernels on GB300); every row
of P is checked against the lattice weights first.  Bars: the oracle's
transfers to 1e-13 relative (FP64; the sums run in another order), solves
within one iteration of the CSR transfers with the solutions to 1e-10 (FP64)
and 1e-8 (mixed); levels that are not lattices keep the CSR transfers.
"""
import numpy as np
import pytest

import parmoon2022_gb300 as pg
import pyoracle as po

pytestmark = pytest.mark.gpu

S3 = 0.57735026918962573
KW = dict(eps=1e-3, b=(S3, S3, S3), c=0.0, supg=True, sdfem_type=2)


def rel(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def params(kw):
    return pg.assembly_params(example=po.EX_POLYEXP, eps=kw["eps"], b=kw["b"], c=kw["c"],
                              space_discretization_type="supg" if kw.get("supg") else "galerkin",
                              sdfem_type=kw.get("sdfem_type", 2))


def sheared(ctx, nref, levels, kw):
    h = pg.Hierarchy(3, 2, nref, n_levels=levels)
    lv = []
    for l in range(levels):
        rp, col = h.pattern(l)
        i = h.info(l)
        v = h.mesh(l).copy()
        v[..., 0] += 0.3 * v[..., 1]
        lv.append(dict(verts=v, dofs=h.dofs(l), gdof=h.dofs(l), ndof=i["ndof"],
                       nactive=i["nactive"], row_ptr=rp, col=col))
    ok = {k: v for k, v in kw.items()}
    o = po.Problem(po.make_config(3, 2, 0, po.EX_POLYEXP, **ok), arrays=lv)
    return pg.ConvectionDiffusion.from_arrays(ctx, pg.CELL_HEXA, 2, lv), o


@pytest.mark.parametrize("shear", [False, True])
def test_lattice_transfers_against_the_oracle(ctx, monkeypatch, shear):
    monkeypatch.setenv("CDG_LAT_TRANSFER", "1")
    levels = 3
    if shear:
        gpu, o = sheared(ctx, 3, levels, KW)
    else:
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, 3, n_levels=levels))
        o = po.Problem(po.make_config(3, 2, 3, po.EX_POLYEXP, **KW), levels)
    gpu.assemble(params(KW))   # the lattices are found at the first assembly
    rng = np.random.default_rng(3)
    for fine in range(levels - 1):
        xc = rng.standard_normal(o.info(fine + 1)["ndof"])
        df = rng.standard_normal(o.info(fine)["ndof"])
        assert rel(gpu.prolongate(xc, fine), o.prolongate(xc, fine)) < 1e-13
        assert rel(gpu.restrict(df, fine), o.restrict(df, fine)) < 1e-13
        lat = gpu.lattice(fine)
        assert lat["transfer"] == 1, (fine, lat)
        assert all(d > 0 for d in lat["dims"])
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lattice_transfers_in_solves(ctx, monkeypatch, precision):
    levels = 4
    s = pg.solver_params("multigrid", precision=precision, max_n_iterations=300,
                         gmres_restart=30, residual_tolerance=0.0, residual_reduction=1e-10,
                         multigrid_n_levels=levels, multigrid_n_pre_smooth=2,
                         multigrid_n_post_smooth=2, jacobi_damp=0.8)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("CDG_LAT_TRANSFER", flag)
        gpu = pg.ConvectionDiffusion(ctx, pg.Hierarchy(3, 2, 4, n_levels=levels))
        gpu.assemble(params(KW))
        st = gpu.solve(s)
        assert st.residual <= 1e-10 * st.initial_residual
        out.append((st.iterations, gpu.solution(), [gpu.lattice(l)["transfer"]
                                                    for l in range(levels - 1)]))
        gpu.close()
    assert out[0][2] == [1] * (levels - 1) and out[1][2] == [-1] * (levels - 1)
    assert abs(out[0][0] - out[1][0]) <= 1
    assert rel(out[0][1], out[1][1]) < (1e-10 if precision == "fp64" else 1e-8)


def test_no_lattice_keeps_the_csr_transfers(ctx, monkeypatch):
    # Neumann faces (active boundary DOFs) and Q1 hexahedra: no lattice
    monkeypatch.setenv("CDG_LAT_TRANSFER", "1")
    for h, a in ((pg.Hierarchy(3, 2, 2, n_levels=2, neumann_mask=36),
                  pg.assembly_params(example=pg.EX_SINE, eps=0.1, b=(1.0, 0.3, -0.2), c=0.5,
                                     neumann_mask=36)),
                 (pg.Hierarchy(3, 1, 3, n_levels=2), params(KW))):
        gpu = pg.ConvectionDiffusion(ctx, h)
        gpu.assemble(a)
        xc = np.ones(gpu.info(1)["ndof"])
        gpu.prolongate(xc, 0)
        assert gpu.lattice(0)["transfer"] in (-1, 0)
        gpu.close()
