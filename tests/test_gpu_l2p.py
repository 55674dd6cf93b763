"""SurfaceL2 of order 1..3 on the GPU against the FP64 oracle (the reference's tests use
SurfaceL2 order 3: tests/test_aca.py:9, tests/test_SLIntegration.py:29).

Dense FP64 operators within 1e-10 of the oracle's dense matrices; FP64 H-matrices within the
ACA tolerance of the oracle's H-matrices in both directions; mixed precision within 1e-6 of
FP64; the reference's ACA test pattern (dense vs ACA below eps, tests/test_aca.py:21-28);
potentials and mass matrices against the oracle.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import icosphere, ellipsoid

pytestmark = pytest.mark.gpu

KERNELS = [("laplace_sl", 0.0), ("laplace_dl", 0.0), ("helmholtz_sl", 3.0), ("helmholtz_dl", 3.0),
           ("helmholtz_cf", 4.0)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _op(kernel, kappa, mesh, p, method="aca", precision="fp64", **kw):
    sp = nb.SurfaceL2(mesh, order=p)
    prm = dict(intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    prm.update(kw)
    io = prm.pop("intorder")
    op = bem.IntegralOperator(kernel, kappa, sp, sp, "id", "id", io, prm.pop("leafsize"), prm.pop("eta"),
                              prm.pop("eps"), method, False, precision=precision, **prm)
    return op, sp


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("kernel,kappa", KERNELS, ids=[k for k, _ in KERNELS])
def test_dense_parity(oracle, kernel, kappa, p):
    m = icosphere(2 if p < 3 else 1)
    op, sp = _op(kernel, kappa, m, p, "dense", intorder_singular=4, intorder_regular=3)
    D = op.mat.to_dense()
    Do = oracle.dense_matrix(kernel, m, f"L2P{p}", kappa=kappa, intorder_singular=4, intorder_regular=3)
    assert D.shape == (sp.ndof, sp.ndof)
    assert rel(D, Do) < 1e-10


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("kernel,kappa", [("laplace_sl", 0.0), ("helmholtz_cf", 4.0)], ids=["laplace_sl", "helmholtz_cf"])
def test_hmatrix_parity(oracle, kernel, kappa, p):
    m = icosphere(3 if p < 3 else 2)
    op, sp = _op(kernel, kappa, m, p)
    H = oracle.OracleOperator(kernel, m, f"L2P{p}", kappa=kappa, intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    b, ob = op.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    cplx = kappa != 0.0
    rng = np.random.default_rng(7 + p)
    x = rng.standard_normal(sp.ndof) + (1j * rng.standard_normal(sp.ndof) if cplx else 0.0)
    dt = torch.complex128 if cplx else torch.float64
    xd = torch.from_numpy(x).to(dt).cuda()
    y = (op.mat * xd).cpu().numpy()
    assert rel(y, H.mult(x)) < 1e-7
    yt = op.mat.CreateRowVector()
    op.mat.MultTrans(xd, yt)
    assert rel(yt.cpu().numpy(), H.mult(x, trans=True)) < 1e-7


def test_mixed_against_fp64():
    m = icosphere(3)
    for kernel, kappa in [("laplace_sl", 0.0), ("helmholtz_sl", 3.0)]:
        o64, sp = _op(kernel, kappa, m, 3)
        o32, _ = _op(kernel, kappa, m, 3, precision="mixed")
        cplx = kappa != 0.0
        rng = np.random.default_rng(3)
        x = rng.standard_normal(sp.ndof) + (1j * rng.standard_normal(sp.ndof) if cplx else 0.0)
        xd = torch.from_numpy(x).to(torch.complex128 if cplx else torch.float64).cuda()
        y64 = (o64.mat * xd).cpu().numpy()
        y32 = (o32.mat * xd).cpu().numpy()
        assert rel(y32, y64) < 1e-6


def test_reference_aca_pattern():
    """tests/test_aca.py: SL with SurfaceL2 order 3, the ACA product within eps of the dense one."""
    m = ellipsoid(2, (1.0, 0.8, 0.6))
    eps = 1e-6
    Vd, sp = _op("laplace_sl", 0.0, m, 3, "dense", intorder=10)
    Va, _ = _op("laplace_sl", 0.0, m, 3, intorder=10, leafsize=40, eta=3.0, eps=eps)
    x = torch.from_numpy(np.random.default_rng(4711).standard_normal(sp.ndof)).cuda()
    yd, ya = Vd.mat * x, Va.mat * x
    assert (torch.linalg.vector_norm(yd - ya) / torch.linalg.vector_norm(yd)).item() < eps
    assert Va.mat.nze < Vd.mat.nze


@pytest.mark.parametrize("p", [1, 3])
def test_potential_and_mass(oracle, p):
    m = icosphere(2)
    op, sp = _op("laplace_sl", 0.0, m, p)
    dens = np.random.default_rng(11).standard_normal(sp.ndof)
    pts = np.array([[2.0, 0.3, -0.1], [0.1, 0.2, 0.3], [-1.5, 1.0, 0.5]])
    gf = torch.from_numpy(dens).cuda()
    val = op.GetPotential(gf)(pts).cpu().numpy().reshape(len(pts), -1)
    ref = oracle.potential("laplace_sl", m, f"L2P{p}", dens, pts, intorder=3).reshape(len(pts), -1)
    assert rel(val, ref) < 1e-11
    M = nb.MassOperator(sp, sp)
    x = torch.from_numpy(dens).cuda()
    y = (M * x).cpu().numpy()
    Mo = oracle.mass_matrix(m, f"L2P{p}", f"L2P{p}", order=max(4, 2 * p))
    assert rel(y, Mo @ dens) < 1e-12
