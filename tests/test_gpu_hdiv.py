"""HDivSurface of order 1 and 2 on the GPU against the FP64 oracle (the reference's Maxwell
tests use higher-order HDivSurface: tests/test_Maxwell_Mie.py:24, with Curve(order)).

* The Maxwell single layer (DiffOpMaxwellNew traces, src/diffops.hpp:263-338): dense FP64
  within 1e-10 of the oracle on flat and curved meshes; its block on the lowest-order dofs is
  the RT0 operator.
* H-matrices within the ACA tolerance of the oracle's in both directions with the same block
  lists; mixed precision within 1e-6 of FP64.
* Potentials and mass matrices against the oracle.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import ellipsoid, icosphere

pytestmark = pytest.mark.gpu

KAPPA = 2.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _op(sp, method="aca", precision="fp64", **kw):
    prm = dict(intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    prm.update(kw)
    io = prm.pop("intorder")
    return bem.IntegralOperator("maxwell_sl", KAPPA, sp, sp, "maxwell", "maxwell", io, prm.pop("leafsize"),
                                prm.pop("eta"), prm.pop("eps"), method, False, precision=precision, **prm)


@pytest.mark.parametrize("g", [1, 3])
@pytest.mark.parametrize("K", [1, 2])
def test_dense_parity(oracle, K, g):
    m = icosphere(1).Curve(g)
    sp = nb.HDivSurface(m, order=K, complex=True)
    D = _op(sp, "dense", intorder_singular=4, intorder_regular=3).mat.to_dense()
    Do = oracle.dense_matrix("maxwell_sl", m, f"HDIV{K}", kappa=KAPPA, trial_eval="maxwell", intorder_singular=4,
                             intorder_regular=3)
    assert D.shape == (sp.ndof, sp.ndof)
    assert rel(D, Do) < 1e-10
    # the lowest-order dofs carry the RT0 functions with RT0's numbering
    rt = nb.HDivSurface(m, order=0, complex=True)
    R = _op(rt, "dense", intorder_singular=4, intorder_regular=3).mat.to_dense()
    assert rel(D[: rt.ndof, : rt.ndof], R) < 1e-12


@pytest.mark.parametrize("K", [1, 2])
def test_hmatrix_parity(oracle, K):
    m = ellipsoid(3 if K == 1 else 2, (1.0, 0.8, 0.6)).Curve(2)
    kind = f"HDIV{K}"
    sp = nb.HDivSurface(m, order=K, complex=True)
    op = _op(sp)
    H = oracle.OracleOperator("maxwell_sl", m, kind, kappa=KAPPA, trial_eval="maxwell", intorder=3, leafsize=40,
                              eta=2.0, eps=1e-8)
    b, ob = op.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    rng = np.random.default_rng(31 + K)
    x = rng.standard_normal(sp.ndof) + 1j * rng.standard_normal(sp.ndof)
    xd = torch.from_numpy(x).cuda()
    y = (op.mat * xd).cpu().numpy()
    assert rel(y, H.mult(x)) < 1e-7
    yt = op.mat.CreateRowVector()
    op.mat.MultTrans(xd, yt)
    assert rel(yt.cpu().numpy(), H.mult(x, trans=True)) < 1e-7
    y32 = (_op(sp, precision="mixed").mat * xd).cpu().numpy()
    assert rel(y32, y) < 1e-6


@pytest.mark.parametrize("K", [1, 2])
def test_potential_and_mass(oracle, K):
    m = icosphere(2).Curve(3)
    kind = f"HDIV{K}"
    sp = nb.HDivSurface(m, order=K, complex=True)
    rng = np.random.default_rng(5)
    dens = rng.standard_normal(sp.ndof) + 1j * rng.standard_normal(sp.ndof)
    pts = np.array([[2.0, 0.3, -0.1], [0.1, 0.2, 0.3], [-1.5, 1.0, 0.5]])
    op = _op(sp)
    val = op.GetPotential(torch.from_numpy(dens).cuda())(pts).cpu().numpy().reshape(len(pts), -1)
    ref = oracle.potential("maxwell_sl", m, kind, dens, pts, kappa=KAPPA, trial_eval="maxwell",
                           intorder=3).reshape(len(pts), -1)
    assert rel(val, ref) < 1e-11
    M = nb.MassOperator(sp, sp)
    x = rng.standard_normal(sp.ndof)
    y = (M * torch.from_numpy(x).to(torch.complex128 if M.is_complex else torch.float64).cuda()).cpu().numpy()
    assert rel(y, oracle.mass_matrix(m, kind, kind, order=4) @ x) < 1e-12
