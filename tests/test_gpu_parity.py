"""GPU parity: the CUDA path through the C-ABI against the FP64 oracle on the same inputs.

Tolerances: dense FP64 path 1e-10 relative (Frobenius); FP64 H-matrix vs the oracle's
H-matrix within the ACA tolerance (pivots may differ at rounding level); mixed precision
within 1e-6 of the FP64 GPU path.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import icosphere, ellipsoid

pytestmark = pytest.mark.gpu

CASES = [
    ("laplace_sl", "P0", "P0", "id", "id", 0.0),
    ("laplace_sl", "P1", "P1", "id", "id", 0.0),
    ("laplace_sl", "P1", "P0", "id", "id", 0.0),
    ("laplace_dl", "P1", "P0", "id", "id", 0.0),
    ("laplace_dl", "P0", "P1", "id", "id", 0.0),
    ("laplace_hs", "P1", "P1", "rot", "rot", 0.0),
    ("helmholtz_sl", "P0", "P0", "id", "id", 3.0),
    ("helmholtz_dl", "P1", "P1", "id", "id", 3.0),
    ("helmholtz_cf", "P1", "P1", "id", "id", 5.0),
    ("helmholtz_hs", "P1", "P1", "helm", "helm", 3.0),
    ("maxwell_sl", "RT0", "RT0", "maxwell", "maxwell", 2.0),
    ("helmholtz_sl_dkappa", "P1", "P0", "id", "id", 3.0),
    ("maxwell_dl", "HCURL", "RT0", "rotatedtrace", "id", 2.0),
    ("maxwell_dl", "HCURL", "HCURL", "rotatedtrace", "id", 2.0),
    ("maxwell_sl", "HCURL", "HCURL", "maxwellcurl", "maxwellcurl", 2.0),
]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _op(case, mesh, method="aca", **kw):
    k, tr, te, e1, e2, kap = case
    trs = nb.TraceSpace(mesh, tr)
    tes = trs if te == tr else nb.TraceSpace(mesh, te)
    p = dict(intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    p.update(kw)
    io = p.pop("intorder")
    op = bem.IntegralOperator(k, kap, trs, tes, e1, e2, io, p.pop("leafsize"), p.pop("eta"), p.pop("eps"), method,
                              False, **p)
    return op, trs, tes


def _vec(n, cplx, seed):
    r = np.random.default_rng(seed)
    x = r.standard_normal(n)
    return x + 1j * r.standard_normal(n) if cplx else x


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}{c[2]}" for c in CASES])
def test_dense_parity(oracle, case):
    m = icosphere(2)
    op, trs, tes = _op(case, m, "dense", intorder_singular=4, intorder_regular=3)
    Dg = op.mat.to_dense()
    k, tr, te, e1, e2, kap = case
    Do = oracle.dense_matrix(k, m, tr, te, kappa=kap, trial_eval=e1, test_eval=e2, intorder_singular=4,
                             intorder_regular=3)
    assert rel(Dg, Do) < 1e-10


def test_config1_dense_laplace_sl_l3(oracle):
    """Laplace SL dense FP64, icosphere L3 (1280 triangles), P0, SS order 4, regular order 3."""
    m = icosphere(3)
    fes = nb.SurfaceL2(m)
    V = nb.SingleLayerPotentialOperator(fes, method="dense", intorder_singular=4, intorder_regular=3)
    x = np.random.default_rng(20261203).standard_normal(fes.ndof)
    y = (V.mat * torch.from_numpy(x).cuda()).cpu().numpy()
    D = oracle.dense_matrix("laplace_sl", m, "P0", intorder_singular=4, intorder_regular=3)
    assert rel(y, D @ x) < 1e-10
    assert V.mat.info["nblocks"] == 1 and V.mat.info["n_singular_pairs"] == 1280 + 3840 + 11460


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}{c[2]}" for c in CASES])
def test_hmatrix_fp64_parity(oracle, case):
    m = icosphere(3)
    op, trs, tes = _op(case, m)
    k, tr, te, e1, e2, kap = case
    oo = oracle.OracleOperator(k, m, tr, te, kappa=kap, trial_eval=e1, test_eval=e2, intorder=3, leafsize=20,
                               eta=2.0, eps=1e-8)
    cplx = op.mat.is_complex
    x = _vec(trs.ndof, cplx, 1)
    y = (op.mat * torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel(y, oo.mult(x)) < 1e-7
    z = _vec(tes.ndof, cplx, 2)
    yt = op.mat.CreateRowVector()
    op.mat.MultTrans(torch.from_numpy(z).cuda(), yt)
    assert rel(yt.cpu().numpy(), oo.mult(z, trans=True)) < 1e-7
    b, ob = op.mat.blocks(), oo.blocks()
    for key in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[key], ob[key])
    assert np.array_equal(b["fallback"] == 1, ob["fallback"] == 1)   # shared-vertex fallbacks


@pytest.mark.parametrize("case", [CASES[0], CASES[3], CASES[6], CASES[8], CASES[10]],
                         ids=["lsl", "ldl", "hsl", "hcf", "msl"])
def test_mixed_vs_fp64(case):
    m = ellipsoid(3)
    op64, trs, tes = _op(case, m)
    op32, _, _ = _op(case, m, precision="mixed")
    cplx = op64.mat.is_complex
    x = torch.from_numpy(_vec(trs.ndof, cplx, 5)).cuda()
    y64, y32 = op64.mat * x, op32.mat * x
    assert float(torch.linalg.vector_norm(y32 - y64) / torch.linalg.vector_norm(y64)) < 1e-6
    assert op32.mat.info["bytes_dense"] + op32.mat.info["bytes_lowrank"] < \
        op64.mat.info["bytes_dense"] + op64.mat.info["bytes_lowrank"]


def test_multi_rhs_and_host_path():
    m = icosphere(3)
    case = CASES[8]
    op, trs, tes = _op(case, m, precision="mixed")
    X = np.stack([_vec(trs.ndof, True, 10 + r) for r in range(7)], axis=1)
    Y = torch.zeros((tes.ndof, 7), dtype=torch.complex128, device="cuda")
    op.mat.Mult(torch.from_numpy(X).cuda(), Y)
    for r in range(7):
        yr = (op.mat * torch.from_numpy(X[:, r].copy()).cuda()).cpu().numpy()
        assert rel(Y[:, r].cpu().numpy(), yr) < 1e-6
    yh = op.mat.mult_host(X[:, 0].copy())
    assert rel(yh, Y[:, 0].cpu().numpy()) < 1e-6
    # MultAdd semantics y = s A x + y with complex s
    y0 = torch.from_numpy(_vec(tes.ndof, True, 99)).cuda()
    y = y0.clone()
    op.mat.MultAdd(0.5 - 2j, torch.from_numpy(X[:, 1].copy()).cuda(), y)
    ref = y0 + (0.5 - 2j) * Y[:, 1]
    assert float(torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref)) < 1e-6


def test_dense_p0_assembly_is_deterministic():
    m = icosphere(3)
    a = _op(CASES[0], m, "dense")[0].mat.to_dense()
    b = _op(CASES[0], m, "dense")[0].mat.to_dense()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gmres_dirichlet_to_neumann(prec):
    m = icosphere(4)
    P0, P1 = nb.SurfaceL2(m), nb.H1(m)
    V = nb.SingleLayerPotentialOperator(P0, leafsize=20, eps=1e-8, precision=prec)
    K = nb.DoubleLayerPotentialOperator(P1, P0, leafsize=20, eps=1e-8, precision=prec)
    M = nb.MassOperator(P1, P0)
    g = torch.from_numpy(m.vertices[:, 0] ** 2 - m.vertices[:, 1] ** 2).cuda()
    u = nb.GMRes(V.mat, (0.5 * M + K.mat) * g, maxsteps=400, tol=1e-8)
    assert nb.GMRes.last["residual"] < 1e-8
    c = m.centroids()
    c /= np.linalg.norm(c, axis=1)[:, None]
    exact = 2 * (c[:, 0] ** 2 - c[:, 1] ** 2)
    A = m.areas()
    uh = u.cpu().numpy()
    assert np.sqrt(np.sum(A * (uh - exact) ** 2) / np.sum(A * exact ** 2)) < 0.01


def test_burton_miller_solve_against_oracle(oracle):
    """(1/2 M + C) u = f for a plane wave (demos/HelmholtzBurtonMiller.ipynb cell 8), P1, kappa 5."""
    m = icosphere(2)
    P1 = nb.H1(m, complex=True)
    C_ = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=5.0, intorder=4, leafsize=20, eps=1e-10)
    M = nb.MassOperator(P1, P1, complex=True)
    d = np.array([0.0, 0.0, 1.0])
    v = m.vertices
    f_nodes = np.exp(1j * 5.0 * v @ d)
    Mo = oracle.mass_matrix(m, "P1", "P1")
    rhs = Mo @ f_nodes
    u = nb.GMRes(0.5 * M + C_.mat, torch.from_numpy(rhs).cuda(), maxsteps=300, tol=1e-12)
    Co = oracle.dense_matrix("helmholtz_cf", m, "P1", kappa=5.0, intorder=4)
    uo = np.linalg.solve(0.5 * Mo + Co, rhs)
    assert rel(u.cpu().numpy(), uo) < 1e-8


def test_testhmatrix_diagnostic(capsys):
    m = icosphere(3)
    V = nb.SingleLayerPotentialOperator(nb.SurfaceL2(m), leafsize=20, eps=1e-8, testhmatrix=True)
    rate, err = V.testhmatrix_result
    assert 0 < rate < 1.5 and err < 1e-6
    assert "compression rate" in capsys.readouterr().out


def test_host_buffers_pinned_and_pageable():
    """bem_operator_mult_host with page-locked buffers (read and written by the kernels in place)
    and with pageable ones (staged), y = s A x + y, against the device entry point."""
    m = icosphere(3)
    op, trs, tes = _op(CASES[0], m, precision="mixed")
    x = _vec(trs.ndof, False, 21)
    y0 = _vec(tes.ndof, False, 22)
    ref = y0 + 0.75 * (op.mat * torch.from_numpy(x).cuda()).cpu().numpy()
    for pinned in (True, False):
        if pinned:
            xt = torch.from_numpy(x.copy()).pin_memory()
            yt = torch.from_numpy(y0.copy()).pin_memory()
            xh, yh = xt.numpy(), yt.numpy()
        else:
            xh, yh = x.copy(), y0.copy()
        op.mat.mult_host(xh, alpha=0.75, beta=1.0, y=yh)
        assert rel(yh, ref) < 1e-12
