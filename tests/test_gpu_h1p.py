"""H1 of order 2 and 3 on the GPU against the FP64 oracle, in the pairings of the reference's
Laplace test (tests/test_Laplace.py:23-45: V on SurfaceL2 of order p - 1, K from H1 of order p
to SurfaceL2 of order p - 1, W on H1 of order p) and the Helmholtz identity-trace operators.

Dense FP64 operators within 1e-10 of the oracle's dense matrices; FP64 H-matrices within the
ACA tolerance of the oracle's H-matrices in both directions; mixed precision within 1e-6 of
FP64; potentials and mass matrices against the oracle; and the interior Dirichlet-to-Neumann
map of x^2 - y^2 on the sphere solved through V, K and M with H1 of order 3 data.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.forms import load_vector
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu

# (kernel, kappa, trial kind, test kind, evaluator); L2 stands for SurfaceL2 of order p - 1
COMBOS = [("laplace_sl", 0.0, "H1", "H1", "id"), ("laplace_dl", 0.0, "H1", "H1", "id"),
          ("laplace_dl", 0.0, "H1", "L2", "id"), ("laplace_hs", 0.0, "H1", "H1", "rot"),
          ("helmholtz_sl", 3.0, "H1", "H1", "id"), ("helmholtz_dl", 3.0, "H1", "H1", "id"),
          ("helmholtz_cf", 4.0, "H1", "H1", "id"), ("helmholtz_hs", 3.0, "H1", "H1", "helm")]
IDS = [f"{k}-{a}-{b}" for k, _, a, b, _ in COMBOS]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _kinds(p, trial, test):
    k = {"H1": f"H1P{p}", "L2": f"L2P{p - 1}"}
    return k[trial], k[test]


def _space(mesh, kind):
    if kind.startswith("H1P"):
        return nb.H1(mesh, order=int(kind[3:]))
    return nb.SurfaceL2(mesh, order=int(kind[3:]))


def _op(kernel, kappa, mesh, tr, te, ev, method="aca", precision="fp64", **kw):
    s_tr, s_te = _space(mesh, tr), _space(mesh, te)
    prm = dict(intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    prm.update(kw)
    io = prm.pop("intorder")
    tev = ev if te.startswith("H1") else "id"
    op = bem.IntegralOperator(kernel, kappa, s_tr, s_te, ev, tev, io, prm.pop("leafsize"), prm.pop("eta"),
                              prm.pop("eps"), method, False, precision=precision, **prm)
    return op, s_tr, s_te


@pytest.mark.parametrize("p", [2, 3])
@pytest.mark.parametrize("kernel,kappa,trial,test,ev", COMBOS, ids=IDS)
def test_dense_parity(oracle, kernel, kappa, trial, test, ev, p):
    m = icosphere(2 if p == 2 else 1)
    tr, te = _kinds(p, trial, test)
    op, s_tr, s_te = _op(kernel, kappa, m, tr, te, ev, "dense", intorder_singular=4, intorder_regular=3)
    D = op.mat.to_dense()
    Do = oracle.dense_matrix(kernel, m, tr, te, kappa=kappa, trial_eval=ev,
                             test_eval=ev if te.startswith("H1") else "id", intorder_singular=4,
                             intorder_regular=3)
    assert D.shape == (s_te.ndof, s_tr.ndof)
    assert rel(D, Do) < 1e-10


@pytest.mark.parametrize("p", [2, 3])
@pytest.mark.parametrize("kernel,kappa,trial,test,ev", [COMBOS[0], COMBOS[2], COMBOS[3], COMBOS[6]],
                         ids=[IDS[0], IDS[2], IDS[3], IDS[6]])
def test_hmatrix_parity(oracle, kernel, kappa, trial, test, ev, p):
    m = icosphere(3 if p == 2 else 2)
    tr, te = _kinds(p, trial, test)
    op, s_tr, s_te = _op(kernel, kappa, m, tr, te, ev)
    H = oracle.OracleOperator(kernel, m, tr, te, kappa=kappa, trial_eval=ev,
                              test_eval=ev if te.startswith("H1") else "id", intorder=3, leafsize=40,
                              eta=2.0, eps=1e-8)
    b, ob = op.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    cplx = kappa != 0.0
    rng = np.random.default_rng(17 + p)
    dt = torch.complex128 if cplx else torch.float64
    x = rng.standard_normal(s_tr.ndof) + (1j * rng.standard_normal(s_tr.ndof) if cplx else 0.0)
    y = (op.mat * torch.from_numpy(x).to(dt).cuda()).cpu().numpy()
    assert rel(y, H.mult(x)) < 1e-7
    z = rng.standard_normal(s_te.ndof) + (1j * rng.standard_normal(s_te.ndof) if cplx else 0.0)
    yt = op.mat.CreateRowVector()
    op.mat.MultTrans(torch.from_numpy(z).to(dt).cuda(), yt)
    assert rel(yt.cpu().numpy(), H.mult(z, trans=True)) < 1e-7


def test_mixed_against_fp64():
    m = icosphere(2)
    for kernel, kappa, trial, test, ev in [COMBOS[0], COMBOS[2], COMBOS[3], COMBOS[6]]:
        tr, te = _kinds(3, trial, test)
        o64, s_tr, _ = _op(kernel, kappa, m, tr, te, ev)
        o32, _, _ = _op(kernel, kappa, m, tr, te, ev, precision="mixed")
        cplx = kappa != 0.0
        rng = np.random.default_rng(5)
        x = rng.standard_normal(s_tr.ndof) + (1j * rng.standard_normal(s_tr.ndof) if cplx else 0.0)
        xd = torch.from_numpy(x).to(torch.complex128 if cplx else torch.float64).cuda()
        assert rel((o32.mat * xd).cpu().numpy(), (o64.mat * xd).cpu().numpy()) < 1e-6


@pytest.mark.parametrize("p", [2, 3])
def test_potential_and_mass(oracle, p):
    m = icosphere(2)
    kind = f"H1P{p}"
    for kernel in ("laplace_sl", "laplace_dl"):
        op, sp, _ = _op(kernel, 0.0, m, kind, kind, "id")
        dens = np.random.default_rng(13).standard_normal(sp.ndof)
        pts = np.array([[2.0, 0.3, -0.1], [0.1, 0.2, 0.3], [-1.5, 1.0, 0.5]])
        val = op.GetPotential(torch.from_numpy(dens).cuda())(pts).cpu().numpy().reshape(len(pts), -1)
        ref = oracle.potential(kernel, m, kind, dens, pts, intorder=3).reshape(len(pts), -1)
        assert rel(val, ref) < 1e-11
    sp = nb.H1(m, order=p)
    sl = nb.SurfaceL2(m, order=p - 1)
    x = np.random.default_rng(3).standard_normal(sp.ndof)
    for test_sp, test_kind, order in ((sp, kind, 2 * p), (sl, f"L2P{p - 1}", 2 * p - 1)):
        M = nb.MassOperator(sp, test_sp)
        y = (M * torch.from_numpy(x).cuda()).cpu().numpy()
        Mo = oracle.mass_matrix(m, kind, test_kind, order=max(4, order))
        assert rel(y, Mo @ x) < 1e-12


def test_dirichlet_to_neumann_order_3(oracle):
    """The reference's Laplace test pairing on a known answer: g = x^2 - y^2 on the unit sphere
    (H1 of order 3 data) gives the interior Neumann data 2 g.  Solve V u = (M/2 + K) g with V
    on SurfaceL2 of order 2, K from H1 of order 3 and M their mass matrix; the flat triangles
    limit the error to O(h^2), which the refinement shows."""
    errs = []
    for level in (2, 3):
        m = icosphere(level)
        h1 = nb.H1(m, order=3)
        l2 = nb.SurfaceL2(m, order=2)
        V = nb.SingleLayerPotentialOperator(l2, intorder=7, eps=1e-10)
        K = nb.DoubleLayerPotentialOperator(h1, l2, intorder=7, eps=1e-10)
        M = nb.MassOperator(h1, l2)

        def g(x, n):
            return x[..., 0] ** 2 - x[..., 1] ** 2

        # g in H1 of order 3: its L2 projection
        gh = np.linalg.solve(oracle.mass_matrix(m, "H1P3", "H1P3", order=6), load_vector(h1, g, order=8))
        ghd = torch.from_numpy(gh).cuda()
        rhs = 0.5 * (M * ghd) + K.mat * ghd
        u = nb.GMRes(A=V.mat, b=rhs, tol=1e-10, maxsteps=400, printrates=False)
        u = u.cpu().numpy() if isinstance(u, torch.Tensor) else np.asarray(u)
        # the exact Neumann data projected onto SurfaceL2 of order 2 (block-diagonal mass)
        Ml2 = oracle.mass_matrix(m, "L2P2", "L2P2", order=4)
        c = np.linalg.solve(Ml2, load_vector(l2, lambda x, n: 2.0 * g(x, n), order=8))
        e = u - c
        errs.append(float(np.sqrt(e @ Ml2 @ e / (c @ Ml2 @ c))))
    assert errs[1] < 0.05
    assert errs[1] < 0.5 * errs[0]
