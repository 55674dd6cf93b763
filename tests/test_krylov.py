"""Preconditioned GMRES, conjugate gradients, block systems and the mass-matrix inverse of
ngbem_gb300.krylov / bem.GMRes on the CPU, with dense stand-ins for the library's matrices (the
library's own products are tested on the GPU).  The reference's tests solve with
ngsolve.krylovspace.GMRes(A, b, pre=mass inverse or a BlockMatrix of them).  Also the
TestCompression diagnostic (torch on the CPU here)."""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import krylov
from ngbem_gb300.bem import _MassInverse


class Dense:
    """A stand-in with the library matrices' _apply interface, on CPU tensors."""

    def __init__(self, A):
        self.A = torch.as_tensor(A)
        self.height, self.width = self.A.shape
        self.is_complex = self.A.is_complex()

    def _apply(self, trans, alpha, x, beta, y):
        M = self.A.T if trans else self.A
        r = M.to(torch.promote_types(M.dtype, x.dtype)) @ x
        if beta == 0.0:
            y.copy_(alpha * r)
        else:
            y.mul_(beta).add_(alpha * r)


def _rand(n, m=None, cplx=False, seed=0):
    r = np.random.default_rng(seed)
    a = r.standard_normal((n, m or n))
    if cplx:
        a = a + 1j * r.standard_normal((n, m or n))
    return a


def test_cg_solves_spd():
    B = _rand(60, seed=1)
    A = torch.as_tensor(B @ B.T + 60 * np.eye(60))
    b = torch.as_tensor(np.random.default_rng(2).standard_normal(60))
    x, it, rel = krylov.cg(lambda v: A @ v, b, tol=1e-13)
    assert rel < 1e-13 and torch.linalg.vector_norm(A @ x - b) / torch.linalg.vector_norm(b) < 1e-12
    bc = b + 1j * b.flip(0)
    xc, _, _ = krylov.cg(lambda v: A.to(v.dtype) @ v, bc, tol=1e-13)
    assert torch.allclose(A.to(xc.dtype) @ xc, bc, atol=1e-10)


@pytest.mark.parametrize("cplx", [False, True])
def test_gmres_with_and_without_preconditioner(cplx):
    n = 80
    D = np.diag(np.linspace(1.0, 400.0, n))
    A = torch.as_tensor(D + 0.5 * _rand(n, cplx=cplx, seed=3))
    b = torch.as_tensor(_rand(n, 1, cplx=cplx, seed=4)[:, 0])
    ref = torch.linalg.solve(A, b)
    x1, it1, r1 = krylov.gmres(lambda v: A @ v, b, maxsteps=400, tol=1e-12)
    pre = torch.as_tensor(np.diag(1.0 / np.diag(D))).to(A.dtype)
    x2, it2, r2 = krylov.gmres(lambda v: A @ v, b, pre=lambda v: pre @ v, maxsteps=400, tol=1e-12)
    for x in (x1, x2):
        assert torch.linalg.vector_norm(x - ref) / torch.linalg.vector_norm(ref) < 1e-9
    assert it2 < it1
    # restarted
    x3, it3, _ = krylov.gmres(lambda v: A @ v, b, pre=lambda v: pre @ v, maxsteps=400, tol=1e-12, restart=5)
    assert torch.linalg.vector_norm(x3 - ref) / torch.linalg.vector_norm(ref) < 1e-9 and it3 >= it2


def test_gmres_freedofs():
    n = 40
    A = torch.as_tensor(np.diag(np.arange(1.0, n + 1)) + 0.1 * _rand(n, seed=5))
    b = torch.as_tensor(_rand(n, 1, seed=6)[:, 0])
    free = np.ones(n, dtype=bool)
    free[::5] = False
    x, _, _ = krylov.gmres(lambda v: A @ v, b, freedofs=free, maxsteps=200, tol=1e-13)
    f = torch.as_tensor(free)
    assert (x[~f] == 0).all()
    xr = torch.linalg.solve(A[f][:, f], b[f])
    assert torch.allclose(x[f], xr, rtol=0, atol=1e-10)
    # a start vector carries fixed values on the other dofs (a Dirichlet lift)
    x0 = torch.zeros(n, dtype=torch.float64)
    x0[~f] = 2.0
    x2, _, _ = krylov.gmres(lambda v: A @ v, b, x0=x0, freedofs=free, maxsteps=200, tol=1e-13)
    assert (x2[~f] == 2.0).all()
    xr2 = torch.linalg.solve(A[f][:, f], b[f] - A[f][:, ~f] @ x0[~f])
    assert torch.allclose(x2[f], xr2, rtol=0, atol=1e-10)


def test_block_matrix_and_vector():
    A, B, C = _rand(5, seed=7), _rand(5, 3, seed=8), _rand(3, seed=9)
    K = nb.BlockMatrix([[Dense(A), Dense(B)], [None, Dense(C)]])
    full = np.block([[A, B], [np.zeros((3, 5)), C]])
    u, v = torch.as_tensor(_rand(5, 1, seed=10)[:, 0]), torch.as_tensor(_rand(3, 1, seed=11)[:, 0])
    bv = nb.BlockVector([u, v])
    assert len(bv) == 2 and torch.equal(bv[1], v)
    y = K * bv
    assert isinstance(y, nb.BlockVector)
    assert np.allclose(y.data.numpy(), full @ np.concatenate([u, v]))
    yt = torch.zeros(8, dtype=torch.float64)
    K.MultTrans(bv, yt)
    assert np.allclose(yt.numpy(), full.T @ np.concatenate([u, v]))
    with pytest.raises(ValueError):
        nb.BlockMatrix([[Dense(A), Dense(C)]])
    # a real block inside a complex system acts on real and imaginary parts
    Kc = nb.BlockMatrix([[Dense(A.astype(complex) * (1 + 1j)), Dense(B)], [None, Dense(C)]])
    z = torch.as_tensor(_rand(8, 1, cplx=True, seed=12)[:, 0])
    fullc = np.block([[A * (1 + 1j), B], [np.zeros((3, 5)), C]])
    assert np.allclose((Kc * z).numpy(), fullc @ z.numpy())


def test_mass_inverse_and_block_preconditioned_gmres():
    """The pattern of the reference's Laplace test: GMRes(BlockMatrix, BlockVector,
    pre=BlockMatrix of mass-matrix inverses)."""
    B1, B2 = _rand(30, seed=13), _rand(20, seed=14)
    M1 = Dense(B1 @ B1.T + 30 * np.eye(30))
    M2 = Dense(B2 @ B2.T + 20 * np.eye(20))
    inv1, inv2 = _MassInverse(M1, None, 1e-14, 500), _MassInverse(M2, None, 1e-14, 500)
    x = torch.as_tensor(_rand(30, 1, cplx=True, seed=15)[:, 0])
    y = torch.zeros(30, dtype=torch.complex128)
    inv1._apply(False, 1.0, (M1.A.to(x.dtype) @ x), 0.0, y)
    assert torch.allclose(y, x, atol=1e-11)
    # products keep the vector's field: a real inverse on a complex vector
    assert torch.allclose(inv1 * (M1.A.to(x.dtype) @ x), x, atol=1e-11)
    xr = x.real.contiguous()
    assert torch.allclose(inv1 * (M1.A @ xr), xr, atol=1e-11) and not (inv1 * (M1.A @ xr)).is_complex()
    V, K, W = _rand(30, seed=16) + 40 * np.eye(30), 0.3 * _rand(30, 20, seed=17), _rand(20, seed=18) + 30 * np.eye(20)
    lhs = nb.BlockMatrix([[Dense(V), Dense(-K)], [Dense(K.T), Dense(W)]])
    pre = nb.BlockMatrix([[inv1, None], [None, inv2]])
    rhs = nb.BlockVector([torch.as_tensor(_rand(30, 1, seed=19)[:, 0]), torch.as_tensor(_rand(20, 1, seed=20)[:, 0])])
    sol = nb.GMRes(A=lhs, b=rhs, pre=pre, maxsteps=300, tol=1e-12, printrates=False)
    full = np.block([[V, -K], [K.T, W]])
    ref = np.linalg.solve(full, rhs.data.numpy())
    assert isinstance(sol, nb.BlockVector)
    assert np.linalg.norm(sol.data.numpy() - ref) / np.linalg.norm(ref) < 1e-9
    assert nb.GMRes.last["iterations"] > 0
    # freedofs on the mass inverse: zero outside, the restricted inverse inside
    free = np.ones(30, dtype=bool)
    free[:4] = False
    invf = _MassInverse(M1, free, 1e-14, 500)
    r = torch.as_tensor(_rand(30, 1, seed=21)[:, 0])
    z = torch.zeros(30, dtype=torch.float64)
    invf._apply(False, 1.0, r, 0.0, z)
    Mf = M1.A[free][:, free]
    assert (z[:4] == 0).all() and torch.allclose(z[4:], torch.linalg.solve(Mf, r[4:]), atol=1e-11)


def test_compression_diagnostic():
    """TestCompression (the reference's python_bem.cpp:177-193): the truncated SVD leaves an
    error below eps sqrt(rank deficit); the randomized SVD and ACA reach the same order of
    accuracy with ranks near the SVD's; other methods give (0, 0)."""
    eps = 1e-10
    r_svd, e_svd, t = nb.TestCompression(100, 120, 2.0, eps, "svd", seed=3, device="cpu")
    assert 0 < r_svd < 100 and e_svd <= eps * np.sqrt(100) and t >= 0
    r_t, e_t, _ = nb.TestCompression(100, 120, 2.0, eps, "tsvd", seed=3, device="cpu")
    assert abs(r_t - r_svd) <= 3 and e_t < 10 * eps * np.sqrt(100)
    r_a, e_a, _ = nb.TestCompression(100, 120, 2.0, eps, "aca", seed=3, device="cpu")
    assert r_svd <= r_a <= r_svd + 20 and e_a < 1e-8
    # better separated clusters compress further
    assert nb.TestCompression(100, 120, 0.5, eps, "svd", seed=3, device="cpu")[0] < r_svd
    assert nb.TestCompression(method="other", device="cpu") == (0, 0)
