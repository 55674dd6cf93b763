"""The reference tests' solver pattern on the GPU: ngsolve.krylovspace.GMRes with a mass-matrix
inverse as preconditioner (tests/test_Maxwell_Box.py:44-50, tests/test_Laplace.py:56-60), here
with the library's H-matrices, mass matrices and their inverses (a Cholesky factor on the GPU,
or conjugate gradients) inside the preconditioned restarted GMRES (krylov.py), against the
unpreconditioned native GMRES and the exact answer of the Laplace Dirichlet-to-Neumann map on
the sphere (d_n u = 2 u for u = x^2 - y^2), and against a direct solve of a higher-order EFIE."""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu


def test_preconditioned_gmres_dtn():
    m = icosphere(3)
    P0, P1 = nb.SurfaceL2(m), nb.H1(m)
    kw = dict(intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    V = nb.SingleLayerPotentialOperator(P0, **kw)
    K = nb.DoubleLayerPotentialOperator(P1, P0, **kw)
    M10 = nb.MassOperator(P1, P0)
    M00 = nb.MassOperator(P0, P0)
    g = torch.from_numpy(m.vertices[:, 0] ** 2 - m.vertices[:, 1] ** 2).cuda()
    rhs = (0.5 * M10 + K.mat) * g
    u_plain = nb.GMRes(V.mat, rhs, maxsteps=500, tol=1e-10, restart=500)
    it_plain = nb.GMRes.last["iterations"]
    u_pre = nb.GMRes(V.mat, rhs, pre=M00.Inverse(), maxsteps=500, tol=1e-10, restart=200)
    it_pre = nb.GMRes.last["iterations"]
    assert it_pre > 0 and it_plain > 0
    assert (torch.linalg.vector_norm(u_pre - u_plain) / torch.linalg.vector_norm(u_plain)).item() < 1e-8
    c = m.centroids()
    c = c / np.linalg.norm(c, axis=1)[:, None]
    exact = 2.0 * (c[:, 0] ** 2 - c[:, 1] ** 2)
    a = m.areas()
    uh = u_pre.cpu().numpy()
    assert np.sqrt(np.sum(a * (uh - exact) ** 2) / np.sum(a * exact ** 2)) < 0.02


def test_mass_inverse_cholesky_and_cg():
    """The mass-matrix inverse by a Cholesky factor (the default up to 12 000 free dofs) and by
    conjugate gradients agree, solve M z = x, and respect freedofs (the other entries are 0)."""
    m = icosphere(2)
    sp = nb.H1(m, order=2)
    M = nb.MassOperator(sp, sp)
    rng = np.random.default_rng(9)
    x = torch.from_numpy(rng.standard_normal(sp.ndof)).cuda()
    zc = M.Inverse() * x
    zg = M.Inverse(direct_max=0) * x
    assert (torch.linalg.vector_norm(zc - zg) / torch.linalg.vector_norm(zc)).item() < 1e-9
    assert (torch.linalg.vector_norm(M * zc - x) / torch.linalg.vector_norm(x)).item() < 1e-12
    xc = x.to(torch.complex128) * (1 + 2j)
    assert (torch.linalg.vector_norm(M.Inverse() * xc - zc * (1 + 2j)) / torch.linalg.vector_norm(xc)).item() < 1e-12
    free = np.ones(sp.ndof, dtype=bool)
    free[::3] = False
    zf = (M.Inverse(freedofs=free) * x).cpu().numpy()
    assert np.all(zf[~free] == 0.0)
    Md = M.to_dense()
    assert np.abs(Md[np.ix_(free, free)] @ zf[free] - x.cpu().numpy()[free]).max() < 1e-12 * np.abs(x.cpu().numpy()).max()


def test_preconditioned_gmres_efie_order_2():
    """The reference's Maxwell pattern (GMRes with pre = the HDivSurface mass inverse) on the
    EFIE of a sphere with HDivSurface of order 2: the same current as a direct solve."""
    m = icosphere(1, radius=0.25).Curve(3)
    HD = nb.HDivSurface(m, order=2, complex=True)
    V = nb.MaxwellSingleLayerPotentialOperator(HD, 5.0, intorder=6, leafsize=120, eta=3.0, eps=1e-10)
    rng = np.random.default_rng(4)
    b = torch.from_numpy(rng.standard_normal(HD.ndof) + 1j * rng.standard_normal(HD.ndof)).cuda()
    pre = nb.MassOperator(HD, HD, complex=True).Inverse()
    j = nb.GMRes(A=V.mat, b=b, pre=pre, tol=1e-11, maxsteps=2000, restart=400, printrates=False)
    jd = torch.linalg.solve(torch.from_numpy(V.mat.to_dense()).cuda(), b)
    assert (torch.linalg.vector_norm(j - jd) / torch.linalg.vector_norm(jd)).item() < 1e-8
