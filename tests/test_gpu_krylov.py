"""The reference tests' solver pattern on the GPU: ngsolve.krylovspace.GMRes with a mass-matrix
inverse as preconditioner (tests/test_Maxwell_Box.py:44-50, tests/test_Laplace.py:56-60), here
with the library's H-matrices, mass matrices and their conjugate-gradient inverses inside the
preconditioned restarted GMRES (krylov.py), against the unpreconditioned native GMRES and the
exact answer of the Laplace Dirichlet-to-Neumann map on the sphere (d_n u = 2 u for
u = x^2 - y^2)."""
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
