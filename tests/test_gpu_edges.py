"""Edge cases of the operator path on the GPU: the smallest meshes (one triangle, a
tetrahedron's four), zero right-hand sides, and the bounds of the tensor-core path in the
number of right-hand sides (2 and 32 take it, 1 and 33 stay on the CUDA cores, all agreeing).
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import Mesh, ellipsoid

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _tetrahedron():
    X = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    T = np.array([[0, 2, 1], [0, 1, 3], [1, 2, 3], [0, 3, 2]], dtype=np.int32)
    return Mesh(X, T)


@pytest.mark.parametrize("kernel,kind,kappa", [("laplace_sl", "P0", 0.0), ("laplace_dl", "P1", 0.0),
                                                ("helmholtz_sl", "P1", 2.0)])
def test_smallest_meshes_against_the_oracle(oracle, kernel, kind, kappa):
    """A single triangle (all pairs identical) and a tetrahedron (every pair shares an edge):
    dense FP64 operators within 1e-12 of the oracle, and the ACA method (every block near)
    equal to the dense one."""
    one = Mesh(np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.2, 0.9, 0.1]]), np.array([[0, 1, 2]], dtype=np.int32))
    for m in (one, _tetrahedron()):
        sp = nb.TraceSpace(m, kind, complex=kappa != 0.0)
        D = bem.IntegralOperator(kernel, kappa, sp, sp, "id", "id", 4, 40, 2.0, 1e-8, "dense", False).mat.to_dense()
        Do = oracle.dense_matrix(kernel, m, kind, kappa=kappa, intorder=4)
        # the double layer of one flat triangle is zero up to rounding: an absolute floor
        assert np.linalg.norm(D - Do) <= 1e-12 * np.linalg.norm(Do) + 1e-16
        H = bem.IntegralOperator(kernel, kappa, sp, sp, "id", "id", 4, 40, 2.0, 1e-8, "aca", False).mat.to_dense()
        assert np.linalg.norm(H - D) <= 1e-14 * np.linalg.norm(D) + 1e-16


def test_zero_right_hand_sides_give_zero():
    m = ellipsoid(3, (1.0, 0.7, 0.5))
    P1 = nb.H1(m, complex=True)
    A = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=4.0, precision="mixed", intorder=3, leafsize=20,
                                          eps=1e-8).mat
    for acc in (True, False):
        A.set_accuracy(acc)
        for shape in ((P1.ndof,), (P1.ndof, 8)):
            x = torch.zeros(shape, dtype=torch.complex128, device="cuda")
            y = torch.full_like(x, 7.0)
            A.Mult(x, y)
            torch.cuda.synchronize()
            assert torch.count_nonzero(y).item() == 0


@pytest.mark.parametrize("nrhs", [1, 2, 32, 33])
def test_tensor_core_bounds_in_right_hand_sides(nrhs):
    """2..32 right-hand sides take the tensor cores, 1 and 33 the CUDA cores; every count gives
    the FP32 operator's products (the compensated ones) within the tensor cores' 1e-6."""
    m = ellipsoid(3, (1.0, 0.7, 0.5))
    P1 = nb.H1(m, complex=True)
    A = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=4.0, precision="mixed", intorder=3, leafsize=20,
                                          eps=1e-8).mat
    g = torch.Generator().manual_seed(nrhs)
    x = (torch.randn(P1.ndof, nrhs, generator=g, dtype=torch.float64)
         + 1j * torch.randn(P1.ndof, nrhs, generator=g, dtype=torch.float64)).to(torch.complex128).cuda()
    A.set_accuracy(True)
    y_ref = torch.empty_like(x)
    A.Mult(x, y_ref)
    A.set_accuracy(False)
    A.set_tensor_cores(True)
    y = torch.empty_like(x)
    A.Mult(x, y)
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-6
