"""Tensor-core products for several right-hand sides (tc_matvec.cu, tc_host.cpp).

* The encodings of the tcgen05 instruction and shared-memory descriptors pass their
  known-answer product (exact small-integer GEMM).
* The Helmholtz combined-field operator (kappa 8, FP32 storage, plain accuracy) applied to 32
  and to 5 right-hand sides through the tensor cores agrees with the compensated CUDA-core
  products of the same operator to 1e-6, and with the FP64-stored operator to 1.5e-6.  The
  operands are split-TF32 (about 2^-21 per product); tensor memory accumulates with rounding
  toward zero, so no accumulator takes more than 2 TC_CHAIN MMAs before the epilogue adds it
  into sums that round to nearest.
* Switching the path off gives the CUDA-core products again; one right-hand side never takes it.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import ellipsoid

pytestmark = pytest.mark.gpu

KAPPA = 8.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_selftest_exact():
    assert nb.tc_selftest()


@pytest.fixture(scope="module")
def bm():
    m = ellipsoid(4, (1.0, 0.7, 0.5))
    P1 = nb.H1(m, complex=True)
    kw = dict(kappa=KAPPA, intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    C32 = nb.HelmholtzCombinedFieldOperator(P1, P1, precision="mixed", **kw)
    C64 = nb.HelmholtzCombinedFieldOperator(P1, P1, precision="fp64", **kw)
    return P1, C32.mat, C64.mat


def _x(n, nrhs, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(n, nrhs, generator=g, dtype=torch.float64) + 1j * torch.randn(n, nrhs, generator=g,
                                                                                  dtype=torch.float64)
    return x.to(torch.complex128).cuda()


def _apply(A, x):
    y = torch.empty_like(x)
    A.Mult(x, y)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("nrhs", [32, 5])
def test_tensor_core_products(bm, nrhs):
    P1, A32, A64 = bm
    x = _x(P1.ndof, nrhs, 11 + nrhs)
    A32.set_accuracy(True)
    y_comp = _apply(A32, x)
    A32.set_accuracy(False)
    A32.set_tensor_cores(True)
    info = A32.tensor_cores()
    assert info["state"] == 1 and info["bytes"] > 0 and min(info["items"]) > 0
    y_tc = _apply(A32, x)
    y64 = _apply(A64, x)
    # split-TF32 products, accumulators of at most 2 TC_CHAIN MMAs summed with round-to-nearest:
    # the product meets the 1e-6 bar against the FP64 path
    assert rel(y_tc, y_comp) < 1e-6
    assert rel(y_tc, y64) < 1.5e-6
    for r in range(nrhs):
        assert rel(y_tc[:, r], y_comp[:, r]) < 2e-6
    # off: the CUDA-core plain products
    A32.set_tensor_cores(False)
    assert A32.tensor_cores()["state"] == 0
    y_cc = _apply(A32, x)
    assert rel(y_cc, y_comp) < 2e-6
    A32.set_tensor_cores(True)
    A32.set_accuracy(True)


def test_beta_and_single_rhs(bm):
    P1, A32, _ = bm
    A32.set_accuracy(False)
    A32.set_tensor_cores(True)
    x = _x(P1.ndof, 8, 3)
    y0 = _x(P1.ndof, 8, 4)
    ref = _apply(A32, x)
    y = y0.clone()
    A32.MultAdd(0.5, x, y)   # y += 0.5 A x through the same path
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy(), y0.cpu().numpy() + 0.5 * ref) < 1e-12 + 1e-6
    x1 = x[:, :1].contiguous()
    y1 = _apply(A32, x1)
    assert rel(y1[:, 0], ref[:, 0]) < 1e-5
    A32.set_accuracy(True)


def test_stage_plan_autotuner(bm):
    """The tuner times 2, 3 and 4 pipeline stages on the operator, keeps the fastest, and the
    products with the kept plan still agree with the compensated ones."""
    P1, A32, A64 = bm
    A32.set_accuracy(True)
    x = _x(P1.ndof, 32, 5)
    y_comp = _apply(A32, x)
    A32.set_accuracy(False)
    A32.set_tensor_cores(True)
    res = A32.autotune_tensor_cores(reps=2)
    assert res["stages"] in (2, 3, 4)
    assert all(v > 0 for v in res["ms"].values())
    assert res["ms"][res["stages"]] == min(res["ms"].values())
    assert rel(_apply(A32, x), y_comp) < 1e-6


def test_products_against_the_oracle_at_level_5(oracle):
    """The Burton-Miller operator near the benchmark's size (ellipsoid L5, 10 242 P1 dofs, kappa
    8): the tensor-core product of 32 right-hand sides against the oracle's FP64 H-matrix
    (CalcHMatrix and HMatrix::Mult restated) on four of its columns, within the 1e-6 bar."""
    m = ellipsoid(5, (1.0, 0.7, 0.5))
    P1 = nb.H1(m, complex=True)
    kw = dict(kappa=KAPPA, intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    A = nb.HelmholtzCombinedFieldOperator(P1, P1, precision="mixed", **kw).mat
    A.set_accuracy(False)
    A.set_tensor_cores(True)
    x = _x(P1.ndof, 32, 23)
    y = _apply(A, x)
    assert A.tensor_cores()["state"] == 1
    H = oracle.OracleOperator("helmholtz_cf", m, "P1", kappa=KAPPA, intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    xh = x.cpu().numpy()
    for r in (0, 9, 20, 31):
        yo = H.mult(xh[:, r])
        assert rel(y[:, r], yo) < 1e-6
