"""Failure paths of assembly and application, exercised without faulting the GPU.

* Far blocks whose ACA fails are assembled densely, as the reference's CalcHMatrix does when
  CalcFarFieldBlock throws (src/ngbem.cpp:143-153).  The failure is injected on the host
  (NGBEM_GB300_ACA_FAIL) and through the rank cap, whose first round (provisional cap 48)
  sends the blocks that reach it to a second round with the full cap.
* A bounded device wait that runs out is reported (bem_operator_status, and an error return
  of the synchronous host-buffer product) and the operator works again after the reset.  The
  test hook makes every grid-barrier wait of the single-launch product wait for an arrival
  that never comes, with a short poll limit, so the kernel ends by itself.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import _lib
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_injected_aca_failures_fall_back_to_dense(oracle, monkeypatch):
    m = icosphere(3)
    P0 = nb.SurfaceL2(m)
    every = 3
    monkeypatch.setenv("NGBEM_GB300_ACA_FAIL", str(every))
    V = nb.SingleLayerPotentialOperator(P0, intorder=3, leafsize=20, eta=2.0, eps=1e-8, precision="fp64")
    monkeypatch.delenv("NGBEM_GB300_ACA_FAIL")
    b = V.mat.blocks()
    far = np.flatnonzero((b["near"] == 0) & (b["fallback"] != 1))
    hit = far[far % every == 0]
    miss = far[far % every != 0]
    assert len(hit) > 10 and len(miss) > 10
    assert np.all(b["fallback"][hit] == 2) and np.all(b["rank"][hit] == -1)
    assert np.all(b["fallback"][miss] == 0) and np.all(b["rank"][miss] >= 0)
    assert V.mat.info["nfallback"] == int(np.sum(b["fallback"] != 0))
    # the dense blocks are the exact quadrature of those blocks: the product stays within the
    # ACA tolerance of the oracle's H-matrix and of its dense matrix
    x = np.random.default_rng(5).standard_normal(P0.ndof)
    y = (V.mat * torch.from_numpy(x).cuda()).cpu().numpy()
    H = oracle.OracleOperator("laplace_sl", m, "P0", intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    D = oracle.dense_matrix("laplace_sl", m, "P0", intorder=3)
    assert _rel(y, H.mult(x)) < 1e-7
    assert _rel(y, D @ x) < 1e-7


def test_rank_cap_second_round_and_dense_fallback(oracle):
    """eps = 1e-12 needs ranks up to about 70 at L3: with max_rank 60 the blocks of rank 49..60
    finish in the second ACA round, those above 60 are assembled densely."""
    m = icosphere(3)
    P0 = nb.SurfaceL2(m)
    V = nb.SingleLayerPotentialOperator(P0, intorder=3, leafsize=20, eta=2.0, eps=1e-12, precision="fp64",
                                        max_rank=60)
    b = V.mat.blocks()
    r = b["rank"]
    assert r.max() <= 60
    assert np.any((r > 48) & (r <= 60)), "no block finished in the second round"
    assert np.any(b["fallback"] == 2), "no block reached the rank cap"
    x = np.random.default_rng(6).standard_normal(P0.ndof)
    y = (V.mat * torch.from_numpy(x).cuda()).cpu().numpy()
    D = oracle.dense_matrix("laplace_sl", m, "P0", intorder=3)
    H = oracle.OracleOperator("laplace_sl", m, "P0", intorder=3, leafsize=20, eta=2.0, eps=1e-12)
    assert _rel(y, D @ x) < 1e-10
    assert _rel(y, H.mult(x)) < 1e-10


def _status(mat, reset):
    f = C.c_int(-1)
    _lib.check(_lib.lib.bem_operator_status(mat.h, C.byref(f), int(reset)))
    return f.value


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_wait_that_runs_out_is_reported(precision):
    m = icosphere(3)
    P0 = nb.SurfaceL2(m)
    V = nb.SingleLayerPotentialOperator(P0, intorder=3, leafsize=20, eta=2.0, eps=1e-8, precision=precision)
    x = torch.from_numpy(np.random.default_rng(7).standard_normal(P0.ndof)).cuda()
    y_ref = V.mat * x
    assert _status(V.mat, False) == 0
    # every grid-barrier wait of the single-launch product polls 4096 times, then gives up
    _lib.check(_lib.lib.bem_operator_test_waits(V.mat.h, 1 << 12, 1))
    y = V.mat.CreateColVector()
    V.mat.Mult(x, y)
    torch.cuda.synchronize()
    assert _status(V.mat, True) & 4
    assert _status(V.mat, False) == 0  # cleared by the reset
    # the synchronous host-buffer product reports it as an error
    xh = x.cpu().numpy()
    with pytest.raises(_lib.BemError) as e:
        V.mat.mult_host(xh)
    assert e.value.code == _lib.BEM_ERR_INTERNAL and "wait" in str(e.value)
    # back to normal: the same product as before
    _lib.check(_lib.lib.bem_operator_test_waits(V.mat.h, 0, 0))
    V.mat.Mult(x, y)
    torch.cuda.synchronize()
    assert _status(V.mat, False) == 0
    assert (torch.linalg.vector_norm(y - y_ref) / torch.linalg.vector_norm(y_ref)).item() < 1e-12
    yh = V.mat.mult_host(xh)
    assert _rel(yh, y_ref.cpu().numpy()) < 1e-12
