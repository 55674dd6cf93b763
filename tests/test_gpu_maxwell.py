"""Maxwell EFIE operator (single layer on RT0 with [Piola u; div u] traces, kappa = 2) at the
H-matrix accuracy of the Maxwell workload (ACA eps 1e-6): the GPU H-matrix against the FP64
oracle's dense matrix on the same mesh (matvec), FP64 and mixed precision, and the mixed path
against the FP64 path."""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _x(n, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(n) + 1j * r.standard_normal(n)


@pytest.mark.parametrize("precision,tol", [("fp64", 2e-5), ("mixed", 2e-5)])
def test_maxwell_hmatrix_matvec_against_oracle(oracle, precision, tol):
    m = icosphere(3)
    RT = nb.HDivSurface(m, complex=True)
    op = nb.MaxwellSingleLayerPotentialOperator(RT, kappa=2.0, intorder=3, leafsize=20, eps=1e-6,
                                                precision=precision)
    D = oracle.dense_matrix("maxwell_sl", m, "RT0", "RT0", kappa=2.0, trial_eval="maxwell", intorder=3)
    assert op.mat.height == D.shape[0] == RT.ndof
    x = _x(RT.ndof, 3)
    y = (op.mat * torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel(y, D @ x) < tol
    # transpose (no conjugation)
    yt = (op.mat.T * torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel(yt, D.T @ x) < tol


def test_maxwell_mixed_against_fp64():
    m = icosphere(4)
    RT = nb.HDivSurface(m, complex=True)
    ops = {p: nb.MaxwellSingleLayerPotentialOperator(RT, kappa=2.0, intorder=3, leafsize=20, eps=1e-6, precision=p)
           for p in ("fp64", "mixed")}
    x = torch.from_numpy(_x(RT.ndof, 4)).cuda()
    y64 = (ops["fp64"].mat * x).cpu().numpy()
    y32 = (ops["mixed"].mat * x).cpu().numpy()
    assert rel(y32, y64) < 1e-5


def test_maxwell_config_size_against_oracle_hmatrix(oracle):
    """The Maxwell workload's own size: RT0 on the L5 icosphere (30 720 edge dofs), kappa 2,
    leaf 20, eta 2, ACA eps 1e-6.  Both GPU paths against the oracle's H-matrix of the same
    partition (its assembly takes about ten seconds on the host cores), product and transposed
    product, within the ACA tolerance; the block lists are equal block for block."""
    m = icosphere(5)
    RT = nb.HDivSurface(m, complex=True)
    H = oracle.OracleOperator("maxwell_sl", m, "RT0", kappa=2.0, trial_eval="maxwell", intorder=3, leafsize=20,
                              eta=2.0, eps=1e-6)
    x = _x(RT.ndof, 5)
    yo, yto = H.mult(x), H.mult(x, trans=True)
    ob = H.blocks()
    for precision in ("fp64", "mixed"):
        op = nb.MaxwellSingleLayerPotentialOperator(RT, kappa=2.0, intorder=3, leafsize=20, eta=2.0, eps=1e-6,
                                                    precision=precision)
        b = op.mat.blocks()
        for k in ("rowcl", "colcl", "near"):
            assert np.array_equal(b[k], ob[k])
        xd = torch.from_numpy(x).cuda()
        assert rel((op.mat * xd).cpu().numpy(), yo) < 1e-5
        assert rel((op.mat.T * xd).cpu().numpy(), yto) < 1e-5
        del op
