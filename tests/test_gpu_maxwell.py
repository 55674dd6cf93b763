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
