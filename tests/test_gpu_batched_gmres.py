"""Batched GMRES (bem_gmres_batched) on the Burton-Miller system (1/2 M + C) u = f with several
plane waves at once (demos/HelmholtzBurtonMiller.ipynb cell 8; P1, complex).

* FP64 H-matrices (ACA eps 1e-10): every column against the dense oracle solve, 1e-8.
* The batched solve against one single-right-hand-side GMRES per column, 1e-9.
* Mixed precision (FP32 far field, iterative refinement) against the FP64 solution, 1e-5.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.forms import p1_load_vector, plane_wave_bm_source, random_directions
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu

KAPPA = 4.0


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _system(m, precision, eps):
    P1 = nb.H1(m, complex=True)
    C_ = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=KAPPA, intorder=4, leafsize=20, eps=eps,
                                           precision=precision)
    M = nb.MassOperator(P1, P1, complex=True)
    return 0.5 * M + C_.mat


def _rhs(m, nrhs):
    d = random_directions(nrhs, 17)
    return p1_load_vector(m, plane_wave_bm_source(KAPPA, d), order=6)


def test_batched_against_dense_oracle(oracle):
    m = icosphere(2)
    A = _system(m, "fp64", 1e-10)
    F = _rhs(m, 5)
    U = nb.GMRes(A, torch.from_numpy(F).cuda(), maxsteps=300, tol=1e-12)
    assert nb.GMRes.last["residual"] < 1e-11
    assert len(nb.GMRes.last["residuals"]) == 5
    Mo = oracle.mass_matrix(m, "P1", "P1")
    Co = oracle.dense_matrix("helmholtz_cf", m, "P1", kappa=KAPPA, intorder=4)
    Uo = np.linalg.solve(0.5 * Mo + Co, F)
    Un = U.cpu().numpy()
    for r in range(F.shape[1]):
        assert rel(Un[:, r], Uo[:, r]) < 1e-8


def test_batched_equals_single_column_solves():
    m = icosphere(3)
    A = _system(m, "fp64", 1e-8)
    F = _rhs(m, 3)
    U = nb.GMRes(A, torch.from_numpy(F).cuda(), maxsteps=300, tol=1e-10).cpu().numpy()
    for r in range(F.shape[1]):
        u = nb.GMRes(A, torch.from_numpy(np.ascontiguousarray(F[:, r])).cuda(), maxsteps=300, tol=1e-10)
        assert rel(U[:, r], u.cpu().numpy()) < 1e-9


def test_batched_mixed_precision():
    m = icosphere(3)
    F = _rhs(m, 4)
    U64 = nb.GMRes(_system(m, "fp64", 1e-8), torch.from_numpy(F).cuda(), maxsteps=300, tol=1e-9).cpu().numpy()
    U32 = nb.GMRes(_system(m, "mixed", 1e-8), torch.from_numpy(F).cuda(), maxsteps=300, tol=1e-9)
    assert nb.GMRes.last["residual"] < 1e-9
    U32 = U32.cpu().numpy()
    for r in range(F.shape[1]):
        assert rel(U32[:, r], U64[:, r]) < 1e-5
