"""Potential evaluation (bem_operator_potential; reference GetPotential / PotentialCF,
src/ngbem.cpp:1166-1301) against the FP64 oracle's restatement of the reference loop on the
same mesh, trial space and rule: every kernel family with its trial trace, points outside and
inside the sphere (and normals for the kernels that use them), 1e-11 relative.  Plus the
analytic answer for the single layer of the constant density (1/|x| outside, 1 inside)."""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu

CASES = [
    ("laplace_sl", "P0", "id", 0.0),
    ("laplace_sl", "P1", "id", 0.0),
    ("laplace_dl", "P1", "id", 0.0),
    ("laplace_hs", "P1", "rot", 0.0),
    ("helmholtz_sl", "P1", "id", 3.0),
    ("helmholtz_dl", "P0", "id", 3.0),
    ("helmholtz_cf", "P1", "id", 5.0),
    ("helmholtz_hs", "P1", "helm", 3.0),
    ("maxwell_sl", "RT0", "maxwell", 2.0),
    ("helmholtz_sl_dkappa", "P1", "id", 3.0),
    # the curl single layer on HCurl, and the double layer (HCurl rotated trace; tested with the
    # HCurl identity trace, as MaxwellDoubleLayerPotentialOperator pairs them), whose potential
    # is the reference's sum of its six cross-product terms without their signs
    ("maxwell_sl", "HCURL", "maxwellcurl", 2.0),
    ("maxwell_dl", "HCURL", "rotatedtrace", 2.0, "id"),
    # higher-order spaces with the Helmholtz kernels
    ("helmholtz_dl", "L2P2", "id", 3.0),
    ("helmholtz_cf", "L2P3", "id", 4.0),
    ("helmholtz_dl", "H1P3", "id", 3.0),
    ("helmholtz_cf", "H1P2", "id", 4.0),
]


def _points(seed):
    r = np.random.default_rng(seed)
    d = r.standard_normal((40, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    rad = np.concatenate([r.uniform(1.3, 3.0, 30), r.uniform(0.1, 0.7, 10)])
    n = r.standard_normal((40, 3))
    n /= np.linalg.norm(n, axis=1)[:, None]
    return d * rad[:, None], n


@pytest.mark.parametrize("case", CASES, ids=[c[0] + "-" + c[1] for c in CASES])
def test_potential_against_oracle(oracle, case):
    kernel, kind, ev, kappa = case[:4]
    tev = case[4] if len(case) > 4 else ev
    m = icosphere(2)
    sp = nb.TraceSpace(m, kind, complex=kernel not in ("laplace_sl", "laplace_dl", "laplace_hs"))
    op = bem.IntegralOperator(kernel, kappa, sp, sp, ev, tev, 3, 20, 2.0, 1e-8, "aca", False)
    r = np.random.default_rng(7)
    dens = r.standard_normal(sp.ndof)
    if op.mat.is_complex:
        dens = dens + 1j * r.standard_normal(sp.ndof)
    pts, nrm = _points(3)
    pot = op.GetPotential(dens)
    got = pot(pts, nrm).cpu().numpy().reshape(len(pts), -1)
    ref = oracle.potential(kernel, m, kind, dens, pts, normals=nrm, kappa=kappa, trial_eval=ev, intorder=3)
    assert got.shape == ref.shape
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-11


def test_single_layer_potential_of_one():
    m = icosphere(4)
    P0 = nb.SurfaceL2(m)
    V = nb.SingleLayerPotentialOperator(P0, intorder=4)
    pts = np.array([[0.0, 0.0, 2.0], [1.5, 1.0, 0.5], [0.1, -0.2, 0.3]])
    u = V.GetPotential(np.ones(P0.ndof))(pts).cpu().numpy()
    r = np.linalg.norm(pts, axis=1)
    assert np.allclose(u, [1.0 / r[0], 1.0 / r[1], 1.0], rtol=5e-3)
