"""Batched single-layer energy and shape gradient (bem_sl_batch_*) on the GPU.

* The energy u^T V u and V u against the FP64 oracle's dense single-layer matrix on the same
  perturbed meshes and rules (1e-11 relative; the rules are identical).
* dE/dX against central finite differences of the same discrete energy (h = 1e-6, FP64):
  single coordinates and a random direction, relative to the gradient's scale, 1e-5.
* The torch.autograd.Function: X.grad, u.grad = 2 V u and per-problem weights.
* Mixed precision (FP32 regular pairs) against FP64: energy 1e-6, gradient 1e-5.
* The wavenumber derivative of the Helmholtz single-layer energy (HelmholtzEnergy) against
  central differences in kappa and in u, 1e-6.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import icosphere, perturbed_icosphere
from ngbem_gb300.shape import SingleLayerEnergyBatch, SingleLayerEnergy

pytestmark = pytest.mark.gpu


def _batch(levels, precision="fp64", dual=False, seed=7):
    meshes = [perturbed_icosphere(L, 0.05, seed + k) for k, L in enumerate(levels)]
    return meshes, SingleLayerEnergyBatch(meshes, intorder=3, intorder_singular=4, precision=precision,
                                          dual_mapping=dual)


def _density(batch, seed=3):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(batch.nt_total, dtype=torch.float64, generator=g).cuda()


@pytest.mark.parametrize("dual", [False, True])
def test_energy_matches_oracle(oracle, dual):
    meshes, b = _batch([1, 2, 1], dual=dual)
    X, u = b.coordinates(), _density(b)
    E, Vu, _ = b.evaluate(X, u, vu=True)
    un = u.cpu().numpy()
    for k, m in enumerate(meshes):
        V = oracle.dense_matrix("laplace_sl", m, "P0", "P0", intorder_singular=4, intorder_regular=3,
                                trial_dual=dual, test_dual=dual)
        t0, t1 = b.triangle_offsets[k], b.triangle_offsets[k + 1]
        uk = un[t0:t1]
        vu_ref = V @ uk
        assert np.linalg.norm(Vu.cpu().numpy()[t0:t1] - vu_ref) / np.linalg.norm(vu_ref) < 1e-11
        e_ref = uk @ vu_ref
        assert abs(E[k].item() - e_ref) / abs(e_ref) < 1e-11


def _energy(b, X, u):
    E, _, _ = b.evaluate(X, u)
    return E.double().cpu().numpy()


def test_gradient_matches_finite_differences():
    meshes, b = _batch([1, 2])
    X, u = b.coordinates(), _density(b)
    _, _, G = b.evaluate(X, u, grad=True, energy=False)
    G = G.cpu().numpy()
    scale = np.abs(G).max()
    h = 1e-6
    rng = np.random.default_rng(11)
    prob_of_vertex = np.searchsorted(b.vertex_offsets, np.arange(b.nv_total), side="right") - 1
    for _ in range(16):
        v, c = int(rng.integers(b.nv_total)), int(rng.integers(3))
        Xp, Xm = X.clone(), X.clone()
        Xp[v, c] += h
        Xm[v, c] -= h
        k = prob_of_vertex[v]
        fd = (_energy(b, Xp, u)[k] - _energy(b, Xm, u)[k]) / (2 * h)
        assert abs(fd - G[v, c]) < 1e-5 * scale, (v, c, fd, G[v, c])
    # directional derivative over all coordinates at once
    d = torch.as_tensor(rng.standard_normal((b.nv_total, 3)), device="cuda")
    fd = (_energy(b, X + h * d, u) - _energy(b, X - h * d, u)) / (2 * h)
    dn = d.cpu().numpy()
    for k in range(b.nprob):
        s = slice(b.vertex_offsets[k], b.vertex_offsets[k + 1])
        an = float((G[s] * dn[s]).sum())
        assert abs(fd[k] - an) < 1e-6 * max(abs(an), 1.0), (k, fd[k], an)


def test_autograd_function():
    _, b = _batch([1, 2, 2])
    X = b.coordinates().requires_grad_(True)
    u = _density(b).requires_grad_(True)
    w = torch.tensor([0.5, -2.0, 1.5], dtype=torch.float64, device="cuda")
    E = SingleLayerEnergy.apply(X, u, b)
    (E * w).sum().backward()
    _, Vu, G = b.evaluate(X.detach(), u.detach(), weights=w, vu=True, grad=True)
    assert torch.allclose(X.grad, G, rtol=0, atol=1e-13 * G.abs().max().item())
    wt = w[b.triangle_problem]
    ref = 2.0 * Vu * wt
    # FP64 atomics add in a different order on each call: compare against the vector's scale
    assert torch.allclose(u.grad, ref, rtol=0, atol=1e-12 * ref.abs().max().item())
    # energy through the callable form equals the raw evaluation
    E2 = b(X.detach(), u.detach())
    assert torch.allclose(E2, E.detach(), rtol=1e-14, atol=0)


def test_mixed_precision_against_fp64():
    meshes, b64 = _batch([3, 2])
    _, b32 = _batch([3, 2], precision="mixed")
    X, u = b64.coordinates(), _density(b64)
    E64, _, G64 = b64.evaluate(X, u, grad=True)
    E32, _, G32 = b32.evaluate(X, u, grad=True)
    assert ((E32 - E64).abs() / E64.abs()).max().item() < 1e-6
    assert (torch.linalg.vector_norm(G32 - G64) / torch.linalg.vector_norm(G64)).item() < 1e-5


def test_batch_argument_errors():
    _, b = _batch([1])
    X, u = b.coordinates(), _density(b)
    with pytest.raises(ValueError):
        b.evaluate(X[:-1], u)
    with pytest.raises(TypeError):
        b.evaluate(X.float(), u)


def test_helmholtz_energy_kappa_derivative():
    """dE/dkappa and dE/du of E(kappa, u) = u^T V_kappa u (Helmholtz single layer, P0, L2) from
    the kappa-derivative operator, against central differences (h = 1e-5) of the plain FP64
    operator; the derivative operator against FD of the matrix itself is in the parity tests."""
    from ngbem_gb300.shape import HelmholtzEnergy
    m = icosphere(2)
    P0 = nb.SurfaceL2(m)
    en = HelmholtzEnergy(P0, intorder=4, method="dense")
    g = torch.Generator().manual_seed(5)
    u = torch.randn(P0.ndof, generator=g, dtype=torch.float64).cuda().requires_grad_(True)
    kappa = torch.tensor(2.5, dtype=torch.float64, device="cuda", requires_grad=True)
    E = en(kappa, u)
    w = torch.tensor([0.7, -0.3], dtype=torch.float64, device="cuda")
    (E * w).sum().backward()
    h = 1e-5
    with torch.no_grad():
        Ep = en(torch.tensor(2.5 + h, dtype=torch.float64, device="cuda"), u)
        Em = en(torch.tensor(2.5 - h, dtype=torch.float64, device="cuda"), u)
    fd = float(((Ep - Em) / (2 * h) * w).sum())
    assert abs(float(kappa.grad) - fd) <= 1e-6 * abs(fd)
    d = torch.randn(P0.ndof, generator=g, dtype=torch.float64).cuda()
    with torch.no_grad():
        Up = en(kappa.detach(), u + h * d)
        Um = en(kappa.detach(), u - h * d)
    fdu = float(((Up - Um) / (2 * h) * w).sum())
    assert abs(float(torch.dot(u.grad, d)) - fdu) <= 1e-6 * abs(fdu)
