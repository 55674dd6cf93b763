"""Curved geometry on the GPU against the FP64 oracle (Mesh.Curve, order 2 and 3; the
reference's tests curve every mesh: tests/test_aca.py:7, tests/test_SLIntegration.py:28,
tests/test_Laplace.py:25).

* Dense FP64 operators within 1e-10 of the oracle's dense matrices for the scalar spaces and
  their traces (identity, rotated gradient, Helmholtz), with the Sauter-Schwab points mapped
  through the curved elements.
* FP64 H-matrices within the ACA tolerance of the oracle's H-matrices in both directions, with
  the same block lists; mixed precision within 1e-6 of FP64.
* Potentials and mass matrices against the oracle.
* The reference's ACA test (tests/test_aca.py:21-28) and its single-layer integration test
  (tests/test_SLIntegration.py:30-40) on curved meshes.
* The interior Dirichlet-to-Neumann map on the curved sphere: the error of the flat triangles
  (O(h^2)) is gone.
* HDivSurface and HCurl through the Piola map of the curved elements (Maxwell single and double
  layer, curl single layer), and the dual mapping of P0.
* A mesh in use cannot be curved.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.forms import load_vector
from ngbem_gb300.meshes import ellipsoid, icosphere

pytestmark = pytest.mark.gpu

# (kernel, kappa, trial kind, test kind, trial evaluator, test evaluator)
COMBOS = [("laplace_sl", 0.0, "P0", "P0", "id", "id"), ("laplace_dl", 0.0, "P1", "P0", "id", "id"),
          ("laplace_hs", 0.0, "P1", "P1", "rot", "rot"), ("helmholtz_cf", 4.0, "P1", "P1", "id", "id"),
          ("helmholtz_hs", 3.0, "P1", "P1", "helm", "helm"), ("laplace_sl", 0.0, "L2P2", "L2P2", "id", "id"),
          ("laplace_dl", 0.0, "H1P3", "L2P2", "id", "id"), ("laplace_hs", 0.0, "H1P3", "H1P3", "rot", "rot"),
          ("helmholtz_dl", 3.0, "H1P2", "H1P2", "id", "id"), ("maxwell_sl", 2.0, "RT0", "RT0", "maxwell", "maxwell"),
          ("maxwell_dl", 2.0, "HCURL", "RT0", "rotatedtrace", "id"),
          ("maxwell_sl", 2.0, "HCURL", "HCURL", "maxwellcurl", "maxwellcurl"),
          ("laplace_sl", 0.0, "P0D", "P0D", "id", "id")]
IDS = [f"{c[0]}-{c[2]}-{c[3]}" for c in COMBOS]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _space(mesh, kind):
    # P0D: P0 with the dual mapping (v = 1 / |J|)
    if kind == "P0D":
        return nb.TraceSpace(mesh, "P0", dual_mapping=True)
    return nb.TraceSpace(mesh, kind, complex=kind in ("RT0", "HCURL"))


def _okind(kind):
    return ("P0", True) if kind == "P0D" else (kind, False)


def _op(kernel, kappa, mesh, tr, te, ev_tr, ev_te, method="aca", precision="fp64", **kw):
    prm = dict(intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    prm.update(kw)
    io = prm.pop("intorder")
    s_tr, s_te = _space(mesh, tr), _space(mesh, te)
    op = bem.IntegralOperator(kernel, kappa, s_tr, s_te, ev_tr, ev_te, io, prm.pop("leafsize"), prm.pop("eta"),
                              prm.pop("eps"), method, False, precision=precision, **prm)
    return op, s_tr, s_te


@pytest.mark.parametrize("g", [2, 3, 4])
@pytest.mark.parametrize("kernel,kappa,tr,te,ev_tr,ev_te", COMBOS, ids=IDS)
def test_dense_parity(oracle, kernel, kappa, tr, te, ev_tr, ev_te, g):
    m = icosphere(1).Curve(g)
    op, s_tr, s_te = _op(kernel, kappa, m, tr, te, ev_tr, ev_te, "dense", intorder_singular=4,
                         intorder_regular=3)
    D = op.mat.to_dense()
    (otr, dtr), (ote, dte) = _okind(tr), _okind(te)
    Do = oracle.dense_matrix(kernel, m, otr, ote, kappa=kappa, trial_eval=ev_tr, test_eval=ev_te,
                             intorder_singular=4, intorder_regular=3, trial_dual=dtr, test_dual=dte)
    assert D.shape == (s_te.ndof, s_tr.ndof)
    assert rel(D, Do) < 1e-10
    # the curved operator is not the flat one
    flat, _, _ = _op(kernel, kappa, icosphere(1), tr, te, ev_tr, ev_te, "dense", intorder_singular=4,
                     intorder_regular=3)
    assert rel(flat.mat.to_dense(), Do) > 1e-4


@pytest.mark.parametrize("kernel,kappa,tr,te,ev_tr,ev_te", [COMBOS[0], COMBOS[3], COMBOS[7], COMBOS[9]],
                         ids=[IDS[0], IDS[3], IDS[7], IDS[9]])
def test_hmatrix_parity(oracle, kernel, kappa, tr, te, ev_tr, ev_te):
    m = ellipsoid(3 if tr in ("P0", "P1", "RT0") else 2, (1.0, 0.8, 0.6)).Curve(3)
    op, s_tr, s_te = _op(kernel, kappa, m, tr, te, ev_tr, ev_te)
    H = oracle.OracleOperator(kernel, m, tr, te, kappa=kappa, trial_eval=ev_tr, test_eval=ev_te, intorder=3,
                              leafsize=40, eta=2.0, eps=1e-8)
    b, ob = op.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    cplx = kappa != 0.0
    rng = np.random.default_rng(23)
    dt = torch.complex128 if cplx else torch.float64
    x = rng.standard_normal(s_tr.ndof) + (1j * rng.standard_normal(s_tr.ndof) if cplx else 0.0)
    y = (op.mat * torch.from_numpy(x).to(dt).cuda()).cpu().numpy()
    assert rel(y, H.mult(x)) < 1e-7
    z = rng.standard_normal(s_te.ndof) + (1j * rng.standard_normal(s_te.ndof) if cplx else 0.0)
    yt = op.mat.CreateRowVector()
    op.mat.MultTrans(torch.from_numpy(z).to(dt).cuda(), yt)
    assert rel(yt.cpu().numpy(), H.mult(z, trans=True)) < 1e-7
    o32, _, _ = _op(kernel, kappa, m, tr, te, ev_tr, ev_te, precision="mixed")
    xd = torch.from_numpy(x).to(dt).cuda()
    assert rel((o32.mat * xd).cpu().numpy(), y) < 1e-6


@pytest.mark.parametrize("kind", ["P1", "H1P3", "RT0", "HCURL"])
def test_potential_and_mass(oracle, kind):
    m = icosphere(2).Curve(3)
    sp = _space(m, kind)
    rng = np.random.default_rng(13)
    pts = np.array([[2.0, 0.3, -0.1], [0.1, 0.2, 0.3], [-1.5, 1.0, 0.5]])
    if kind in ("RT0", "HCURL"):
        dens = rng.standard_normal(sp.ndof) + 1j * rng.standard_normal(sp.ndof)
        ev = "maxwell" if kind == "RT0" else "maxwellcurl"
        op, _, _ = _op("maxwell_sl", 2.0, m, kind, kind, ev, ev)
        cases = [("maxwell_sl", 2.0, ev, op)]
    else:
        dens = rng.standard_normal(sp.ndof)
        cases = [(k, 0.0, "id", _op(k, 0.0, m, kind, kind, "id", "id")[0]) for k in ("laplace_sl", "laplace_dl")]
    for kernel, kappa, ev, op in cases:
        val = op.GetPotential(torch.from_numpy(dens).cuda())(pts).cpu().numpy().reshape(len(pts), -1)
        ref = oracle.potential(kernel, m, kind, dens, pts, kappa=kappa, trial_eval=ev, intorder=3).reshape(len(pts), -1)
        assert rel(val, ref) < 1e-11
    M = nb.MassOperator(sp, sp)
    x = rng.standard_normal(sp.ndof)
    y = (M * torch.from_numpy(x).to(torch.complex128 if M.is_complex else torch.float64).cuda()).cpu().numpy()
    order = 6 if kind == "H1P3" else 4
    assert rel(y, oracle.mass_matrix(m, kind, kind, order=order) @ x) < 1e-12


def test_reference_aca_pattern():
    """tests/test_aca.py on a curved mesh: Curve(3), SurfaceL2 of order 3, the ACA product
    within eps of the dense one."""
    m = ellipsoid(2, (1.0, 0.8, 0.6)).Curve(3)
    eps = 1e-6
    Vd, sp, _ = _op("laplace_sl", 0.0, m, "L2P3", "L2P3", "id", "id", "dense", intorder=10)
    Va, _, _ = _op("laplace_sl", 0.0, m, "L2P3", "L2P3", "id", "id", intorder=10, leafsize=40, eta=3.0, eps=eps)
    x = torch.from_numpy(np.random.default_rng(4711).standard_normal(sp.ndof)).cuda()
    yd, ya = Vd.mat * x, Va.mat * x
    assert (torch.linalg.vector_norm(yd - ya) / torch.linalg.vector_norm(yd)).item() < eps
    assert Va.mat.nze < Vd.mat.nze


def test_reference_sl_integration_pattern():
    """tests/test_SLIntegration.py on a curved mesh (Curve(2), SurfaceL2 of order 3): the dense
    single layer converges to the high-order one as the integration order grows."""
    m = icosphere(1).Curve(2)
    ref, _, _ = _op("laplace_sl", 0.0, m, "L2P3", "L2P3", "id", "id", "dense", intorder=20)
    R = ref.mat.to_dense()
    errs = []
    for io in (4, 6, 8, 10):
        a, _, _ = _op("laplace_sl", 0.0, m, "L2P3", "L2P3", "id", "id", "dense", intorder=io)
        errs.append(rel(a.mat.to_dense(), R))
    assert errs[-1] < 1e-6
    assert all(e2 < e1 for e1, e2 in zip(errs, errs[1:]))


def _dtn_error(mesh, oracle):
    h1 = nb.H1(mesh, order=3)
    l2 = nb.SurfaceL2(mesh, order=2)
    V = nb.SingleLayerPotentialOperator(l2, intorder=7, eps=1e-10)
    K = nb.DoubleLayerPotentialOperator(h1, l2, intorder=7, eps=1e-10)
    M = nb.MassOperator(h1, l2)

    def g(x, n):
        return x[..., 0] ** 2 - x[..., 1] ** 2

    gh = np.linalg.solve(oracle.mass_matrix(mesh, "H1P3", "H1P3", order=8), load_vector(h1, g, order=10))
    ghd = torch.from_numpy(gh).cuda()
    rhs = 0.5 * (M * ghd) + K.mat * ghd
    u = nb.GMRes(A=V.mat, b=rhs, tol=1e-11, maxsteps=400, printrates=False)
    u = u.cpu().numpy() if isinstance(u, torch.Tensor) else np.asarray(u)
    Ml2 = oracle.mass_matrix(mesh, "L2P2", "L2P2", order=8)
    c = np.linalg.solve(Ml2, load_vector(l2, lambda x, n: 2.0 * g(x, n), order=10))
    e = u - c
    return float(np.sqrt(e @ Ml2 @ e / (c @ Ml2 @ c)))


def test_dirichlet_to_neumann_on_the_curved_sphere(oracle):
    """g = x^2 - y^2 on the unit sphere has the interior Neumann data 2 g: on flat triangles the
    error stalls at the geometry's O(h^2); with Curve(3) it is far smaller."""
    flat = _dtn_error(icosphere(2), oracle)
    curved = _dtn_error(icosphere(2).Curve(3), oracle)
    assert curved < 0.1 * flat
    assert curved < 5e-3


def test_a_mesh_in_use_cannot_be_curved():
    from ngbem_gb300 import _lib
    from ngbem_gb300.bem import _MeshHandle
    m = icosphere(1)
    nb.SingleLayerPotentialOperator(nb.SurfaceL2(m), intorder=3)
    G = np.ascontiguousarray(icosphere(1).Curve(2).curve_nodes)
    rc = _lib.lib.bem_mesh_set_geometry(_MeshHandle.of(m).h, 2, G.ctypes.data_as(_lib._dp))
    assert rc == _lib.BEM_ERR_STATE


@pytest.mark.parametrize("b_curved", [True, False], ids=["both-curved", "curved-and-flat"])
def test_trial_and_test_on_two_curved_meshes(oracle, b_curved):
    """Trial space on one mesh, test space on another, at least one of them curved: the library
    joins them into one mesh of the higher geometry order (a flat mesh takes nodes on its flat
    triangles); the operator equals the block of the oracle's operator on that union."""
    from ngbem_gb300.meshes import Mesh
    a = icosphere(2).Curve(3)
    c = np.array([1.6, 0.3, -0.2])
    b0 = icosphere(1)

    def proj(x):
        d = np.asarray(x) - c
        return c + 0.4 * d / np.linalg.norm(d, axis=-1, keepdims=True)

    b = Mesh(0.4 * b0.vertices + c, b0.triangles, project=proj)
    bn = Mesh(b.vertices, b.triangles, project=proj if b_curved else (lambda x: np.asarray(x))).Curve(3).curve_nodes
    if b_curved:
        b.Curve(3)
    union = Mesh(np.vstack([a.vertices, b.vertices]), np.vstack([a.triangles, b.triangles + a.nv]))
    union.curve_order, union.curve_nodes = 3, np.ascontiguousarray(np.vstack([a.curve_nodes, bn]))
    for k, tr, te, e1, e2, kap in (("laplace_dl", "P1", "P0", "id", "id", 0.0),
                                   ("maxwell_sl", "RT0", "RT0", "maxwell", "maxwell", 2.0)):
        trs, tes = nb.TraceSpace(b, tr, complex=kap != 0), nb.TraceSpace(a, te, complex=kap != 0)
        D = bem.IntegralOperator(k, kap, trs, tes, e1, e2, 3, 10, 2.0, 1e-8, "dense", False).mat.to_dense()
        Do = oracle.dense_matrix(k, union, tr, te, kappa=kap, trial_eval=e1, test_eval=e2, intorder=3)
        Db = Do[np.ix_(np.arange(tes.ndof), oracle.ndof(a, tr) + np.arange(trs.ndof))]
        assert D.shape == Db.shape and rel(D, Db) < 1e-10
