"""HDivSurface and HCurl of order 1 to 4 on the GPU against the FP64 oracle (the reference's
Maxwell tests use higher orders: tests/test_Maxwell_Mie.py:24, tests/test_Maxwell_Box.py:19-21).

* The Maxwell single layer (DiffOpMaxwellNew traces, src/diffops.hpp:263-338): dense FP64
  within 1e-10 of the oracle on flat and curved meshes; its block on the lowest-order dofs is
  the RT0 operator.
* H-matrices within the ACA tolerance of the oracle's in both directions with the same block
  lists; mixed precision within 1e-6 of FP64.
* Potentials and mass matrices against the oracle.
* HCurl of order 1, 2: the curl single layer and the Maxwell double layer (HCurl to HDivSurface
  or HCurl) against the oracle, with their lowest-order blocks the order-0 operators; and the
  Calderon identity of the reference's Maxwell test, V j = (-1/2 M + K) m, on the exact traces
  of a dipole field, whose residual falls with the order.
* Orders 3 and 4 (the reference's Maxwell tests): the single layer on HDivSurface of order 3, 4,
  the double layer from HCurl to HDivSurface of order 3 (dense, H-matrix, mixed, potential,
  mass), and the Calderon identity at order 3.
* The reference's Maxwell box test (tests/test_Maxwell_Box.py: V j = (-1/2 M + K) m solved with
  GMRES for a dipole field, the current's L2 error below 0.015 at order 3) on the curved sphere.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import ellipsoid, icosphere

pytestmark = pytest.mark.gpu

KAPPA = 2.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _op(sp, method="aca", precision="fp64", **kw):
    prm = dict(intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    prm.update(kw)
    io = prm.pop("intorder")
    return bem.IntegralOperator("maxwell_sl", KAPPA, sp, sp, "maxwell", "maxwell", io, prm.pop("leafsize"),
                                prm.pop("eta"), prm.pop("eps"), method, False, precision=precision, **prm)


@pytest.mark.parametrize("g", [1, 3])
@pytest.mark.parametrize("K", [1, 2])
def test_dense_parity(oracle, K, g):
    m = icosphere(1).Curve(g)
    sp = nb.HDivSurface(m, order=K, complex=True)
    D = _op(sp, "dense", intorder_singular=4, intorder_regular=3).mat.to_dense()
    Do = oracle.dense_matrix("maxwell_sl", m, f"HDIV{K}", kappa=KAPPA, trial_eval="maxwell", intorder_singular=4,
                             intorder_regular=3)
    assert D.shape == (sp.ndof, sp.ndof)
    assert rel(D, Do) < 1e-10
    # the lowest-order dofs carry the RT0 functions with RT0's numbering
    rt = nb.HDivSurface(m, order=0, complex=True)
    R = _op(rt, "dense", intorder_singular=4, intorder_regular=3).mat.to_dense()
    assert rel(D[: rt.ndof, : rt.ndof], R) < 1e-12


@pytest.mark.parametrize("K", [1, 2])
def test_hmatrix_parity(oracle, K):
    m = ellipsoid(3 if K == 1 else 2, (1.0, 0.8, 0.6)).Curve(2)
    kind = f"HDIV{K}"
    sp = nb.HDivSurface(m, order=K, complex=True)
    op = _op(sp)
    H = oracle.OracleOperator("maxwell_sl", m, kind, kappa=KAPPA, trial_eval="maxwell", intorder=3, leafsize=40,
                              eta=2.0, eps=1e-8)
    b, ob = op.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    rng = np.random.default_rng(31 + K)
    x = rng.standard_normal(sp.ndof) + 1j * rng.standard_normal(sp.ndof)
    xd = torch.from_numpy(x).cuda()
    y = (op.mat * xd).cpu().numpy()
    assert rel(y, H.mult(x)) < 1e-7
    yt = op.mat.CreateRowVector()
    op.mat.MultTrans(xd, yt)
    assert rel(yt.cpu().numpy(), H.mult(x, trans=True)) < 1e-7
    y32 = (_op(sp, precision="mixed").mat * xd).cpu().numpy()
    assert rel(y32, y) < 1e-6


@pytest.mark.parametrize("K", [1, 2])
def test_potential_and_mass(oracle, K):
    m = icosphere(2).Curve(3)
    kind = f"HDIV{K}"
    sp = nb.HDivSurface(m, order=K, complex=True)
    rng = np.random.default_rng(5)
    dens = rng.standard_normal(sp.ndof) + 1j * rng.standard_normal(sp.ndof)
    pts = np.array([[2.0, 0.3, -0.1], [0.1, 0.2, 0.3], [-1.5, 1.0, 0.5]])
    op = _op(sp)
    val = op.GetPotential(torch.from_numpy(dens).cuda())(pts).cpu().numpy().reshape(len(pts), -1)
    ref = oracle.potential("maxwell_sl", m, kind, dens, pts, kappa=KAPPA, trial_eval="maxwell",
                           intorder=3).reshape(len(pts), -1)
    assert rel(val, ref) < 1e-11
    M = nb.MassOperator(sp, sp)
    x = rng.standard_normal(sp.ndof)
    y = (M * torch.from_numpy(x).to(torch.complex128 if M.is_complex else torch.float64).cuda()).cpu().numpy()
    assert rel(y, oracle.mass_matrix(m, kind, kind, order=4) @ x) < 1e-12


HC_COMBOS = [("maxwell_sl", "HCURL", "HCURL", "maxwellcurl", "maxwellcurl"),
             ("maxwell_dl", "HCURL", "HDIV", "rotatedtrace", "id"),
             ("maxwell_dl", "HCURL", "HCURL", "rotatedtrace", "id")]
ORDER0 = {"HCURL": "HCURL", "HDIV": "RT0"}


def _space(m, fam, K):
    kind = (fam + str(K)) if K else ORDER0[fam]
    return kind, nb.TraceSpace(m, kind, complex=True)


@pytest.mark.parametrize("g", [1, 3])
@pytest.mark.parametrize("K", [1, 2])
@pytest.mark.parametrize("kernel,ftr,fte,e1,e2", HC_COMBOS, ids=[f"{c[0]}-{c[2]}" for c in HC_COMBOS])
def test_hcurl_dense_parity(oracle, kernel, ftr, fte, e1, e2, K, g):
    m = icosphere(1).Curve(g)
    (ktr, str_), (kte, ste) = _space(m, ftr, K), _space(m, fte, K)
    kw = dict(intorder_singular=4, intorder_regular=3)
    D = bem.IntegralOperator(kernel, KAPPA, str_, ste, e1, e2, 3, 40, 2.0, 1e-8, "dense", False, **kw).mat.to_dense()
    Do = oracle.dense_matrix(kernel, m, ktr, kte, kappa=KAPPA, trial_eval=e1, test_eval=e2, **kw)
    assert rel(D, Do) < 1e-10
    (_, s0), (_, t0) = _space(m, ftr, 0), _space(m, fte, 0)
    R = bem.IntegralOperator(kernel, KAPPA, s0, t0, e1, e2, 3, 40, 2.0, 1e-8, "dense", False, **kw).mat.to_dense()
    assert rel(D[: t0.ndof, : s0.ndof], R) < 1e-12


def test_hcurl_hmatrix_potential_and_mass(oracle):
    m = ellipsoid(2, (1.0, 0.8, 0.6)).Curve(2)
    HC, HD = nb.HCurl(m, order=1, complex=True), nb.HDivSurface(m, order=1, complex=True)
    op = nb.MaxwellDoubleLayerPotentialOperator(HC, HD, KAPPA, intorder=3, leafsize=40, eps=1e-8)
    H = oracle.OracleOperator("maxwell_dl", m, "HCURL1", "HDIV1", kappa=KAPPA, trial_eval="rotatedtrace",
                              test_eval="id", intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    b, ob = op.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    rng = np.random.default_rng(41)
    x = rng.standard_normal(HC.ndof) + 1j * rng.standard_normal(HC.ndof)
    assert rel((op.mat * torch.from_numpy(x).cuda()).cpu().numpy(), H.mult(x)) < 1e-7
    pts = np.array([[2.0, 0.3, -0.1], [-1.5, 1.0, 0.5]])
    for kernel, ev, o in (("maxwell_dl", "rotatedtrace", op),
                          ("maxwell_sl", "maxwellcurl",
                           nb.MaxwellSingleLayerPotentialOperatorCurl(HC, KAPPA, intorder=3, eps=1e-8))):
        val = o.GetPotential(torch.from_numpy(x).cuda())(pts).cpu().numpy().reshape(len(pts), -1)
        ref = oracle.potential(kernel, m, "HCURL1", x, pts, kappa=KAPPA, trial_eval=ev, intorder=3)
        assert rel(val, ref.reshape(len(pts), -1)) < 1e-11
    M = nb.MassOperator(HC, HD, complex=True)
    y = (M * torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel(y, oracle.mass_matrix(m, "HCURL1", "HDIV1", order=4) @ x) < 1e-12


def test_calderon_identity_higher_order(oracle):
    """The reference's Maxwell test identity V j = (-1/2 M + K) m with the L2 projections of the
    exact traces of a dipole field, on the curved sphere: the residual falls with the order.
    Order 1 keeps the piecewise-constant divergences of order 0 (BDM_1), which bound the
    single layer's div-div part, so its gain is small; order 2 has linear divergences
    (measured on a GB300: 6.9e-3, 4.0e-3, 2.6e-4)."""
    from _maxwell_fields import calderon_residual, curl, field
    from ngbem_gb300.forms import load_vector
    m = icosphere(2).Curve(3)
    kappa = 1.0
    res = []
    for K in (0, 1, 2):
        HC, HD = nb.HCurl(m, order=K, complex=True), nb.HDivSurface(m, order=K, complex=True)
        kc, kd = HC.kind, HD.kind

        def mex(x, n):
            return -np.cross(np.cross(n, field(x, kappa)), n)

        def jex(x, n):
            return np.cross(n, curl(x, kappa) / kappa)

        mh = np.linalg.solve(oracle.mass_matrix(m, kc, kc, order=8), load_vector(HC, mex, order=10))
        jh = np.linalg.solve(oracle.mass_matrix(m, kd, kd, order=8), load_vector(HD, jex, order=10))
        kw = dict(intorder=6, leafsize=40, eps=1e-10)
        V = nb.MaxwellSingleLayerPotentialOperator(HD, kappa, **kw)
        Kop = nb.MaxwellDoubleLayerPotentialOperator(HC, HD, kappa, **kw)
        M = nb.MassOperator(HC, HD, complex=True)

        def mv(A, v):
            return (A * torch.from_numpy(np.ascontiguousarray(v)).cuda()).cpu().numpy()

        res.append(calderon_residual(mv(V.mat, jh), mv(Kop.mat, mh), mv(M, mh)))
    assert res[1] < 0.8 * res[0] and res[2] < 0.1 * res[1], res


@pytest.mark.parametrize("g", [1, 3])
@pytest.mark.parametrize("K", [3, 4])
def test_order_3_4_single_layer(oracle, K, g):
    """The Maxwell single layer on HDivSurface of order 3 and 4 (the orders of the reference's
    Maxwell tests; 20 and 30 dofs per element) against the oracle, dense, with its lowest-order
    block the RT0 operator."""
    m = icosphere(1).Curve(g)
    sp = nb.HDivSurface(m, order=K, complex=True)
    D = _op(sp, "dense", intorder_singular=4, intorder_regular=3).mat.to_dense()
    Do = oracle.dense_matrix("maxwell_sl", m, f"HDIV{K}", kappa=KAPPA, trial_eval="maxwell", intorder_singular=4,
                             intorder_regular=3)
    assert rel(D, Do) < 1e-10
    rt = nb.HDivSurface(m, order=0, complex=True)
    R = _op(rt, "dense", intorder_singular=4, intorder_regular=3).mat.to_dense()
    assert rel(D[: rt.ndof, : rt.ndof], R) < 1e-12


def test_order_3_double_layer_hmatrix_potential_mass(oracle):
    m = icosphere(2).Curve(3)
    HC, HD = nb.HCurl(m, order=3, complex=True), nb.HDivSurface(m, order=3, complex=True)
    kw = dict(intorder=3, leafsize=40, eps=1e-8)
    K3 = nb.MaxwellDoubleLayerPotentialOperator(HC, HD, KAPPA, **kw)
    H = oracle.OracleOperator("maxwell_dl", m, "HCURL3", "HDIV3", kappa=KAPPA, trial_eval="rotatedtrace",
                              test_eval="id", intorder=3, leafsize=40, eta=2.0, eps=1e-8)
    b, ob = K3.mat.blocks(), H.blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(b[k], ob[k])
    rng = np.random.default_rng(43)
    x = rng.standard_normal(HC.ndof) + 1j * rng.standard_normal(HC.ndof)
    xd = torch.from_numpy(x).cuda()
    y = (K3.mat * xd).cpu().numpy()
    assert rel(y, H.mult(x)) < 1e-7
    y32 = (nb.MaxwellDoubleLayerPotentialOperator(HC, HD, KAPPA, precision="mixed", **kw).mat * xd).cpu().numpy()
    assert rel(y32, y) < 1e-6
    pts = np.array([[2.0, 0.3, -0.1], [-1.5, 1.0, 0.5]])
    val = K3.GetPotential(xd)(pts).cpu().numpy().reshape(len(pts), -1)
    ref = oracle.potential("maxwell_dl", m, "HCURL3", x, pts, kappa=KAPPA, trial_eval="rotatedtrace", intorder=3)
    assert rel(val, ref.reshape(len(pts), -1)) < 1e-11
    M = nb.MassOperator(HC, HD, complex=True)
    assert rel((M * xd).cpu().numpy(), oracle.mass_matrix(m, "HCURL3", "HDIV3", order=6) @ x) < 1e-12


def test_calderon_identity_order_3(oracle):
    """The identity of the reference's Maxwell test (tests/test_Maxwell_Box.py uses order 3) on
    the curved sphere: the residual at order 3 is below order 2's."""
    from _maxwell_fields import calderon_residual, curl, field
    from ngbem_gb300.forms import load_vector
    m = icosphere(2).Curve(3)
    kappa = 1.0
    res = []
    for K in (2, 3):
        HC, HD = nb.HCurl(m, order=K, complex=True), nb.HDivSurface(m, order=K, complex=True)

        def mex(x, n):
            return -np.cross(np.cross(n, field(x, kappa)), n)

        def jex(x, n):
            return np.cross(n, curl(x, kappa) / kappa)

        mh = np.linalg.solve(oracle.mass_matrix(m, HC.kind, HC.kind, order=10), load_vector(HC, mex, order=12))
        jh = np.linalg.solve(oracle.mass_matrix(m, HD.kind, HD.kind, order=10), load_vector(HD, jex, order=12))
        kw = dict(intorder=7, leafsize=40, eps=1e-11)
        V = nb.MaxwellSingleLayerPotentialOperator(HD, kappa, **kw)
        Kop = nb.MaxwellDoubleLayerPotentialOperator(HC, HD, kappa, **kw)
        M = nb.MassOperator(HC, HD, complex=True)

        def mv(A, v):
            return (A * torch.from_numpy(np.ascontiguousarray(v)).cuda()).cpu().numpy()

        res.append(calderon_residual(mv(V.mat, jh), mv(Kop.mat, mh), mv(M, mh)))
    assert res[1] < 0.5 * res[0], res


def _hdiv_values(sp, coef, order):
    """Values (nt, nq, 3) of the HDivSurface function with coefficients coef at the points of a
    triangle rule on every element, and the weights w |J| (nt, nq)."""
    from ngbem_gb300.forms import _geometry, _lagrange, hdiv_fields, triangle_rule
    m = sp.mesh
    x, n, detj, lam, w = _geometry(m, order)
    xi, eta, _ = triangle_rule(order)
    _, Dxi, Deta = _lagrange(m.curve_order, xi, eta)
    J0 = np.einsum("qn,tnc->tqc", Dxi, m.curve_nodes)
    J1 = np.einsum("qn,tnc->tqc", Deta, m.curve_nodes)
    _, signs = sp.element_dofs()
    fields, _ = hdiv_fields(int(sp.kind[4:]), lam, signs)
    psi = (J0[:, :, None, :] * fields[..., 0, None] + J1[:, :, None, :] * fields[..., 1, None]) / detj[:, :, None, None]
    return x, n, np.einsum("tqac,ta->tqc", psi, coef[sp.dof_table()]), w[None, :] * detj


def test_reference_maxwell_box_pattern(oracle):
    """tests/test_Maxwell_Box.py on the curved unit sphere: the dipole field's current j solved
    from V j = (-1/2 M + K) m with GMRES (m the L2 projection of the exact tangential trace), at
    orders 1, 2, 3; the relative L2 error of j falls with the order and meets the reference
    test's bar (0.015) at order 3."""
    from _maxwell_fields import curl, field
    from ngbem_gb300.forms import load_vector
    m = icosphere(1).Curve(3)
    kappa = 1.0
    errs = []
    for K in (1, 2, 3):
        HC, HD = nb.HCurl(m, order=K, complex=True), nb.HDivSurface(m, order=K, complex=True)
        mh = np.linalg.solve(oracle.mass_matrix(m, HC.kind, HC.kind, order=10),
                             load_vector(HC, lambda x, n: -np.cross(np.cross(n, field(x, kappa)), n), order=12))
        kw = dict(intorder=8, leafsize=40, eps=1e-10)
        V = nb.MaxwellSingleLayerPotentialOperator(HD, kappa, **kw)
        Kop = nb.MaxwellDoubleLayerPotentialOperator(HC, HD, kappa, **kw)
        M = nb.MassOperator(HC, HD, complex=True)
        md = torch.from_numpy(mh).cuda()
        rhs = -0.5 * (M * md) + Kop.mat * md
        j = nb.GMRes(A=V.mat, b=rhs, tol=1e-10, maxsteps=2000, printrates=False)
        j = j.cpu().numpy() if isinstance(j, torch.Tensor) else np.asarray(j)
        x, n, jh, W = _hdiv_values(HD, j, 10)
        jex = np.cross(n, curl(x, kappa) / kappa)
        errs.append(float(np.sqrt(np.einsum("tq,tqc->", W, np.abs(jh - jex) ** 2) /
                                  np.einsum("tq,tqc->", W, np.abs(jex) ** 2))))
    assert errs[0] > errs[1] > errs[2], errs
    assert errs[2] < 0.015, errs


def test_reference_maxwell_mie_pattern():
    """tests/test_Maxwell_Mie.py: the electric-field integral equation of a perfectly conducting
    sphere (radius 0.25, kappa 5, a plane wave x_hat exp(i kappa z)) with the Maxwell single
    layer on HDivSurface of order 2 and 3 (mesh curved to order 4), solved directly on the
    assembled H-matrix; the current against the Mie series (tests/_mie.py).  The oracle's
    dense solve gives 8.3e-3 and 1.1e-3 (and 3.5e-4 at order 4, which tests/test_hdiv_cpu.py
    checks against the reference's bar; the GPU order-4 operator equals the oracle's by
    test_order_3_4_single_layer)."""
    from _mie import mie_current
    from ngbem_gb300.forms import load_vector
    a, kappa = 0.25, 5.0
    m = icosphere(1, radius=a).Curve(4)  # the reference curves to the element order

    def einc(x, n):
        z = x[..., 2]
        return np.stack([np.exp(1j * kappa * z), 0 * z, 0 * z], -1)

    rel_err = []
    for K in (2, 3):
        HD = nb.HDivSurface(m, order=K, complex=True)
        V = nb.MaxwellSingleLayerPotentialOperator(HD, kappa, intorder=8, leafsize=120, eta=3.0, eps=1e-10)
        b = torch.from_numpy(load_vector(HD, lambda x, n: 1j * einc(x, n), order=14)).cuda()
        A = torch.from_numpy(V.mat.to_dense()).cuda()
        J = torch.linalg.solve(A, b).cpu().numpy()
        x, n, Jh, W = _hdiv_values(HD, J, 12)
        Jm = mie_current(x.reshape(-1, 3), a, kappa).reshape(x.shape)
        rel_err.append(float(np.sqrt(np.einsum("tq,tqc->", W, np.abs(Jh - Jm) ** 2) /
                                     np.einsum("tq,tqc->", W, np.abs(Jm) ** 2))))
    assert rel_err[0] < 1e-2 and rel_err[1] < 1.3e-3 and rel_err[1] < rel_err[0] / 5, rel_err
