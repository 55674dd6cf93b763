"""HDivSurface and HCurl of order 1 to 4 on the CPU (the reference's Maxwell tests use higher-order
HDivSurface: tests/test_Maxwell_Mie.py:24).  The oracle's basis against the properties that
define the space, and the library's spaces against the oracle's:

* normal continuity: on every interior edge the flux of each global function through the edge
  is the same from both sides (outward conormals opposite), and functions of one element only
  have no flux through it;
* the divergence trace: on every element the integral of the surface divergence equals the
  flux through the element's boundary (divergence theorem), for every local function;
* the span: on one flat triangle the (K + 1)(K + 2) functions span all tangential vector
  polynomials of degree K;
* the lowest-order dofs are the RT0 functions with RT0's numbering;
* dof tables, cluster trees and partitions of the library equal the oracle's, bit for bit;
* the reference's Mie test at order 4 with the oracle's operator: the current against the Mie
  series within the reference's bar;
* HCurl of order 1..4 (n x those shapes): tangential continuity, the order-0 HCurl functions as
  its lowest-order part, the library's space and load vectors against the oracle.
"""
import numpy as np
import pytest

import ngbem_gb300 as nb
from ngbem_gb300.forms import triangle_rule
from ngbem_gb300.meshes import ellipsoid, icosphere

GAUSS = np.polynomial.legendre.leggauss(5)


def _ref_point(k, s):
    """(xi, eta) at parameter s along local edge k from vertex k to vertex k+1."""
    v = np.array([[1.0, 0.0], [0.0, 1.0], [0.0, 0.0]])
    return (1 - s) * v[k] + s * v[(k + 1) % 3]


def _conormal(X, tri, k):
    """Outward unit conormal of local edge k of a flat triangle (in its plane)."""
    p = X[tri]
    n = np.cross(p[0] - p[2], p[1] - p[2])
    t = p[(k + 1) % 3] - p[k]
    nu = np.cross(t, n)
    nu /= np.linalg.norm(nu)
    if nu @ (p[(k + 2) % 3] - p[k]) > 0:
        nu = -nu
    return nu


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_normal_continuity(oracle, K):
    m = ellipsoid(1)
    kind = f"HDIV{K}"
    X, T = m.vertices, m.triangles
    seen = {}
    checked = 0
    for e, t in enumerate(T):
        for k in range(3):
            key = tuple(sorted((t[k], t[(k + 1) % 3])))
            if key not in seen:
                seen[key] = (e, k)
                continue
            e1, k1 = seen[key]
            nu1, nu2 = _conormal(X, T[e1], k1), _conormal(X, t, k)
            for s in (0.17, 0.5, 0.83):
                # the same physical point from both elements
                x1 = _ref_point(k1, s)
                s2 = s if T[e1][k1] == t[k] else 1 - s
                x2 = _ref_point(k, s2)
                S1, d1 = oracle.eval_trace(m, kind, "id", e1, *x1)
                S2, d2 = oracle.eval_trace(m, kind, "id", e, *x2)
                f1 = dict(zip(d1.tolist(), S1[:, :3] @ nu1))
                f2 = dict(zip(d2.tolist(), S2[:, :3] @ nu2))
                for d in set(f1) | set(f2):
                    assert abs(f1.get(d, 0.0) + f2.get(d, 0.0)) < 1e-13
            checked += 1
    assert checked == len(seen) > 0  # a closed surface: every edge is shared


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_divergence_theorem(oracle, K):
    m = icosphere(1)
    kind = f"HDIV{K}"
    X, T = m.vertices, m.triangles
    xi, eta, w = triangle_rule(6)
    for e in (0, 11, 47):
        p = X[T[e]]
        detj = np.linalg.norm(np.cross(p[0] - p[2], p[1] - p[2]))
        lhs = sum(w[q] * detj * oracle.eval_trace(m, kind, "maxwell", e, xi[q], eta[q])[0][:, 3]
                  for q in range(len(w)))
        rhs = 0.0
        for k in range(3):
            nu = _conormal(X, T[e], k)
            length = np.linalg.norm(p[(k + 1) % 3] - p[k])
            for g, wg in zip(*GAUSS):
                S, _ = oracle.eval_trace(m, kind, "maxwell", e, *_ref_point(k, 0.5 * (g + 1)))
                rhs = rhs + 0.5 * wg * length * (S[:, :3] @ nu)
        assert np.abs(lhs - rhs).max() < 1e-12 * np.abs(rhs).max()


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_span(oracle, K):
    """On a flat triangle, every tangential field (a(x) t1 + b(x) t2) with a, b of degree K is a
    combination of the element's functions."""
    m = icosphere(1)
    kind = f"HDIV{K}"
    e = 5
    p = m.vertices[m.triangles[e]]
    t1 = p[0] - p[2]
    t2 = np.cross(np.cross(t1, p[1] - p[2]), t1)
    t1, t2 = t1 / np.linalg.norm(t1), t2 / np.linalg.norm(t2)
    xi, eta, _ = triangle_rule(2 * K + 4)
    B = np.stack([oracle.eval_trace(m, kind, "id", e, a, b)[0][:, :3] for a, b in zip(xi, eta)])  # (nq, nd, 3)
    assert B.shape[1] == (K + 1) * (K + 2)
    for i in range(K + 1):
        for j in range(K + 1 - i):
            for t in (t1, t2):
                target = ((xi ** i) * (eta ** j))[:, None] * t[None, :]
                A = B.transpose(0, 2, 1).reshape(-1, B.shape[1])
                c, *_ = np.linalg.lstsq(A, target.ravel(), rcond=None)
                assert np.abs(A @ c - target.ravel()).max() < 1e-12


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_lowest_order_dofs_are_rt0(oracle, K):
    m = icosphere(1)
    for e in (0, 30):
        S, d = oracle.eval_trace(m, f"HDIV{K}", "maxwell", e, 0.21, 0.33)
        R, dr = oracle.eval_trace(m, "RT0", "maxwell", e, 0.21, 0.33)
        for k in range(3):
            assert d[k * (K + 1)] == dr[k]
            assert np.abs(S[k * (K + 1)] - R[k]).max() < 1e-15


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_library_space_matches_the_oracle(oracle, K):
    m = ellipsoid(3).Curve(2)
    kind = f"HDIV{K}"
    sp = nb.HDivSurface(m, order=K)
    assert sp.ndof == oracle.ndof(m, kind)
    t = sp.dof_table()
    for e in (0, 200, m.nt - 1):
        assert np.array_equal(t[e], oracle.eval_trace(m, kind, "id", e, 0.2, 0.3)[1])
    assert np.array_equal(sp.global_dofs, np.arange(sp.ndof))
    for leaf in (20, 40):
        p1, ci1, cd1 = nb.cluster_tree(sp, leaf)
        p2, ci2, cd2 = oracle.cluster_tree(m, kind, leaf)
        assert np.array_equal(p1, p2) and np.array_equal(ci1, ci2)
        assert np.array_equal(cd1.view(np.int64), cd2.view(np.int64))
    part = nb.partition(sp, sp, 40, 2.0)
    ob = oracle.OracleOperator("maxwell_sl", m, kind, kappa=1.0, trial_eval="maxwell", intorder=2, leafsize=40,
                               eta=2.0, eps=1e-3).blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(part[k], ob[k])


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_hcurl_tangential_continuity_and_lowest_order(oracle, K):
    """HCurl of order K (n x the HDivSurface shapes): the tangential component along every edge
    is the same from both sides, and the lowest-order dofs are the order-0 HCurl functions."""
    m = ellipsoid(1)
    kind = f"HCURL{K}"
    X, T = m.vertices, m.triangles
    seen = {}
    for e, t in enumerate(T):
        for k in range(3):
            key = tuple(sorted((t[k], t[(k + 1) % 3])))
            if key not in seen:
                seen[key] = (e, k)
                continue
            e1, k1 = seen[key]
            tau = X[key[1]] - X[key[0]]
            for s in (0.2, 0.6):
                x1 = _ref_point(k1, s)
                x2 = _ref_point(k, s if T[e1][k1] == t[k] else 1 - s)
                S1, d1 = oracle.eval_trace(m, kind, "id", e1, *x1)
                S2, d2 = oracle.eval_trace(m, kind, "id", e, *x2)
                f1 = dict(zip(d1.tolist(), S1[:, :3] @ tau))
                f2 = dict(zip(d2.tolist(), S2[:, :3] @ tau))
                for d in set(f1) | set(f2):
                    assert abs(f1.get(d, 0.0) - f2.get(d, 0.0)) < 1e-13
    for ev in ("id", "rotatedtrace", "maxwellcurl"):
        S, d = oracle.eval_trace(m, kind, ev, 3, 0.21, 0.33)
        R, dr = oracle.eval_trace(m, "HCURL", ev, 3, 0.21, 0.33)
        for k in range(3):
            assert d[k * (K + 1)] == dr[k]
            assert np.abs(S[k * (K + 1)] - R[k]).max() < 1e-15


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_hcurl_library_space_and_load_vector(oracle, K):
    from ngbem_gb300.forms import _geometry, load_vector
    m = icosphere(2).Curve(3)
    kind = f"HCURL{K}"
    sp = nb.HCurl(m, order=K)
    assert sp.ndof == oracle.ndof(m, kind)
    assert np.array_equal(sp.dof_table()[7], oracle.eval_trace(m, kind, "id", 7, 0.2, 0.3)[1])
    p1, ci1, cd1 = nb.cluster_tree(sp, 30)
    p2, ci2, cd2 = oracle.cluster_tree(m, kind, 30)
    assert np.array_equal(p1, p2) and np.array_equal(cd1.view(np.int64), cd2.view(np.int64))

    def f(x, n):
        return np.stack([x[..., 1], x[..., 2] * x[..., 0], np.ones(x.shape[:2])], axis=-1)

    b = load_vector(sp, f, order=4)
    x, n, detj, lam, w = _geometry(m, 4)
    xi, eta, _ = triangle_rule(4)
    fv = f(x, n)
    ref = np.zeros(sp.ndof)
    for e in range(m.nt):
        for q in range(len(w)):
            S, d = oracle.eval_trace(m, kind, "id", e, xi[q], eta[q])
            ref[d] += w[q] * detj[e, q] * (S[:, :3] @ fv[e, q])
    assert np.abs(b - ref).max() < 1e-13 * np.abs(ref).max()


def test_mie_current_at_order_4(oracle):
    """The reference's Mie test (tests/test_Maxwell_Mie.py: a conducting sphere of radius 0.25,
    kappa 5, HDivSurface of order 4 on a mesh curved to order 4, intorder 16; L2 error of the
    current below 0.0015) with the oracle's dense Maxwell single layer at intorder 12 and a
    direct solve: the current against the Mie series (tests/_mie.py)."""
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from _mie import mie_current
    from ngbem_gb300.forms import _geometry, _lagrange, hdiv_fields, load_vector
    a, kappa = 0.25, 5.0
    m = icosphere(1, radius=a).Curve(4)
    sp = nb.HDivSurface(m, order=4, complex=True)
    V = oracle.dense_matrix("maxwell_sl", m, "HDIV4", kappa=kappa, trial_eval="maxwell", intorder=12)
    b = load_vector(sp, lambda x, n: 1j * np.stack([np.exp(1j * kappa * x[..., 2]), 0 * x[..., 2],
                                                   0 * x[..., 2]], -1), order=14)
    J = np.linalg.solve(V, b)
    x, n, detj, lam, w = _geometry(m, 12)
    xi, eta, _ = triangle_rule(12)
    _, Dxi, Deta = _lagrange(4, xi, eta)
    J0 = np.einsum("qn,tnc->tqc", Dxi, m.curve_nodes)
    J1 = np.einsum("qn,tnc->tqc", Deta, m.curve_nodes)
    fields, _ = hdiv_fields(4, lam, sp.element_dofs()[1])
    psi = (J0[:, :, None, :] * fields[..., 0, None] + J1[:, :, None, :] * fields[..., 1, None]) / detj[:, :, None, None]
    Jh = np.einsum("tqac,ta->tqc", psi, J[sp.dof_table()])
    Jm = mie_current(x.reshape(-1, 3), a, kappa).reshape(x.shape)
    W = w[None, :] * detj
    err = np.sqrt(np.einsum("tq,tqc->", W, np.abs(Jh - Jm) ** 2))
    assert err < 0.0015
    assert err / np.sqrt(np.einsum("tq,tqc->", W, np.abs(Jm) ** 2)) < 5e-4
