"""H1 of order 2 and 3 on the CPU: the oracle's hierarchical basis against its known
properties (continuity across edges, its surface curl against finite differences, exact
L2 projection of polynomials of degree p), and the library's spaces (dof tables, cluster
trees, partitions) against the oracle's, bit for bit.  The reference's Laplace test
(tests/test_Laplace.py:23-45) uses H1 of order 3 with SurfaceL2 of order 2.
"""
import numpy as np
import pytest

import ngbem_gb300 as nb
from ngbem_gb300.forms import _geometry, h1p_shapes, load_vector, triangle_rule
from ngbem_gb300.meshes import ellipsoid, icosphere


def _edge_pairs(mesh, count):
    """(element, local edge, element, local edge) of the first `count` interior edges."""
    seen, out = {}, []
    for e, t in enumerate(mesh.triangles):
        for k in range(3):
            key = tuple(sorted((t[k], t[(k + 1) % 3])))
            if key in seen:
                e1, k1 = seen[key]
                out.append((e1, k1, e, k))
                if len(out) == count:
                    return out
            else:
                seen[key] = (e, k)
    return out


def _point_on_edge(tri, k, vfirst, s):
    """(xi, eta) of the point (1 - s) v + s w on local edge k of a triangle, v = vertex vfirst."""
    lam = np.zeros(3)
    i, j = k, (k + 1) % 3
    if tri[i] == vfirst:
        lam[i], lam[j] = 1 - s, s
    else:
        lam[j], lam[i] = 1 - s, s
    return lam[0], lam[1]


@pytest.mark.parametrize("p", [2, 3])
def test_basis_is_continuous_across_edges(oracle, p):
    """Every global function takes the same values on an edge from both of its elements, and
    the functions of one element that the other lacks vanish on the edge."""
    m = ellipsoid(1)
    kind = f"H1P{p}"
    for e1, k1, e2, k2 in _edge_pairs(m, 25):
        v = m.triangles[e1][k1]
        for s in (0.13, 0.5, 0.77):
            x1 = _point_on_edge(m.triangles[e1], k1, v, s)
            x2 = _point_on_edge(m.triangles[e2], k2, v, s)
            a1, d1 = oracle.eval_trace(m, kind, "id", e1, *x1)
            a2, d2 = oracle.eval_trace(m, kind, "id", e2, *x2)
            f1 = dict(zip(d1.tolist(), a1[:, 0]))
            f2 = dict(zip(d2.tolist(), a2[:, 0]))
            for d in set(f1) | set(f2):
                assert abs(f1.get(d, 0.0) - f2.get(d, 0.0)) < 1e-14


@pytest.mark.parametrize("p", [2, 3])
def test_rot_trace_is_the_surface_curl(oracle, p):
    """The ROT trace n x grad_Gamma phi: (rot x n) . J0 and . J1 (J the columns of the element
    map) are the derivatives of phi in xi and eta (central differences)."""
    m = ellipsoid(1)
    kind = f"H1P{p}"
    X, T = m.vertices, m.triangles
    h = 1e-6
    for e in (0, 7, 31):
        J0, J1 = X[T[e, 0]] - X[T[e, 2]], X[T[e, 1]] - X[T[e, 2]]
        n = np.cross(J0, J1)
        n /= np.linalg.norm(n)
        xi, eta = 0.21, 0.33
        rot, _ = oracle.eval_trace(m, kind, "rot", e, xi, eta)
        grad = np.cross(rot[:, :3], n)
        dxi = (oracle.eval_trace(m, kind, "id", e, xi + h, eta)[0][:, 0]
               - oracle.eval_trace(m, kind, "id", e, xi - h, eta)[0][:, 0]) / (2 * h)
        deta = (oracle.eval_trace(m, kind, "id", e, xi, eta + h)[0][:, 0]
                - oracle.eval_trace(m, kind, "id", e, xi, eta - h)[0][:, 0]) / (2 * h)
        assert np.abs(grad @ J0 - dxi).max() < 1e-8
        assert np.abs(grad @ J1 - deta).max() < 1e-8


@pytest.mark.parametrize("p", [2, 3])
def test_projection_reproduces_polynomials(oracle, p):
    """A polynomial of degree p restricted to the flat triangles is continuous and of degree p on
    each: its L2 projection is itself, so b . M^-1 b = int f^2 (the library's numbering and
    load vector, the oracle's mass matrix)."""
    m = icosphere(2)
    sp = nb.H1(m, order=p)
    M = oracle.mass_matrix(m, f"H1P{p}", f"H1P{p}", order=2 * p)

    def f(x, n):
        return x[..., 0] * x[..., 1] * (x[..., 2] if p == 3 else 1.0) + 0.3 * x[..., 2] - 0.7

    b = load_vector(sp, f, order=8)
    c = np.linalg.solve(M, b)
    x, nrm, detj, lam, w = _geometry(m, 8)
    int_f2 = np.einsum("q,tq->t", w, f(x, nrm) ** 2) @ detj
    assert abs(b @ c - int_f2) < 1e-13 * int_f2


@pytest.mark.parametrize("p", [2, 3])
def test_shapes_span_the_polynomials(p):
    """On one triangle the (p+1)(p+2)/2 functions span the polynomials of degree p, for either
    orientation of the edges."""
    xi, eta, _ = triangle_rule(2 * p + 2)
    lam = np.stack([xi, eta, 1 - xi - eta], axis=1)
    for signs in ([1, 1, 1], [-1, 1, -1]):
        phi = h1p_shapes(p, lam, np.array([signs]))[0]
        for a in range(p + 1):
            for b in range(p + 1 - a):
                g = xi ** a * eta ** b
                c, *_ = np.linalg.lstsq(phi, g, rcond=None)
                assert np.abs(phi @ c - g).max() < 1e-12


@pytest.mark.parametrize("p", [2, 3])
def test_library_space_and_tree_match_the_oracle(oracle, p):
    m = icosphere(3)
    kind = f"H1P{p}"
    sp = nb.H1(m, order=p)
    assert sp.ndof == oracle.ndof(m, kind)
    t = sp.dof_table()
    for e in (0, 100, m.nt - 1):
        assert np.array_equal(t[e], oracle.eval_trace(m, kind, "id", e, 0.2, 0.3)[1])
    # every dof of the whole-mesh space maps to itself
    assert np.array_equal(sp.global_dofs, np.arange(sp.ndof))
    for leaf in (20, 40):
        p1, ci1, cd1 = nb.cluster_tree(sp, leaf)
        p2, ci2, cd2 = oracle.cluster_tree(m, kind, leaf)
        assert np.array_equal(p1, p2) and np.array_equal(ci1, ci2)
        assert np.array_equal(cd1.view(np.int64), cd2.view(np.int64))
    part = nb.partition(sp, sp, 40, 2.0)
    ob = oracle.OracleOperator("laplace_sl", m, kind, intorder=2, leafsize=40, eta=2.0, eps=1e-3).blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(part[k], ob[k])


def test_region_space_numbers_like_the_submesh():
    """H1 of order 3 on a region has the dof table of H1 of order 3 on the region's submesh, and
    global_dofs maps its dofs to the same functions of the space on the whole mesh."""
    from ngbem_gb300.meshes import Region
    m = icosphere(2)
    reg = Region(m, m.centroids()[:, 2] > 0.1)
    sp = nb.H1(m, order=3, definedon=reg)
    full = nb.H1(m, order=3)
    sub, vids, tids = m.submesh(reg)
    spsub = nb.H1(sub, order=3)
    assert sp.ndof == spsub.ndof
    tr, tf, ts = sp.dof_table(), full.dof_table(), spsub.dof_table()
    assert np.array_equal(tr[tids], ts)
    assert np.all(tr[~reg.mask] == -1)
    assert np.array_equal(sp.global_dofs[tr[tids]], tf[tids])


@pytest.mark.parametrize("p", [2, 3])
def test_hypersingular_annihilates_constants(oracle, p):
    """The surface curl of a constant is zero: the oracle's hypersingular matrix on H1 of order p
    maps the constant (the vertex hats' coefficients 1, the bubbles' 0) to zero."""
    m = icosphere(1)
    kind = f"H1P{p}"
    W = oracle.OracleOperator("laplace_hs", m, kind, trial_eval="rot", intorder=4, method="dense").to_dense()
    one = np.zeros(oracle.ndof(m, kind))
    one[: m.nv] = 1.0
    assert np.abs(W @ one).max() < 1e-12 * np.abs(W).max()
