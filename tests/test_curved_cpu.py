"""Curved geometry on the CPU (Mesh.Curve; the reference's tests curve every mesh, e.g.
tests/test_aca.py:7 Curve(3), tests/test_SLIntegration.py:28 Curve(2)).

* The oracle's isoparametric map against known answers on the unit sphere: the area converges
  like h^2 for flat triangles and like h^4 for curved ones of order 2 and 3, and the Laplace
  single layer reproduces V 1 = 1 far better on the curved sphere.
* Mesh.Curve: the corner nodes are the vertices, nodes on a shared edge agree bit for bit
  between the two elements, and every node lies on the surface.
* The library's cluster trees on curved meshes equal the oracle's bit for bit (the cluster data
  read the mapped points and the curved element weights), and differ from the flat mesh's.
* Load vectors on curved meshes integrate through the map (the Piola-mapped RT0 and HCurl
  shapes against the oracle's); the C-ABI rejects bad geometry.
"""
import ctypes as C

import numpy as np
import pytest

import ngbem_gb300 as nb
from ngbem_gb300 import _lib
from ngbem_gb300.forms import load_vector
from ngbem_gb300.meshes import Mesh, ellipsoid, icosphere


def test_area_converges_with_the_geometry_order(oracle):
    err = {}
    for g in (1, 2, 3, 4):
        err[g] = [abs(oracle.mass_matrix(icosphere(lev).Curve(g), "P0", "P0", order=12).sum() - 4 * np.pi)
                  for lev in (1, 2)]
    assert 3.5 < err[1][0] / err[1][1] < 4.5          # h^2
    for g in (2, 3):
        assert err[g][0] / err[g][1] > 12.0            # h^4
        assert err[g][1] < 0.01 * err[1][1]
    assert err[4][0] / err[4][1] > 48.0                # h^6
    assert err[4][1] < 0.02 * err[3][1]


def test_single_layer_of_one_on_the_curved_sphere(oracle):
    """V 1 = 1 on the unit sphere: (V 1, v_e) = (1, v_e) for the P0 functions v_e."""
    dev = {}
    for g in (1, 3):
        m = icosphere(1).Curve(g)
        V = oracle.dense_matrix("laplace_sl", m, "P0", intorder=6)
        M = oracle.mass_matrix(m, "P0", "P0", order=10)
        dev[g] = np.abs(V.sum(1) - M.sum(1)).max() / M.sum(1).max()
    assert dev[3] < 1e-3
    assert dev[3] < 0.02 * dev[1]


@pytest.mark.parametrize("g", [2, 3, 4])
def test_curve_nodes(g):
    m = ellipsoid(2, (1.0, 0.7, 0.5)).Curve(g)
    G = m.curve_nodes
    nn = (g + 1) * (g + 2) // 2
    assert G.shape == (m.nt, nn, 3) and m.curve_order == g
    corners = [0, nn - (g + 1), nn - 1]
    for k in range(3):
        assert np.array_equal(G[:, corners[k]], m.vertices[m.triangles[:, k]])
    # every node on the ellipsoid
    assert np.abs(((G / np.array([1.0, 0.7, 0.5])) ** 2).sum(-1) - 1.0).max() < 1e-14
    # the nodes of a shared edge: the node at barycentric (i, j, 0) of (v0, v1) in one element is
    # the node at the same weights of the same vertices in the other
    idx = [(i, j, g - i - j) for i in range(g, -1, -1) for j in range(g - i, -1, -1)]
    pos = {}
    for e, t in enumerate(m.triangles):
        for n, w in enumerate(idx):
            key = tuple(sorted((int(t[a]), w[a]) for a in range(3) if w[a]))
            if key in pos:
                assert np.array_equal(pos[key], G[e, n])
            else:
                pos[key] = G[e, n]
    assert m.Curve(1).curve_order == 1 and m.curve_nodes is None


@pytest.mark.parametrize("g", [2, 3, 4])
@pytest.mark.parametrize("kind", ["P0", "P1", "L2P2", "H1P3"])
def test_cluster_trees_match_the_oracle(oracle, g, kind):
    m = ellipsoid(3).Curve(g)
    sp = nb.TraceSpace(m, kind)
    for leaf in (20, 40):
        p1, ci1, cd1 = nb.cluster_tree(sp, leaf)
        p2, ci2, cd2 = oracle.cluster_tree(m, kind, leaf)
        assert np.array_equal(p1, p2) and np.array_equal(ci1, ci2)
        assert np.array_equal(cd1.view(np.int64), cd2.view(np.int64))
    flat = nb.cluster_tree(nb.TraceSpace(ellipsoid(3), kind), 20)[2]
    assert not np.array_equal(flat, nb.cluster_tree(sp, 20)[2])
    part = nb.partition(sp, sp, 40, 2.0)
    ob = oracle.OracleOperator("laplace_sl", m, kind, intorder=2, leafsize=40, eta=2.0, eps=1e-3).blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(part[k], ob[k])


@pytest.mark.parametrize("kind", ["P0", "P1", "L2P2", "H1P3"])
def test_load_vectors_on_curved_meshes(oracle, kind):
    """b = int f v over the curved triangles: for f = 1 the sum of b over a partition of unity
    (P0, P1, and the vertex hats of H1) is the curved area, which the oracle's mass matrix gives."""
    m = icosphere(2).Curve(3)
    sp = nb.TraceSpace(m, kind)
    b = load_vector(sp, lambda x, n: np.ones(x.shape[:2]), order=10)
    area = oracle.mass_matrix(m, "P0", "P0", order=10).sum()
    if kind == "H1P3":
        b = b[: m.nv]
    if kind == "L2P2":
        b = b[:: 6]  # the constant of each element's Dubiner basis
    assert abs(b.sum() - area) < 1e-12 * area
    # normals per point on curved meshes: n . x = 1 on the unit sphere up to the map's error
    bn = load_vector(nb.TraceSpace(m, "P0"), lambda x, n: np.einsum("tqc,tqc->tq", n, x), order=10)
    assert abs(bn.sum() - area) < 1e-3 * area


def test_c_abi_rejects_bad_geometry():
    m = icosphere(1)
    X = np.ascontiguousarray(m.vertices)
    T = np.ascontiguousarray(m.triangles)
    h = C.c_void_p()
    assert _lib.lib.bem_mesh_create(m.nv, X.ctypes.data_as(_lib._dp), m.nt, T.ctypes.data_as(_lib._ip),
                                    C.byref(h)) == 0
    try:
        G = np.ascontiguousarray(icosphere(1).Curve(2).curve_nodes)
        assert _lib.lib.bem_mesh_set_geometry(h, 4, G.ctypes.data_as(_lib._dp)) == _lib.BEM_ERR_ARG
        assert _lib.lib.bem_mesh_set_geometry(h, 2, None) == _lib.BEM_ERR_ARG
        bad = G.copy()
        bad[5, 0, 1] += 1e-3  # a corner node off its vertex
        assert _lib.lib.bem_mesh_set_geometry(h, 2, bad.ctypes.data_as(_lib._dp)) == _lib.BEM_ERR_ARG
        bad = G.copy()
        bad[7, 4] = np.nan
        assert _lib.lib.bem_mesh_set_geometry(h, 2, bad.ctypes.data_as(_lib._dp)) == _lib.BEM_ERR_ARG
        assert _lib.lib.bem_mesh_set_geometry(h, 2, G.ctypes.data_as(_lib._dp)) == 0
        assert _lib.lib.bem_mesh_set_geometry(h, 1, None) == 0
        # once a space lives on the mesh, its geometry is fixed
        sp = C.c_void_p()
        assert _lib.lib.bem_space_create(h, 0, 0, C.byref(sp)) == 0
        assert _lib.lib.bem_mesh_set_geometry(h, 2, G.ctypes.data_as(_lib._dp)) == _lib.BEM_ERR_STATE
        _lib.lib.bem_space_destroy(sp)
    finally:
        _lib.lib.bem_mesh_destroy(h)


def test_mesh_without_projection_needs_one():
    m = Mesh(icosphere(1).vertices, icosphere(1).triangles)
    with pytest.raises(ValueError):
        m.Curve(2)
    m.Curve(2, project=lambda x: x / np.linalg.norm(x, axis=-1, keepdims=True))
    assert m.curve_order == 2
    with pytest.raises(ValueError):
        m.Curve(4)


@pytest.mark.parametrize("kind", ["RT0", "HCURL"])
def test_piola_load_vectors_match_the_oracle_shapes(oracle, kind):
    """b_i = int f . v_i on a curved mesh with the library's Piola-mapped RT0 (and n x RT0)
    shapes against the same sum over the oracle's shapes at every rule point."""
    from ngbem_gb300.forms import _geometry, triangle_rule
    m = icosphere(1).Curve(3)
    sp = nb.TraceSpace(m, kind)

    def f(x, n):
        return np.stack([x[..., 2], x[..., 0] * x[..., 1], np.ones(x.shape[:2])], axis=-1)

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
