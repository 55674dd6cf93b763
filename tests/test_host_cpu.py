"""Host-side logic on the CPU: the C-ABI library loads and exports every declared symbol,
the cluster tree and block partition are bit-exact with the oracle, and invalid arguments
come back as status codes (no GPU compute is called here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import ngbem_gb300 as nb
from ngbem_gb300 import _lib
from ngbem_gb300.meshes import icosphere, ellipsoid, perturbed_icosphere

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ngbem_gb300.h")


def test_library_exports_header_symbols():
    src = open(HEADER).read()
    names = set(re.findall(r"^\s*(?:int|const char\*)\s+(bem_\w+)\s*\(", src, re.M))
    assert len(names) >= 20
    for n in names:
        assert hasattr(_lib.lib, n), n
    assert set(_lib.SIGNATURES) >= names


@pytest.mark.parametrize("mesh_fn,kind,leaf", [
    (lambda: icosphere(2), "P0", 20), (lambda: icosphere(3), "P0", 20), (lambda: icosphere(3), "P1", 20),
    (lambda: icosphere(3), "RT0", 40), (lambda: ellipsoid(3), "P0", 40), (lambda: ellipsoid(3), "P1", 10),
    (lambda: perturbed_icosphere(3, 0.05, 7), "P0", 20), (lambda: icosphere(4), "P0", 40),
    (lambda: icosphere(2), "P0", 2 ** 31 - 1),
    # 4096 dofs and more: levels split over the host thread team
    (lambda: icosphere(5), "P1", 20), (lambda: icosphere(4), "RT0", 20), (lambda: ellipsoid(5), "P0", 20)])
def test_cluster_tree_bit_exact(oracle, mesh_fn, kind, leaf):
    m = mesh_fn()
    sp = nb.TraceSpace(m, kind)
    p1, ci1, cd1 = nb.cluster_tree(sp, leaf)
    p2, ci2, cd2 = oracle.cluster_tree(m, kind, leaf)
    assert np.array_equal(p1, p2)
    assert np.array_equal(ci1, ci2)
    assert np.array_equal(cd1.view(np.int64), cd2.view(np.int64))  # bit for bit
    # a valid binary tree: children partition the parent's dof range
    for c in range(len(ci1)):
        lvl, par, c1, c2, num, pos, _ = ci1[c]
        if c1 >= 0:
            assert ci1[c1][5] == pos and ci1[c2][5] == pos + ci1[c1][4] and ci1[c1][4] + ci1[c2][4] == num
    assert sorted(p1.tolist()) == list(range(sp.ndof))


@pytest.mark.parametrize("trial,test,leaf,eta", [("P0", "P0", 20, 2.0), ("P1", "P0", 20, 2.0),
                                                 ("P1", "P1", 10, 3.0), ("RT0", "RT0", 40, 2.0),
                                                 ("P0", "P0", 20, 0.0)])
def test_partition_matches_oracle_blocks(oracle, trial, test, leaf, eta):
    m = icosphere(3)
    tr = nb.TraceSpace(m, trial)
    te = tr if test == trial else nb.TraceSpace(m, test)
    part = nb.partition(tr, te, leaf, eta)
    # the oracle builds the same partition inside its operator (blocks in assembly order)
    H = oracle.OracleOperator("laplace_sl", m, trial, test, intorder=2, leafsize=leaf, eta=eta, eps=1e-3)
    ob = H.blocks()
    assert np.array_equal(part["rowcl"], ob["rowcl"])
    assert np.array_equal(part["colcl"], ob["colcl"])
    assert np.array_equal(part["near"], ob["near"])
    if eta == 0.0:
        assert part["near"].all()


def test_argument_errors_are_status_codes():
    m = icosphere(1)
    h = C.c_void_p()
    X = np.ascontiguousarray(m.vertices)
    T = np.ascontiguousarray(m.triangles).copy()
    T[0, 0] = 10 ** 6
    st = _lib.lib.bem_mesh_create(m.nv, X.ctypes.data_as(_lib._dp), m.nt, T.ctypes.data_as(_lib._ip), C.byref(h))
    assert st == _lib.BEM_ERR_ARG and b"out of range" in _lib.lib.bem_last_error()
    with pytest.raises(_lib.BemError):
        nb.TraceSpace(m, "P1", dual_mapping=True)
    with pytest.raises(ValueError):
        nb.TraceSpace(m, "P2")
    with pytest.raises(NotImplementedError):
        nb.SurfaceL2(m, order=4)
    sp = nb.SurfaceL2(m)
    with pytest.raises(_lib.BemError):
        nb.cluster_tree(sp, 0)
    # region spaces and operator regions
    out = C.c_void_p()
    assert _lib.lib.bem_space_create_on(None, 0, 0, None, C.byref(out)) == _lib.BEM_ERR_ARG
    assert _lib.lib.bem_space_create_on(sp._mh.h, 17, 0, None, C.byref(out)) == _lib.BEM_ERR_ARG
    none = np.zeros(m.nt, dtype=np.uint8)
    assert _lib.lib.bem_space_create_on(sp._mh.h, 0, 0, C.c_void_p(none.ctypes.data), C.byref(out)) == \
        _lib.BEM_ERR_ARG and b"no elements" in _lib.lib.bem_last_error()
    assert _lib.lib.bem_space_global_dofs(None, None) == _lib.BEM_ERR_ARG
    assert _lib.lib.bem_operator_set_definedon(None, None, None) == _lib.BEM_ERR_ARG


def test_status_plumbing_without_a_device():
    """The device-status query and the wait test hook check their arguments on the host."""
    flags = C.c_int(-1)
    assert _lib.lib.bem_operator_status(None, C.byref(flags), 0) == _lib.BEM_ERR_ARG
    assert b"null" in _lib.lib.bem_last_error()
    assert _lib.lib.bem_operator_test_waits(None, 0, 0) == _lib.BEM_ERR_ARG
    assert _lib.lib.bem_operator_mult_noalloc(None, 0, None, None, None, None, 1, None) == _lib.BEM_ERR_ARG


def test_maxwell_factory_argument_checks():
    """The HCurl space and the Maxwell double-layer / curl factories check their spaces before
    any assembly (no GPU needed)."""
    m = icosphere(1)
    HC, RT, P0 = nb.HCurl(m), nb.HDivSurface(m), nb.SurfaceL2(m)
    assert HC.ndof == RT.ndof and HC.kind == "HCURL"
    with pytest.raises(TypeError):
        nb.MaxwellDoubleLayerPotentialOperator(RT, RT, 1.0)
    with pytest.raises(TypeError):
        nb.MaxwellDoubleLayerPotentialOperator(HC, P0, 1.0)
    with pytest.raises(TypeError):
        nb.MaxwellSingleLayerPotentialOperatorCurl(RT, 1.0)
    with pytest.raises(TypeError):
        nb.MaxwellSingleLayerPotentialOperator(RT, None)
    with pytest.raises(NotImplementedError):
        nb.HCurl(m, order=5)


def test_mesh_generators():
    for L in range(4):
        m = icosphere(L)
        assert m.nt == 20 * 4 ** L and m.nv == 10 * 4 ** L + 2
        # outward orientation and closed surface (each edge shared by two triangles, opposite directions)
        assert (np.einsum("ij,ij->i", m.normals(), m.centroids()) > 0).all()
        e = np.concatenate([m.triangles[:, [0, 1]], m.triangles[:, [1, 2]], m.triangles[:, [2, 0]]])
        fwd = set(map(tuple, e.tolist()))
        assert all((b, a) in fwd for a, b in fwd)
    el = ellipsoid(2)
    assert np.allclose(np.abs(el.vertices).max(axis=0), [1.0, 0.7, 0.5], atol=0.02)


def test_edge_numbering_matches_oracle(oracle):
    m = icosphere(2)
    sp = nb.HDivSurface(m)
    edges, te = oracle.mesh_edges(m)
    assert sp.ndof == len(edges) == 3 * m.nt // 2


def _capped_sphere(level=3, z0=0.3):
    from ngbem_gb300.meshes import Mesh
    m0 = icosphere(level)
    cap = (m0.centroids()[:, 2] > z0).astype(np.int32)
    return Mesh(m0.vertices, m0.triangles, regions=cap, region_names=["rest", "cap"])


@pytest.mark.parametrize("kind", ["P0", "P1", "RT0", "HCURL"])
def test_region_space_is_the_submesh_space(oracle, kind):
    """A space on a region (definedon) numbers its dofs like the space on the mesh made of the
    region's triangles, and has the same cluster tree and block partition, bit for bit."""
    m = _capped_sphere()
    R = m.Boundaries("cap")
    sub, vids, tids = m.submesh(R)
    sr, ss = nb.TraceSpace(m, kind, definedon=R), nb.TraceSpace(sub, kind)
    assert sr.ndof == ss.ndof
    g = sr.global_dofs
    if kind == "P0":
        assert np.array_equal(g, tids)
    elif kind == "P1":
        assert np.array_equal(g, vids)
    else:
        E, _ = oracle.mesh_edges(m)
        Es, _ = oracle.mesh_edges(sub)
        assert np.array_equal(np.sort(E[g], axis=1), np.sort(vids[Es], axis=1))
    for leaf in (10, 40):
        p1, ci1, cd1 = nb.cluster_tree(sr, leaf)
        p2, ci2, cd2 = nb.cluster_tree(ss, leaf)
        assert np.array_equal(p1, p2) and np.array_equal(ci1, ci2)
        assert np.array_equal(cd1.view(np.int64), cd2.view(np.int64))
        b1, b2 = nb.partition(sr, leafsize=leaf), nb.partition(ss, leafsize=leaf)
        for k in b1:
            assert np.array_equal(b1[k], b2[k])


def test_regions_and_masks():
    from ngbem_gb300.meshes import Mesh
    m = _capped_sphere(2)
    cap, rest, both = m.Boundaries("cap"), m.Boundaries("rest"), m.Boundaries("cap|rest")
    assert not (cap.Mask() & rest.Mask()).any() and (cap | rest).Mask().all() and both.Mask().all()
    assert m.Boundaries(".*").Mask().all() and not m.Boundaries("outer").Mask().any()
    with pytest.raises(ValueError):
        Mesh(m.vertices, m.triangles, regions=np.zeros(3, dtype=np.int32))
    with pytest.raises(ValueError):
        Mesh(m.vertices, m.triangles, regions=np.full(m.nt, 2), region_names=["a", "b"])
    other = icosphere(2)
    with pytest.raises(ValueError):
        nb.SurfaceL2(other, definedon=cap)
    with pytest.raises(TypeError):
        nb.SurfaceL2(m, definedon=cap.Mask())
    # a region without triangles is refused by the library
    with pytest.raises(Exception):
        nb.H1(m, definedon=m.Boundaries("outer"))
    # the whole mesh as a region gives the plain space
    a, b = nb.HDivSurface(m, definedon=m.Boundaries(".*")), nb.HDivSurface(m)
    assert a.ndof == b.ndof and np.array_equal(a.global_dofs, np.arange(b.ndof))


def test_handles_keep_what_they_point_into():
    """A space keeps its mesh alive (and an operator its spaces): destroying the handles in any
    order leaves the others usable.  The space's cluster tree needs the mesh coordinates."""
    m = icosphere(3)
    X = np.ascontiguousarray(m.vertices)
    T = np.ascontiguousarray(m.triangles, dtype=np.int32)
    mh, sh = C.c_void_p(), C.c_void_p()
    _lib.check(_lib.lib.bem_mesh_create(m.nv, X.ctypes.data_as(_lib._dp), m.nt, T.ctypes.data_as(_lib._ip),
                                        C.byref(mh)))
    _lib.check(_lib.lib.bem_space_create(mh, _lib.KINDS["P1"], 0, C.byref(sh)))

    def tree():
        perm = np.zeros(m.nv, dtype=np.int32)
        nc = C.c_int()
        maxc = 4 * m.nv
        ci = np.zeros(7 * maxc, dtype=np.int64)
        cd = np.zeros(23 * maxc, dtype=np.float64)
        _lib.check(_lib.lib.bem_cluster_tree(sh, 20, perm.ctypes.data_as(_lib._ip), maxc, C.byref(nc),
                                             ci.ctypes.data_as(_lib._lp), cd.ctypes.data_as(_lib._dp)))
        return perm, cd[: 23 * nc.value].copy()

    p0, c0 = tree()
    _lib.check(_lib.lib.bem_mesh_destroy(mh))
    X[:] = 0.0  # the caller's arrays are not what the space reads either
    p1, c1 = tree()
    assert np.array_equal(p0, p1) and np.array_equal(c0.view(np.int64), c1.view(np.int64))
    _lib.check(_lib.lib.bem_space_destroy(sh))
