"""Triangle surface meshes used as operator inputs, flat or curved.

NGSolve/Netgen meshes (OCC spheres, boxes) are not available here, so the operator path
works on plain triangle meshes given as vertex coordinates and vertex triples.  The
generators below build deterministic, consistently outward-oriented meshes:

* ``icosphere(level)``: the icosahedron subdivided ``level`` times (each triangle split in
  four at its edge midpoints) with every vertex projected to the unit sphere:
  20*4**level triangles, 10*4**level + 2 vertices.
* ``ellipsoid(level, axes)``: the icosphere scaled by the semi-axes.
* ``perturbed_icosphere(level, sigma, seed)``: vertices moved radially by sigma*N(0,1).

``mesh.Curve(order)`` (NGSolve's ``Mesh.Curve``) makes the triangles isoparametric Lagrange
elements of order 2 to 4 whose nodes lie on the exact surface (the generators above carry
their surface's projection; other meshes pass ``project``).

Consistent orientation matters: the common-edge Sauter-Schwab permutation assumes that
two triangles sharing an edge traverse it in opposite directions (reference
src/ngbem.cpp:583-586).
"""
from __future__ import annotations

import numpy as np

__all__ = ["Mesh", "Region", "icosphere", "ellipsoid", "perturbed_icosphere"]


class Region:
    """A set of boundary elements of a mesh (the role of NGSolve's Region, e.g.
    ``mesh.Boundaries("outer")``): ``mask`` holds one flag per triangle."""

    def __init__(self, mesh: "Mesh", mask):
        self.mesh = mesh
        self.mask = np.ascontiguousarray(mask, dtype=bool)
        if self.mask.shape != (mesh.nt,):
            raise ValueError("a region mask has one flag per triangle")

    def Mask(self) -> np.ndarray:
        return self.mask

    def __or__(self, other: "Region") -> "Region":
        if other.mesh is not self.mesh:
            raise ValueError("regions of different meshes")
        return Region(self.mesh, self.mask | other.mask)

    __add__ = __or__

    def __repr__(self):
        return f"Region({int(self.mask.sum())} of {self.mesh.nt} triangles)"


class Mesh:
    """A triangle surface mesh: ``vertices`` (nv x 3 float64), ``triangles`` (nt x 3 int32), and
    optionally a boundary-region index per triangle (``regions``, default 0) with the regions'
    names (``region_names``, default ``["default"]``)."""

    def __init__(self, vertices, triangles, regions=None, region_names=None, project=None):
        self.project = project
        self.curve_order = 1
        self.curve_nodes = None
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64)
        self.triangles = np.ascontiguousarray(triangles, dtype=np.int32)
        if self.vertices.ndim != 2 or self.vertices.shape[1] != 3:
            raise ValueError("vertices must be (nv, 3)")
        if self.triangles.ndim != 2 or self.triangles.shape[1] != 3:
            raise ValueError("triangles must be (nt, 3)")
        if self.triangles.size and (self.triangles.min() < 0 or self.triangles.max() >= len(self.vertices)):
            raise ValueError("triangle vertex index out of range")
        nt = self.triangles.shape[0]
        self.regions = np.zeros(nt, dtype=np.int32) if regions is None else \
            np.ascontiguousarray(regions, dtype=np.int32)
        if self.regions.shape != (nt,):
            raise ValueError("regions must hold one index per triangle")
        nreg = int(self.regions.max()) + 1 if nt else 1
        self.region_names = list(region_names) if region_names is not None else \
            (["default"] if nreg == 1 else [f"region{i}" for i in range(nreg)])
        if nt and (self.regions.min() < 0 or nreg > len(self.region_names)):
            raise ValueError("region index without a name")

    def Curve(self, order: int, project=None) -> "Mesh":
        """Curve the triangles (NGSolve's ``Mesh.Curve(order)``, in place; returns the mesh).

        Order 1 keeps flat triangles.  Order 2, 3 or 4 makes each triangle an isoparametric
        Lagrange element: node (i, j, k), i + j + k = order, at barycentric (i, j, k) / order
        of the triangle's vertices (v0, v1, v2), listed for i = order..0, j = order-i..0, is
        moved to the surface by ``project`` (points (n, 3) -> points on the surface; default:
        the projection the mesh was made with).  Nodes on a shared edge are computed from the
        edge's two vertices alone, so neighbouring elements share them bit for bit.  Curve a
        mesh before creating spaces on it."""
        order = int(order)
        if order == 1:
            self.curve_order, self.curve_nodes = 1, None
            return self
        if order not in (2, 3, 4):
            raise ValueError("curved geometry of order 2 to 4")
        proj = project if project is not None else self.project
        if proj is None:
            raise ValueError("a mesh without a surface projection needs project=")
        idx = [(i, j, order - i - j) for i in range(order, -1, -1) for j in range(order - i, -1, -1)]
        p = self.vertices[self.triangles]  # (nt, 3, 3)
        nodes = np.empty((self.nt, len(idx), 3))
        for n, (i, j, k) in enumerate(idx):
            if order in (i, j, k):
                nodes[:, n] = p[:, 0 if i == order else (1 if j == order else 2)]
            else:
                nodes[:, n] = np.asarray(proj((i * p[:, 0] + j * p[:, 1] + k * p[:, 2]) / order), dtype=np.float64)
        self.curve_order, self.curve_nodes = order, np.ascontiguousarray(nodes)
        return self

    def Boundaries(self, pattern: str) -> Region:
        """The triangles whose region name matches the regular expression ``pattern`` (as
        NGSolve's ``mesh.Boundaries("outer|inner")``)."""
        import re
        rx = re.compile(pattern)
        hit = np.array([rx.fullmatch(n) is not None for n in self.region_names], dtype=bool)
        return Region(self, hit[self.regions])

    def submesh(self, region: Region):
        """The mesh made of the region's triangles (in order), its vertices renumbered in
        ascending order: (mesh, vertex ids, triangle ids) in this mesh's numbering."""
        tids = np.flatnonzero(region.mask).astype(np.int32)
        vids = np.unique(self.triangles[tids])
        remap = np.full(self.nv, -1, dtype=np.int32)
        remap[vids] = np.arange(len(vids), dtype=np.int32)
        sub = Mesh(self.vertices[vids], remap[self.triangles[tids]], project=self.project)
        if self.curve_order > 1:
            sub.curve_order, sub.curve_nodes = self.curve_order, np.ascontiguousarray(self.curve_nodes[tids])
        return sub, vids.astype(np.int32), tids

    @property
    def nv(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def ne(self) -> int:
        return int(self.triangles.shape[0])

    nt = ne

    # areas, normals and centroids of the flat triangles (the vertices' triangles)
    def areas(self) -> np.ndarray:
        p = self.vertices[self.triangles]
        return 0.5 * np.linalg.norm(np.cross(p[:, 0] - p[:, 2], p[:, 1] - p[:, 2]), axis=1)

    def normals(self) -> np.ndarray:
        p = self.vertices[self.triangles]
        c = np.cross(p[:, 0] - p[:, 2], p[:, 1] - p[:, 2])
        return c / np.linalg.norm(c, axis=1)[:, None]

    def centroids(self) -> np.ndarray:
        return self.vertices[self.triangles].mean(axis=1)

    def __repr__(self):
        return f"Mesh(nv={self.nv}, nt={self.nt})"


def _icosahedron():
    t = (1.0 + np.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    v = v / np.linalg.norm(v, axis=1)[:, None]
    f = np.array(f, dtype=np.int64)
    # orient every face outward
    p = v[f]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    flip = np.einsum("ij,ij->i", n, p.mean(axis=1)) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f


def _subdivide(v, f):
    verts = [tuple(x) for x in v]
    cache = {}
    out = np.empty((4 * len(f), 3), dtype=np.int64)

    def mid(a, b):
        key = (a, b) if a < b else (b, a)
        idx = cache.get(key)
        if idx is None:
            pa, pb = verts[a], verts[b]
            m = np.array([(pa[0] + pb[0]) * 0.5, (pa[1] + pb[1]) * 0.5, (pa[2] + pb[2]) * 0.5])
            m = m / np.sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2])
            idx = len(verts)
            verts.append((m[0], m[1], m[2]))
            cache[key] = idx
        return idx

    for k, (a, b, c) in enumerate(f.tolist()):
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        out[4 * k + 0] = (a, ab, ca)
        out[4 * k + 1] = (b, bc, ab)
        out[4 * k + 2] = (c, ca, bc)
        out[4 * k + 3] = (ab, bc, ca)
    return np.array(verts, dtype=np.float64), out


class _SphereProjection:
    """Radial projection onto the sphere of the given radius about the origin."""

    def __init__(self, radius):
        self.radius = float(radius)

    def __call__(self, x):
        x = np.asarray(x, dtype=np.float64)
        return self.radius * x / np.linalg.norm(x, axis=-1, keepdims=True)


class _EllipsoidProjection:
    """Projection onto the ellipsoid sum (x_i / a_i)^2 = 1 along the rays of the scaled
    coordinates x_i / a_i (the map of the unit sphere's radial projection)."""

    def __init__(self, axes):
        self.axes = np.asarray(axes, dtype=np.float64)

    def __call__(self, x):
        u = np.asarray(x, dtype=np.float64) / self.axes
        return self.axes * u / np.linalg.norm(u, axis=-1, keepdims=True)


def icosphere(level: int, radius: float = 1.0) -> Mesh:
    """Unit icosphere with 20*4**level triangles (outward normals)."""
    if level < 0:
        raise ValueError("level must be >= 0")
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    return Mesh(v * radius, f.astype(np.int32), project=_SphereProjection(radius))


def ellipsoid(level: int, axes=(1.0, 0.7, 0.5)) -> Mesh:
    """Icosphere scaled by semi-axes ``axes``."""
    m = icosphere(level)
    a = np.asarray(axes, dtype=np.float64)
    return Mesh(m.vertices * a[None, :], m.triangles, project=_EllipsoidProjection(a))


def perturbed_icosphere(level: int, sigma: float = 0.05, seed: int = 0) -> Mesh:
    """Icosphere with vertices moved radially: r = 1 + sigma * N(0,1) (seeded)."""
    m = icosphere(level)
    rng = np.random.default_rng(seed)
    r = 1.0 + sigma * rng.standard_normal(m.nv)
    return Mesh(m.vertices * r[:, None], m.triangles)
