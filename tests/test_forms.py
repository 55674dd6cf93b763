"""Host-side load vectors (ngbem_gb300.forms): rule exactness and integrals of known functions."""
from math import factorial

import numpy as np

from ngbem_gb300.forms import p0_load_vector, p1_load_vector, plane_wave_bm_source, random_directions, triangle_rule
from ngbem_gb300.meshes import icosphere


def test_triangle_rule_exactness():
    for order in (2, 4, 6):
        xi, eta, w = triangle_rule(order)
        for a in range(order + 1):
            for b in range(order + 1 - a):
                exact = factorial(a) * factorial(b) / factorial(a + b + 2)
                assert abs((w * xi ** a * eta ** b).sum() - exact) < 1e-14


def test_load_vectors_integrate_polynomials():
    m = icosphere(3)
    area = m.areas().sum()
    one = lambda x, n: np.ones(x.shape[:2])
    assert abs(p1_load_vector(m, one).sum() - area) < 1e-12
    assert abs(p0_load_vector(m, one).sum() - area) < 1e-12
    # sum_i int f phi_i = int f for the P1 partition of unity; f = z^2 over the polyhedron
    z2 = lambda x, n: x[..., 2] ** 2
    assert abs(p1_load_vector(m, z2).sum() - p0_load_vector(m, z2).sum()) < 1e-12


def test_plane_wave_source_shapes_and_values():
    m = icosphere(1)
    d = random_directions(3, 5)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)
    F = p1_load_vector(m, plane_wave_bm_source(2.0, d))
    assert F.shape == (m.nv, 3) and np.iscomplexobj(F)
    # each column equals the single-direction load vector
    for r in range(3):
        Fr = p1_load_vector(m, plane_wave_bm_source(2.0, d[r:r + 1]))
        assert np.allclose(F[:, r], Fr[:, 0], rtol=0, atol=1e-14)


def _capped(level=3):
    from ngbem_gb300.meshes import Mesh
    m0 = icosphere(level)
    return Mesh(m0.vertices, m0.triangles, regions=(m0.centroids()[:, 2] > 0.3).astype(np.int32),
                region_names=["rest", "cap"])


def test_space_load_vector_scalar_spaces_and_regions():
    """load_vector(space, f): on whole-mesh P0 / P1 it equals the mesh load vectors; on a region
    space it equals the load vector of the space on the region's submesh."""
    import ngbem_gb300 as nb
    from ngbem_gb300.forms import load_vector
    m = _capped()
    f = lambda x, n: np.cos(x[..., 0]) + x[..., 2] * n[:, None, 1]
    fm = lambda x, n: np.stack([f(x, n), 2 * f(x, n)], axis=-1)
    assert np.allclose(load_vector(nb.SurfaceL2(m), f), p0_load_vector(m, f), rtol=0, atol=1e-15)
    assert np.allclose(load_vector(nb.H1(m), f), p1_load_vector(m, f), rtol=0, atol=1e-15)
    assert np.allclose(load_vector(nb.H1(m), fm), p1_load_vector(m, fm), rtol=0, atol=1e-15)
    d = load_vector(nb.SurfaceL2(m, dual_mapping=True), f)
    assert np.allclose(d, p0_load_vector(m, f) / (2 * m.areas()), rtol=1e-14)
    R = m.Boundaries("cap")
    sub, _, _ = m.submesh(R)
    for sp in (nb.SurfaceL2, nb.H1):
        a, b = load_vector(sp(m, definedon=R), f), load_vector(sp(sub), f)
        assert np.allclose(a, b, rtol=0, atol=1e-15)


def test_space_load_vector_vector_spaces(oracle):
    """RT0 / HCURL: the load vector of a field that lies in the space (sum_j c_j v_j) is the
    mass matrix times c (the rule integrates the quadratic products exactly), on the whole mesh
    and on a region."""
    import ngbem_gb300 as nb
    from ngbem_gb300.forms import load_vector
    m = _capped(2)
    R = m.Boundaries("cap")
    sub, _, _ = m.submesh(R)
    rng = np.random.default_rng(3)
    for kind, make in (("RT0", nb.HDivSurface), ("HCURL", nb.HCurl)):
        for space, mesh in ((make(m), m), (make(m, definedon=R), sub)):
            dofs, signs = space.element_dofs()
            c = rng.standard_normal(space.ndof)
            P = m.vertices[m.triangles]
            cr = np.cross(P[:, 0] - P[:, 2], P[:, 1] - P[:, 2])
            detj = np.linalg.norm(cr, axis=1)
            nrm = cr / detj[:, None]

            def field(x, n, dofs=dofs, signs=signs, c=c, kind=kind):
                v = np.zeros(x.shape)
                for k in range(3):
                    on = dofs[:, k] >= 0
                    psi = signs[:, k, None, None] * (x - P[:, (k + 2) % 3][:, None, :]) / detj[:, None, None]
                    if kind == "HCURL":
                        psi = np.cross(nrm[:, None, :], psi)
                    v[on] += c[dofs[on, k], None, None] * psi[on]
                return v
            b = load_vector(space, field, order=4)
            M = oracle.mass_matrix(mesh, kind, kind)
            assert np.allclose(b, M @ c, rtol=0, atol=1e-13 * np.abs(M @ c).max())
