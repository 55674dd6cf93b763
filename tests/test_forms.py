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
