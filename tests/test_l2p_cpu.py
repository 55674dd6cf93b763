"""SurfaceL2 of order 1..3 on the CPU: the oracle's Dubiner basis against its known properties,
the library's spaces and cluster trees against the oracle's (bit for bit), and the quadrature
convergence pattern of the reference's SL integration test (tests/test_SLIntegration.py:27-39,
which uses SurfaceL2 order 3) on the oracle.
"""
import numpy as np
import pytest

import ngbem_gb300 as nb
from ngbem_gb300.forms import dubiner, load_vector, triangle_rule
from ngbem_gb300.meshes import icosphere, ellipsoid


@pytest.mark.parametrize("p", [1, 2, 3])
def test_dubiner_basis_is_orthogonal(oracle, p):
    """The Dubiner basis is L2-orthogonal on every triangle: the oracle's mass matrix is
    diagonal, with the element's first function the constant 1 (mass = area)."""
    m = ellipsoid(1)
    kind = f"L2P{p}"
    M = oracle.mass_matrix(m, kind, kind, order=8)
    nd = (p + 1) * (p + 2) // 2
    assert M.shape == (m.nt * nd, m.nt * nd)
    off = M - np.diag(np.diag(M))
    assert np.abs(off).max() < 1e-13 * np.abs(M).max()
    areas = m.areas()
    assert np.allclose(np.diag(M)[::nd], areas, rtol=1e-13)
    assert np.all(np.diag(M) > 0)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_dubiner_spans_the_polynomials(p):
    """The (p+1)(p+2)/2 functions on one triangle span the polynomials of degree p: the
    monomials x^a y^b (a + b <= p) are reproduced by least squares exactly."""
    xi, eta, w = triangle_rule(2 * p + 2)
    lam = np.stack([xi, eta, 1 - xi - eta], axis=1)
    for f0, f1 in [(0, 1), (2, 0), (1, 2)]:
        phi = dubiner(p, lam, np.array([f0]), np.array([f1]))[0]  # (nq, nd)
        for a in range(p + 1):
            for b in range(p + 1 - a):
                g = xi ** a * eta ** b
                c, *_ = np.linalg.lstsq(phi, g, rcond=None)
                assert np.abs(phi @ c - g).max() < 1e-12


@pytest.mark.parametrize("p", [1, 2, 3])
def test_library_space_and_tree_match_the_oracle(oracle, p):
    m = icosphere(3)
    kind = f"L2P{p}"
    sp = nb.SurfaceL2(m, order=p)
    nd = (p + 1) * (p + 2) // 2
    assert sp.ndof == m.nt * nd == oracle.ndof(m, kind)
    d, s = sp.element_dofs()
    assert np.array_equal(d[:, 0], np.arange(m.nt) * nd) and np.all(d[:, 1:] == -1)
    # signs: the local vertices in the order of their global numbers
    assert np.array_equal(np.take_along_axis(m.triangles, s, axis=1), np.sort(m.triangles, axis=1))
    for leaf in (20, 40):
        p1, ci1, cd1 = nb.cluster_tree(sp, leaf)
        p2, ci2, cd2 = oracle.cluster_tree(m, kind, leaf)
        assert np.array_equal(p1, p2) and np.array_equal(ci1, ci2)
        assert np.array_equal(cd1.view(np.int64), cd2.view(np.int64))
    part = nb.partition(sp, sp, 40, 2.0)
    ob = oracle.OracleOperator("laplace_sl", m, kind, intorder=2, leafsize=40, eta=2.0, eps=1e-3).blocks()
    for k in ("rowcl", "colcl", "near"):
        assert np.array_equal(part[k], ob[k])


def test_load_vector_of_the_constant():
    """<1, phi_a>: the element's area for its first (constant) function, 0 for the others."""
    m = icosphere(2)
    sp = nb.SurfaceL2(m, order=3)
    b = load_vector(sp, lambda x, n: np.ones(x.shape[:2]))
    b = b.reshape(m.nt, 10)
    assert np.allclose(b[:, 0], m.areas(), rtol=1e-13)
    assert np.abs(b[:, 1:]).max() < 1e-14


def test_sl_integration_converges_in_intorder(oracle):
    """The reference's quadrature test pattern: SL with SurfaceL2 order 3, the error of the
    dense matrix at intorder n against a high-order reference falls with n."""
    m = icosphere(1)
    ref = oracle.dense_matrix("laplace_sl", m, "L2P3", intorder_singular=14, intorder_regular=14)
    errs = []
    for n in (2, 4, 6, 8, 10):
        D = oracle.dense_matrix("laplace_sl", m, "L2P3", intorder_singular=n, intorder_regular=n)
        errs.append(np.linalg.norm(D - ref, 2) / np.linalg.norm(ref, 2))
    assert all(errs[k + 1] < errs[k] for k in range(len(errs) - 1)), errs
    assert errs[-1] < 1e-5 * errs[0]
