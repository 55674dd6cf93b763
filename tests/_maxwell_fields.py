"""Manufactured exterior Maxwell solution for the double-layer checks (pattern of the
reference's tests/test_Maxwell_Box.py): the radiating field of an electric dipole at the
origin, its tangential trace m = -(n x E) x n on the HCurl space, the surface current
j = n x curl E / kappa on the RT0 space, and the Calderon identity the reference solves,
    V j = (-1/2 M + K) m,
with V the Maxwell single layer (RT0, [u; div u]), K the Maxwell double layer (rotated HCurl
trace, RT0 test) and M the HCurl-RT0 mass matrix.  Helpers only: the oracle provides edges,
rules and mass matrices."""
import numpy as np

DIPOLE = np.array([1.192, -0.189, 2.745]) / np.linalg.norm([1.192, -0.189, 2.745])


def field(X, kappa, e=DIPOLE):
    r = np.linalg.norm(X, axis=-1)[..., None]
    f = (-kappa ** 2 * r ** 2 - 1j * kappa * r + 1.0) / r ** 3
    g = (X @ e)[..., None] * (-kappa ** 2 * r ** 2 - 3j * kappa * r + 3.0) / r ** 5
    return np.exp(1j * kappa * r) * (f * e - g * X)


def curl(X, kappa, e=DIPOLE, h=1e-5):
    """curl E by central differences (relative error ~1e-10)."""
    J = np.zeros(X.shape + (3,), dtype=complex)
    for j in range(3):
        d = np.zeros(3)
        d[j] = h
        J[..., :, j] = (field(X + d, kappa, e) - field(X - d, kappa, e)) / (2 * h)
    return np.stack([J[..., 2, 1] - J[..., 1, 2], J[..., 0, 2] - J[..., 2, 0], J[..., 1, 0] - J[..., 0, 1]], -1)


def shapes(mesh, kind, xi, eta):
    """Quadrature points (nt, nq, 3), shape functions (nt, nq, 3 local dofs, 3), |J| and normals.
    RT0: sigma_k (x - p_{k+2}) / |J| on edge k = (k, k+1), sigma_k = +1 when the edge runs from
    the lower to the higher vertex number; HCURL: n x that."""
    P = mesh.vertices[mesh.triangles]
    T = mesh.triangles
    lam = np.stack([xi, eta, 1 - xi - eta], -1)
    X = np.einsum("qa,tac->tqc", lam, P)
    cr = np.cross(P[:, 0] - P[:, 2], P[:, 1] - P[:, 2])
    detJ = np.linalg.norm(cr, axis=-1)
    n = cr / detJ[:, None]
    S = np.zeros((mesh.nt, len(xi), 3, 3))
    for k in range(3):
        sg = np.where(T[:, k] < T[:, (k + 1) % 3], 1.0, -1.0)
        psi = sg[:, None, None] * (X - P[:, (k + 2) % 3][:, None, :]) / detJ[:, None, None]
        S[:, :, k, :] = np.cross(n[:, None, :], psi) if kind == "HCURL" else psi
    return X, S, detJ, n


def traces(oracle, mesh, kappa):
    """L2 projections of the exact m (HCurl) and j (RT0), and the mass matrix M (HCurl -> RT0)."""
    _, TE = oracle.mesh_edges(mesh)
    ne = oracle.ndof(mesh, "RT0")
    xi, eta, w = oracle.trig_rule(8)
    X, Sc, detJ, n = shapes(mesh, "HCURL", xi, eta)
    _, Sd, _, _ = shapes(mesh, "RT0", xi, eta)
    nn = np.broadcast_to(n[:, None, :], X.shape)
    W = w[None, :] * detJ[:, None]
    E = field(X, kappa)
    mex = -np.cross(np.cross(nn, E), nn)
    jex = np.cross(nn, curl(X, kappa) / kappa)

    def project(kind, S, vals):
        b = np.zeros(ne, dtype=complex)
        np.add.at(b, TE, np.einsum("tq,tqc,tqkc->tk", W, vals, S))
        return np.linalg.solve(oracle.mass_matrix(mesh, kind, kind, order=4), b)

    M = oracle.mass_matrix(mesh, "HCURL", "RT0", order=4)
    return project("HCURL", Sc, mex), project("RT0", Sd, jex), M


def calderon_residual(Vj, Km, Mm):
    """|V j - (-1/2 M m + K m)| / |V j|."""
    return np.linalg.norm(Vj - (-0.5 * Mm + Km)) / np.linalg.norm(Vj)
