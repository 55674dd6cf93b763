"""Load vectors <f, v> on the trace spaces (the role of NGSolve's LinearForm(f*v*ds) beside the
operators in the reference demos, e.g. demos/HelmholtzBurtonMiller.ipynb), host-side numpy.

f is evaluated at the points of a collapsed Gauss triangle rule on every flat triangle; it is
called as f(x, n) with x (nt, nq, 3) the points and n (nt, 3) the unit normals, and returns
(nt, nq) values (or (nt, nq, m) for m right-hand sides at once).
"""
from __future__ import annotations

import numpy as np

from .meshes import Mesh

__all__ = ["triangle_rule", "load_vector", "hdiv_fields", "p1_load_vector", "p0_load_vector", "plane_wave_bm_source",
           "random_directions", "dubiner", "h1p_shapes"]


def triangle_rule(order: int):
    """Collapsed Gauss-Legendre rule on the reference triangle (1,0), (0,1), (0,0): with n =
    order//2 + 2 points per direction, xi = u, eta = v (1 - u), weight w_u w_v (1 - u); exact for
    polynomials of degree order on the triangle.  Weights sum to 1/2."""
    n = order // 2 + 2
    g, wg = np.polynomial.legendre.leggauss(n)
    u, wu = (g + 1.0) / 2.0, wg / 2.0
    xi = np.repeat(u, n)
    eta = np.outer(1.0 - u, u).ravel()
    wt = np.outer(wu * (1.0 - u), wu).ravel()
    return xi, eta, wt


def _lagrange(order: int, xi: np.ndarray, eta: np.ndarray):
    """Shape functions of the curved (Lagrange) element map and their xi / eta derivatives at
    the points (xi, eta): three (nq, nn) arrays in the node order of Mesh.Curve."""
    lam = [xi, eta, 1.0 - xi - eta]

    def one(i, t):
        v, d = np.ones_like(t), np.zeros_like(t)
        for m in range(i):
            f = (order * t - m) / (m + 1)
            d = d * f + v * order / (m + 1)
            v = v * f
        return v, d
    N, Dxi, Deta = [], [], []
    for i in range(order, -1, -1):
        for j in range(order - i, -1, -1):
            k = order - i - j
            (a, da), (b, db), (c, dc) = one(i, lam[0]), one(j, lam[1]), one(k, lam[2])
            N.append(a * b * c)
            Dxi.append(da * b * c - a * b * dc)
            Deta.append(a * db * c - a * b * dc)
    return np.stack(N, 1), np.stack(Dxi, 1), np.stack(Deta, 1)


def _geometry(mesh: Mesh, order: int):
    """Rule points x (nt, nq, 3), normals n, |J| detj, barycentrics lam (nq, 3) and weights w of
    a triangle rule of the given order on every element.  Flat meshes: n (nt, 3) and detj (nt,)
    per element; curved meshes (Mesh.Curve): n (nt, nq, 3) and detj (nt, nq) per point."""
    X, T = mesh.vertices, mesh.triangles
    xi, eta, w = triangle_rule(order)
    lam = np.stack([xi, eta, 1.0 - xi - eta], axis=1)            # (nq, 3) for (p0, p1, p2)
    if getattr(mesh, "curve_order", 1) > 1:
        N, Dxi, Deta = _lagrange(mesh.curve_order, xi, eta)
        G = mesh.curve_nodes                                       # (nt, nn, 3)
        x = np.einsum("qn,tnc->tqc", N, G)
        n = np.cross(np.einsum("qn,tnc->tqc", Dxi, G), np.einsum("qn,tnc->tqc", Deta, G))
        detj = np.linalg.norm(n, axis=2)
        return x, n / detj[..., None], detj, lam, w
    p0, p1, p2 = X[T[:, 0]], X[T[:, 1]], X[T[:, 2]]
    n = np.cross(p0 - p2, p1 - p2)
    detj = np.linalg.norm(n, axis=1)
    n = n / detj[:, None]
    x = (lam[None, :, 0, None] * p0[:, None] + lam[None, :, 1, None] * p1[:, None]
         + lam[None, :, 2, None] * p2[:, None])                    # (nt, nq, 3)
    return x, n, detj, lam, w


def _weights(w: np.ndarray, detj: np.ndarray) -> np.ndarray:
    """w_q |J| per element and rule point (nt, nq)."""
    return w[None, :] * (detj[:, None] if detj.ndim == 1 else detj)


def p1_load_vector(mesh: Mesh, f, order: int = 6) -> np.ndarray:
    """b_i = int_Gamma f phi_i for the continuous piecewise-linear basis (vertex dofs)."""
    x, n, detj, lam, w = _geometry(mesh, order)
    fv = np.asarray(f(x, n))
    multi = fv.ndim == 3
    if not multi:
        fv = fv[..., None]
    m = fv.shape[2]
    out = np.zeros((mesh.nv, m), dtype=np.result_type(fv.dtype, np.float64))
    W = _weights(w, detj)
    for a in range(3):
        contrib = np.einsum("tq,q,tqm->tm", W, lam[:, a], fv)
        np.add.at(out, mesh.triangles[:, a], contrib)
    return out if multi else out[:, 0]


def p0_load_vector(mesh: Mesh, f, order: int = 6) -> np.ndarray:
    """b_e = int_{T_e} f for the piecewise-constant basis (element dofs)."""
    x, n, detj, lam, w = _geometry(mesh, order)
    fv = np.asarray(f(x, n))
    W = _weights(w, detj)
    if fv.ndim == 3:
        return np.einsum("tq,tqm->tm", W, fv)
    return np.einsum("tq,tq->t", W, fv)


def dubiner(p: int, lam: np.ndarray, f0: np.ndarray, f1: np.ndarray) -> np.ndarray:
    """The SurfaceL2 basis of order p at barycentric points lam (nq, 3) of every triangle, whose
    vertices in the order of their global numbers start with local vertices f0, f1 (nt,):
    (nt, nq, (p+1)(p+2)/2) values of t^i P_i(s/t) P_j^(2i+1,0)(z), x = lam_f0, y = lam_f1,
    s = 2x + y - 1, t = 1 - y, z = 2y - 1, i outer, j inner (the library's basis)."""
    x = lam[:, f0].T  # (nt, nq)
    y = lam[:, f1].T
    s, t, z = 2 * x + y - 1, 1 - y, 2 * y - 1
    leg = [np.ones_like(s), s]
    for n in range(1, p):
        leg.append(((2 * n + 1) * s * leg[n] - n * t * t * leg[n - 1]) / (n + 1))
    out = []
    for i in range(p + 1):
        al = 2 * i + 1
        jac = [np.ones_like(z), ((al + 2) * z + al) / 2]
        for n in range(2, p - i + 1):
            jac.append(((2 * n + al - 1) * ((2 * n + al) * (2 * n + al - 2) * z + al * al) * jac[n - 1]
                        - 2 * (n + al - 1) * (n - 1) * (2 * n + al) * jac[n - 2]) / (2 * n * (n + al) * (2 * n + al - 2)))
        for j in range(p - i + 1):
            out.append(leg[i] * jac[j])
    return np.stack(out, axis=-1)


def h1p_shapes(p: int, lam: np.ndarray, signs: np.ndarray) -> np.ndarray:
    """The H1 basis of order p (2 or 3) at barycentric points lam (nq, 3) of every triangle
    whose local edges (0,1), (1,2), (2,0) have the orientations signs (nt, 3) (+1: the edge's
    first vertex has the lower global number): (nt, nq, (p+1)(p+2)/2) values of the vertex hats
    l_a, the edge bubbles l_i l_j (l_j - l_i)^m times the orientation to the power m, and the
    face bubble l_0 l_1 l_2 (the library's basis and local order)."""
    nt = signs.shape[0]
    out = [np.broadcast_to(lam[:, a], (nt, lam.shape[0])) for a in range(3)]
    for k in range(3):
        i, j = k, (k + 1) % 3
        q = lam[:, i] * lam[:, j]
        for m in range(p - 1):
            out.append(signs[:, k, None] ** m * (q * (lam[:, j] - lam[:, i]) ** m)[None, :])
    if p == 3:
        out.append(np.broadcast_to(lam[:, 0] * lam[:, 1] * lam[:, 2], (nt, lam.shape[0])))
    return np.stack(out, axis=-1)


def hdiv_fields(k: int, lam: np.ndarray, signs: np.ndarray):
    """The HDivSurface basis of order k (1..4) as reference fields at barycentric points lam
    (nq, 3) of every triangle with local edge orientations signs (nt, 3): ((nt, nq, nd, 2) fields,
    (nt, nq, nd) reference divergences) in the library's local order (per edge: the RT0 shape,
    the curls (d/deta, -d/dxi) of sg^e l_i l_j (l_j - l_i)^e, e = 0..k-1; then the interior
    l_j l_k xi^p eta^q curl(l_i), i outer, p + q <= k - 2 with p outer, only p = 0 for i = 2)."""
    nt, nq = signs.shape[0], lam.shape[0]
    dxi, deta = np.array([1.0, 0.0, -1.0]), np.array([0.0, 1.0, -1.0])
    vhat = np.array([[1.0, 0.0], [0.0, 1.0], [0.0, 0.0]])
    xy = lam[:, :2]
    V, D = [], []
    for e in range(3):
        i, j, o = e, (e + 1) % 3, (e + 2) % 3
        sg = signs[:, e, None].astype(np.float64)                          # (nt, 1)
        V.append(sg[:, :, None] * (xy - vhat[o])[None])                    # RT0
        D.append(np.broadcast_to(2.0 * sg, (nt, nq)))
        for m in range(1, k + 1):
            ex = m - 1
            s_ = lam[:, j] - lam[:, i]
            pw = s_ ** ex
            pw1 = ex * s_ ** (ex - 1) if ex > 0 else np.zeros(nq)
            d = np.zeros((nq, 3))
            d[:, i] = lam[:, j] * pw - lam[:, i] * lam[:, j] * pw1
            d[:, j] = lam[:, i] * pw + lam[:, i] * lam[:, j] * pw1
            scale = sg if ex % 2 else np.ones((nt, 1))
            v = np.stack([d @ deta, -(d @ dxi)], axis=1)                   # (nq, 2)
            V.append(scale[:, :, None] * v[None])
            D.append(np.zeros((nt, nq)))
    xi, eta = lam[:, 0], lam[:, 1]
    for i in range(3):
        j, kk = (i + 1) % 3, (i + 2) % 3
        for p in range(k - 1):
            for q in range(k - 1 - p):
                if i == 2 and p > 0:
                    continue
                mon = xi ** p * eta ** q
                mx = p * xi ** (p - 1) * eta ** q if p > 0 else np.zeros(nq)
                my = q * xi ** p * eta ** (q - 1) if q > 0 else np.zeros(nq)
                b = lam[:, j] * lam[:, kk]
                bx = lam[:, kk] * dxi[j] + lam[:, j] * dxi[kk]
                by = lam[:, kk] * deta[j] + lam[:, j] * deta[kk]
                c = np.array([deta[i], -dxi[i]])
                V.append(np.broadcast_to(((b * mon)[:, None] * c[None])[None], (nt, nq, 2)))
                D.append(np.broadcast_to(((bx * mon + b * mx) * c[0] + (by * mon + b * my) * c[1])[None], (nt, nq)))
    return np.stack(V, axis=2), np.stack(D, axis=2)


def load_vector(space, f, order: int = 6) -> np.ndarray:
    """b_i = int f v_i over the space's triangles for the basis v_i of any trace space (the
    role of LinearForm(f * v.Trace() * ds).Assemble() on that space; a space on a region
    integrates over the region only).  P0 / P1: f(x, n) returns (nt, nq) or (nt, nq, m)
    values.  RT0 / HCURL (the RT0 shape sigma (x - p_opp) / |J|, or n x it): f returns
    (nt, nq, 3) vectors or (nt, nq, 3, m); b_i = int f . v_i.  P0 with the dual mapping uses
    v = 1 / |J|.  f receives the rule points x (nt, nq, 3) and the normals n: (nt, 3) per
    element on flat meshes, (nt, nq, 3) per point on curved ones."""
    mesh = space.mesh
    dofs, signs = space.element_dofs()
    on = dofs[:, 0] >= 0
    x, n, detj, lam, w = _geometry(mesh, order)
    fv = np.asarray(f(x, n))
    vector = space.kind == "RT0" or space.kind.startswith(("HCURL", "HDIV"))
    multi = fv.ndim == (4 if vector else 3)
    if not multi:
        fv = fv[..., None]
    out = np.zeros((space.ndof, fv.shape[-1]), dtype=np.result_type(fv.dtype, np.float64))
    curved = getattr(mesh, "curve_order", 1) > 1
    W = _weights(w, detj)
    if space.kind == "P0":
        if space.dual_mapping:
            np.add.at(out, dofs[on, 0], np.einsum("q,tqm->tm", w, fv)[on])
        else:
            np.add.at(out, dofs[on, 0], np.einsum("tq,tqm->tm", W, fv)[on])
    elif space.kind == "P1":
        for a in range(3):
            np.add.at(out, dofs[on, a], np.einsum("tq,q,tqm->tm", W, lam[:, a], fv)[on])
    elif space.kind.startswith("H1P"):
        p = int(space.kind[3:])
        phi = h1p_shapes(p, lam, signs)  # (nt, nq, nd)
        contrib = np.einsum("tq,tqa,tqm->tam", W, phi, fv)
        table = space.dof_table()
        np.add.at(out, table[on].ravel(), contrib[on].reshape(-1, contrib.shape[-1]))
    elif space.kind.startswith("L2P"):
        p = int(space.kind[3:])
        phi = dubiner(p, lam, signs[:, 0], signs[:, 1])  # (nt, nq, nd)
        contrib = np.einsum("tq,tqa,tqm->tam", W, phi, fv)
        nd = phi.shape[-1]
        idx = dofs[on, 0][:, None] + np.arange(nd)[None, :]
        np.add.at(out, idx.ravel(), contrib[on].reshape(-1, contrib.shape[-1]))
    elif space.kind.startswith("HDIV") or (space.kind.startswith("HCURL") and space.kind != "HCURL"):
        # the Piola map J v / |J| of the reference fields, J per element (flat) or per point
        xi, eta, _ = triangle_rule(order)
        if curved:
            _, Dxi, Deta = _lagrange(mesh.curve_order, xi, eta)
            J0 = np.einsum("qn,tnc->tqc", Dxi, mesh.curve_nodes)
            J1 = np.einsum("qn,tnc->tqc", Deta, mesh.curve_nodes)
            dj = detj
        else:
            P = mesh.vertices[mesh.triangles]
            J0 = np.broadcast_to((P[:, 0] - P[:, 2])[:, None], x.shape)
            J1 = np.broadcast_to((P[:, 1] - P[:, 2])[:, None], x.shape)
            dj = np.broadcast_to(detj[:, None], x.shape[:2])
        fields, _ = hdiv_fields(int(space.kind[-1]), lam, signs)           # (nt, nq, nd, 2)
        psi = (J0[:, :, None, :] * fields[..., 0, None] + J1[:, :, None, :] * fields[..., 1, None]) \
            / dj[:, :, None, None]
        if space.kind.startswith("HCURL"):  # n x the HDivSurface shape
            nn = n if n.ndim == 3 else np.broadcast_to(n[:, None, :], x.shape)
            psi = np.cross(nn[:, :, None, :], psi)
        contrib = np.einsum("tq,tqcm,tqac->tam", W, fv, psi)
        table = space.dof_table()
        np.add.at(out, table[on].ravel(), contrib[on].reshape(-1, contrib.shape[-1]))
    elif curved:
        # the Piola map per point: sigma J (xhat - vhat_o) / |J|
        xi, eta, _ = triangle_rule(order)
        _, Dxi, Deta = _lagrange(mesh.curve_order, xi, eta)
        J0 = np.einsum("qn,tnc->tqc", Dxi, mesh.curve_nodes)
        J1 = np.einsum("qn,tnc->tqc", Deta, mesh.curve_nodes)
        vhat = np.array([[1.0, 0.0], [0.0, 1.0], [0.0, 0.0]])
        for k in range(3):
            o = (k + 2) % 3
            off = J0 * (xi - vhat[o, 0])[None, :, None] + J1 * (eta - vhat[o, 1])[None, :, None]
            psi = signs[:, k, None, None] * off / detj[:, :, None]
            if space.kind == "HCURL":
                psi = np.cross(n, psi)
            contrib = np.einsum("tq,tqcm,tqc->tm", W, fv, psi)
            np.add.at(out, dofs[on, k], contrib[on])
    else:
        P = mesh.vertices[mesh.triangles]
        for k in range(3):
            psi = signs[:, k, None, None] * (x - P[:, (k + 2) % 3][:, None, :]) / detj[:, None, None]
            if space.kind == "HCURL":
                psi = np.cross(n[:, None, :], psi)
            contrib = np.einsum("q,tqcm,tqc->tm", w, fv, psi) * detj[:, None]
            np.add.at(out, dofs[on, k], contrib[on])
    return out if multi else out[:, 0]


def plane_wave_bm_source(kappa: float, directions: np.ndarray):
    """Burton-Miller data of incident plane waves exp(i kappa d.x), one per row of directions:
    f = i kappa exp(i kappa d.x) (d.n - 1) (reference demos/HelmholtzBurtonMiller.ipynb, cell 8,
    for d = e_x)."""
    d = np.asarray(directions, dtype=np.float64)

    def f(x, n):
        ph = np.einsum("tqc,mc->tqm", x, d)
        dn = np.einsum("...c,mc->...m", n, d)
        if n.ndim == 2:  # per-element normals of a flat mesh
            dn = dn[:, None, :]
        return 1j * kappa * np.exp(1j * kappa * ph) * (dn - 1.0)
    return f


def random_directions(m: int, seed: int) -> np.ndarray:
    """m unit vectors, uniform on the sphere (normalised standard normal draws, seeded)."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((m, 3))
    return v / np.linalg.norm(v, axis=1)[:, None]
