"""ctypes wrapper of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py, never by
the product package.  See oracle.hpp for the reference files this oracle restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

KERNELS = {"laplace_sl": 0, "laplace_dl": 1, "laplace_hs": 2, "helmholtz_sl": 3,
           "helmholtz_dl": 4, "helmholtz_hs": 5, "helmholtz_cf": 6, "maxwell_sl": 7,
           "helmholtz_sl_dkappa": 8, "maxwell_dl": 9}
KINDS = {"P0": 0, "P1": 1, "RT0": 2, "HCURL": 3, "L2P1": 4, "L2P2": 5, "L2P3": 6, "H1P2": 7, "H1P3": 8,
         "HDIV1": 9, "HDIV2": 10, "HCURL1": 11, "HCURL2": 12, "HDIV3": 13, "HDIV4": 14, "HCURL3": 15,
         "HCURL4": 16}
EVALS = {"id": 0, "rot": 1, "helm": 2, "maxwell": 3, "rotatedtrace": 4, "maxwellcurl": 5}


class Params(C.Structure):
    _fields_ = [("intorder_singular", C.c_int), ("intorder_regular", C.c_int),
                ("leafsize", C.c_int), ("eta", C.c_double), ("eps", C.c_double),
                ("nthreads", C.c_int)]


def build():
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        dp, ip, lp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_long)
        L.orc_mesh_edges.argtypes = [C.c_int, C.c_int, ip, ip, ip]
        L.orc_trig_rule.argtypes = [C.c_int, dp, dp, dp]
        L.orc_set_geometry.argtypes = [C.c_int, C.c_int, dp]
        L.orc_eval_trace.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     dp, ip]
        L.orc_ss_rule.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp, dp]
        L.orc_cluster_tree.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, C.c_int, ip, C.c_int, lp, dp]
        L.orc_operator_create.restype = C.c_void_p
        L.orc_operator_create.argtypes = [C.c_int, C.c_double, C.c_int, dp, C.c_int, ip,
                                          C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(Params)]
        L.orc_operator_info.argtypes = [C.c_void_p, lp]
        L.orc_operator_mult.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.orc_operator_mult_multi.argtypes = [C.c_void_p, C.c_int, dp, dp]
        L.orc_operator_blocks.argtypes = [C.c_void_p, ip, ip, ip, ip, ip]
        L.orc_operator_to_dense.argtypes = [C.c_void_p, dp]
        L.orc_dense_matrix.argtypes = [C.c_int, C.c_double, C.c_int, dp, C.c_int, ip,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(Params), dp]
        L.orc_operator_destroy.argtypes = [C.c_void_p]
        L.orc_mass_matrix.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, C.c_int, C.c_int, dp]
        L.orc_potential.argtypes = [C.c_int, C.c_double, C.c_int, dp, C.c_int, ip, C.c_int, C.c_int, C.c_int,
                                    C.c_int, dp, C.c_int, dp, dp, dp]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _lp(a):
    return a.ctypes.data_as(C.POINTER(C.c_long))


def mesh_edges(mesh):
    tri = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
    edges = np.zeros(6 * mesh.nt, dtype=np.int32)
    te = np.zeros(3 * mesh.nt, dtype=np.int32)
    ne = lib().orc_mesh_edges(mesh.nv, mesh.nt, _ip(tri), _ip(edges), _ip(te))
    return edges[: 2 * ne].reshape(-1, 2), te.reshape(-1, 3)


def trig_rule(order):
    n = (order // 2 + 1) ** 2
    xi, eta, w = np.zeros(n), np.zeros(n), np.zeros(n)
    k = lib().orc_trig_rule(order, _dp(xi), _dp(eta), _dp(w))
    return xi[:k], eta[:k], w[:k]


def ss_rule(cls, order):
    ns = order // 2 + 1
    n = 6 * ns ** 4
    a = [np.zeros(n) for _ in range(5)]
    k = lib().orc_ss_rule(cls, order, *[_dp(x) for x in a])
    return [x[:k] for x in a]


def _geometry(mesh):
    """Set the oracle's geometry to the mesh's: flat, or its curved nodes (Mesh.Curve)."""
    order = int(getattr(mesh, "curve_order", 1))
    if order > 1:
        nodes = np.ascontiguousarray(mesh.curve_nodes, dtype=np.float64)
        rc = lib().orc_set_geometry(order, mesh.nt, _dp(nodes))
    else:
        rc = lib().orc_set_geometry(1, 0, None)
    if rc != 0:
        raise ValueError("bad geometry order")


def eval_trace(mesh, kind, ev, e, xi, eta):
    """(values (nd, 4), dofs (nd,)): the trace values of element e's local dofs at (xi, eta)."""
    _geometry(mesh)
    X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
    out = np.zeros(120)
    dofs = np.zeros(30, dtype=np.int32)
    nd = lib().orc_eval_trace(mesh.nv, _dp(X), mesh.nt, _ip(T), KINDS[kind], EVALS[ev], int(e), float(xi),
                              float(eta), _dp(out), _ip(dofs))
    return out.reshape(30, 4)[:nd], dofs[:nd]


def ndof(mesh, kind):
    if kind == "P0":
        return mesh.nt
    if kind.startswith("L2P"):
        p = int(kind[3:])
        return mesh.nt * (p + 1) * (p + 2) // 2
    if kind == "P1":
        return mesh.nv
    ne = len(mesh_edges(mesh)[0])
    if kind.startswith("H1P"):
        p = int(kind[3:])
        return mesh.nv + ne * (p - 1) + mesh.nt * (p - 1) * (p - 2) // 2
    if kind.startswith("HDIV") or (kind.startswith("HCURL") and kind != "HCURL"):
        k = int(kind[-1])
        return ne * (k + 1) + mesh.nt * (k + 1) * (k - 1)
    return ne


def cluster_tree(mesh, kind, leafsize):
    n = ndof(mesh, kind)
    maxc = 4 * n + 8
    perm = np.zeros(n, dtype=np.int32)
    ci = np.zeros(7 * maxc, dtype=np.int64)
    cd = np.zeros(23 * maxc, dtype=np.float64)
    X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
    _geometry(mesh)
    nc = lib().orc_cluster_tree(mesh.nv, _dp(X), mesh.nt, _ip(T), KINDS[kind], leafsize,
                                _ip(perm), maxc, _lp(ci), _dp(cd))
    if nc < 0:
        raise RuntimeError("too many clusters")
    return perm, ci[: 7 * nc].reshape(nc, 7), cd[: 23 * nc].reshape(nc, 23)


def _params(intorder_singular, intorder_regular, leafsize, eta, eps, nthreads):
    return Params(intorder_singular, intorder_regular, leafsize, eta, eps, nthreads)


class OracleOperator:
    """FP64 H-matrix operator assembled on the CPU by the oracle."""

    def __init__(self, kernel, mesh, trial="P0", test=None, kappa=0.0, trial_eval="id",
                 test_eval=None, intorder=3, intorder_singular=None, intorder_regular=None,
                 leafsize=40, eta=2.0, eps=1e-6, method="aca", nthreads=0,
                 trial_dual=False, test_dual=False):
        test = trial if test is None else test
        test_eval = trial_eval if test_eval is None else test_eval
        if method == "dense":
            leafsize, eta = 2 ** 31 - 1, 0.0
        self.p = _params(intorder_singular or intorder, intorder_regular or intorder,
                         leafsize, eta, eps, nthreads)
        self.X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
        self.T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
        _geometry(mesh)
        self.h = lib().orc_operator_create(KERNELS[kernel], float(kappa), mesh.nv, _dp(self.X),
                                           mesh.nt, _ip(self.T), KINDS[trial], EVALS[trial_eval],
                                           int(trial_dual), KINDS[test], EVALS[test_eval],
                                           int(test_dual), C.byref(self.p))
        if not self.h:
            raise RuntimeError("oracle operator creation failed")
        info = np.zeros(10, dtype=np.int64)
        lib().orc_operator_info(self.h, _lp(info))
        self.is_complex = bool(info[0])
        self.height, self.width = int(info[1]), int(info[2])
        self.nblocks, self.nnear, self.nfar, self.nze = (int(v) for v in info[3:7])
        self.nfallback, self.max_rank, self.sum_rank = (int(v) for v in info[7:10])
        self.dtype = np.complex128 if self.is_complex else np.float64

    def mult(self, x, trans=False):
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.zeros(self.width if trans else self.height, dtype=self.dtype)
        lib().orc_operator_mult(self.h, int(trans), _dp(x.view(np.float64)), _dp(y.view(np.float64)))
        return y

    def blocks(self):
        n = self.nblocks
        arrs = [np.zeros(n, dtype=np.int32) for _ in range(5)]
        lib().orc_operator_blocks(self.h, *[_ip(a) for a in arrs])
        return dict(zip(["rowcl", "colcl", "near", "rank", "fallback"], arrs))

    def to_dense(self):
        out = np.zeros((self.height, self.width), dtype=self.dtype)
        lib().orc_operator_to_dense(self.h, _dp(out.view(np.float64)))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_operator_destroy(self.h)
            self.h = None


def dense_matrix(kernel, mesh, trial="P0", test=None, kappa=0.0, trial_eval="id", test_eval=None,
                 intorder=3, intorder_singular=None, intorder_regular=None, nthreads=0,
                 trial_dual=False, test_dual=False):
    test = trial if test is None else test
    test_eval = trial_eval if test_eval is None else test_eval
    p = _params(intorder_singular or intorder, intorder_regular or intorder, 2 ** 31 - 1, 0.0, 1e-6, nthreads)
    X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
    H, W = ndof(mesh, test), ndof(mesh, trial)
    dt = np.complex128 if KERNELS[kernel] >= 3 else np.float64
    out = np.zeros((H, W), dtype=dt)
    _geometry(mesh)
    lib().orc_dense_matrix(KERNELS[kernel], float(kappa), mesh.nv, _dp(X), mesh.nt, _ip(T),
                           KINDS[trial], EVALS[trial_eval], int(trial_dual), KINDS[test],
                           EVALS[test_eval], int(test_dual), C.byref(p), _dp(out.view(np.float64)))
    return out


def potential(kernel, mesh, trial, density, points, normals=None, kappa=0.0, trial_eval="id", intorder=3,
              trial_dual=False):
    """Potential of `density` (trial dofs) at `points` (reference PotentialCF): (npts, dim)."""
    X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
    cplx = KERNELS[kernel] >= 3
    dens = np.ascontiguousarray(density, dtype=np.complex128 if cplx else np.float64)
    P = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    Nn = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, 3)
    if trial_eval == "id":
        dim = 3 if trial in ("RT0", "HCURL") else 1
    else:
        dim = 3 if trial_eval in ("rot", "rotatedtrace") else 4
    out = np.zeros((P.shape[0], dim), dtype=dens.dtype)
    _geometry(mesh)
    lib().orc_potential(KERNELS[kernel], float(kappa), mesh.nv, _dp(X), mesh.nt, _ip(T), KINDS[trial],
                        EVALS[trial_eval], int(trial_dual), int(intorder), _dp(dens.view(np.float64)), P.shape[0],
                        _dp(P), None if Nn is None else _dp(Nn), _dp(out.view(np.float64)))
    return out


def mass_matrix(mesh, trial="P1", test="P0", order=4):
    X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
    out = np.zeros((ndof(mesh, test), ndof(mesh, trial)))
    _geometry(mesh)
    lib().orc_mass_matrix(mesh.nv, _dp(X), mesh.nt, _ip(T), KINDS[trial], KINDS[test], order, _dp(out))
    return out
