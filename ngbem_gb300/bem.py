"""Python mirror of ngbem's operator API (reference src/python_bem.cpp:11-194).

Factories keep the reference names, argument order, keyword names and defaults
(intorder=3, leafsize=40, eta=2., eps=1e-6, method="aca", testhmatrix=False).  The NGSolve
FESpace argument becomes a trace space on a triangle mesh (SurfaceL2 order 0 = P0,
H1 order 1 = P1, HDivSurface order 0 = RT0), flat or curved by ``Mesh.Curve(order)``.
``.mat`` is an H-matrix resident in GPU memory with the BaseMatrix surface the reference's
callers use: Mult, MultAdd, MultTrans,
MultTransAdd, ``*``, ``.T``, ``nze``, CreateRowVector, CreateColVector, and sums/scalings
of matrices (``0.5 * M.mat + K.mat``).

GB300 extensions (keyword-only): precision ("fp64" plain path or "mixed"),
intorder_singular / intorder_regular (separate Sauter-Schwab and regular orders),
max_rank (ACA rank cap; capped blocks are assembled densely), aca_eps_floor.

Vectors are torch tensors on the GPU (float64 or complex128); numpy arrays are accepted and
go through the host-buffer entry point (copies inside the call).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import KERNELS, KINDS, EVALS, check, cplx2, lib
from .meshes import Mesh, Region

__all__ = ["SurfaceL2", "H1", "HDivSurface", "HCurl", "TraceSpace", "BaseMatrix", "HMatrix", "MassMatrix",
           "IntegralOperator", "IntegralOperatorC",
           "SingleLayerPotentialOperator", "DoubleLayerPotentialOperator", "HypersingularOperator",
           "HelmholtzSingleLayerPotentialOperator", "HelmholtzDoubleLayerPotentialOperator",
           "HelmholtzCombinedFieldOperator", "HelmholtzHypersingularOperator",
           "HelmholtzSingleLayerPotentialOperatorDKappa",
           "MaxwellSingleLayerPotentialOperator", "MaxwellSingleLayerPotentialOperatorCurl",
           "MaxwellDoubleLayerPotentialOperator", "MassOperator", "GMRes", "cluster_tree", "partition",
           "tc_selftest", "TestCompression"]


def _torch():
    import torch
    return torch


# ----------------------------------------------------------------------------------------
# meshes and spaces
# ----------------------------------------------------------------------------------------
class _MeshHandle:
    _cache: dict = {}

    def __init__(self, mesh: Mesh):
        self.mesh = mesh
        self.h = C.c_void_p()
        X = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
        T = np.ascontiguousarray(mesh.triangles, dtype=np.int32)
        check(lib.bem_mesh_create(mesh.nv, X.ctypes.data_as(_lib._dp), mesh.nt, T.ctypes.data_as(_lib._ip),
                                  C.byref(self.h)))
        self.curve = (getattr(mesh, "curve_order", 1), id(getattr(mesh, "curve_nodes", None)))
        if self.curve[0] > 1:
            G = np.ascontiguousarray(mesh.curve_nodes, dtype=np.float64)
            check(lib.bem_mesh_set_geometry(self.h, self.curve[0], G.ctypes.data_as(_lib._dp)))
        ne = C.c_int()
        check(lib.bem_mesh_num_edges(self.h, C.byref(ne)))
        self.ne = ne.value

    @classmethod
    def of(cls, mesh: Mesh):
        key = id(mesh)
        h = cls._cache.get(key)
        curve = (getattr(mesh, "curve_order", 1), id(getattr(mesh, "curve_nodes", None)))
        if h is None or h.mesh is not mesh or h.curve != curve:
            h = cls(mesh)
            cls._cache[key] = h
        return h

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib.bem_mesh_destroy(self.h)
            self.h = C.c_void_p()


class TraceSpace:
    """Surface trace space: kind "P0" (SurfaceL2 order 0), "P1" (H1 order 1), "RT0" (HDivSurface order 0),
    "HCURL" (surface trace of HCurl order 0), "L2P1".."L2P3" (SurfaceL2 orders 1-3), "H1P2",
    "H1P3" (H1 orders 2, 3), "HDIV1".."HDIV4" (HDivSurface orders 1-4), "HCURL1".."HCURL4" (HCurl
    orders 1-4)."""

    def __init__(self, mesh: Mesh, kind: str, dual_mapping: bool = False, complex: bool = False, definedon=None):
        if kind not in KINDS:
            raise ValueError(f"unknown space kind {kind!r}")
        self.mesh = mesh
        self.kind = kind
        self.dual_mapping = bool(dual_mapping)
        self.is_complex = bool(complex)
        self.definedon = definedon
        self._mh = _MeshHandle.of(mesh)
        self.h = C.c_void_p()
        if definedon is None:
            check(lib.bem_space_create(self._mh.h, KINDS[kind], int(self.dual_mapping), C.byref(self.h)))
        else:
            mask = _region_mask(definedon, mesh)
            check(lib.bem_space_create_on(self._mh.h, KINDS[kind], int(self.dual_mapping),
                                          C.c_void_p(mask.ctypes.data), C.byref(self.h)))
        n = C.c_int()
        check(lib.bem_space_ndof(self.h, C.byref(n)))
        self.ndof = n.value

    def element_dofs(self):
        """(dofs, signs), each (nt, 3): the dofs of every triangle (FESpace::GetDofNrs; P0 uses
        column 0; -1 off the space's region) and the RT0 / HCURL edge orientations."""
        nt = self.mesh.nt
        d = np.zeros((nt, 3), dtype=np.int32)
        s = np.zeros((nt, 3), dtype=np.int32)
        check(lib.bem_space_element_dofs(self.h, d.ctypes.data_as(_lib._ip), s.ctypes.data_as(_lib._ip)))
        return d, s

    def dof_table(self):
        """(nt, nd) array of every local dof of every triangle in the basis's local order
        (FESpace::GetDofNrs for any kind; -1 off the space's region)."""
        nd = C.c_int()
        check(lib.bem_space_dof_table(self.h, C.byref(nd), None))
        t = np.zeros((self.mesh.nt, nd.value), dtype=np.int32)
        check(lib.bem_space_dof_table(self.h, C.byref(nd), t.ctypes.data_as(_lib._ip)))
        return t

    @property
    def global_dofs(self) -> np.ndarray:
        """dof -> element (P0), vertex (P1) or edge (RT0, HCURL) of the whole mesh.  A space on a
        region numbers its dofs like the mesh made of the region's elements (Mesh.submesh)."""
        out = np.zeros(self.ndof, dtype=np.int32)
        check(lib.bem_space_global_dofs(self.h, out.ctypes.data_as(_lib._ip)))
        return out

    def __repr__(self):
        return f"TraceSpace({self.kind}, ndof={self.ndof})"

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib.bem_space_destroy(self.h)
            self.h = C.c_void_p()


def _region_mask(region, mesh: Mesh) -> np.ndarray:
    if not isinstance(region, Region):
        raise TypeError("definedon must be a Region (mesh.Boundaries(...))")
    if region.mesh is not mesh:
        raise ValueError("the region belongs to another mesh")
    return np.ascontiguousarray(region.mask, dtype=np.uint8)


def SurfaceL2(mesh: Mesh, order: int = 0, dual_mapping: bool = False, complex: bool = False,
              definedon=None) -> TraceSpace:
    """Discontinuous polynomials of degree `order` on the surface triangles (NGSolve SurfaceL2):
    order 0 the piecewise constants, orders 1..3 the Dubiner basis ((p+1)(p+2)/2 dofs per
    triangle, numbered consecutively per triangle, built on the triangle's vertices in the order
    of their global numbers).  dual_mapping (order 0 only): the basis 1/|J|.  definedon: a
    Region; the space then lives on those triangles only."""
    if order not in (0, 1, 2, 3):
        raise NotImplementedError("SurfaceL2: orders 0 to 3 are supported")
    if order > 0 and dual_mapping:
        raise NotImplementedError("SurfaceL2: dual_mapping is defined for order 0")
    return TraceSpace(mesh, "P0" if order == 0 else f"L2P{order}", dual_mapping, complex, definedon)


def H1(mesh: Mesh, order: int = 1, complex: bool = False, definedon=None) -> TraceSpace:
    """Continuous piecewise polynomials of degree `order` on the surface (NGSolve H1 on a
    surface mesh).  Order 1: the hat functions (one dof per vertex).  Orders 2, 3: a
    hierarchical basis: the vertex hats, then p - 1 edge bubbles l_i l_j (l_j - l_i)^m per edge
    (oriented from the lower to the higher vertex number), then the face bubble l_0 l_1 l_2
    (order 3); dofs numbered vertices, edges (by first appearance), faces.  The traces are the
    identity and the surface curl (hypersingular operator)."""
    if order not in (1, 2, 3):
        raise NotImplementedError("H1: orders 1 to 3 are supported")
    return TraceSpace(mesh, "P1" if order == 1 else f"H1P{order}", False, complex, definedon)


def HDivSurface(mesh: Mesh, order: int = 0, complex: bool = False, definedon=None) -> TraceSpace:
    """Normal-continuous tangential fields on the surface (NGSolve HDivSurface): order 0 the
    lowest-order Raviart-Thomas space (one dof per edge), order K = 1..4 all vector polynomials of
    degree K (K + 1 dofs per edge, (K + 1)(K - 1) per element) in a hierarchical basis of our
    own: the RT0 shapes, the surface curls of H1 edge bubbles and the interior fields
    l_j l_k xi^p eta^q curl(l_i), all Piola-mapped.  Orders 3, 4 serve the Maxwell single layer
    (and the double layer from HCurl of order 3)."""
    if order not in (0, 1, 2, 3, 4):
        raise NotImplementedError("HDivSurface: orders 0 to 4 are supported")
    return TraceSpace(mesh, ("RT0", "HDIV1", "HDIV2", "HDIV3", "HDIV4")[order], False, complex, definedon)


def HCurl(mesh: Mesh, order: int = 0, complex: bool = False, definedon=None) -> TraceSpace:
    """Surface trace of the Nedelec space (NGSolve HCurl restricted to the boundary): order 0
    one dof per edge, on each triangle n x the RT0 shape function of that edge; order 1..4 n x the
    HDivSurface shapes of that order, with the same dofs (order 3 serves the Maxwell double
    layer, order 4 mass matrices and load vectors)."""
    if order not in (0, 1, 2, 3, 4):
        raise NotImplementedError("HCurl: orders 0 to 4 are supported")
    return TraceSpace(mesh, ("HCURL", "HCURL1", "HCURL2", "HCURL3", "HCURL4")[order], False, complex, definedon)


def cluster_tree(space: TraceSpace, leafsize: int = 40):
    """Cluster tree of a space (host): (perm, int fields [nc,7], float fields [nc,23])."""
    maxc = 4 * space.ndof + 8
    perm = np.zeros(space.ndof, dtype=np.int32)
    ci = np.zeros(7 * maxc, dtype=np.int64)
    cd = np.zeros(23 * maxc, dtype=np.float64)
    nc = C.c_int()
    check(lib.bem_cluster_tree(space.h, leafsize, perm.ctypes.data_as(_lib._ip), maxc, C.byref(nc),
                               ci.ctypes.data_as(_lib._lp), cd.ctypes.data_as(_lib._dp)))
    n = nc.value
    return perm, ci[: 7 * n].reshape(n, 7), cd[: 23 * n].reshape(n, 23)


class Potential:
    """Field of a density at arbitrary points (the role of the reference's PotentialCF): FP64,
    the trial space's elements (within the operator's trial definedon region, if any) and the
    regular rule's points, the operator's kernel terms without their factors (as there)."""

    def __init__(self, op: "IntegralOperator", gf):
        torch = _torch()
        self.op = op
        h = op.mat.h
        d = C.c_int()
        check(lib.bem_operator_potential_dim(h, C.byref(d)))
        if d.value == 0:
            raise ValueError("this operator has no potential")
        self.dim = d.value
        dt = torch.complex128 if op.mat.is_complex else torch.float64
        if not isinstance(gf, torch.Tensor):
            gf = torch.as_tensor(np.asarray(gf)).cuda()
        self.density = _as_device(gf, dt).contiguous()
        if self.density.shape[0] != op.mat.width:
            raise ValueError("density length does not match the trial space")

    def __call__(self, points, normals=None):
        torch = _torch()

        def dev(a):
            return _as_device(a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a)).cuda(),
                              torch.float64).reshape(-1, 3).contiguous()
        P = dev(points)
        Nn = None if normals is None else dev(normals)
        out = torch.empty((P.shape[0], self.dim), dtype=self.density.dtype, device=P.device)
        stream = torch.cuda.current_stream().cuda_stream
        check(lib.bem_operator_potential(self.op.mat.h, C.c_void_p(self.density.data_ptr()), P.shape[0],
                                         C.c_void_p(P.data_ptr()),
                                         C.c_void_p(Nn.data_ptr()) if Nn is not None else None,
                                         C.c_void_p(out.data_ptr()), C.c_void_p(stream)))
        return out[:, 0] if self.dim == 1 else out


def tc_selftest() -> bool:
    """Known-answer check of the tensor-core encodings on the current GPU (True: exact)."""
    ok = C.c_int()
    check(lib.bem_tc_selftest(C.byref(ok)))
    return bool(ok.value)


def partition(trial: TraceSpace, test: TraceSpace | None = None, leafsize: int = 40, eta: float = 2.0):
    """Block partition (host): dict of rowcl, colcl, near arrays in the reference order."""
    test = trial if test is None else test
    maxb = 64 * max(trial.ndof, test.ndof) + 64
    arrs = [np.zeros(maxb, dtype=np.int32) for _ in range(3)]
    nb = C.c_int()
    check(lib.bem_partition(trial.h, test.h, leafsize, float(eta), maxb, C.byref(nb),
                            *[a.ctypes.data_as(_lib._ip) for a in arrs]))
    n = nb.value
    return dict(rowcl=arrs[0][:n], colcl=arrs[1][:n], near=arrs[2][:n])


# ----------------------------------------------------------------------------------------
# matrices
# ----------------------------------------------------------------------------------------
def _as_device(x, dtype):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            raise ValueError("torch vectors must live on the GPU")
        if x.dtype != dtype:
            x = x.to(dtype)
        return x.contiguous()
    raise TypeError("expected a torch CUDA tensor")


class BaseMatrix:
    """Linear operator algebra (sums, scalings, transposes) over GPU vectors."""

    height: int
    width: int
    is_complex: bool

    # y = s * A x + y
    def MultAdd(self, s, x, y):
        self._apply(False, s, x, 1.0, y)

    def MultTransAdd(self, s, x, y):
        self._apply(True, s, x, 1.0, y)

    def Mult(self, x, y):
        self._apply(False, 1.0, x, 0.0, y)

    def MultTrans(self, x, y):
        self._apply(True, 1.0, x, 0.0, y)

    @property
    def T(self):
        return _Transposed(self)

    def CreateRowVector(self):
        return self._vec(self.width)

    def CreateColVector(self):
        return self._vec(self.height)

    def _vec(self, n):
        torch = _torch()
        return torch.zeros(n, dtype=torch.complex128 if self.is_complex else torch.float64, device="cuda")

    def __mul__(self, x):
        if isinstance(x, BaseMatrix):
            raise NotImplementedError("matrix products are not supported")
        if isinstance(x, np.ndarray):
            return self._apply_host(False, x)
        y = self.CreateColVector() if not (x.is_complex() and not self.is_complex) else None
        if y is None:
            raise TypeError("complex vector on a real operator")
        self.Mult(x, y)
        return y

    def __rmul__(self, s):
        return _Scaled(self, s)

    def __add__(self, other):
        return _Sum([(1.0, self), (1.0, other)])

    def __sub__(self, other):
        return _Sum([(1.0, self), (-1.0, other)])

    def __neg__(self):
        return _Scaled(self, -1.0)

    def _terms(self):
        return [(1.0, self)]

    def _apply_host(self, trans, x):
        torch = _torch()
        xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        y = self._vec(self.width if trans else self.height)
        self._apply(trans, 1.0, xd, 0.0, y)
        return y.cpu().numpy()


class _Scaled(BaseMatrix):
    def __init__(self, A, s):
        self.A, self.s = A, s
        self.height, self.width = A.height, A.width
        self.is_complex = A.is_complex or isinstance(s, complex)

    def _apply(self, trans, alpha, x, beta, y):
        self.A._apply(trans, alpha * self.s, x, beta, y)

    def _terms(self):
        return [(self.s * c, M) for c, M in self.A._terms()]


class _Sum(BaseMatrix):
    def __init__(self, terms):
        self.parts = terms
        self.height, self.width = terms[0][1].height, terms[0][1].width
        for _, M in terms:
            if (M.height, M.width) != (self.height, self.width):
                raise ValueError("matrix sizes differ")
        self.is_complex = any(M.is_complex or isinstance(c, complex) for c, M in terms)

    def _apply(self, trans, alpha, x, beta, y):
        b = beta
        for c, M in self.parts:
            M._apply(trans, alpha * c, x, b, y)
            b = 1.0

    def _terms(self):
        out = []
        for c, M in self.parts:
            out += [(c * c2, M2) for c2, M2 in M._terms()]
        return out


class _Transposed(BaseMatrix):
    def __init__(self, A):
        self.A = A
        self.height, self.width = A.width, A.height
        self.is_complex = A.is_complex

    def _apply(self, trans, alpha, x, beta, y):
        self.A._apply(not trans, alpha, x, beta, y)

    @property
    def T(self):
        return self.A


class _NativeMatrix(BaseMatrix):
    """A matrix owned by the C library (H-matrix or sparse mass matrix)."""

    def __init__(self, handle):
        self.h = handle
        info = _lib.OperatorInfo()
        check(lib.bem_operator_info(self.h, C.byref(info)))
        self.info = {k: (list(getattr(info, k)) if k in ("mv_items", "mv_ranges") else getattr(info, k))
                     for k, _ in _lib.OperatorInfo._fields_}
        self.height, self.width = info.height, info.width
        self.is_complex = bool(info.is_complex)

    @property
    def nze(self):
        return int(self.info["nze"])

    def _apply(self, trans, alpha, x, beta, y):
        torch = _torch()
        dt = torch.complex128 if self.is_complex else torch.float64
        nin, nout = (self.height, self.width) if trans else (self.width, self.height)
        if not (isinstance(y, torch.Tensor) and y.is_cuda and y.dtype == dt and y.is_contiguous()):
            raise TypeError(f"y must be a contiguous CUDA tensor of dtype {dt}")
        xd = _as_device(x, dt)
        if xd.shape[0] != nin or y.shape[0] != nout:
            raise ValueError("vector length does not match the matrix")
        nrhs = 1 if xd.dim() == 1 else xd.shape[1]
        if xd.dim() == 2:
            # column-major right-hand sides: each column contiguous
            xd = xd.t().contiguous()
            yt = y.t().contiguous() if beta != 0 else torch.empty((nrhs, nout), dtype=dt, device=y.device)
        else:
            yt = y
        stream = torch.cuda.current_stream().cuda_stream
        check(lib.bem_operator_mult(self.h, int(trans), cplx2(alpha), C.c_void_p(xd.data_ptr()), cplx2(beta),
                                    C.c_void_p(yt.data_ptr()), nrhs, C.c_void_p(stream)))
        if xd.dim() == 2:
            y.copy_(yt.t())

    def mult_host(self, x: np.ndarray, trans=False, alpha=1.0, beta=0.0, y: np.ndarray | None = None):
        """Apply with host buffers through bem_operator_mult_host: page-locked buffers are read and
        written by the kernels in place, others are staged through device copies."""
        dt = np.complex128 if self.is_complex else np.float64
        x = np.ascontiguousarray(x, dtype=dt)
        nrhs = 1 if x.ndim == 1 else x.shape[1]
        xc = x if x.ndim == 1 else np.asfortranarray(x)
        nout = self.width if trans else self.height
        if y is None:
            y = np.zeros((nout,) if x.ndim == 1 else (nout, nrhs), dtype=dt, order="F")
        check(lib.bem_operator_mult_host(self.h, int(trans), cplx2(alpha), C.c_void_p(xc.ctypes.data),
                                         cplx2(beta), C.c_void_p(y.ctypes.data), nrhs))
        return y

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            lib.bem_operator_destroy(self.h)
            self.h = C.c_void_p()


class HMatrix(_NativeMatrix):
    """H-matrix (reference HMatrix<T>, src/hmat.hpp:162-201) resident in GPU memory."""

    def blocks(self):
        n = self.info["nblocks"]
        arrs = [np.zeros(n, dtype=np.int32) for _ in range(5)]
        check(lib.bem_operator_blocks(self.h, *[a.ctypes.data_as(_lib._ip) for a in arrs]))
        return dict(zip(["rowcl", "colcl", "near", "rank", "fallback"], arrs))

    def set_accuracy(self, compensated: bool = True):
        """FP32-stored operators: error-free (True, default) or plain FP32 (False) matvec arithmetic."""
        check(lib.bem_operator_set_accuracy(self.h, int(bool(compensated))))

    def autotune(self, reps: int = 10) -> dict:
        """Time the single-vector matvec for each piece size and schedule; keep the fastest."""
        piece, fused, ms = C.c_int(), C.c_int(), C.c_double()
        check(lib.bem_operator_autotune(self.h, int(reps), C.byref(piece), C.byref(fused), C.byref(ms)))
        self.tuned = {"piece": piece.value, "fused": bool(fused.value), "ms": ms.value}
        return self.tuned

    def save(self, path: str):
        """Write the assembled H-matrix (partition, ranks, dense blocks, factors) to a file."""
        check(lib.bem_operator_save(self.h, str(path).encode()))

    @classmethod
    def load(cls, path: str, trial_space: "TraceSpace", test_space: "TraceSpace | None" = None) -> "HMatrix":
        """An H-matrix saved by save(), on the same trial and test spaces, without assembly."""
        h = C.c_void_p()
        check(lib.bem_operator_load(str(path).encode(), trial_space.h,
                                    (test_space or trial_space).h, C.byref(h)))
        return cls(h)

    def set_global_dofs(self, trial_map, trial_nglobal: int, test_map=None, test_nglobal: int | None = None):
        """Apply the matrix to vectors in a global dof numbering (the reference's HMatrix acts on
        the FE space's full vectors, width_vol_dof x height_vol_dof, src/hmat.hpp:178-179):
        dof d of the trial space is entry trial_map[d] of a vector of trial_nglobal entries
        (test likewise; test_map None: the compact test numbering).  Entries that hold no dof of
        the output are
        set to beta * y (Mult: 0).  trial_map None restores the compact numbering.  Solves with
        GMRes keep the compact numbering and refuse a matrix with global numbering."""
        def arr(m):
            return None if m is None else np.ascontiguousarray(m, dtype=np.int32)
        tm, em = arr(trial_map), arr(test_map)
        check(lib.bem_operator_set_global_dofs(self.h, int(trial_nglobal or 0),
                                               None if tm is None else tm.ctypes.data_as(_lib._ip),
                                               int(test_nglobal or 0),
                                               None if em is None else em.ctypes.data_as(_lib._ip)))
        self.width = int(trial_nglobal) if tm is not None else self.info["width"]
        self.height = int(test_nglobal) if em is not None else self.info["height"]
        self.global_numbering = tm is not None or em is not None

    def set_tensor_cores(self, enable: bool = True):
        """Tensor-core products for 2..32 right-hand sides at plain accuracy (complex FP32 storage):
        True builds the packed panels now when the operator qualifies, False turns them off."""
        check(lib.bem_operator_set_tensor_cores(self.h, int(bool(enable))))

    def tensor_cores(self) -> dict:
        """State of the tensor-core path: 1 built, 0 not built, -1 not applicable."""
        st, nb_, i0, i1, ms = C.c_int(), C.c_longlong(), C.c_int(), C.c_int(), C.c_double()
        check(lib.bem_operator_tensor_cores(self.h, C.byref(st), C.byref(nb_), C.byref(i0), C.byref(i1),
                                            C.byref(ms)))
        return {"state": st.value, "bytes": nb_.value, "items": (i0.value, i1.value), "ms_build": ms.value}

    def autotune_tensor_cores(self, reps: int = 5) -> dict:
        """Tune the tensor-core stage plan (2, 3 or 4 pipeline stages) on this operator: the kept
        stage count and the time per 32-right-hand-side application of each."""
        n = C.c_int()
        ms = (C.c_double * 3)()
        check(lib.bem_operator_autotune_tc(self.h, int(reps), C.byref(n), ms))
        return {"stages": n.value, "ms": {2: ms[0], 3: ms[1], 4: ms[2]}}

    def set_profiling(self, enable: bool = True):
        check(lib.bem_operator_set_profiling(self.h, int(bool(enable))))

    def kernel_times(self):
        """Accumulated (ms, launches) of [permute_in, stage1, apply, permute_out]."""
        ms = (C.c_double * 4)()
        n = (C.c_longlong * 4)()
        check(lib.bem_operator_kernel_times(self.h, ms, n))
        return list(ms), list(n)

    def to_dense(self) -> np.ndarray:
        dt = np.complex128 if self.is_complex else np.float64
        out = np.zeros((self.height, self.width), dtype=dt)
        check(lib.bem_operator_to_dense(self.h, C.c_void_p(out.ctypes.data)))
        return out


class MassMatrix(_NativeMatrix):
    """Sparse Galerkin mass matrix <u, v> of identity traces (rows = test dofs)."""

    def to_dense(self) -> np.ndarray:
        """The matrix as a dense (height, width) array (real entries)."""
        dt = np.complex128 if self.is_complex else np.float64
        out = np.zeros((self.height, self.width), dtype=dt)
        check(lib.bem_operator_to_dense(self.h, C.c_void_p(out.ctypes.data)))
        return out.real.copy() if self.is_complex else out

    def Inverse(self, freedofs=None, tol=1e-14, maxiter=2000, direct_max=12000):
        """The inverse (the role of ``BilinearForm(...).Assemble().mat.Inverse(freedofs=...)`` as
        the reference's tests use it for GMRes preconditioners); dofs outside freedofs map to 0.
        Up to direct_max free dofs: a Cholesky factorisation on the GPU, once; above: conjugate
        gradients with this matrix's products, to tol relative."""
        if self.height != self.width:
            raise ValueError("only square mass matrices have an inverse")
        nfree = self.height if freedofs is None else int(np.count_nonzero(freedofs))
        if nfree <= direct_max:
            return _MassCholesky(self, freedofs)
        return _MassInverse(self, freedofs, tol, maxiter)


class _MassCholesky(BaseMatrix):
    """M^-1 of a symmetric positive definite mass matrix through its Cholesky factor on the GPU,
    computed once (real M; it applies to real and complex vectors alike)."""
    any_field = True

    def __init__(self, M, freedofs):
        torch = _torch()
        self.height = self.width = M.height
        self.is_complex = M.is_complex
        D = M.to_dense()
        self.free = None if freedofs is None else np.flatnonzero(np.asarray(freedofs, dtype=bool))
        if self.free is not None:
            D = D[np.ix_(self.free, self.free)]
        self.L = torch.linalg.cholesky(torch.from_numpy(np.ascontiguousarray(D)).cuda())
        self.idx = None if self.free is None else torch.from_numpy(self.free).cuda()

    def _solve(self, x):
        torch = _torch()
        b = x if self.idx is None else x[self.idx]
        if torch.is_complex(b):
            Lc = self.L.to(b.dtype)
            z = torch.cholesky_solve(b.reshape(len(b), -1), Lc).reshape(b.shape)
        else:
            z = torch.cholesky_solve(b.reshape(len(b), -1), self.L).reshape(b.shape)
        if self.idx is None:
            return z
        out = torch.zeros_like(x)
        out[self.idx] = z
        return out

    def _apply(self, trans, alpha, x, beta, y):
        z = self._solve(x)
        torch = _torch()
        z = z.to(y.dtype) if torch.is_complex(y) else z.real
        if beta == 0.0:
            y.copy_(alpha * z)
        else:
            y.mul_(beta).add_(alpha * z)

    def __mul__(self, x):
        torch = _torch()
        if isinstance(x, np.ndarray):
            return (self * torch.from_numpy(np.ascontiguousarray(x)).cuda()).cpu().numpy()
        y = torch.zeros(self.height, dtype=x.dtype if x.is_complex() else torch.float64, device=x.device)
        self._apply(False, 1.0, x, 0.0, y)
        return y


class _MassInverse(BaseMatrix):
    """M^-1 of a symmetric positive definite mass matrix by conjugate gradients (real M; it
    applies to real and complex vectors alike)."""
    any_field = True

    def __init__(self, M, freedofs, tol, maxiter):
        self.M, self.tol, self.maxiter = M, float(tol), int(maxiter)
        self.height = self.width = M.height
        self.is_complex = M.is_complex
        self.freedofs = None if freedofs is None else np.asarray(freedofs, dtype=bool)
        self.last = None

    def _apply(self, trans, alpha, x, beta, y):
        from . import krylov
        torch = _torch()
        mask = None if self.freedofs is None else torch.as_tensor(self.freedofs).to(x.device)
        Mop = krylov.as_operator(self.M)

        def proj(v):
            return v if mask is None else torch.where(mask, v, torch.zeros((), dtype=v.dtype, device=v.device))
        z, it, rel = krylov.cg(lambda v: proj(Mop(proj(v))), proj(x), self.tol, self.maxiter)
        self.last = dict(iterations=it, residual=rel)
        z = z.to(y.dtype) if torch.is_complex(y) else z.real
        if beta == 0.0:
            y.copy_(alpha * z)
        else:
            y.mul_(beta).add_(alpha * z)

    def __mul__(self, x):
        # the result lives in the vector's field (a real inverse applies to complex vectors)
        torch = _torch()
        if isinstance(x, np.ndarray):
            return (self * torch.from_numpy(np.ascontiguousarray(x)).cuda()).cpu().numpy()
        y = torch.zeros(self.height, dtype=x.dtype if x.is_complex() else torch.float64, device=x.device)
        self._apply(False, 1.0, x, 0.0, y)
        return y


def MassOperator(trial_space: TraceSpace, test_space: TraceSpace | None = None, complex: bool = False) -> MassMatrix:
    test_space = trial_space if test_space is None else test_space
    h = C.c_void_p()
    check(lib.bem_mass_create(trial_space.h, test_space.h, int(bool(complex)), C.byref(h)))
    return MassMatrix(h)


# ----------------------------------------------------------------------------------------
# integral operators
# ----------------------------------------------------------------------------------------
class IntegralOperator:
    """Assembled layer-potential operator (reference IntegralOperator<T>, src/ngbem.hpp:32-87)."""

    def __init__(self, kernel, kappa, trial, test, trial_eval, test_eval, intorder, leafsize, eta, eps, method,
                 testhmatrix, precision="fp64", intorder_singular=None, intorder_regular=None, max_rank=None,
                 aca_eps_floor=None, trial_definedon=None, test_definedon=None):
        test = trial if test is None else test
        p = _lib.Params()
        check(lib.bem_params_default(C.byref(p)))
        p.intorder = int(intorder)
        p.intorder_singular = int(intorder_singular or 0)
        p.intorder_regular = int(intorder_regular or 0)
        p.leafsize = int(leafsize)
        p.eta = float(eta)
        p.eps = float(eps)
        p.method = _lib.METHODS[method]
        p.precision = _lib.PRECISIONS[precision]
        p.max_rank = int(max_rank or 0)
        p.aca_eps_floor = float(aca_eps_floor or 0.0)
        self.params = p
        self.kernel, self.kappa = kernel, kappa
        self.trial_space, self.test_space = trial, test
        self._evals = (trial_eval, test_eval)
        h = C.c_void_p()
        check(lib.bem_operator_create(KERNELS[kernel], float(kappa), trial.h, test.h, EVALS[trial_eval],
                                      EVALS[test_eval], C.byref(p), C.byref(h)))
        self.mat = HMatrix(h)
        # definedon regions (reference IntegralOperator ctor, src/ngbem.cpp:17-113): as there,
        # the assembled matrix does not read them; GetPotential sums over the trial region only
        self.trial_definedon, self.test_definedon = trial_definedon, test_definedon
        if trial_definedon is not None or test_definedon is not None:
            masks = [None if r is None else _region_mask(r, sp.mesh)
                     for r, sp in ((trial_definedon, trial), (test_definedon, test))]
            check(lib.bem_operator_set_definedon(h, *[None if m is None else C.c_void_p(m.ctypes.data)
                                                      for m in masks]))
        if testhmatrix:
            self._test_hmatrix()

    @property
    def info(self):
        return self.mat.info

    def GetPotential(self, gf):
        """Potential of the trial-space density gf (reference GetPotential, src/ngbem.cpp:1166-1172):
        a callable ``pot(points, normals=None)`` giving the field at points (n, 3) on the GPU, shape
        (n,) for scalar trial traces, else (n, dim).  As the reference's PotentialCF, the sum leaves
        out the kernel terms' factors; for the Maxwell double layer (six cross-product terms with
        factors +-1) it is therefore the reference's field, not the signed double-layer field."""
        return Potential(self, gf)

    def _test_hmatrix(self):
        """Reference testhmatrix diagnostic (src/ngbem.cpp:332-369): dense assembly plus 30
        power iterations of (D - H)^H (D - H); prints compression rate and 2-norm error."""
        torch = _torch()
        p = self.params
        dense = IntegralOperator(self.kernel, self.kappa, self.trial_space, self.test_space, *self._evals,
                                 p.intorder, p.leafsize, p.eta, p.eps, "dense", False,
                                 precision="fp64", intorder_singular=p.intorder_singular or None,
                                 intorder_regular=p.intorder_regular or None)
        print(f"dense: {self.mat.height} x {self.mat.width}")
        D, H = dense.mat, self.mat
        x = H.CreateRowVector()
        x.fill_(1.0)
        y = H.CreateColVector()
        for _ in range(30):
            x /= torch.linalg.vector_norm(x)
            D.Mult(x, y)
            H.MultAdd(-1.0, x, y)
            y = y.conj()
            D.MultTrans(y, x)
            H.MultTransAdd(-1.0, y, x)
            x = x.conj()
        rate = self.mat.nze / (float(self.mat.height) * self.mat.width)
        err = float(torch.sqrt(torch.linalg.vector_norm(x)))
        print(f"compression rate {rate}  2-norm error {err}")
        self.testhmatrix_result = (rate, err)


IntegralOperatorC = IntegralOperator


def _dense_args(method, leafsize, eta):
    # reference python_bem.cpp:30-33: method "dense" means one root block
    return method, leafsize, eta




def SingleLayerPotentialOperator(space, intorder=3, leafsize=40, eta=2., eps=1e-6, method="aca",
                                 testhmatrix=False, **gb):
    """Laplace single layer V (reference python_bem.cpp:27-38)."""
    return IntegralOperator("laplace_sl", 0.0, space, space, "id", "id", intorder, leafsize, eta, eps, method,
                            testhmatrix, **gb)


def DoubleLayerPotentialOperator(trial_space, test_space, trial_definedon=None, test_definedon=None, intorder=3,
                                 leafsize=40, eta=2., eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Laplace double layer K (reference python_bem.cpp:41-60)."""
    return IntegralOperator("laplace_dl", 0.0, trial_space, test_space, "id", "id", intorder, leafsize, eta, eps,
                            method, testhmatrix, trial_definedon=trial_definedon, test_definedon=test_definedon,
                            **gb)


def HypersingularOperator(space, definedon=None, intorder=3, leafsize=40, eta=2., eps=1e-6, method="aca",
                          testhmatrix=False, **gb):
    """Laplace hypersingular W with surface-curl traces (reference python_bem.cpp:63-75).
    As in the reference, method is not consulted (always an ACA H-matrix)."""
    return IntegralOperator("laplace_hs", 0.0, space, space, "rot", "rot", intorder, leafsize, eta, eps, "aca",
                            testhmatrix, trial_definedon=definedon, test_definedon=definedon, **gb)


def _kappa(kappa):
    if kappa is None:
        raise TypeError("kappa is required")
    return float(kappa)


def HelmholtzSingleLayerPotentialOperator(trial_space, test_space=None, kappa=None, intorder=3, leafsize=40, eta=2.,
                                          eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Helmholtz single layer (reference python_bem.cpp:79-87).  test_space=None uses the
    trial space (the reference dereferences the null test space there)."""
    return IntegralOperator("helmholtz_sl", _kappa(kappa), trial_space, test_space, "id", "id", intorder, leafsize,
                            eta, eps, "aca", testhmatrix, **gb)


def HelmholtzSingleLayerPotentialOperatorDKappa(trial_space, test_space=None, kappa=None, intorder=3, leafsize=40,
                                                eta=2., eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Derivative of the Helmholtz single layer with respect to kappa (no counterpart in the
    reference): the operator of the bilinear form d/dkappa <V_kappa u, v>, kernel
    i e^{i kappa |x-y|}/(4 pi).  Same arguments and assembly as
    HelmholtzSingleLayerPotentialOperator."""
    return IntegralOperator("helmholtz_sl_dkappa", _kappa(kappa), trial_space, test_space, "id", "id", intorder,
                            leafsize, eta, eps, method, testhmatrix, **gb)


def HelmholtzDoubleLayerPotentialOperator(trial_space, test_space=None, kappa=None, intorder=3, leafsize=40,
                                          eta=2., eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Helmholtz double layer (reference python_bem.cpp:91-99)."""
    return IntegralOperator("helmholtz_dl", _kappa(kappa), trial_space, test_space, "id", "id", intorder, leafsize,
                            eta, eps, "aca", testhmatrix, **gb)


def HelmholtzCombinedFieldOperator(trial_space, test_space=None, kappa=None, intorder=3, leafsize=40, eta=2.,
                                   eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Helmholtz combined field DL - i kappa SL (reference python_bem.cpp:102-110)."""
    return IntegralOperator("helmholtz_cf", _kappa(kappa), trial_space, test_space, "id", "id", intorder, leafsize,
                            eta, eps, "aca", testhmatrix, **gb)


def HelmholtzHypersingularOperator(trial_space, test_space=None, kappa=None, intorder=3, leafsize=40, eta=2.,
                                   eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Helmholtz hypersingular with [n x grad u; u] traces (reference python_bem.cpp:113-119)."""
    return IntegralOperator("helmholtz_hs", _kappa(kappa), trial_space, test_space, "helm", "helm", intorder,
                            leafsize, eta, eps, "aca", testhmatrix, **gb)


def MaxwellSingleLayerPotentialOperator(space, kappa, definedon=None, intorder=3, leafsize=40, eta=2., eps=1e-6,
                                        method="aca", testhmatrix=False, **gb):
    """Maxwell single layer on HDivSurface with [Piola u; div u] traces (reference
    python_bem.cpp:122-134): kappa <u,v> - 1/kappa <div u, div v> weighted by G."""
    return IntegralOperator("maxwell_sl", _kappa(kappa), space, space, "maxwell", "maxwell", intorder, leafsize,
                            eta, eps, "aca", testhmatrix, trial_definedon=definedon, test_definedon=definedon, **gb)


def _need_hcurl(space, what):
    if not space.kind.startswith("HCURL"):
        raise TypeError(f"{what} needs an HCurl space, got {space.kind}")


def MaxwellSingleLayerPotentialOperatorCurl(space, kappa, definedon=None, intorder=3, leafsize=40, eta=2.,
                                            eps=1e-6, method="aca", testhmatrix=False, **gb):
    """Maxwell single layer on HCurl with DiffOpMaxwell traces [n x u; curl u] (reference
    python_bem.cpp:137-150): kappa <n x u, n x v> - 1/kappa <curl u, curl v> weighted by G."""
    _need_hcurl(space, "MaxwellSingleLayerPotentialOperatorCurl")
    return IntegralOperator("maxwell_sl", _kappa(kappa), space, space, "maxwellcurl", "maxwellcurl", intorder,
                            leafsize, eta, eps, "aca", testhmatrix, trial_definedon=definedon,
                            test_definedon=definedon, **gb)


def MaxwellDoubleLayerPotentialOperator(trial_space, test_space, kappa, trial_definedon=None, test_definedon=None,
                                        intorder=3, leafsize=40, eta=2., eps=1e-6, method="aca", testhmatrix=False,
                                        **gb):
    """Maxwell double layer (reference python_bem.cpp:154-171): MaxwellDLKernel on the rotated
    trace n x u of the HCurl trial space and the identity trace of the test space (HDivSurface,
    as in the reference's Maxwell tests, or HCurl).  method "dense" gives one root block."""
    _need_hcurl(trial_space, "MaxwellDoubleLayerPotentialOperator (trial space)")
    if not (test_space.kind == "RT0" or test_space.kind.startswith(("HDIV", "HCURL"))):
        raise TypeError("MaxwellDoubleLayerPotentialOperator: the test space must be HDivSurface or HCurl")
    return IntegralOperator("maxwell_dl", _kappa(kappa), trial_space, test_space, "rotatedtrace", "id", intorder,
                            leafsize, eta, eps, method, testhmatrix, trial_definedon=trial_definedon,
                            test_definedon=test_definedon, **gb)


# ----------------------------------------------------------------------------------------
# GMRES
# ----------------------------------------------------------------------------------------
def GMRes(A, b, pre=None, freedofs=None, x=None, maxsteps=100, tol=1e-7, innerproduct=None, callback=None,
          restart=None, startiteration=0, printrates=False, reltol=None):
    """Restarted GMRES on the GPU for sums of native matrices (the role of
    ngsolve.krylovspace.GMRes in the reference tests).  Returns the solution vector; the
    iteration count and final relative residual are in GMRes.last."""
    torch = _torch()
    from . import krylov
    if innerproduct is not None:
        raise NotImplementedError("GMRes: inner products other than the Euclidean one are not supported")
    if pre is not None or freedofs is not None or isinstance(A, krylov.BlockMatrix) or \
            isinstance(b, krylov.BlockVector):
        # preconditioned or block systems: the Krylov iteration in torch on the GPU, every
        # operator and preconditioner application the library's own
        bd = krylov._data(b)
        if not isinstance(bd, torch.Tensor):
            bd = torch.as_tensor(np.asarray(bd)).cuda()
        cplx = bd.is_complex() or A.is_complex
        dt = torch.complex128 if cplx else torch.float64
        bd = bd.to(dt)
        x0 = None if x is None else krylov._data(x).to(dt)
        sol, it, res = krylov.gmres(krylov.as_operator(A), bd, pre=krylov.as_operator(pre), x0=x0,
                                    maxsteps=int(maxsteps), tol=float(reltol if reltol is not None else tol),
                                    restart=restart, freedofs=freedofs, callback=callback, printrates=printrates)
        GMRes.last = dict(iterations=it, residual=res)
        if x is not None:
            krylov._data(x).copy_(sol)
            return x
        return krylov.BlockVector.wrap(sol, b.sizes) if isinstance(b, krylov.BlockVector) else sol
    terms = A._terms() if isinstance(A, BaseMatrix) else [(1.0, A)]
    for _, M in terms:
        if not isinstance(M, _NativeMatrix):
            raise TypeError("GMRes needs sums of H-matrices and mass matrices")
        if getattr(M, "global_numbering", False):
            raise ValueError("GMRes works in the compact dof numbering: reset the matrix's global numbering "
                             "(set_global_dofs(None, 0))")
    cplx = any(M.is_complex or isinstance(c, complex) for c, M in terms)
    dt = torch.complex128 if cplx else torch.float64
    bd = _as_device(b, dt)
    xd = torch.zeros_like(bd) if x is None else _as_device(x, dt).clone()
    ops = (C.c_void_p * len(terms))(*[M.h for _, M in terms])
    coef = (C.c_double * (2 * len(terms)))()
    for k, (c, _) in enumerate(terms):
        z = complex(c)
        coef[2 * k], coef[2 * k + 1] = z.real, z.imag
    it, res = C.c_int(), C.c_double()
    stream = torch.cuda.current_stream().cuda_stream
    rtol = float(reltol if reltol is not None else tol)
    if bd.dim() == 2:
        # several right-hand sides (columns): solved together, one operator pass per step
        nrhs = bd.shape[1]
        bc = bd.t().contiguous()
        xc = xd.t().contiguous()
        resv = (C.c_double * nrhs)()
        check(lib.bem_gmres_batched(len(terms), ops, coef, nrhs, C.c_void_p(bc.data_ptr()), C.c_void_p(xc.data_ptr()),
                                    int(maxsteps), int(restart or min(maxsteps, 200)), rtol, C.byref(it), resv,
                                    C.c_void_p(stream)))
        GMRes.last = dict(iterations=it.value, residual=max(resv), residuals=list(resv))
        if printrates:
            print(f"GMRes iteration {it.value}, max residual = {max(resv)}")
        xd = xc.t().contiguous()
        if x is not None:
            x.copy_(xd)
            return x
        return xd
    check(lib.bem_gmres(len(terms), ops, coef, C.c_void_p(bd.data_ptr()), C.c_void_p(xd.data_ptr()), int(maxsteps),
                        int(restart or min(maxsteps, 200)), rtol, C.byref(it), C.byref(res), C.c_void_p(stream)))
    GMRes.last = dict(iterations=it.value, residual=res.value)
    if printrates:
        print(f"GMRes iteration {it.value}, residual = {res.value}")
    if x is not None:
        x.copy_(xd)
        return x
    return xd


GMRes.last = {}


# ----------------------------------------------------------------------------------------
# compression diagnostic
# ----------------------------------------------------------------------------------------
def TestCompression(nx=100, ny=100, eta=2.0, eps=1e-10, method="svd", seed=None, device=None):
    """The reference's compression diagnostic (python_bem.cpp:177-193, test_compression.cpp):
    the block 1/|x - y| between nx and ny random points of two unit cubes, the second shifted
    by 1 + sqrt(3)/eta along x (admissible for eta), compressed by a full SVD ("svd"), a
    randomized SVD of growing rank ("tsvd") or ACA with the eps scaling 2/3 eps / sqrt(nx ny)
    ("aca").  Returns (rank, Frobenius error, seconds), or (0, 0) for another method.  The
    reference draws the points with an unseeded rand(); here seed picks them (None: fresh).
    Runs in torch on device (default: the GPU when there is one)."""
    import time
    torch = _torch()
    if method not in ("svd", "tsvd", "aca"):
        return (0, 0)
    dev = torch.device(device) if device is not None else torch.device("cuda" if torch.cuda.is_available() else "cpu")
    rng = np.random.default_rng(seed)
    ax = rng.random((nx, 3))
    ay = rng.random((ny, 3))
    ay[:, 0] += 1.0 + np.sqrt(3.0) / eta
    A = torch.as_tensor(1.0 / np.linalg.norm(ax[:, None, :] - ay[None, :, :], axis=2), device=dev)

    def sync():
        if dev.type == "cuda":
            torch.cuda.synchronize(dev)

    sync()
    t0 = time.perf_counter()
    if method == "svd":
        U, S, Vh = torch.linalg.svd(A, full_matrices=False)
        num = int((S.abs() > eps).sum())
        Uk, Vk = U[:, :num] * S[:num].sqrt(), S[:num].sqrt()[:, None] * Vh[:num]
    elif method == "tsvd":
        Uk, Vk, num = _tsvd(A, eps, rng)
    else:
        Uk, Vk, num = _aca_dense(A, eps)
    sync()
    t = time.perf_counter() - t0
    err = float(torch.linalg.norm(A - Uk[:, :num] @ Vk[:num]))
    return (num, err, t)


def _tsvd(A, eps, rng):
    """Randomized SVD of growing rank (test_compression.cpp:80-122): ranks 5, 7, 10, ... until
    the last singular value drops below eps; rank = the index before the first one below eps."""
    torch = _torch()
    p = min(A.shape)
    rank = 5

    def cut(S):
        for j in range(1, len(S)):
            if S[j] < eps:
                return j - 1
        return None

    while rank < p:
        V = torch.as_tensor(rng.random((rank, A.shape[1])), device=A.device)
        U, S, _ = torch.linalg.svd(A @ V.T, full_matrices=False)
        U2, S, Vh = torch.linalg.svd(U.T @ A, full_matrices=False)
        U = U @ U2
        if float(S[rank - 1]) < eps:
            num = cut(S)
            if num is not None:
                return U * S.sqrt(), S.sqrt()[:, None] * Vh, num
        rank = int(rank * 1.5)
    U, S, Vh = torch.linalg.svd(A, full_matrices=False)
    num = cut(S)
    num = p if num is None else num
    return U * S.sqrt(), S.sqrt()[:, None] * Vh, num


def _aca_dense(A, eps):
    """ACA with partial pivoting on a dense matrix (test_compression.cpp:155-207): row pivot,
    column pivot excluding the previous ones, stop when |u_k||v_k| < eps' |A_k|_F with
    eps' = 2/3 eps / sqrt(m n)."""
    torch = _torch()
    m, n = A.shape
    U = torch.zeros((m, m), dtype=A.dtype, device=A.device)
    V = torch.zeros((n, n), dtype=A.dtype, device=A.device)
    epsk = 2.0 / 3.0 * eps / np.sqrt(m * n)
    ik, jk, ikm1, jkm1 = 0, 0, -1, -1
    norm2 = 0.0
    kmax = min(m, n)
    for k in range(kmax):
        v = A[ik] - V[:k].T @ U[ik, :k]
        av = v.abs()
        if jkm1 >= 0:
            av[jkm1] = -1.0
        jk = int(torch.argmax(av))
        v = v / v[jk]
        V[k] = v
        u = A[:, jk] - U[:, :k] @ V[:k, jk]
        U[:, k] = u
        au = u.abs()
        if ikm1 >= 0:
            au[ikm1] = -1.0
        ik = int(torch.argmax(au))
        nk = float(torch.linalg.vector_norm(v) * torch.linalg.vector_norm(u))
        norm2 += nk * nk
        if k:
            norm2 += 2.0 * float(((V[:k] @ v) * (U[:, :k].T @ u)).sum())
        ikm1, jkm1 = ik, jk
        if nk < epsk * np.sqrt(norm2):
            return U, V, k + 1
    return U, V, kmax

