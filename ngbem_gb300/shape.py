"""Batched Laplace single-layer energy E_b = u_b^T V(X_b) u_b and its adjoint derivatives.

The reference has no derivatives; the energy is what ``u^T (V.mat * u)`` gives for
``V = SingleLayerPotentialOperator(SurfaceL2(mesh, order=0), ...)`` with dense assembly
(reference src/python_bem.cpp:27-40, src/ngbem.cpp:373-738).  Here it is evaluated for a
whole batch of meshes in one pass of device kernels (bem_sl_batch_eval), and
``SingleLayerEnergy.apply`` makes it a ``torch.autograd.Function``: the backward pass calls
the hand-written derivative kernels again (the quadrature is recomputed, not stored) and
returns dE/dX (exact for the discrete energy) and dE/du = 2 V u.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib
from .meshes import Mesh

__all__ = ["SingleLayerEnergyBatch", "SingleLayerEnergy", "HelmholtzEnergy"]


def _torch():
    import torch
    return torch


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class SingleLayerEnergyBatch:
    """Topology of a batch of closed triangle meshes (built once) for the energy kernels.

    meshes: list of ``Mesh``; intorder: order of the tensor triangle rule on element pairs
    without a common vertex; intorder_singular: Sauter-Schwab order on the others;
    precision: "fp64" or "mixed" (FP32 regular pairs, FP64 singular pairs);
    dual_mapping: P0 basis 1/|J| (then V_ij carries no |J| factors).
    """

    def __init__(self, meshes: list[Mesh], intorder: int = 3, intorder_singular: int = 4,
                 precision: str = "fp64", dual_mapping: bool = False):
        torch = _torch()
        self.meshes = list(meshes)
        self.nprob = len(self.meshes)
        nv = np.array([m.nv for m in self.meshes], dtype=np.int32)
        nt = np.array([m.nt for m in self.meshes], dtype=np.int32)
        tris = np.ascontiguousarray(np.concatenate([m.triangles for m in self.meshes]).astype(np.int32))
        self.vertex_offsets = np.concatenate([[0], np.cumsum(nv)]).astype(np.int64)
        self.triangle_offsets = np.concatenate([[0], np.cumsum(nt)]).astype(np.int64)
        self.nv_total, self.nt_total = int(nv.sum()), int(nt.sum())
        self.h = C.c_void_p()
        check(lib.bem_sl_batch_create(self.nprob, nv.ctypes.data_as(_lib._ip), nt.ctypes.data_as(_lib._ip),
                                      tris.ctypes.data_as(_lib._ip), int(intorder), int(intorder_singular),
                                      _lib.PRECISIONS[precision], int(bool(dual_mapping)), C.byref(self.h)))
        self.precision = precision
        problem = np.repeat(np.arange(self.nprob), nt)
        self.triangle_problem = torch.as_tensor(problem, dtype=torch.long, device="cuda")

    def __del__(self):
        try:
            if self.h:
                lib.bem_sl_batch_destroy(self.h)
        except Exception:
            pass

    def info(self) -> dict:
        nu, ns, npr = C.c_int(), C.c_int(), C.c_longlong()
        check(lib.bem_sl_batch_info(self.h, C.byref(nu), C.byref(ns), C.byref(npr)))
        return {"work_units": nu.value, "singular_pairs": ns.value, "regular_pairs": npr.value}

    def coordinates(self):
        """Vertex coordinates of all meshes, concatenated: (sum nv, 3) float64 on the GPU."""
        torch = _torch()
        return torch.as_tensor(np.concatenate([m.vertices for m in self.meshes]), dtype=torch.float64,
                               device="cuda").contiguous()

    def evaluate(self, X, u, weights=None, energy=True, vu=False, grad=False):
        """Raw evaluation: returns (energy[nprob] | None, vu[nt] | None, grad[nv, 3] | None)."""
        torch = _torch()
        X = X.detach().contiguous()
        u = u.detach().contiguous()
        if X.dtype != torch.float64 or u.dtype != torch.float64 or not X.is_cuda or not u.is_cuda:
            raise TypeError("X and u must be float64 CUDA tensors")
        if X.shape != (self.nv_total, 3) or u.shape != (self.nt_total,):
            raise ValueError(f"expected X of shape ({self.nv_total}, 3) and u of shape ({self.nt_total},)")
        E = torch.empty(self.nprob, dtype=torch.float64, device=X.device) if energy else None
        V = torch.empty(self.nt_total, dtype=torch.float64, device=X.device) if vu else None
        G = torch.empty_like(X) if grad else None
        w = weights.detach().to(torch.float64).contiguous() if weights is not None else None
        stream = torch.cuda.current_stream().cuda_stream
        check(lib.bem_sl_batch_eval(self.h, _ptr(X), _ptr(u), _ptr(w), _ptr(E), _ptr(V), _ptr(G),
                                    C.c_void_p(stream)))
        return E, V, G

    def __call__(self, X, u):
        return _function().apply(X, u, self)


def _make_function():
    torch = _torch()

    class _SingleLayerEnergy(torch.autograd.Function):
        """E_b(X, u) = u_b^T V(X_b) u_b for every problem b of a SingleLayerEnergyBatch."""

        @staticmethod
        def forward(ctx, X, u, batch):
            E, _, _ = batch.evaluate(X, u, energy=True)
            ctx.save_for_backward(X, u)
            ctx.batch = batch
            return E

        @staticmethod
        def backward(ctx, gE):
            X, u = ctx.saved_tensors
            batch = ctx.batch
            need_x, need_u = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
            gE = gE.contiguous()
            _, V, G = batch.evaluate(X, u, weights=gE, energy=False, vu=need_u, grad=need_x)
            gu = 2.0 * V * gE[batch.triangle_problem] if need_u else None
            return G if need_x else None, gu, None

    return _SingleLayerEnergy


class _Lazy:
    fn = None


def _function():
    if _Lazy.fn is None:
        _Lazy.fn = _make_function()
    return _Lazy.fn


def __getattr__(name):
    if name == "SingleLayerEnergy":
        return _function()
    raise AttributeError(name)


class HelmholtzEnergy:
    """E(kappa, u) = u^T V_kappa u for the Helmholtz single layer on a fixed trace space, as a
    function of the wavenumber and of a real density, returned as (Re E, Im E).

    ``energy(kappa, u)`` is differentiable (``torch.autograd``): the backward pass assembles the
    kappa-derivative operator (kernel i e^{i kappa r}/(4 pi), the same quadrature and
    H-matrix compression as V_kappa) and gives dE/dkappa = u^T (dV/dkappa) u and
    dE/du = (V_kappa + V_kappa^T) u.  The reference has no derivatives; E is what
    ``u^T (V.mat * u)`` gives for ``V = HelmholtzSingleLayerPotentialOperator(space, kappa=...)``.
    Operators are reassembled when kappa changes.
    """

    def __init__(self, space, intorder=3, leafsize=40, eta=2.0, eps=1e-8, method="aca", precision="fp64"):
        self.space = space
        self.kw = dict(intorder=intorder, leafsize=leafsize, eta=eta, eps=eps, method=method, precision=precision)
        self._ops = {}

    def operator(self, kappa: float, derivative: bool = False):
        from . import bem
        key = (float(kappa), bool(derivative))
        if key not in self._ops:
            if len(self._ops) >= 4:
                self._ops.clear()
            f = bem.HelmholtzSingleLayerPotentialOperatorDKappa if derivative else \
                bem.HelmholtzSingleLayerPotentialOperator
            self._ops[key] = f(self.space, self.space, kappa=float(kappa), **self.kw)
        return self._ops[key].mat

    def __call__(self, kappa, u):
        return _helmholtz_function().apply(kappa, u, self)


def _make_helmholtz_function():
    torch = _torch()

    def apply_op(A, u, trans=False):
        uc = u.to(torch.complex128)
        y = torch.empty_like(uc)
        (A.MultTrans if trans else A.Mult)(uc, y)
        return y

    class _HelmholtzEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, kappa, u, energy):
            k = float(kappa)
            V = energy.operator(k)
            E = torch.dot(u.to(torch.complex128), apply_op(V, u))
            ctx.save_for_backward(kappa, u)
            ctx.energy = energy
            return torch.stack([E.real, E.imag])

        @staticmethod
        def backward(ctx, gE):
            kappa, u = ctx.saved_tensors
            energy = ctx.energy
            k = float(kappa)
            gk = gu = None
            if ctx.needs_input_grad[0]:
                dE = torch.dot(u.to(torch.complex128), apply_op(energy.operator(k, derivative=True), u))
                gk = (gE[0] * dE.real + gE[1] * dE.imag).to(kappa.dtype).reshape(kappa.shape)
            if ctx.needs_input_grad[1]:
                V = energy.operator(k)
                w = apply_op(V, u) + apply_op(V, u, trans=True)
                gu = (gE[0] * w.real + gE[1] * w.imag).to(u.dtype)
            return gk, gu, None

    return _HelmholtzEnergy


class _LazyH:
    fn = None


def _helmholtz_function():
    if _LazyH.fn is None:
        _LazyH.fn = _make_helmholtz_function()
    return _LazyH.fn
