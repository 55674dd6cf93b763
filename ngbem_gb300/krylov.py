"""Preconditioned Krylov solves and block systems (the role of ngsolve.krylovspace.GMRes with
``pre=`` / ``freedofs=`` and of ngsolve's BlockMatrix / BlockVector, as the reference's tests
use them: tests/test_Laplace.py:56-60, tests/test_Maxwell_Box.py:44-50,
tests/test_FEMBEM_sphere.py:45-49).

Without a preconditioner, ``bem.GMRes`` runs the native GMRES of the library (operator
application captured in a CUDA graph).  With one, the iteration below runs in torch on the
vectors' device while every operator and preconditioner application is the library's own
(H-matrix products, sparse mass matrices and their inverses).  The functions here take
callables on vectors and are device-agnostic.

This module is a convenience for the solver pattern of the reference's tests, outside the
accelerated path: its loops are torch operations on a handful of vectors, launched one by one.
The accelerated solves are the library's native GMRES (CUDA-graph matvec) and its batched GMRES
for many right-hand sides.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["cg", "gmres", "BlockMatrix", "BlockVector", "as_operator"]


def _torch():
    import torch
    return torch


def _dot(a, b):
    torch = _torch()
    return torch.vdot(a, b) if a.is_complex() or b.is_complex() else torch.dot(a, b)


def cg(apply, b, tol=1e-14, maxiter=2000, x0=None):
    """Conjugate gradients for a Hermitian positive definite operator: (x, iterations, relative
    residual).  Stops when |r| <= tol |b|."""
    torch = _torch()
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    r = b - apply(x) if x0 is not None else b.clone()
    nb = float(torch.linalg.vector_norm(b))
    if nb == 0.0:
        return x, 0, 0.0
    p = r.clone()
    rr = _dot(r, r).real
    it = 0
    while it < maxiter and math.sqrt(float(rr)) > tol * nb:
        q = apply(p)
        a = rr / _dot(p, q).real
        x += a * p
        r -= a * q
        rr_new = _dot(r, r).real
        p = r + (rr_new / rr) * p
        rr = rr_new
        it += 1
    return x, it, math.sqrt(float(rr)) / nb


def gmres(apply, b, pre=None, x0=None, maxsteps=100, tol=1e-7, restart=None, freedofs=None, callback=None,
          printrates=False):
    """Restarted GMRES, left preconditioned: minimises |pre (b - A x)| over the Krylov space of
    pre A (classical Gram-Schmidt applied twice, Givens rotations).  Stops when that residual
    is below tol times its initial value.  freedofs (boolean mask) restricts the unknowns:
    entries outside it keep their initial values (x0, else zero), as with a Dirichlet lift.
    Returns (x, iterations, relative preconditioned residual)."""
    torch = _torch()
    dev, dt = b.device, b.dtype
    cplx = torch.is_complex(b)
    mask = None
    if freedofs is not None:
        mask = torch.as_tensor(np.asarray(freedofs, dtype=bool)).to(dev)

    def proj(v):
        return v if mask is None else torch.where(mask, v, torch.zeros((), dtype=v.dtype, device=dev))

    def P(v):
        return proj(v) if pre is None else proj(pre(proj(v)))

    def scal(z):  # a host scalar in the vectors' field
        return complex(z) if cplx else float(complex(z).real)

    x = torch.zeros_like(b) if x0 is None else x0.clone().to(dt)
    m = int(restart or min(maxsteps, 200))
    r = P(b - apply(x))
    beta0 = float(torch.linalg.vector_norm(r))
    if beta0 == 0.0:
        return x, 0, 0.0
    total, rel = 0, 1.0
    while total < maxsteps:
        beta = float(torch.linalg.vector_norm(r))
        rel = beta / beta0
        if rel <= tol:
            break
        V = [r / beta]
        H = np.zeros((m + 1, m), dtype=complex)
        g = np.zeros(m + 1, dtype=complex)
        g[0] = beta
        cs, sn = [], []
        k = 0
        while k < m and total < maxsteps:
            w = P(apply(V[k]))
            for _ in range(2):
                for j in range(k + 1):
                    h = scal(_dot(V[j], w))
                    H[j, k] += h
                    w = w - h * V[j]
            hn = float(torch.linalg.vector_norm(w))
            H[k + 1, k] = hn
            for j in range(k):
                t = cs[j] * H[j, k] + sn[j] * H[j + 1, k]
                H[j + 1, k] = -np.conj(sn[j]) * H[j, k] + cs[j] * H[j + 1, k]
                H[j, k] = t
            a, bb = H[k, k], H[k + 1, k]
            den = math.hypot(abs(a), abs(bb))
            if den == 0.0:
                c, sg = 1.0, 0.0
            elif a == 0:
                c, sg = 0.0, np.conj(bb) / abs(bb)
            else:
                c, sg = abs(a) / den, (a / abs(a)) * np.conj(bb) / den
            H[k, k] = c * a + sg * bb
            H[k + 1, k] = 0.0
            cs.append(c)
            sn.append(sg)
            g[k + 1] = -np.conj(sg) * g[k]
            g[k] = c * g[k]
            total += 1
            k += 1
            rel = abs(g[k]) / beta0
            if callback is not None:
                callback(total, rel)
            if printrates:
                print(f"GMRes iteration {total}, residual = {rel}")
            if rel <= tol or hn == 0.0:
                break
            V.append(w / hn)
        y = np.linalg.solve(np.triu(H[:k, :k]), g[:k]) if k else np.zeros(0)
        for j in range(k):
            x = x + scal(y[j]) * V[j]
        r = P(b - apply(x))
        rel = float(torch.linalg.vector_norm(r)) / beta0
        if rel <= tol:
            break
    return x, total, rel


class BlockVector:
    """Vectors of a block system side by side (the role of ngsolve's BlockVector): ``data`` is
    the concatenation, ``[i]`` the view of block i."""

    def __init__(self, blocks):
        torch = _torch()
        self.sizes = [int(v.shape[0]) for v in blocks]
        dt = torch.complex128 if any(v.is_complex() for v in blocks) else torch.float64
        self.data = torch.cat([v.to(dt) for v in blocks])

    @classmethod
    def wrap(cls, data, sizes):
        bv = cls.__new__(cls)
        bv.sizes = list(sizes)
        bv.data = data
        return bv

    def __getitem__(self, i):
        o = sum(self.sizes[:i])
        return self.data[o:o + self.sizes[i]]

    def __len__(self):
        return len(self.sizes)


class BlockMatrix:
    """A matrix of blocks, None for zero blocks (the role of ngsolve's BlockMatrix): rows of
    blocks with the library's matrices (or their sums, scalings, transposes, inverses).
    Applies to concatenated vectors or BlockVectors."""

    def __init__(self, rows):
        self.rows = [list(r) for r in rows]
        nr, nc = len(self.rows), len(self.rows[0])
        if any(len(r) != nc for r in self.rows):
            raise ValueError("every block row needs the same number of blocks")
        self.heights, self.widths = [None] * nr, [None] * nc
        for i, r in enumerate(self.rows):
            for j, M in enumerate(r):
                if M is None:
                    continue
                for lst, k, v in ((self.heights, i, M.height), (self.widths, j, M.width)):
                    if lst[k] is not None and lst[k] != v:
                        raise ValueError("block sizes do not fit together")
                    lst[k] = v
        if None in self.heights or None in self.widths:
            raise ValueError("every block row and column needs one block")
        self.height, self.width = sum(self.heights), sum(self.widths)
        self.is_complex = any(M is not None and M.is_complex for r in self.rows for M in r)

    def _apply(self, trans, alpha, x, beta, y):
        hs, ws = (self.widths, self.heights) if trans else (self.heights, self.widths)
        xo = [0] + [int(v) for v in np.cumsum(ws)]
        yo = [0] + [int(v) for v in np.cumsum(hs)]
        if beta == 0.0:
            y.zero_()
        elif beta != 1.0:
            y.mul_(beta)
        for i, r in enumerate(self.rows):
            for j, M in enumerate(r):
                if M is None:
                    continue
                oi, oj = (j, i) if trans else (i, j)
                _apply_block(M, trans, alpha, x[xo[oj]:xo[oj + 1]], y[yo[oi]:yo[oi + 1]])

    def Mult(self, x, y):
        self._apply(False, 1.0, _data(x), 0.0, _data(y))

    def MultTrans(self, x, y):
        self._apply(True, 1.0, _data(x), 0.0, _data(y))

    def __mul__(self, x):
        torch = _torch()
        xd = _data(x)
        dt = torch.complex128 if (self.is_complex or xd.is_complex()) else torch.float64
        y = torch.zeros(self.height, dtype=dt, device=xd.device)
        self._apply(False, 1.0, xd.to(dt), 0.0, y)
        return BlockVector.wrap(y, self.heights) if isinstance(x, BlockVector) else y


def _data(v):
    return v.data if isinstance(v, BlockVector) else v


def _apply_block(M, trans, alpha, x, y):
    """y += alpha M x (or M^T x); a real block in a complex system acts on the real and
    imaginary parts separately."""
    torch = _torch()
    if (torch.is_complex(x) or torch.is_complex(y)) and not M.is_complex and not getattr(M, "any_field", False):
        n = y.shape[0]
        tr = torch.zeros(n, dtype=torch.float64, device=y.device)
        ti = torch.zeros(n, dtype=torch.float64, device=y.device)
        M._apply(trans, 1.0, x.real.contiguous(), 0.0, tr)
        if torch.is_complex(x):
            M._apply(trans, 1.0, x.imag.contiguous(), 0.0, ti)
        y += alpha * torch.complex(tr, ti) if torch.is_complex(y) else alpha * tr
        return
    M._apply(trans, alpha, x, 1.0, y)


def as_operator(M):
    """A callable v -> M v for the matrices this package applies: the library's matrices and
    their algebra (anything with ``_apply``), BlockMatrix, dense torch tensors and callables."""
    torch = _torch()
    if M is None:
        return None
    if hasattr(M, "_apply"):
        def f(v):
            dt = torch.complex128 if (M.is_complex or torch.is_complex(v)) else torch.float64
            y = torch.zeros(M.height, dtype=dt, device=v.device)
            vv = v.to(dt)
            if torch.is_complex(vv) and not M.is_complex and not getattr(M, "any_field", False):
                # a real operator on a complex vector: real and imaginary parts separately
                yr = torch.zeros(M.height, dtype=torch.float64, device=v.device)
                yi = torch.zeros(M.height, dtype=torch.float64, device=v.device)
                M._apply(False, 1.0, vv.real.contiguous(), 0.0, yr)
                M._apply(False, 1.0, vv.imag.contiguous(), 0.0, yi)
                return torch.complex(yr, yi)
            M._apply(False, 1.0, vv, 0.0, y)
            return y
        return f
    if isinstance(M, torch.Tensor):
        return lambda v: M.to(torch.promote_types(M.dtype, v.dtype)) @ v.to(torch.promote_types(M.dtype, v.dtype))
    if callable(M):
        return M
    raise TypeError(f"cannot apply {type(M).__name__} as an operator")

