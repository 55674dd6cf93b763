"""Products on vectors in a global dof numbering (bem_operator_set_global_dofs).

The reference's HMatrix is width_vol_dof x height_vol_dof (src/hmat.hpp:178-179): its blocks
gather x and scatter y through the FE space's global dof numbers, and a boundary space defined
on part of a volume mesh leaves most of them unused (src/ngbem.cpp:43-65,
tests/test_Laplace.py:27).  Here a random injective map into a longer vector plays that
numbering.  Every product form must give, on the mapped entries, the compact product of the
gathered input, and beta * y on the unused entries (the reference's Mult zeroes them, MultAdd
leaves them): same kernels, so 1e-12 (the order of FP64 atomic additions).
"""
import ctypes as C

import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import _lib
from ngbem_gb300.meshes import ellipsoid, icosphere

pytestmark = pytest.mark.gpu


def _map(ndof, extra, seed):
    n = 3 * ndof + extra
    return np.random.default_rng(seed).permutation(n)[:ndof].astype(np.int32), n


def _vec(n, nrhs, cplx, seed):
    g = np.random.default_rng(seed)
    v = g.standard_normal((n, nrhs))
    if cplx:
        v = v + 1j * g.standard_normal((n, nrhs))
    return v


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _check(mat, trans, nrhs, alpha, beta, seed, host=False):
    cplx = mat.is_complex
    tmap, tn = _map(mat.info["width"], 11, seed)
    emap, en = _map(mat.info["height"], 5, seed + 1)
    (imap, inn), (omap, on) = ((emap, en), (tmap, tn)) if trans else ((tmap, tn), (emap, en))
    xg = _vec(inn, nrhs, cplx, seed + 2)
    y0 = _vec(on, nrhs, cplx, seed + 3)
    # the compact product of the gathered input (no global numbering set)
    mat.set_global_dofs(None, 0)
    dt = torch.complex128 if cplx else torch.float64
    xc = torch.from_numpy(np.ascontiguousarray(xg[imap])).to(dt).cuda()
    yc = torch.zeros((len(omap), nrhs), dtype=dt, device="cuda")
    (mat.T if trans else mat).Mult(xc, yc)
    expect = beta * y0
    expect[omap] += alpha * yc.cpu().numpy()
    mat.set_global_dofs(tmap, tn, emap, en)
    assert (mat.width, mat.height) == (tn, en)
    if host:
        y = mat.mult_host(xg, trans=trans, alpha=alpha, beta=beta, y=np.asfortranarray(y0.copy()))
    else:
        x = torch.from_numpy(xg).to(dt).cuda()
        y = torch.from_numpy(y0.copy()).to(dt).cuda()
        (mat.MultTransAdd if trans else mat.MultAdd)(alpha, x, y) if beta == 1.0 else \
            mat._apply(trans, alpha, x, beta, y)
        torch.cuda.synchronize()
        y = y.cpu().numpy()
    mat.set_global_dofs(None, 0)
    assert _rel(y, expect) < 1e-12
    # untouched scaling on the unused entries
    free = np.setdiff1d(np.arange(on), omap)
    assert np.array_equal(np.asarray(y)[free], expect[free])


@pytest.fixture(scope="module")
def ops():
    m = icosphere(3)
    P0, P1 = nb.SurfaceL2(m), nb.H1(m)
    kw = dict(intorder=3, leafsize=20, eta=2.0, eps=1e-8)
    V = nb.SingleLayerPotentialOperator(P0, precision="mixed", **kw).mat
    K = nb.DoubleLayerPotentialOperator(P1, P0, precision="fp64", **kw).mat
    return V, K


@pytest.mark.parametrize("which,trans,nrhs,alpha,beta", [
    ("V", 0, 1, 1.0, 0.0),     # single launch, Mult
    ("V", 1, 1, 2.0, 1.0),     # transposed, MultAdd
    ("K", 0, 1, 1.0, 0.0),     # trial and test numberings differ
    ("K", 1, 1, -1.0, 0.5),
    ("K", 0, 3, 0.5, 1.0),     # several right-hand sides
    ("K", 1, 2, 1.0, 0.0),
])
def test_global_numbering_products(ops, which, trans, nrhs, alpha, beta):
    V, K = ops
    _check(V if which == "V" else K, trans, nrhs, alpha, beta, 10 + 7 * trans + nrhs)


def test_global_numbering_host_buffers_and_noalloc(ops):
    V, K = ops
    _check(K, 0, 1, 1.0, 0.0, 40, host=True)
    # the no-allocation product in the same numbering
    tmap, tn = _map(K.info["width"], 11, 41)
    emap, en = _map(K.info["height"], 5, 42)
    xg = torch.from_numpy(_vec(tn, 1, False, 43)[:, 0]).cuda()
    K.set_global_dofs(tmap, tn, emap, en)
    y1 = torch.full((en,), 3.0, dtype=torch.float64, device="cuda")
    y2 = y1.clone()
    K.Mult(xg, y1)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.lib.bem_operator_mult_noalloc(K.h, 0, _lib.cplx2(1.0), C.c_void_p(xg.data_ptr()),
                                                  _lib.cplx2(0.0), C.c_void_p(y2.data_ptr()), 1,
                                                  C.c_void_p(stream)))
    torch.cuda.synchronize()
    K.set_global_dofs(None, 0)
    assert (torch.linalg.vector_norm(y1 - y2) / torch.linalg.vector_norm(y1)).item() < 1e-12
    free = np.setdiff1d(np.arange(en), emap)
    assert torch.all(y2[torch.from_numpy(free).cuda()] == 0)


def test_global_numbering_tensor_cores():
    """Several complex right-hand sides at plain accuracy: the tensor-core product reads x and
    writes y through the same composed numbering."""
    m = ellipsoid(3, (1.0, 0.7, 0.5))
    P1 = nb.H1(m, complex=True)
    C32 = nb.HelmholtzCombinedFieldOperator(P1, P1, kappa=4.0, intorder=3, leafsize=20, eta=2.0, eps=1e-8,
                                            precision="mixed").mat
    C32.set_accuracy(False)
    C32.set_tensor_cores(True)
    assert C32.tensor_cores()["state"] == 1
    _check(C32, 0, 32, 1.0 + 0.5j, 0.0, 50)
    _check(C32, 0, 8, 1.0, 1.0, 51)
    C32.set_accuracy(True)


def test_global_numbering_argument_checks(ops):
    V, _ = ops
    n = V.info["width"]
    bad = np.zeros(n, dtype=np.int32)  # not injective
    with pytest.raises(_lib.BemError):
        V.set_global_dofs(bad, 2 * n)
    with pytest.raises(_lib.BemError):
        V.set_global_dofs(np.arange(n, dtype=np.int32), n - 1)  # too short
    with pytest.raises(_lib.BemError):
        V.set_global_dofs(np.arange(n, dtype=np.int32) + n, 2 * n - 1)  # out of range
    V.set_global_dofs(np.arange(n, dtype=np.int32)[::-1].copy(), n, np.arange(n, dtype=np.int32), n)
    with pytest.raises(ValueError):
        nb.GMRes(V, torch.ones(n, dtype=torch.float64, device="cuda"))
    V.set_global_dofs(None, 0)
