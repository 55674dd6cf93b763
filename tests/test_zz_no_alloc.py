"""bem_operator_mult_noalloc (fixed device scratch, no allocation) against bem_operator_mult.

Both entry points run the same kernels on the same operator data, so they agree up to the
order of the FP64 atomic additions: 1e-12 relative is the tolerance.  Each case calls the
no-allocation entry point twice in a row with different inputs (and then the first input
again), which checks that every call starts from cleared accumulators even though the
scratch area keeps the previous call's contents.  The reference products come first: they
build the work lists of each form, which the no-allocation entry point uses but never builds.  Kept last in collection order so that it
runs both after the other GPU tests and, alone, in a fresh process.
"""
import ctypes as C

import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import _lib, bem
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _operator(kernel, trial, test, kappa, precision, level=3):
    m = icosphere(level)
    trs = nb.TraceSpace(m, trial)
    tes = trs if test == trial else nb.TraceSpace(m, test)
    return bem.IntegralOperator(kernel, kappa, trs, tes, "id", "id", 3, 20, 2.0, 1e-8, "aca", False,
                                precision=precision).mat


def _call(fn, mat, trans, alpha, x, beta, y, nrhs):
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(fn(mat.h, int(trans), _lib.cplx2(alpha), C.c_void_p(x.data_ptr()), _lib.cplx2(beta),
                  C.c_void_p(y.data_ptr()), nrhs, C.c_void_p(stream)))


def _vectors(mat, trans, nrhs, seed):
    dt = torch.complex128 if mat.is_complex else torch.float64
    nin, nout = (mat.height, mat.width) if trans else (mat.width, mat.height)
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(nrhs * nin, dtype=dt, generator=g).cuda()
    y0 = torch.randn(nrhs * nout, dtype=dt, generator=g).cuda()
    return x, y0


def _rel(a, b):
    return (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()


CASES = [
    # kernel, trial, test, kappa, precision, trans, alpha, beta, nrhs
    ("laplace_sl", "P0", "P0", 0.0, "mixed", 0, 1.0, 0.0, 1),
    ("laplace_sl", "P0", "P0", 0.0, "fp64", 0, 1.0, 0.0, 1),
    ("laplace_dl", "P1", "P0", 0.0, "mixed", 0, 2.0, 0.5, 1),
    ("laplace_dl", "P1", "P0", 0.0, "fp64", 1, -1.5, 1.0, 1),
    ("helmholtz_sl", "P0", "P0", 3.0, "mixed", 0, 1.0 + 0.5j, 0.0, 3),
    ("helmholtz_dl", "P1", "P1", 3.0, "fp64", 1, 1.0, 0.25j, 2),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}{c[2]}-{c[4]}-t{c[5]}-r{c[8]}" for c in CASES])
def test_noalloc_matches_mult(case):
    kernel, trial, test, kappa, precision, trans, alpha, beta, nrhs = case
    mat = _operator(kernel, trial, test, kappa, precision)
    x1, y1 = _vectors(mat, trans, nrhs, 1)
    x2, y2 = _vectors(mat, trans, nrhs, 2)
    ref1, ref2 = y1.clone(), y2.clone()
    _call(_lib.lib.bem_operator_mult, mat, trans, alpha, x1, beta, ref1, nrhs)
    _call(_lib.lib.bem_operator_mult, mat, trans, alpha, x2, beta, ref2, nrhs)
    a1, a2, a3 = y1.clone(), y2.clone(), y1.clone()
    _call(_lib.lib.bem_operator_mult_noalloc, mat, trans, alpha, x1, beta, a1, nrhs)
    _call(_lib.lib.bem_operator_mult_noalloc, mat, trans, alpha, x2, beta, a2, nrhs)
    _call(_lib.lib.bem_operator_mult_noalloc, mat, trans, alpha, x1, beta, a3, nrhs)
    torch.cuda.synchronize()
    assert _rel(a1, ref1) < TOL
    assert _rel(a2, ref2) < TOL
    assert _rel(a3, ref1) < TOL


def test_noalloc_leaves_device_memory_alone():
    # the first call on the device looks the array up (and may load the device code holding it)
    warm = _operator("laplace_sl", "P0", "P0", 0.0, "mixed", level=2)
    xw, yw = _vectors(warm, 0, 1, 3)
    _call(_lib.lib.bem_operator_mult_noalloc, warm, 0, 1.0, xw, 0.0, yw, 1)
    # a fresh operator: already its first no-allocation product allocates nothing
    mat = _operator("laplace_sl", "P0", "P0", 0.0, "mixed")
    x, y = _vectors(mat, 0, 1, 3)
    ref = y.clone()
    _call(_lib.lib.bem_operator_mult, mat, 0, 1.0, x, 0.0, ref, 1)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        _call(_lib.lib.bem_operator_mult_noalloc, mat, 0, 1.0, x, 0.0, y, 1)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0
    assert _rel(y, ref) < TOL


def test_noalloc_never_builds_work_lists():
    """A form whose work lists the operator does not have yet is refused (BEM_ERR_STATE)
    instead of building them; one bem_operator_mult of that form builds them."""
    mat = _operator("laplace_dl", "P1", "P0", 0.0, "mixed")
    x, y = _vectors(mat, 1, 1, 5)
    with pytest.raises(_lib.BemError) as e:
        _call(_lib.lib.bem_operator_mult_noalloc, mat, 1, 1.0, x, 0.0, y, 1)
    assert e.value.code == _lib.BEM_ERR_STATE and "bem_operator_mult" in str(e.value)
    ref = y.clone()
    _call(_lib.lib.bem_operator_mult, mat, 1, 1.0, x, 0.0, ref, 1)
    _call(_lib.lib.bem_operator_mult_noalloc, mat, 1, 1.0, x, 0.0, y, 1)
    torch.cuda.synchronize()
    assert _rel(y, ref) < TOL


def test_noalloc_rejects_oversized_scratch():
    mat = _operator("laplace_sl", "P0", "P0", 0.0, "mixed")
    nrhs = 1200  # permuted input + accumulator alone exceed the fixed area
    assert 2 * 8 * mat.width * nrhs > _lib.NOALLOC_SCRATCH_BYTES
    x, y = _vectors(mat, 0, nrhs, 4)
    with pytest.raises(_lib.BemError) as e:
        _call(_lib.lib.bem_operator_mult_noalloc, mat, 0, 1.0, x, 0.0, y, nrhs)
    assert e.value.code == _lib.BEM_ERR_ARG and "scratch" in str(e.value)


def test_noalloc_rejects_mass_operator():
    M = bem.MassOperator(nb.TraceSpace(icosphere(2), "P0"))
    x = torch.zeros(M.width, dtype=torch.float64, device="cuda")
    y = torch.zeros(M.height, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.BemError) as e:
        _call(_lib.lib.bem_operator_mult_noalloc, M, 0, 1.0, x, 0.0, y, 1)
    assert e.value.code == _lib.BEM_ERR_STATE
