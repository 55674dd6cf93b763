"""Saving and loading an assembled H-matrix (bem_operator_save / bem_operator_load): the loaded
operator applies like the saved one (same blocks and factors; only the order of the FP64
atomic additions differs, 1e-12), keeps the partition and ranks, serves the tensor-core and
multi-RHS products, and refuses spaces whose cluster trees differ."""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300 import bem
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


@pytest.mark.parametrize("kernel,kind,kappa,prec", [("laplace_sl", "P0", 0.0, "mixed"),
                                                    ("helmholtz_cf", "P1", 5.0, "mixed"),
                                                    ("laplace_dl", "P1", 0.0, "fp64")])
def test_save_load_roundtrip(tmp_path, kernel, kind, kappa, prec):
    m = icosphere(3)
    cplx = kernel.startswith("helmholtz")
    sp = nb.TraceSpace(m, kind, complex=cplx)
    op = bem.IntegralOperator(kernel, kappa, sp, sp, "id", "id", 3, 20, 2.0, 1e-8, "aca", False, precision=prec)
    path = tmp_path / "op.bin"
    op.mat.save(str(path))
    sp2 = nb.TraceSpace(m, kind, complex=cplx)
    loaded = bem.HMatrix.load(str(path), sp2)
    assert loaded.info["nblocks"] == op.mat.info["nblocks"] and loaded.info["nze"] == op.mat.info["nze"]
    a, b = op.mat.blocks(), loaded.blocks()
    for k in a:
        assert np.array_equal(a[k], b[k])
    dt = torch.complex128 if cplx else torch.float64
    g = torch.Generator().manual_seed(3)
    x = torch.randn(sp.ndof, 4, generator=g, dtype=torch.float64).to(dt).cuda()
    y1, y2 = torch.empty_like(x), torch.empty_like(x)
    op.mat.Mult(x, y1)
    loaded.Mult(x, y2)
    assert rel(y2, y1) < 1e-12
    v1 = op.mat * x[:, 0].contiguous()
    v2 = loaded * x[:, 0].contiguous()
    assert rel(v2, v1) < 1e-12
    if cplx:  # plain accuracy, several right-hand sides: the tensor-core products on the loaded factors
        op.mat.set_accuracy(False)
        loaded.set_accuracy(False)
        op.mat.Mult(x, y1)
        loaded.Mult(x, y2)
        assert rel(y2, y1) < 1e-6


def test_load_refuses_other_spaces(tmp_path):
    m = icosphere(3)
    V = nb.SingleLayerPotentialOperator(nb.SurfaceL2(m), leafsize=20)
    path = tmp_path / "v.bin"
    V.mat.save(str(path))
    with pytest.raises(Exception):
        bem.HMatrix.load(str(path), nb.SurfaceL2(icosphere(2)))
    with pytest.raises(Exception):
        bem.HMatrix.load(str(path), nb.H1(m))
