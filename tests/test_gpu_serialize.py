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


def _dense_descriptor_offset(raw, op):
    """Byte offset of the first dense-block descriptor (MVDense: ptr, r0, m, c0, n) in a saved
    operator file, found by walking the file's layout (the save order of serialize.cpp)."""
    import ctypes as C

    from ngbem_gb300 import _lib

    def count(o):
        return int(np.frombuffer(raw[o:o + 8], dtype=np.int64)[0])

    o = 8 + 4 + 8 + 4 + 4 + 4 + C.sizeof(_lib.Params) + 6 * 4 + 4 + 4 + 4 + 8  # ... nv, nt, geometry
    for _ in range(4):  # the two permutations and the two dof maps (int32)
        o += 8 + 4 * count(o)
    nb_ = count(o)
    assert nb_ == op.mat.info["nblocks"]
    o += 8 + 12 * nb_  # blocks: (rowcl, colcl, near) of 12 bytes
    for _ in range(2):  # ranks and fallback flags
        assert count(o) == nb_
        o += 8 + 4 * nb_
    o += C.sizeof(_lib.OperatorInfo)
    assert count(o) == op.mat.info["nnear"]
    return o + 8


def test_load_refuses_corrupt_files(tmp_path):
    """A truncated file, a precision out of range and a dense block reaching past the matrix
    are refused with BEM_ERR_ARG before anything is uploaded."""
    from ngbem_gb300._lib import BemError
    m = icosphere(2)
    sp = nb.SurfaceL2(m)
    V = nb.SingleLayerPotentialOperator(sp, leafsize=20, precision="mixed")
    path = tmp_path / "v.bin"
    V.mat.save(str(path))
    raw = bytearray(path.read_bytes())
    cases = {"truncated": raw[:-100]}
    bad = bytearray(raw)
    bad[28:32] = np.int32(7).tobytes()  # the precision field
    cases["precision"] = bad
    bad = bytearray(raw)
    o = _dense_descriptor_offset(raw, V)
    bad[o + 8:o + 12] = np.int32(sp.ndof).tobytes()  # r0 of the first dense block
    cases["extent"] = bad
    for name, data in cases.items():
        p = tmp_path / f"{name}.bin"
        p.write_bytes(bytes(data))
        with pytest.raises(BemError) as e:
            bem.HMatrix.load(str(p), nb.SurfaceL2(m))
        assert e.value.code == 1, name  # BEM_ERR_ARG
    # the intact file still loads
    assert bem.HMatrix.load(str(path), nb.SurfaceL2(m)).info["nblocks"] == V.mat.info["nblocks"]


def test_load_refuses_another_geometry(tmp_path):
    """An operator assembled on a curved mesh does not load onto the flat mesh of the same
    triangles (nor onto another curving), and loads onto its own."""
    from ngbem_gb300._lib import BemError
    mc = icosphere(2).Curve(3)
    V = nb.SingleLayerPotentialOperator(nb.SurfaceL2(mc), intorder=3, leafsize=20, eps=1e-8)
    path = tmp_path / "curved.bin"
    V.mat.save(str(path))
    for other in (icosphere(2), icosphere(2).Curve(2)):
        with pytest.raises(BemError) as e:
            bem.HMatrix.load(str(path), nb.SurfaceL2(other))
        assert e.value.code == 1
    W = bem.HMatrix.load(str(path), nb.SurfaceL2(mc))
    x = torch.from_numpy(np.random.default_rng(2).standard_normal(W.width)).cuda()
    y, z = W * x, V.mat * x
    assert (torch.linalg.vector_norm(y - z) / torch.linalg.vector_norm(z)).item() < 1e-12
