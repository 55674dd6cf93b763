"""Maxwell double layer and the curl form of the Maxwell single layer on the HCurl space
(reference python_bem.cpp:137-171; kernels src/ngbem.hpp:440-510, traces src/diffops.hpp:62-255)
on the GPU.  Entry-level parity with the oracle is in the parity tests; here:
* the Calderon identity of the reference's Maxwell test, V j = (-1/2 M + K) m, on the exact
  traces of a dipole field with the GPU H-matrices (FP64 and mixed) and the GPU mass matrix:
  residual below the oracle's dense value at the same level plus the ACA tolerance;
* the single layer with DiffOpMaxwell traces equals the RT0 single layer (dense, 1e-13);
* the factories' argument checks.
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import icosphere
from _maxwell_fields import traces, calderon_residual

pytestmark = pytest.mark.gpu


def _mv(op, x):
    return (op.mat * torch.from_numpy(np.ascontiguousarray(x)).cuda()).cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_calderon_identity_hmatrix(oracle, precision):
    m = icosphere(3)
    kappa = 1.0
    HC, RT = nb.HCurl(m, complex=True), nb.HDivSurface(m, complex=True)
    kw = dict(intorder=3, leafsize=20, eps=1e-6, precision=precision)
    V = nb.MaxwellSingleLayerPotentialOperator(RT, kappa, **kw)
    K = nb.MaxwellDoubleLayerPotentialOperator(HC, RT, kappa, **kw)
    assert K.mat.height == RT.ndof and K.mat.width == HC.ndof and K.mat.info["nfar"] > 0 and K.mat.info["sum_rank"] > 0
    mh, jh, M = traces(oracle, m, kappa)
    Mg = nb.MassOperator(HC, RT, complex=True)
    Mm = (Mg * torch.from_numpy(mh).cuda()).cpu().numpy()
    assert np.linalg.norm(Mm - M @ mh) / np.linalg.norm(M @ mh) < 1e-12
    r = calderon_residual(_mv(V, jh), _mv(K, mh), Mm)
    assert r < 0.0069 + 1e-3, r


def test_curl_single_layer_equals_rt0_single_layer():
    m = icosphere(2)
    HC, RT = nb.HCurl(m, complex=True), nb.HDivSurface(m, complex=True)
    Vc = nb.MaxwellSingleLayerPotentialOperatorCurl(HC, 2.0, intorder=4, leafsize=10 ** 6, eta=0.0)
    Vd = nb.MaxwellSingleLayerPotentialOperator(RT, 2.0, intorder=4, leafsize=10 ** 6, eta=0.0)
    Dc, Dd = Vc.mat.to_dense(), Vd.mat.to_dense()
    assert np.linalg.norm(Dc - Dd) / np.linalg.norm(Dd) < 1e-13


def test_factory_argument_checks():
    m = icosphere(1)
    HC, RT, P0 = nb.HCurl(m), nb.HDivSurface(m), nb.SurfaceL2(m)
    with pytest.raises(TypeError):
        nb.MaxwellDoubleLayerPotentialOperator(RT, RT, 1.0)
    with pytest.raises(TypeError):
        nb.MaxwellDoubleLayerPotentialOperator(HC, P0, 1.0)
    with pytest.raises(TypeError):
        nb.MaxwellSingleLayerPotentialOperatorCurl(RT, 1.0)
    with pytest.raises(NotImplementedError):
        nb.HCurl(m, order=5)
