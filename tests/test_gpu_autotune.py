"""Matvec autotuner (bem_operator_autotune): the chosen piece size and schedule are among the
candidates, and the operator applies the same matrix afterwards (FP64: 1e-12; mixed: 1e-12 in
the compensated mode, whose only rounding is that of the stored entries)."""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import icosphere

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_keeps_the_matvec(precision):
    m = icosphere(3)
    V = nb.SingleLayerPotentialOperator(nb.SurfaceL2(m), leafsize=20, eps=1e-8, precision=precision)
    x = torch.from_numpy(np.random.default_rng(5).standard_normal(m.nt)).cuda()
    y0 = (V.mat * x).cpu().numpy()
    t = V.mat.autotune(reps=3)
    assert t["piece"] in (256, 384, 512, 768, 1024, 1536, 2048) and t["ms"] > 0
    y1 = (V.mat * x).cpu().numpy()
    assert np.linalg.norm(y1 - y0) / np.linalg.norm(y0) < 1e-12
