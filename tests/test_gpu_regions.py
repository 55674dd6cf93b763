"""Spaces and operators on mesh regions (`definedon`) on the GPU.

* A space on a region is the space of the mesh made of the region's triangles: the operators
  between region spaces equal the operators on that submesh (GPU against GPU, dense 1e-12 and
  H-matrix matvec 1e-12) and the oracle's dense operator on the submesh (1e-10).
* A region test space with a whole-mesh trial space (the FEM-BEM coupling pattern
  K(fesH1, fesL2 on "outer")) gives the whole-mesh matrix's rows of the region's dofs.
* The mass matrix between region spaces equals the oracle's on the submesh.
* Operator definedon regions do not change the matrix (as in the reference) and restrict
  GetPotential's elements to the trial region (PotentialCF, reference src/ngbem.cpp:1205).
"""
import numpy as np
import pytest
import torch

import ngbem_gb300 as nb
from ngbem_gb300.meshes import Mesh, icosphere

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _mesh(level=3):
    m0 = icosphere(level)
    cap = (m0.centroids()[:, 2] > 0.3).astype(np.int32)
    return Mesh(m0.vertices, m0.triangles, regions=cap, region_names=["rest", "cap"])


CASES = [("laplace_sl", "P0", "P0", "id", "id", 0.0), ("laplace_dl", "P1", "P0", "id", "id", 0.0),
         ("helmholtz_sl", "P1", "P1", "id", "id", 3.0), ("maxwell_sl", "RT0", "RT0", "maxwell", "maxwell", 2.0)]


@pytest.mark.parametrize("case", CASES, ids=[c[0] + "-" + c[1] + c[2] for c in CASES])
def test_region_operator_is_the_submesh_operator(oracle, case):
    k, tr, te, e1, e2, kap = case
    m = _mesh()
    R = m.Boundaries("cap")
    sub, _, _ = m.submesh(R)
    ops = []
    for mesh, reg in ((m, R), (sub, None)):
        trs = nb.TraceSpace(mesh, tr, definedon=reg)
        tes = trs if te == tr else nb.TraceSpace(mesh, te, definedon=reg)
        dense = nb.bem.IntegralOperator(k, kap, trs, tes, e1, e2, 3, 20, 2.0, 1e-8, "dense", False)
        hmat = nb.bem.IntegralOperator(k, kap, trs, tes, e1, e2, 3, 10, 2.0, 1e-8, "aca", False)
        ops.append((dense, hmat, trs))
    Dr, Ds = ops[0][0].mat.to_dense(), ops[1][0].mat.to_dense()
    assert rel(Dr, Ds) < 1e-12
    Do = oracle.dense_matrix(k, sub, tr, te, kappa=kap, trial_eval=e1, test_eval=e2, intorder=3)
    assert rel(Dr, Do) < 1e-10
    assert ops[0][1].mat.info["nfar"] > 0
    cplx = ops[0][1].mat.is_complex
    r = np.random.default_rng(4)
    x = r.standard_normal(ops[0][2].ndof) + (1j * r.standard_normal(ops[0][2].ndof) if cplx else 0)
    xt = torch.from_numpy(x).cuda()
    yr, ys = (ops[0][1].mat * xt).cpu().numpy(), (ops[1][1].mat * xt).cpu().numpy()
    assert rel(yr, ys) < 1e-12


def test_region_test_space_rows():
    m = _mesh()
    R = m.Boundaries("cap")
    P1 = nb.H1(m)
    P0r, P0 = nb.SurfaceL2(m, definedon=R), nb.SurfaceL2(m)
    Kr = nb.DoubleLayerPotentialOperator(P1, P0r, test_definedon=R, method="dense").mat.to_dense()
    K = nb.DoubleLayerPotentialOperator(P1, P0, method="dense").mat.to_dense()
    assert Kr.shape == (P0r.ndof, P1.ndof)
    assert rel(Kr, K[P0r.global_dofs]) < 1e-12


def test_region_mass_matrix(oracle):
    m = _mesh()
    R = m.Boundaries("cap")
    sub, _, _ = m.submesh(R)
    M = nb.MassOperator(nb.H1(m, definedon=R), nb.SurfaceL2(m, definedon=R))
    Mo = oracle.mass_matrix(sub, "P1", "P0")
    x = np.random.default_rng(2).standard_normal(Mo.shape[1])
    y = (M * torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel(y, Mo @ x) < 1e-13


def test_definedon_leaves_the_matrix_and_restricts_the_potential(oracle):
    m = _mesh()
    R = m.Boundaries("cap")
    P0 = nb.SurfaceL2(m)
    V = nb.bem.IntegralOperator("helmholtz_sl", 2.0, P0, P0, "id", "id", 3, 40, 2.0, 1e-6, "dense", False)
    Vd = nb.bem.IntegralOperator("helmholtz_sl", 2.0, P0, P0, "id", "id", 3, 40, 2.0, 1e-6, "dense", False,
                                 trial_definedon=R, test_definedon=R)
    assert np.array_equal(V.mat.to_dense(), Vd.mat.to_dense())
    u = np.random.default_rng(8).standard_normal(P0.ndof) + 0j
    pts = np.array([[0.0, 0.0, 2.5], [1.5, -1.0, 0.5], [0.1, 0.2, -0.1]])
    pd = Vd.GetPotential(torch.from_numpy(u).cuda())(torch.from_numpy(pts).cuda()).cpu().numpy()
    # the same as the potential of the density restricted to the region, on a region space
    P0r = nb.SurfaceL2(m, definedon=R)
    Vr = nb.HelmholtzSingleLayerPotentialOperator(P0r, kappa=2.0)
    ur = u[P0r.global_dofs]
    pr = Vr.GetPotential(torch.from_numpy(ur).cuda())(torch.from_numpy(pts).cuda()).cpu().numpy()
    assert rel(pd, pr) < 1e-12
    sub, _, tids = m.submesh(R)
    po = oracle.potential("helmholtz_sl", sub, "P0", u[tids], pts, kappa=2.0, intorder=3)[:, 0]
    assert rel(pr, po) < 1e-11
    # without the region every element counts
    pf = V.GetPotential(torch.from_numpy(u).cuda())(torch.from_numpy(pts).cuda()).cpu().numpy()
    assert rel(pf, pd) > 1e-3


TWO_MESH_CASES = [("laplace_sl", "P0", "P1", "id", "id", 0.0), ("helmholtz_dl", "P1", "P0", "id", "id", 2.0),
                  ("maxwell_sl", "RT0", "RT0", "maxwell", "maxwell", 2.0)]


def _union(a, b):
    return Mesh(np.vstack([a.vertices, b.vertices]), np.vstack([a.triangles, b.triangles + a.nv]))


@pytest.mark.parametrize("case", TWO_MESH_CASES, ids=[c[0] for c in TWO_MESH_CASES])
def test_trial_and_test_on_two_meshes(oracle, case):
    """Trial space on one mesh, test space on another (the reference's trial and test
    MeshAccess): the operator equals the block of the oracle's operator on the union of both
    meshes (test rows of the first, trial columns of the second).  Dense 1e-10 with a small
    sphere 0.24 from the unit sphere (close regular pairs); H-matrix within the ACA tolerance
    with it 1.6 away (the root block is admissible, low rank); the potential sums over the
    trial mesh."""
    k, tr, te, e1, e2, kap = case
    a = icosphere(3)
    b0 = icosphere(2)
    r = np.random.default_rng(6)
    for centre, method in (((1.6, 0.3, -0.2), "dense"), ((3.0, 0.3, -0.2), "aca")):
        b = Mesh(0.4 * b0.vertices + np.array(centre), b0.triangles)
        trs, tes = nb.TraceSpace(b, tr), nb.TraceSpace(a, te)
        op = nb.bem.IntegralOperator(k, kap, trs, tes, e1, e2, 3, 10, 2.0, 1e-8, method, False)
        Do = oracle.dense_matrix(k, _union(a, b), tr, te, kappa=kap, trial_eval=e1, test_eval=e2, intorder=3)
        Db = Do[np.ix_(np.arange(tes.ndof), oracle.ndof(a, tr) + np.arange(trs.ndof))]
        if method == "dense":
            D = op.mat.to_dense()
            assert D.shape == Db.shape and rel(D, Db) < 1e-10
            continue
        assert op.mat.info["nfar"] > 0
        cplx = op.mat.is_complex
        x = r.standard_normal(trs.ndof) + (1j * r.standard_normal(trs.ndof) if cplx else 0)
        y = (op.mat * torch.from_numpy(x).cuda()).cpu().numpy()
        assert rel(y, Db @ x) < 1e-6
        z = r.standard_normal(tes.ndof) + (1j * r.standard_normal(tes.ndof) if cplx else 0)
        yt = (op.mat.T * torch.from_numpy(z).cuda()).cpu().numpy()
        assert rel(yt, Db.T @ z) < 1e-6
        if k == "laplace_sl":
            pts = np.array([[0.0, 0.0, 0.0], [4.0, 0.0, 0.0]])
            p = op.GetPotential(torch.from_numpy(x).cuda())(torch.from_numpy(pts).cuda()).cpu().numpy()
            po = oracle.potential(k, b, tr, x, pts, intorder=3)[:, 0]
            assert rel(p, po) < 1e-11
