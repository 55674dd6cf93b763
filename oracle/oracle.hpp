// FP64 CPU oracle for the ngbem operator path: TEST INFRASTRUCTURE ONLY.
//
// This is a plain C++17 restatement of the reference algorithms (Weggler/ngbem):
//   src/intrules.cpp:13-136      Sauter-Schwab rules
//   src/ngbem.hpp:215-510        fundamental-solution kernels and KernelTerm tables
//   src/diffops.hpp:12-338       trace evaluators (BoundaryRot, Helmholtz, MaxwellNew)
//   src/ngbem.cpp:14-157         operator set-up and CalcHMatrix (with dense fallback)
//   src/ngbem.cpp:373-738        CalcBlockMatrix (near field)
//   src/ngbem.cpp:743-1163       CalcFarFieldBlock (ACA + projection)
//   src/hmat.cpp:13-681          cluster data, PCA cluster tree, admissibility, partition, matvec
// NGSolve pieces the reference calls (quadrature rule tables, element transformation,
// LAPACK dsyev) are restated with documented choices: Golub-Welsch Gauss rules, the
// collapsed Gauss-Jacobi x Gauss-Legendre triangle rule, a cyclic Jacobi 3x3 eigen solver.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library.  It is the checker and the timed CPU baseline, never the product.
//
// Parity status: the reference cannot be built or run here (it links NGSolve, which is
// absent), so this oracle is pinned by known-answer tests (rule weight sums, analytic
// Laplace spectra on the sphere, the harmonic Dirichlet-to-Neumann answer, ACA-vs-dense
// error) rather than by outputs of the reference itself: parity with ngbem-as-shipped
// is unpinned at the bit level.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// kernel ids (same numbering as include/ngbem_gb300.h)
enum {
  ORC_LAPLACE_SL = 0, ORC_LAPLACE_DL = 1, ORC_LAPLACE_HS = 2,
  ORC_HELMHOLTZ_SL = 3, ORC_HELMHOLTZ_DL = 4, ORC_HELMHOLTZ_HS = 5,
  ORC_HELMHOLTZ_CF = 6, ORC_MAXWELL_SL = 7,
  // d/dkappa of the Helmholtz single layer, i e^{i kappa r}/(4 pi): no counterpart in the
  // reference (which has no derivatives); pinned by central differences of ORC_HELMHOLTZ_SL
  ORC_HELMHOLTZ_SL_DKAPPA = 8,
  // MaxwellDLKernel<3>, src/ngbem.hpp:475-510
  ORC_MAXWELL_DL = 9
};
// space kinds
// (ORC_HCURL: surface Nedelec order 0, shape n x the RT0 shape of the same edge and sign)
// ORC_L2P1..3: SurfaceL2 of order 1..3 (Dubiner basis on the vertices sorted by global number)
// ORC_H1P2, ORC_H1P3: H1 of order 2, 3: vertex hats, edge bubbles l_lo l_hi (l_hi - l_lo)^m
// (lo, hi: the edge's vertices by global number), the face bubble l_0 l_1 l_2; dofs vertices,
// then p - 1 per edge (edge order of orc_mesh_edges), then per element
// ORC_HDIV1, ORC_HDIV2: HDivSurface of order K = 1, 2 (BDM_K): per local edge K + 1 dofs (the
// edge id, then ne + edge K + m - 1), then (K + 1)(K - 1) per element after all edge dofs
// ORC_HCURL1, ORC_HCURL2: HCurl of order K = 1, 2: n x the HDIV shapes, the same dofs
// ORC_HDIV3, ORC_HDIV4, ORC_HCURL3, ORC_HCURL4: the same of order 3, 4
enum { ORC_P0 = 0, ORC_P1 = 1, ORC_RT0 = 2, ORC_HCURL = 3, ORC_L2P1 = 4, ORC_L2P2 = 5, ORC_L2P3 = 6,
       ORC_H1P2 = 7, ORC_H1P3 = 8, ORC_HDIV1 = 9, ORC_HDIV2 = 10, ORC_HCURL1 = 11, ORC_HCURL2 = 12,
       ORC_HDIV3 = 13, ORC_HDIV4 = 14, ORC_HCURL3 = 15, ORC_HCURL4 = 16 };
// trace evaluators; on ORC_HCURL: ID the tangential trace, ROTATED_TRACE DiffOpRotatedTrace,
// MAXWELL_CURL DiffOpMaxwell
enum { ORC_EV_ID = 0, ORC_EV_ROT = 1, ORC_EV_HELM = 2, ORC_EV_MAXWELL = 3,
       ORC_EV_ROTATED_TRACE = 4, ORC_EV_MAXWELL_CURL = 5 };

typedef struct {
  int intorder_singular;   // Sauter-Schwab rules (reference: param.intorder)
  int intorder_regular;    // disjoint tensor rule and far-field points (reference: param.intorder)
  int leafsize;
  double eta;
  double eps;
  int nthreads;            // 0 = all hardware threads
} orc_params_t;

// Edge table of a triangle mesh: edges numbered by first appearance, scanning elements
// in order and local edges (0,1),(1,2),(2,0).  Returns the number of edges.
int orc_mesh_edges(int nv, int nt, const int* tri, int* edges /*2*3nt*/, int* tri_edges /*3nt*/);

// Geometry of the meshes that the following calls build (a setting of the library, kept until
// the next call): order 1 flat triangles; order 2..4 isoparametric Lagrange triangles with
// nodes[nt][(order+1)(order+2)/2][3], node (i, j, k) (i + j + k = order) at barycentric
// (i, j, k) / order of the element's vertices, listed for i = order..0, j = order-i..0.  A
// mesh with another element count is built flat.  Returns 0, or -1 for a bad order.
int orc_set_geometry(int order, int nt, const double* nodes);

// Trace values of the local dofs of element e at (xi, eta) (for known-answer tests):
// out[4 a + c] component c of local dof a, dofs[a] its global dof; returns the dofs per element.
int orc_eval_trace(int nv, const double* xyz, int nt, const int* tri, int kind, int ev, int e, double xi,
                   double eta, double* out /*120*/, int* dofs /*30*/);

// Quadrature tables (for known-answer tests).
int orc_trig_rule(int order, double* xi, double* eta, double* w);            // returns npts
int orc_ss_rule(int cls /*0 identic,1 edge,2 vertex*/, int order,
                double* x0, double* x1, double* y0, double* y1, double* w);   // returns npts

// Cluster tree (reference ClusterTree ctor, src/hmat.cpp:409-453).
// clusters_i: 7 longs per cluster (Level, Parent, Child1, Child2, Number, PermuPos, BasisElement)
// clusters_d: 23 doubles per cluster (Radius, EVec[9], EVal[3], XMin[3], XMax[3], Centre[3], DiagLength)
int orc_cluster_tree(int nv, const double* xyz, int nt, const int* tri, int kind, int leafsize,
                     int* perm /*ndof*/, int max_clusters, long* clusters_i, double* clusters_d);

// Operator: builds trees, partition and assembles the H-matrix in FP64 (constructor).
void* orc_operator_create(int kernel, double kappa,
                          int nv, const double* xyz, int nt, const int* tri,
                          int trial_kind, int trial_eval, int trial_dual,
                          int test_kind, int test_eval, int test_dual,
                          const orc_params_t* params);
// info: [is_complex, height, width, nblocks, nnear, nfar, nze, nfallback, max_rank, sum_rank]
int orc_operator_info(void* op, long* info);
// y = A x (trans=0) or y = A^T x (trans=1, no conjugation); complex vectors interleaved.
int orc_operator_mult(void* op, int trans, const double* x, double* y);
// y = A X for nrhs column-major right-hand sides (leading dimension = vector length)
int orc_operator_mult_multi(void* op, int nrhs, const double* x, double* y);
// block list in assembly order: row cluster, col cluster, near flag (1 near, 0 far),
// rank (-1 for dense), dense-fallback flag.
int orc_operator_blocks(void* op, int* rowcl, int* colcl, int* near, int* rank, int* fallback);
// full dense matrix of the H-matrix (height x width, row-major; complex interleaved)
int orc_operator_to_dense(void* op, double* out);
// Dense matrix of CalcBlockMatrix over all dofs (reference testhmatrix path, ngbem.cpp:332-336)
int orc_dense_matrix(int kernel, double kappa, int nv, const double* xyz, int nt, const int* tri,
                     int trial_kind, int trial_eval, int trial_dual,
                     int test_kind, int test_eval, int test_dual,
                     const orc_params_t* params, double* out);
void orc_operator_destroy(void* op);
// Galerkin mass matrix <u, v> for scalar/vector identity traces (dense, row = test)
int orc_mass_matrix(int nv, const double* xyz, int nt, const int* tri,
                    int trial_kind, int test_kind, int order, double* out);
// Potential of a density at points (reference PotentialCF::T_Evaluate, src/ngbem.cpp:1187-1238):
// out[p * dim + tec] = sum over elements, regular points y and kernel terms of
// w_y K_kc(x_p, y, n_p, n_y) (trial evaluator applied to the density)_trc, dim = trial
// evaluator dimension; normals (3 per point) may be NULL for kernels without n_x.
int orc_potential(int kernel, double kappa, int nv, const double* xyz, int nt, const int* tri,
                  int trial_kind, int trial_eval, int trial_dual, int intorder, const double* density,
                  int npts, const double* pts, const double* normals, double* out);

#ifdef __cplusplus
}
#endif
