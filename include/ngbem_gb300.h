/* ngbem_gb300: C-ABI of the GB300-native boundary-element operator path.
 *
 * Drop-in boundary for ngbem's operator construction and H-matrix application
 * (Weggler/ngbem).  Each entry point names the reference interface it replaces.
 * Conventions:
 *   - every function returns an int status (BEM_OK = 0); bem_last_error() gives a
 *     thread-local message for the last failure; no C++ exception crosses this ABI;
 *   - handles are opaque; host arrays are caller-owned; vectors are float64 (real
 *     operators) or interleaved complex128 (complex operators);
 *   - device pointers and cudaStream_t are passed as void*.
 */
#ifndef NGBEM_GB300_H
#define NGBEM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define BEM_OK 0
#define BEM_ERR_ARG 1      /* invalid argument */
#define BEM_ERR_CUDA 2     /* CUDA runtime failure or no device */
#define BEM_ERR_ALLOC 3    /* device or host allocation failed */
#define BEM_ERR_STATE 4    /* call not valid for this object */
#define BEM_ERR_INTERNAL 5 /* device-side check failed (capacity, rank cap, ...) */

/* kernel ids: reference src/ngbem.hpp:226-434 (LaplaceSL/DL/HS, HelmholtzSL/DL/HS,
 * CombinedField, MaxwellSL).  BEM_HELMHOLTZ_SL_DKAPPA (no counterpart in the reference) is the
 * derivative of the Helmholtz single layer with respect to kappa, kernel i e^{i kappa r}/(4 pi):
 * its operator is the kappa-derivative of the single-layer bilinear form.  BEM_MAXWELL_DL is
 * MaxwellDLKernel<3> (src/ngbem.hpp:475-510): three components e^{i kappa r}(i kappa r - 1)
 * (x - y)/(4 pi r^3) and six cross-product terms. */
enum {
  BEM_LAPLACE_SL = 0, BEM_LAPLACE_DL = 1, BEM_LAPLACE_HS = 2,
  BEM_HELMHOLTZ_SL = 3, BEM_HELMHOLTZ_DL = 4, BEM_HELMHOLTZ_HS = 5,
  BEM_HELMHOLTZ_CF = 6, BEM_MAXWELL_SL = 7, BEM_HELMHOLTZ_SL_DKAPPA = 8, BEM_MAXWELL_DL = 9
};
/* trace spaces: SurfaceL2 order 0 (P0), H1 order 1 trace (P1), HDivSurface order 0 (RT0),
 * and the surface trace of HCurl order 0 (HCURL: lowest-order Nedelec on the surface
 * triangles, one dof per edge like RT0; on each triangle its shape functions are n x the RT0
 * shape functions of the same edges and signs) */
/* BEM_L2P1..3: SurfaceL2 of order 1..3 (NGSolve SurfaceL2(mesh, order=p)): (p+1)(p+2)/2
 * consecutive dofs per element, the Dubiner basis on the element's vertices taken in the order
 * of their global numbers; identity trace only.
 * BEM_H1P2, BEM_H1P3: H1 of order 2, 3 (NGSolve H1(mesh, order=p) on a surface mesh): the
 * vertex dofs (ascending vertex numbers), then p - 1 dofs per edge (edges by first
 * appearance), then (p - 1)(p - 2) / 2 per element; a hierarchical basis (vertex hats, edge
 * bubbles l_i l_j (l_j - l_i)^m oriented from the lower to the higher vertex number, the face
 * bubble l_0 l_1 l_2).  Traces ID and ROT.
 * BEM_HDIV1, BEM_HDIV2: HDivSurface of order 1, 2 (NGSolve HDivSurface(mesh, order=K): all
 * tangential vector polynomials of degree K, normal-continuous): per edge K + 1 dofs, per
 * element (K + 1)(K - 1); numbered: the lowest-order edge dofs (edges by first appearance, as
 * BEM_RT0), then K per edge, then the interior ones per element.  A hierarchical basis of our
 * own (the RT0 shape, surface curls of H1 edge bubbles, interior l_j l_k curl l_i), Piola-mapped.
 * Traces ID and MAXWELL.
 * BEM_HCURL1, BEM_HCURL2: HCurl of order 1, 2 on the surface (tangential traces of NGSolve
 * HCurl(mesh, order=K)): n x the BEM_HDIV1 / BEM_HDIV2 shapes with the same dofs; traces ID,
 * ROTATED_TRACE and MAXWELL_CURL as on BEM_HCURL.
 * BEM_HDIV3, BEM_HDIV4, BEM_HCURL3, BEM_HCURL4: the same of order 3, 4 (20 and 30 dofs per
 * element), for the operators of the reference's Maxwell tests: the Maxwell single layer on
 * HDivSurface of order 3, 4 and the double layer from HCurl to HDivSurface of order 3. */
enum { BEM_P0 = 0, BEM_P1 = 1, BEM_RT0 = 2, BEM_HCURL = 3, BEM_L2P1 = 4, BEM_L2P2 = 5, BEM_L2P3 = 6,
       BEM_H1P2 = 7, BEM_H1P3 = 8, BEM_HDIV1 = 9, BEM_HDIV2 = 10, BEM_HCURL1 = 11, BEM_HCURL2 = 12,
       BEM_HDIV3 = 13, BEM_HDIV4 = 14, BEM_HCURL3 = 15, BEM_HCURL4 = 16 };
/* trace evaluators: GetEvaluator(BND) (ID), DiffOpBoundaryRot (ROT), DiffOpHelmholtz (HELM),
 * DiffOpMaxwellNew (MAXWELL); reference src/diffops.hpp:12-338.  On BEM_HCURL: ID is the
 * tangential trace (GetEvaluator(BND) of an HCurl space), ROTATED_TRACE is
 * DiffOpRotatedTrace (src/diffops.hpp:62-104: n x the shape function) and MAXWELL_CURL is
 * DiffOpMaxwell (src/diffops.hpp:172-255: [n x shape; surface curl]). */
enum { BEM_EV_ID = 0, BEM_EV_ROT = 1, BEM_EV_HELM = 2, BEM_EV_MAXWELL = 3,
       BEM_EV_ROTATED_TRACE = 4, BEM_EV_MAXWELL_CURL = 5 };
/* precision modes: plain FP64 on the GPU, or mixed (FP64 singular pairs, FP32 regular
 * near field, ACA and factors) */
enum { BEM_FP64 = 0, BEM_MIXED = 1 };
/* assembly methods (reference python_bem.cpp:30-33: "dense" = one root block) */
enum { BEM_METHOD_ACA = 0, BEM_METHOD_DENSE = 1 };

typedef struct bem_mesh_s* bem_mesh_t;
typedef struct bem_space_s* bem_space_t;
typedef struct bem_operator_s* bem_operator_t;
typedef struct bem_slbatch_s* bem_slbatch_t;

/* BEMParameters (reference src/ngbem.hpp:13-27) plus the GB300 extensions. */
typedef struct {
  int intorder;           /* reference intorder: both rules unless overridden */
  int intorder_singular;  /* <= 0: intorder.  Sauter-Schwab rules */
  int intorder_regular;   /* <= 0: intorder.  disjoint tensor rule and far-field points */
  int leafsize;           /* minimal cluster size (reference default 40) */
  double eta;             /* admissibility parameter (default 2) */
  double eps;             /* ACA tolerance (default 1e-6) */
  int method;             /* BEM_METHOD_ACA or BEM_METHOD_DENSE */
  int precision;          /* BEM_FP64 or BEM_MIXED */
  int max_rank;           /* ACA rank cap per block; a block reaching it is assembled densely (0: 128).
                             ACA runs first with a cap of 48; blocks reaching that run again with this cap */
  double aca_eps_floor;   /* mixed precision: ACA tolerance floor (0: 2e-7) */
  long long scratch_bytes;/* ACA scratch budget in bytes (0: an eighth of the device memory, at most 16 GiB) */
} bem_params_t;

/* Assembly and storage summary (reference HMatrix::NZE, src/hmat.cpp:623-630). */
typedef struct {
  int is_complex;
  int height, width;           /* test ndof, trial ndof */
  int nblocks, nnear, nfar, nfallback;
  long long nze;               /* sum m*n (dense) + r*(m+n) (low rank) */
  int max_rank;
  long long sum_rank;
  long long bytes_dense, bytes_lowrank;  /* device storage */
  long long bytes_lowrank_u;             /* of which U factors (m x R per block) */
  int n_singular_pairs;        /* Sauter-Schwab element pairs assembled */
  long long n_regular_pairs;   /* disjoint element pairs assembled (tensor rule) */
  double ms_setup, ms_aca, ms_nearfield, ms_projection, ms_total;  /* assembly phases */
  int mv_items[4];             /* matvec work items per pass (t=V2x, y+=Dx+U2t, t=U2^Tx, y+=D^Tx+V2^Tt) */
  int mv_segments;             /* matvec segments (block pieces) */
  int mv_ranges[4];            /* staged input ranges per pass */
  double ms_mvitems;           /* host time grouping the blocks into matvec work items */
  long long nf_regular_evals;  /* kernel evaluations of the regular near-field pairs (pairs x nq^2) */
  long long aca_evals;         /* kernel evaluations of ACA: per block and kernel component,
                                  (steps + 1) x (row points + column points), every round */
} bem_operator_info_t;

/* Fill *p with the reference defaults (intorder 3, leafsize 40, eta 2, eps 1e-6, aca). */
int bem_params_default(bem_params_t* p);

/* Mesh of triangles (flat until bem_mesh_set_geometry curves them); vertex order per
 * triangle defines the outward normal.
 * Replaces NGSolve MeshAccess for the surface (reference src/ngbem.cpp:33-34). */
int bem_mesh_create(int nv, const double* xyz, int nt, const int* tri, bem_mesh_t* out);
int bem_mesh_num_edges(bem_mesh_t mesh, int* ne);
int bem_mesh_destroy(bem_mesh_t mesh);
/* Curved geometry (NGSolve's Mesh.Curve(order), which the reference's tests call before
 * assembly, e.g. tests/test_aca.py:7; the operators then integrate through the curved element
 * maps, mesh->GetTrafo in src/ngbem.cpp:501-737).  order 1: flat triangles; order 2..4:
 * isoparametric Lagrange triangles with nodes[nt][(order+1)(order+2)/2][3]: node (i, j, k),
 * i + j + k = order, at barycentric (i, j, k) / order of the triangle's vertices
 * (v0, v1, v2), listed for i = order..0, j = order-i..0; the corner nodes must equal the
 * vertices.  Every space lives on curved meshes (RT0 and HCurl through the Piola map of the
 * curved element at each point).  Call before the first space on the mesh is created
 * (BEM_ERR_STATE after: spaces cache cluster trees of the mesh's geometry). */
int bem_mesh_set_geometry(bem_mesh_t mesh, int order, const double* nodes);

/* Trace space on a mesh (replaces the NGSolve FESpace argument of the factories,
 * reference src/python_bem.cpp:27-173).  RT0 dofs are edges numbered by first
 * appearance (element order, local edges (0,1),(1,2),(2,0)). */
int bem_space_create(bem_mesh_t mesh, int kind, int dual_mapping, bem_space_t* out);
/* Trace space on a region of the mesh: element_mask holds nt flags (nonzero: the space lives
 * on that element); null means every element.  Replaces a `definedon` FESpace (NGSolve's
 * SurfaceL2(..., definedon=...)): the reference's operators read only the dofs of the
 * boundary elements the space has (src/ngbem.cpp:43-66, src/hmat.cpp:19-41).  The dofs are
 * numbered as on the mesh made of the region's elements (elements in order, vertices in
 * ascending order, edges by first appearance); bem_space_global_dofs maps them back. */
int bem_space_create_on(bem_mesh_t mesh, int kind, int dual_mapping, const unsigned char* element_mask,
                        bem_space_t* out);
/* dof -> element (P0), vertex (P1) or mesh edge (RT0, HCURL); out holds ndof entries.
 * BEM_H1P2/3: the dof of the same basis function in the space on the whole mesh (vertex v:
 * v; dof j of mesh edge g: nv + g (p - 1) + j; face dof j of element e: nv + ne (p - 1) +
 * e (p - 1)(p - 2) / 2 + j). */
int bem_space_global_dofs(bem_space_t space, int* out);
/* The dofs of every element (FESpace::GetDofNrs, as the reference reads them throughout
 * src/ngbem.cpp): dofs holds 3 ints per element (P0: the element's dof in the first; -1 on
 * elements outside the space's region); signs (may be null) the RT0 / HCURL orientation
 * +1/-1 of the local edges (0,1), (1,2), (2,0).  BEM_L2P1..3: the first holds the element's
 * first dof (its (p+1)(p+2)/2 dofs are consecutive), the others -1, and signs the element's
 * local vertices in the order of their global numbers. */
int bem_space_element_dofs(bem_space_t space, int* dofs, int* signs);
/* Every local dof of every element (FESpace::GetDofNrs for any space kind): *nd = the dofs per
 * element; dofs (may be null to query nd) holds nd ints per element in the local order of the
 * basis (-1 on elements outside the space's region).  BEM_H1P2/3: vertices 0..2, the p - 1
 * dofs of the local edges (0,1), (1,2), (2,0), then the face dofs; bem_space_element_dofs
 * gives their vertex dofs and, in signs, the edges' orientations. */
int bem_space_dof_table(bem_space_t space, int* nd, int* dofs);
int bem_space_ndof(bem_space_t space, int* ndof);
int bem_space_destroy(bem_space_t space);

/* Cluster tree of a space (reference ClusterTree ctor, src/hmat.cpp:409-453); host only.
 * perm: ndof ints (mapcluster2glob).  ci: 7 longs per cluster (Level, Parent, Child1,
 * Child2, Number, PermuPos, BasisElement).  cd: 23 doubles per cluster (Radius, EVec[9],
 * EVal[3], XMin[3], XMax[3], Centre[3], DiagLength). */
int bem_cluster_tree(bem_space_t space, int leafsize, int* perm, int max_clusters,
                     int* nclusters, long* ci, double* cd);

/* Block partition (reference HMatrix ctor / HMatrix_help, src/hmat.cpp:587-621); host only.
 * Returns blocks in the reference order: row (test) cluster, col (trial) cluster, near flag. */
int bem_partition(bem_space_t trial, bem_space_t test, int leafsize, double eta, int max_blocks,
                  int* nblocks, int* rowcl, int* colcl, int* near);

/* Operator construction = assembly on the GPU (reference GenericIntegralOperator ctor,
 * src/ngbem.cpp:314-330, and CalcHMatrix :118-157; factories src/python_bem.cpp:27-173).
 * test may equal trial.  The spaces may live on two meshes (the reference's trial and test
 * MeshAccess, src/ngbem.cpp:33-34): elements of different meshes share no vertex, so every
 * pair between them is regular.  Synchronous: returns when the H-matrix is resident in HBM. */
int bem_operator_create(int kernel, double kappa, bem_space_t trial, bem_space_t test,
                        int trial_eval, int test_eval, const bem_params_t* params,
                        bem_operator_t* out);

/* Galerkin mass matrix <u, v> of identity traces as a sparse operator (replaces the NGSolve
 * BilinearForm(u*v*ds) used beside the BEM operators, e.g. reference tests/test_Laplace.py:50).
 * complex_vectors: 1 if it acts on complex128 vectors. */
int bem_mass_create(bem_space_t trial, bem_space_t test, int complex_vectors, bem_operator_t* out);

int bem_operator_info(bem_operator_t op, bem_operator_info_t* info);

/* Block list after assembly: row/col cluster, near flag, rank (-1 dense), dense fallback. */
int bem_operator_blocks(bem_operator_t op, int* rowcl, int* colcl, int* near, int* rank,
                        int* fallback);

/* y = alpha * op(A) x + beta * y on the device (reference HMatrix::Mult / MultAdd /
 * MultTrans / MultTransAdd, src/hmat.cpp:632-666).  trans=1 is the plain transpose (no
 * conjugation).  alpha/beta point to (re, im) pairs.  nrhs column-major right-hand sides
 * (leading dimension = vector length).  Stream-ordered, asynchronous.  Assembly builds the
 * work lists of the single right-hand-side product; the first call of another form (the
 * transpose, several right-hand sides) builds its lists then, so make it outside a stream
 * capture (BEM_ERR_STATE inside one). */
int bem_operator_mult(bem_operator_t op, int trans, const double* alpha, const void* x,
                      const double* beta, void* y, int nrhs, void* stream);

/* Bytes of the fixed device scratch area used by bem_operator_mult_noalloc (one per device). */
#define BEM_NOALLOC_SCRATCH_BYTES (16u << 20)

/* bem_operator_mult for callers that must not have device memory allocated on their behalf
 * (no counterpart in the reference).  bem_operator_mult grows operator-owned scratch on first
 * use and when nrhs grows (cudaFree + cudaMalloc; cudaFree waits for the whole device).  This
 * entry point allocates nothing: its scratch is a fixed file-scope device array of
 * BEM_NOALLOC_SCRATCH_BYTES, and it never builds work lists (which would allocate).  Same
 * arguments, same result (up to the order of FP64 atomic additions).  H-matrix operators only
 * (BEM_ERR_STATE for a mass operator).  A call whose scratch would exceed the area -- about
 * 2 * (height + width + sum of block ranks) * nrhs values -- returns BEM_ERR_ARG before
 * launching anything.  The work lists of the non-transposed single-vector product exist from
 * assembly (or loading); those of another form (trans = 1, or nrhs > 1) are built by one
 * bem_operator_mult call of that form, and until then this call returns BEM_ERR_STATE.  The
 * first call on a device looks the array up (and may load device code): make it before any
 * stream capture.  The area is shared by every call on a device, so overlapping calls
 * (several streams or host threads) race: serialise them.  Bounded device waits that run out
 * are reported by bem_operator_status. */
int bem_operator_mult_noalloc(bem_operator_t op, int trans, const double* alpha, const void* x,
                              const double* beta, void* y, int nrhs, void* stream);

/* Global dof numbering of the vectors the products act on (reference: the HMatrix of an
 * IntegralOperator is width_vol_dof x height_vol_dof, src/hmat.hpp:178-179, and its blocks
 * gather x and scatter y through the FE space's global dof numbers, src/hmat.cpp:473-515, from
 * the boundary maps of src/ngbem.cpp:43-65).  trial_map[d] (test_map[d]) is the global number
 * of dof d of the trial (test) space in a vector of trial_nglobal (test_nglobal) entries: e.g.
 * the volume dof of a boundary dof of a definedon space.  Maps are injective; entries that hold
 * no dof of the output space are set to beta * y (0 for a plain product), as the reference's
 * Mult zeroes y and MultAdd leaves them.  After this call bem_operator_mult,
 * bem_operator_mult_noalloc and bem_operator_mult_host take x and y in the global numbering
 * (leading dimension trial_nglobal / test_nglobal for several right-hand sides); a NULL map
 * restores the compact numbering of that space.  bem_gmres and bem_operator_to_dense keep the
 * compact numbering.  H-matrix operators only. */
int bem_operator_set_global_dofs(bem_operator_t op, int trial_nglobal, const int* trial_map, int test_nglobal,
                                 const int* test_map);

/* Same with HOST buffers (synchronous).  When x and y together hold at most
 * BEM_HOST_MAPPED_MAX_BYTES and both are page-locked (cudaHostAlloc, torch pin_memory), the
 * kernels read and write them in place through their device mapping; larger products and
 * other host memory are copied up, applied and copied back. */
#define BEM_HOST_MAPPED_MAX_BYTES (1u << 20)
int bem_operator_mult_host(bem_operator_t op, int trans, const double* alpha, const void* x,
                           const double* beta, void* y, int nrhs);

/* Error flags of the operator's products on the device (no counterpart in the reference,
 * whose products run on host threads and raise C++ exceptions).  Every wait of the product
 * kernels is bounded; a wait that runs out sets a flag (2: a pipeline wait of the CUDA-core
 * product kernels; 4: a grid barrier of the single-launch product; 0x100: a pipeline wait of
 * the tensor-core products) and the kernel finishes without
 * hanging, leaving y invalid.  bem_operator_mult and bem_operator_mult_noalloc are
 * stream-ordered and do not read the flags; this call synchronizes the device and returns
 * them in *flags (0 = every product since the last reset was complete).  reset != 0 clears
 * the flags and the operator's scheduling counters and accumulators, which a product whose
 * waits ran out leaves in an unknown state.  bem_operator_mult_host checks the flags itself
 * and returns BEM_ERR_INTERNAL (after the reset) when one is set. */
int bem_operator_status(bem_operator_t op, int* flags, int reset);

/* Test hook of the bounded waits (no counterpart in the reference): the grid-barrier waits of
 * the single-launch product poll at most `limit` times (0: the default, about a second) and,
 * with extra_arrivals = 1, wait for one arrival more than the grid can make, so that every
 * such wait runs out.  Lets a test check that a wait that runs out is reported, without a
 * fault or a hang.  (0, 0) restores normal operation. */
int bem_operator_test_waits(bem_operator_t op, long long limit, int extra_arrivals);

/* Dense height x width matrix of the operator (row-major, host, in the operator's vector
 * type), for small cases; mass matrices too (their real entries). */
int bem_operator_to_dense(bem_operator_t op, void* out);

int bem_operator_destroy(bem_operator_t op);

/* ---- Batched single-layer energy and shape gradient (no counterpart in the reference, which
 * has no derivatives; the energy u^T V(X) u is what u^T (SingleLayerPotentialOperator(...).mat
 * * u) gives for a P0 space, src/python_bem.cpp:27-40 and src/ngbem.cpp:373-738).
 * Topology of nprob closed triangle meshes: nverts[b], ntris[b], tris = concatenated triangles
 * (3 vertex ids local to their mesh).  Quadrature: tensor triangle rule of order
 * intorder_regular (0..5) on pairs sharing no vertex, Sauter-Schwab rules of order
 * intorder_singular on the others, as the dense near-field assembly uses them.
 * precision: BEM_FP64 (all FP64) or BEM_MIXED (regular pairs in FP32 with hi+lo centroid
 * differences, singular pairs FP64).  dual_mapping: the P0 basis 1/|J|. */
int bem_sl_batch_create(int nprob, const int* nverts, const int* ntris, const int* tris, int intorder_regular,
                        int intorder_singular, int precision, int dual_mapping, bem_slbatch_t* out);

/* One evaluation on the device (stream-ordered).  X: 3 * sum(nverts) coordinates (problems
 * concatenated), u: sum(ntris) densities.  Outputs (device, overwritten; any may be NULL):
 * energy[nprob] = u_b^T V(X_b) u_b, vu[sum ntris] = V(X_b) u_b, grad[3 * sum nverts] =
 * weights[b] * dE_b/dX (weights NULL: 1).  grad = NULL skips the derivative kernels.  The
 * derivative is exact for the discrete energy (the rule moves with the mesh). */
int bem_sl_batch_eval(bem_slbatch_t batch, const double* X, const double* u, const double* weights,
                      double* energy, double* vu, double* grad, void* stream);

/* nunits: regular work units, nsing: singular element pairs, npairs_regular: regular pairs. */
int bem_sl_batch_info(bem_slbatch_t batch, int* nunits, int* nsing, long long* npairs_regular);

int bem_sl_batch_destroy(bem_slbatch_t batch);

/* Arithmetic of the matvec for FP32-stored operators (no counterpart in the reference, which is
 * FP64 throughout): compensated = 1 (default) forms every product and sum error-free (x split
 * into FP32 hi+lo, TwoProd/TwoSum), so the only rounding is that of the stored entries;
 * compensated = 0 uses plain FP32 FMAs (about 1e-7 relative rounding, faster); complex
 * operators applied to 2..32 right-hand sides then use the tensor cores (about 5e-7, see
 * bem_operator_set_tensor_cores).  FP64-stored operators ignore it.  bem_gmres uses the plain
 * form inside its Krylov iterations and the compensated form for its residuals (iterative
 * refinement). */
int bem_operator_set_accuracy(bem_operator_t op, int compensated);

/* Autotuner of the single right-hand-side matvec (no counterpart in the reference): times
 * `reps` applications for each candidate piece size (stored elements per warp task: 256, 384,
 * 512, 768, 1024, 1536, 2048) and schedule (one cooperative launch or the four-pass pipeline) and keeps the
 * fastest.  Outputs (may be NULL): the chosen piece size, 1 if the single launch won, and the
 * best time per matvec in milliseconds.  Synchronous; allocates two vectors. */
int bem_operator_autotune(bem_operator_t op, int reps, int* piece, int* fused, double* ms);

/* Tensor-core products for several right-hand sides (no counterpart in the reference, which
 * applies HMatrix::MultAdd, src/hmat.cpp:647-655, one vector at a time).  For complex
 * operators with FP32 storage, plain accuracy (bem_operator_set_accuracy(op, 0)) and 2..32
 * right-hand sides, bem_operator_mult runs the low-rank products T = V2 X and Y += U2 T on the
 * tcgen05 tensor cores with split-TF32 operands (high + low parts; FP32 accumulation in tensor
 * memory over at most 8 MMAs per accumulator, summed with rounding to nearest; about 5e-7
 * relative), the dense blocks included.  The packed operand panels
 * (about 3x the low-rank storage) are built on the first such call outside a stream capture,
 * or here.
 * enable = 1 (default) builds them now when the operator qualifies; 0 turns the path off and
 * frees them.  bem_operator_tensor_cores reports the state (1 built, 0 not built, -1 the
 * operator or device does not qualify), the device bytes of the panels, the work items of the
 * two passes and the build time in ms (outputs may be NULL). */
int bem_operator_set_tensor_cores(bem_operator_t op, int enable);
int bem_operator_tensor_cores(bem_operator_t op, int* state, long long* bytes, int* items0, int* items1,
                              double* ms_build);
/* Autotuner of the tensor-core stage plan (no counterpart in the reference): builds the panels
 * if needed, times `reps` applications to 32 right-hand sides (zero vectors: the kernels do the
 * same work for any values) with the pipeline ring cut into 2, 3 and 4 stages, and keeps the
 * fastest.  nstages: the stages kept; ms: the time per application of 2, 3, 4 stages (3
 * doubles; either may be NULL).  BEM_ERR_STATE if the operator has no tensor-core path. */
int bem_operator_autotune_tc(bem_operator_t op, int reps, int* nstages, double* ms);

/* An assembled H-matrix to a file and back (no counterpart in the reference, which reassembles
 * each session).  The file holds the partition, ranks, dense blocks and factors, and the mesh's
 * geometry order with a hash of its curved nodes; loading needs the same trial and test spaces
 * on the same geometry (checked through their cluster trees and that record) and applies
 * exactly like the saved operator.  test may be NULL (= trial). */
int bem_operator_save(bem_operator_t op, const char* path);
int bem_operator_load(const char* path, bem_space_t trial, bem_space_t test, bem_operator_t* out);

/* Potential of a density (reference GenericIntegralOperator::GetPotential / PotentialCF,
 * src/ngbem.cpp:1166-1301): out[p * dim + c] = sum over the trial elements, the points y of
 * the regular rule (the operator's intorder) and the kernel terms of
 * w_y K(x_p, y, n_p, n_y) (trial evaluator applied to the density)_c, in FP64; as in the
 * reference, term factors are not applied.  density: trial dofs (double, or complex128 for
 * complex kernels); points, normals: 3 doubles per point (normals may be NULL unless the
 * kernel uses n_x: the Helmholtz hypersingular); out: dim values per point.  All device
 * pointers; synchronous on `stream`.  dim is the trial evaluator's dimension (1 for P0/P1
 * identity traces), 0 when the operator has no potential. */
int bem_operator_potential_dim(bem_operator_t op, int* dim);

/* The operator's trial / test `definedon` regions (reference IntegralOperator ctor,
 * src/ngbem.cpp:17-113): one flag per element of the trial space's mesh and of the test
 * space's mesh, null for none.  As in the reference, the
 * assembled matrix does not depend on them (its dofs are the spaces' dofs); the trial region
 * restricts the elements bem_operator_potential sums over (PotentialCF, src/ngbem.cpp:1205). */
int bem_operator_set_definedon(bem_operator_t op, const unsigned char* trial_mask, const unsigned char* test_mask);
int bem_operator_potential(bem_operator_t op, const void* density, int npts, const double* points,
                           const double* normals, void* out, void* stream);

/* Known-answer check of the tensor-core encodings on the current device (one 128 x 32 x 16
 * split-TF32 product of exactly representable values).  passed = 1 when every entry is exact. */
int bem_tc_selftest(int* passed);

/* Diagnostics (no counterpart in the reference, whose Timer/RegionTimer instrumentation at
 * src/hmat.cpp:650 plays this role): when enabled, every bem_operator_mult records CUDA
 * events on its stream around its four launches; bem_operator_kernel_times returns the
 * accumulated milliseconds and launch counts of [permute-in, low-rank stage 1, apply,
 * permute-out].  Enabling resets the counters. */
int bem_operator_set_profiling(bem_operator_t op, int enable);
int bem_operator_kernel_times(bem_operator_t op, double* ms, long long* launches);

/* Restarted GMRES on A = sum_k coef[k] * ops[k] (ngsolve.krylovspace.GMRes as used by the
 * reference tests, e.g. tests/test_Laplace.py:60).  b, x: device vectors; x holds the
 * initial guess.  FP64 Arnoldi with classical Gram-Schmidt and re-orthogonalisation; the
 * operator application is replayed from a CUDA graph.  coef: 2*nterms doubles (re, im).
 * iters/resid: iterations done and final relative residual. */
int bem_gmres(int nterms, const bem_operator_t* ops, const double* coef, const void* b, void* x,
              int maxiter, int restart, double tol, int* iters, double* resid, void* stream);

/* GMRES for nrhs right-hand sides at once (the reference calls GMRes once per right-hand
 * side; here the nrhs independent solves advance in lockstep so that every Arnoldi step applies
 * the operators once to all of them, streaming the H-matrix once per step).  b, x: nrhs
 * column-major device vectors (leading dimension = n).  Per column: FP64 Arnoldi with CGS2,
 * Givens rotations, own convergence; resid[nrhs] = final relative residuals; iters = steps. */
int bem_gmres_batched(int nterms, const bem_operator_t* ops, const double* coef, int nrhs, const void* b,
                      void* x, int maxiter, int restart, double tol, int* iters, double* resid, void* stream);

const char* bem_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
