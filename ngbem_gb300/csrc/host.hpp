// Host-side structures of the operator path: quadrature rules, mesh, trace spaces, cluster
// trees, the block partition and the assembled H-matrix.  Compiled with -ffp-contract=off so
// that the cluster tree is bit-identical across hosts (it must match the oracle bit for bit).
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <climits>
#include <cstdint>
#include <atomic>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ngbem_gb300.h"
#include "bem_shared.h"
#include "kernels.h"

namespace bem {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define BEM_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw ::bem::Error(BEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

// Device buffer owned by RAII.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t n) {
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error(BEM_ERR_ALLOC, std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
    }
    bytes = n;
  }
  template <class T>
  void upload(const std::vector<T>& v, cudaStream_t s = 0) {
    alloc(v.size() * sizeof(T));
    if (!v.empty()) BEM_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  template <class T> T* as() const { return (T*)p; }
};

// ---- quadrature (quadrature.cpp) -------------------------------------------------------
void sym_eigen(int n, std::vector<double> A, std::vector<double>& evals, std::vector<double>& evecs);
void sym_eigen3(const double* A, double* evals, double* evecs);  // n = 3, same bits
struct TrigRule { std::vector<double> xi, eta, w; };
TrigRule make_trig_rule(int order);
// Sauter-Schwab rule of a singularity class (0 identical, 1 common edge, 2 common vertex).
// Every point is xi * (a, b, c, d) for a direction (a, b, c, d) and a Gauss point xi in (0, 1),
// with weight xi^3 w_dir w_xi.  radial = true returns one point per direction at xi = 1 with
// weight w_dir, and c1 = sum w_xi xi, c2 = sum w_xi xi^2: for an integrand homogeneous of
// degree -1 in x - y (1/|x - y|) the sum over xi of a direction is c2 times the xi = 1 term,
// and for degree -2 (grad 1/|x - y|) c1 times it.
struct SSRule { std::vector<double> x0, x1, y0, y1, w; double c1 = 0.0, c2 = 0.0; };
SSRule make_ss_rule(int cls, int order, bool radial = false);

// ---- mesh and spaces (geometry.cpp) -----------------------------------------------------
struct MeshH {
  int nv = 0, nt = 0, ne = 0;
  std::vector<double> X;      // 3*nv
  std::vector<int> T;         // 3*nt
  std::vector<int> E;         // 2*ne
  std::vector<int> TE;        // 3*nt
  std::vector<ElemRec64> rec;
  // curved geometry (gorder 2, 3): (gorder+1)(gorder+2)/2 nodes per element (curved_map)
  int gorder = 1;
  std::vector<double> G;
  // device tables, built on first use
  std::mutex mu;
  bool dev_ready = false;
  std::atomic<int> nspaces{0};  // spaces built on the mesh (their trees read the geometry)
  DevBuf d_tri, d_rec64, d_gnodes;
  struct RuleTables {
    int nq = 0;
    DevBuf rec[2], qoff[2], apts[2], rq[2];  // [0] fp64, [1] fp32
    DevBuf pgeo[2];                          // PGeo per rule point (curved meshes)
  };
  std::map<int, std::unique_ptr<RuleTables>> tables;  // by regular order
  void build(int nv_, const double* xyz, int nt_, const int* tri);
  // curve the elements (before any device table is built)
  void set_geometry(int order, const double* nodes);
  bool curved() const { return gorder > 1; }
  int gnodes() const { return (gorder + 1) * (gorder + 2) / 2; }
  void map(int e, double xi, double eta, double* x) const;
  // the map at (xi, eta): point, |J0 x J1|, normal and n x grad_Gamma(lambda_a); J0, J1 the
  // derivatives when asked for
  double frame(int e, double xi, double eta, double* x, double* n, double rot[3][3], double* J0 = nullptr,
               double* J1 = nullptr) const;
  // the element's weight in the cluster data: the flat area, or |J0 x J1| / 2 at the
  // centroid of a curved element
  double area(int e) const;
  void ensure_device();
  RuleTables& rule_tables(int order);
};

// HDivSurface / HCurl of order K >= 1: K (0 for other kinds), and whether the kind is HCurl
inline int bdm_kind_order(int kind) {
  switch (kind) {
    case BEM_HDIV1: case BEM_HCURL1: return 1;
    case BEM_HDIV2: case BEM_HCURL2: return 2;
    case BEM_HDIV3: case BEM_HCURL3: return 3;
    case BEM_HDIV4: case BEM_HCURL4: return 4;
    default: return 0;
  }
}
inline bool bdm_kind_curl(int kind) {
  return kind == BEM_HCURL1 || kind == BEM_HCURL2 || kind == BEM_HCURL3 || kind == BEM_HCURL4;
}

struct ClusterTreeH;
class LevelTeam;  // host threads kept for the levels of a cluster-tree build (geometry.cpp)

struct SpaceH {
  MeshH* mesh = nullptr;
  int kind = BEM_P0, nd = 1, ndof = 0, dual = 0;
  std::vector<int> dofs;      // 3*nt (P0: the element's dof three times; -1 off the region)
  std::vector<int> sign;      // 3*nt
  std::vector<int> e4d_ptr, e4d;  // dof -> elements (CSR, element order)
  std::vector<int> global_dof;    // dof -> element (P0), vertex (P1) or mesh edge (RT0, HCURL);
                                  // H1 of order p: the dof of the space on the whole mesh
  std::vector<int> xdof;          // H1 of order p >= 2: nd dofs per element (local order)
  std::vector<int> elems;         // the elements the space lives on, ascending
  DevBuf d_dofs, d_sign;
  // mask: nt flags of the elements the space lives on (null: all of them)
  void build(MeshH* m, int kind_, int dual_, const unsigned char* mask = nullptr);
  bool on(int e) const { return dofs[3 * e] >= 0; }
  const int* el_dofs(int e) const { return &dofs[3 * e]; }  // kinds with at most 3 dofs per element
  // dof of local dof a of element e (SurfaceL2 of order >= 1: consecutive from dofs[3 e]; H1
  // of order >= 2: the element's row of xdof)
  int dof(int e, int a) const {
    if (kind >= BEM_H1P2) return xdof[(size_t)nd * e + a];
    return kind >= BEM_L2P1 ? dofs[3 * e] + a : dofs[3 * e + a];
  }
  void ensure_device();
  // cluster tree with element patches for a leaf size, built on first use and shared by the
  // operators on this space (a tree depends only on the space and the leaf size)
  std::shared_ptr<ClusterTreeH> tree(int leafsize);
  std::mutex tree_mu;
  std::map<int, std::shared_ptr<ClusterTreeH>> trees;
};

// device view of a space's dofs, signs and cluster positions (operator.cpp)
SpaceDev space_dev(const SpaceH& s, int tr, const DevBuf& pinv);

// ---- cluster tree and partition (geometry.cpp) -----------------------------------------
struct ClusterH {
  long Level = 0, Parent = -1, Child1 = -1, Child2 = -1, Number = 0, PermuPos = 0, BasisElement = 0;
  double Radius = 0, EVec[9] = {0}, EVal[3] = {0}, XMin[3] = {0}, XMax[3] = {0}, Centre[3] = {0};
  double DiagLength = 0;
};

struct ClusterTreeH {
  std::vector<int> perm;      // cluster position -> dof (mapcluster2glob)
  std::vector<int> pinv;      // dof -> cluster position
  std::vector<ClusterH> cl;
  // element patches per cluster (elements touching a dof of the cluster)
  std::vector<int> patch_ptr, patch;
  std::vector<double> patch_rad;  // radius of the patch vertices around Centre
  // team: threads to split the work of a level on (null: a team of its own for large trees)
  void build(const SpaceH& sp, int leafsize, LevelTeam* team = nullptr);
  void build_patches(const SpaceH& sp, LevelTeam* team = nullptr);
};

struct BlockH {
  int rowcl, colcl;
  bool near;
};
void partition_blocks(const ClusterTreeH& row, const ClusterTreeH& col, double eta, std::vector<BlockH>& out);

// ---- operators (assembly operator.cpp, products apply.cpp, solvers gmres.cpp) ---------------
struct OperatorBase {
  virtual ~OperatorBase() = default;
  bool cplx = false;
  int height = 0, width = 0;
  DevBuf stage_x, stage_y;  // device staging for the host-buffer entry point
  virtual void mult(int trans, const double* alpha, const void* x, const double* beta, void* y, int nrhs,
                    cudaStream_t s) = 0;
};

struct HOperator : OperatorBase {
  int kid = 0;
  double kappa = 0.0;
  SpaceH* trial = nullptr;
  SpaceH* test = nullptr;
  // Spaces on two meshes: merge_meshes() builds one mesh of both (the test mesh's vertices and
  // elements first, then the trial mesh's) and rebuilds each space on its part as a region
  // space, which has the same dofs in the same order; trial / test then point at those.
  std::unique_ptr<MeshH> own_mesh;
  std::unique_ptr<SpaceH> own_trial_space, own_test_space;
  int trial_e0 = 0;       // first element of the trial space's mesh in trial->mesh
  int trial_nt0 = 0, test_nt0 = 0;  // elements of the meshes the caller's spaces live on
  void merge_meshes();
  int trial_ev = 0, test_ev = 0, trt = 0, tet = 0;
  bem_params_t prm{};
  int prec = 0;           // 0 fp64, 1 mixed
  size_t vsize = 8;       // bytes of one stored value
  std::shared_ptr<ClusterTreeH> own_trial, own_test;
  ClusterTreeH* ttrial = nullptr;
  ClusterTreeH* ttest = nullptr;
  std::vector<BlockH> blocks;
  std::vector<int> block_rank, block_fallback;

  // device data
  DevBuf d_perm_trial, d_perm_test, d_pinv_trial, d_pinv_test;
  // Optional global numbering of the vectors the C-ABI products act on (the FE space's full dof
  // numbering, of which the operator's spaces hold the boundary dofs): dof d of the trial
  // (test) space is entry map[d] of a vector of gn_trial (gn_test) entries; 0 = the compact
  // numbering.  d_gperm_* are the cluster permutations composed with the maps, d_gfree_* the
  // global entries that hold no dof (an output's such entries are scaled by beta).
  int gn_trial = 0, gn_test = 0, n_gfree_trial = 0, n_gfree_test = 0;
  DevBuf d_gperm_trial, d_gperm_test, d_gfree_trial, d_gfree_test;
  bool apply_gmap = false;  // set by the C-ABI product entry points for the call
  void set_global_dofs(int trial_n, const int* trial_map, int test_n, const int* test_map);
  // what a product in direction `trans` reads and writes: permutations into x and y, leading
  // dimensions of x and y, and the output entries outside the output space
  struct VecMap {
    const int* pin;
    const int* pout;
    int ld_in, ld_out;
    const int* free_out;
    int n_free_out;
  };
  VecMap vec_map(int trans) const;
  std::vector<std::unique_ptr<DevBuf>> pools;  // dense and factor pools
  DevBuf d_mvdense, d_mvlr, d_err, d_sched;
  // per pass: 0 t=V2 x, 1 y+=Dx+U2 t, 2 t=U2^T x, 3 y+=D^T x+V2^T t; 4-7 the two phases of the
  // single-launch matvec (4: t=V2 x and y+=Dx, 5: y+=U2 t; 6, 7 the same for the transpose)
  DevBuf d_items[MV_NPASS], d_pieces[MV_NPASS], d_ranges[MV_NPASS];
  int n_items[MV_NPASS] = {};
  // several right-hand sides, not transposed: one piece per block (passes 0 and 1)
  DevBuf d_mr_items[2], d_mr_pieces[2];
  int n_mr_items[2] = {0, 0};
  DevBuf d_ro_leaves, d_ro_ents;  // owner-computes lists of the second pass (several right-hand sides)
  int n_ro_leaves = 0;
  bool mv_fused = true;  // one cooperative launch per single-RHS matvec (else the 4-pass pipeline)
  int mv_piece = 0;      // stored elements per piece (0: the kernel's default); set by autotune
  double autotune(int reps, int* best_piece, int* best_fused);
  int mv_grid = 152;
  int mv_compensated = 1;  // fp32 storage: error-free products/sums (1) or plain FP32 (0)
  int t_len = 0;
  DevBuf d_t, d_tx, d_xp, d_yp;

  int ws_nrhs = 0;
  std::vector<MVDense> mvdense;
  std::vector<MVLowRank> mvlr;
  // tensor-core products for 2..32 right-hand sides at plain accuracy (complex FP32 storage;
  // tc_host.cpp, tc_matvec.cu): packed operand panels built on first use
  int tc_mode = 1;   // 0: off (CUDA-core products)
  int tc_state = 0;  // 0 not built, 1 built, -1 not applicable to this operator or device
  DevBuf d_tc_xa, d_tc_xa2, d_tc_ta, d_tc_vp, d_tc_up, d_tc_dp, d_tc_y;
  DevBuf d_tc_items[2], d_tc_stages[2], d_tc_chunks[2], d_tc_sched[2], d_tc_outs;
  DevBuf d_tc_leaves, d_tc_deltas;  // per leaf: the partial-row offsets of the row clusters holding it
  int tc_grid[2] = {0, 0}, tc_items[2] = {0, 0}, tc_nkc_x = 0, tc_nkc_x2 = 0, n_tc_leaves = 0;
  long long tc_bytes = 0;
  double tc_ms_build = 0.0;
  // the stage plan: ring stages (2..4, TC_NST_DEFAULT until autotune_tc), the balanced items,
  // segments and CTA schedules it is planned from, and the tuner's timings of 2, 3, 4 stages
  int tc_nst = TC_NST_DEFAULT;
  std::vector<TCItem> tc_it[2];
  std::vector<TCSeg> tc_sg[2];
  std::vector<int2> tc_sch[2];
  double tc_tune_ms[3] = {0.0, 0.0, 0.0};
  bool tc_eligible(int trans, int nrhs, cudaStream_t s);
  void build_tc();
  void plan_tc(int nst);  // stage plans of both passes for nst stages, uploaded
  // times `reps` 32-right-hand-side applications with each stage count and keeps the fastest;
  // returns its time per application (ms)
  double autotune_tc(int reps);
  void release_tc();
  void mult_tc(const double* alpha, const void* x, const double* beta, void* y, int nrhs, cudaStream_t s);
  bem_operator_info_t info{};
  // optional per-kernel timing of mult (CUDA events on the launch stream)
  bool profiling = false;
  cudaEvent_t pev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<std::array<cudaEvent_t, 5>> pending;  // recorded, not yet read
  std::vector<bool> pending_fused;                   // ... by a single-launch matvec
  double kms[4] = {0, 0, 0, 0};                     // permute_in, stage1, apply, permute_out
  long long kcount[4] = {0, 0, 0, 0};
  void collect_profile();
  ~HOperator() override;

  void assemble();
  // Matvec work lists.  Bit p of `mask` builds pass list p (see d_items); `multi` the lists of
  // several right-hand sides.  keep = false drops every other list (piece size changed).  The
  // lists a matvec needs are built on its first call (ensure_mv) outside a stream capture.
  void build_mv_items(unsigned mask, bool multi, bool keep);
  void ensure_mv(unsigned mask, bool multi, cudaStream_t s);
  unsigned mv_built = 0;
  bool mv_multi_built = false;
  int device_status();   // matvec pipeline error flags (0 = ok)
  // the same flags copied on stream s into a page-locked word (no device-wide synchronisation):
  // queue_status before the caller synchronises s, queued_status after
  void queue_status(cudaStream_t s);
  int queued_status() const { return h_status ? *(volatile int*)h_status : 0; }
  int* h_status = nullptr;
  // Clears the error flags, the claim counters and the accumulators of the products (after a
  // product whose bounded waits ran out: its schedule state is not the one a product leaves).
  void reset_device_state();
  // test hook of the single-launch product's grid-barrier waits (MVFusedArgs)
  long long wait_limit = 0;
  unsigned long long bar_extra = 0;
  void mult(int trans, const double* alpha, const void* x, const double* beta, void* y, int nrhs,
            cudaStream_t s) override;
  void to_dense(void* out);
  // potential of a trial-space density at points (device buffers; synchronous)
  void potential(const void* density, int npts, const double* pts, const double* normals, void* out,
                 cudaStream_t s);
  // trial / test definedon regions (nt element flags; empty: none).  As in the reference they
  // do not change the assembled matrix; the trial region restricts the potential's elements.
  std::vector<unsigned char> def_trial, def_test;
};

struct MassOperator : OperatorBase {
  // cplx (from OperatorBase) = the vectors it acts on are complex128
  DevBuf rowptr, col, val;
  int nrows = 0, ncols = 0;
  std::vector<int> h_rowptr, h_col;
  std::vector<double> h_val;
  void build(SpaceH* trial, SpaceH* test, bool complex_vectors);
  void mult(int trans, const double* alpha, const void* x, const double* beta, void* y, int nrhs,
            cudaStream_t s) override;
};

// Batched single-layer energy (energy_host.cpp / energy.cu): element topology of a batch of
// closed meshes, built once; eval() takes new coordinates and densities each call.
struct SLBatch {
  int nprob = 0, ntri = 0, nvert = 0, nq = 0, prec = 0, dual = 0;
  int nunits = 0, nsing = 0;
  long long npairs_regular = 0;
  double rxi[16] = {}, reta[16] = {}, rw[16] = {};
  int ss_n[3] = {0, 0, 0};
  double ss_c1 = 0.0, ss_c2 = 0.0;
  DevBuf d_tri, d_tprob, d_t0, d_nt, d_units, d_sing, d_ss[3];
  DevBuf d_D, d_dD, d_cf, d_off, d_q64, scratch_out;
  void build(int nprob, const int* nverts, const int* ntris, const int* tris, int order_reg, int order_sing, int prec,
             int dual);
  void eval(const double* X, const double* u, const double* wprob, double* energy, double* vu, double* grad,
            cudaStream_t s);
};

// op.mult with the scratch taken from a fixed device array instead of operator buffers
// (mult_noalloc.cu); allocates nothing.
// 1 when the tensor-core encodings passed their known-answer product on this device (run once)
int tc_selftest();

// an assembled H-matrix to / from a file (serialize.cpp)
void save_operator(const HOperator& op, const char* path);
std::unique_ptr<HOperator> load_operator(const char* path, SpaceH* trial, SpaceH* test);

void mult_noalloc(HOperator& op, int trans, const double* alpha, const void* x, const double* beta, void* y,
                  int nrhs, cudaStream_t s);

int trace_kind(int space_kind, int ev);
bool pairs_overflow(size_t ntiles);
int gmres_solve(int nterms, OperatorBase* const* ops, const double* coef, const void* b, void* x, int maxiter,
                int restart, double tol, int* iters, double* resid, cudaStream_t s);
int gmres_batched_solve(int nterms, OperatorBase* const* ops, const double* coef, int nrhs, const void* b, void* x,
                        int maxiter, int restart, double tol, int* iters, double* resid, cudaStream_t s);

}  // namespace bem

// Handles share what they point into: a space keeps its mesh alive and an operator its spaces,
// so the caller may destroy the handles in any order.
struct bem_mesh_s {
  std::shared_ptr<bem::MeshH> m = std::make_shared<bem::MeshH>();
};
struct bem_space_s {
  std::shared_ptr<bem::MeshH> mesh;
  std::shared_ptr<bem::SpaceH> s = std::make_shared<bem::SpaceH>();
};
struct bem_operator_s {
  std::shared_ptr<bem::MeshH> keep_mesh_trial, keep_mesh_test;  // declared before op: destroyed after it
  std::shared_ptr<bem::SpaceH> keep_trial, keep_test;
  std::unique_ptr<bem::OperatorBase> op;
  void keep(bem_space_s* trial, bem_space_s* test) {
    keep_trial = trial->s;
    keep_mesh_trial = trial->mesh;
    keep_test = test->s;
    keep_mesh_test = test->mesh;
  }
};
struct bem_slbatch_s {
  bem::SLBatch b;
};
