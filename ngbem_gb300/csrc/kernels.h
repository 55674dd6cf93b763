// Host-side declarations of the CUDA kernel launchers and their argument blocks.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bem_shared.h"

namespace bem {

struct SpaceDev {
  int tr;              // TraceKind
  int nd;              // local dofs per element
  int dual;            // P0 dual mapping (1/|J| scaling)
  const int4* dofs;    // element -> dofs
  const int4* sign;    // RT0 edge orientation per element (+1/-1)
  const int* pinv;     // dof -> position in the cluster permutation
};

// Points of the regular triangle rule on element e: offsets from the centroid and the
// weight w_q*|J| (QPt), or absolute position as a hi+lo pair (APt) for ACA.
template <class P> struct QPt { P x, y, z, w; };
template <class P> struct APt { P hx, hy, hz, lx, ly, lz, w, pad; };

struct NFArgs {
  const NFTile* tiles;
  int ntiles;
  const DenseDesc* blocks;
  const int* patch_test;
  const int* patch_trial;
  const int4* tri;
  SpaceDev test, trial;
  const void* erecP;      // ElemRecP<P>[nt]
  const void* qoff;       // QPt<P>[nt*nq]
  const void* rq;         // reference points (xi, eta) of the regular rule, P2[nq]
  const void* pgeo;       // PGeo<P>[nt*nq] of curved meshes, else null
  int nq;
  double kappa;
  void* pool;             // dense pool, value type of the operator in storage precision
  int atomic_scatter;     // 0: every dense entry is owned by one element pair (P0 x P0)
  SingItem* sing;
  int* sing_count;
  int sing_cap;
  int* err;
  // singular kernel
  const ElemRec64* erec64;
  const double* gnodes;   // curved meshes: the element nodes (curved_map), else null
  int gorder;
  const double* ss[3];    // Sauter-Schwab tables: x0[n], x1[n], y0[n], y1[n], w[n]
  int ss_n[3];
  int ss_smem_bytes;      // > 0: stage all three tables in shared memory
  int sing_grid;
};

struct AcaArgs {
  const FarDesc* far;
  int nfar;
  const int* patch_test;
  const int* patch_trial;
  const void* apts;       // APt<P>[nt*nq]
  const void* erecP;      // normals
  const void* pgeo;       // PGeo<P>[nt*nq] of curved meshes (normals per point), else null
  int nq;
  double kappa;
  double eps;
  void* U;                // scratch, value type in precision P
  void* V;
  int* ranks;             // [nfar][NC]
  int* status;            // [nfar] 1 = rank cap reached
};

struct ProjArgs {
  const FarDesc* far;
  const LRDesc* lr;
  int nfar;
  const int* ranks;
  const int* patch_test;
  const int* patch_trial;
  const void* erecP;
  const void* qoff;
  const void* rq;
  const void* pgeo;       // PGeo<P>[nt*nq] of curved meshes, else null
  int nq;
  double kappa;
  SpaceDev test, trial;
  const void* U;          // ACA scratch
  const void* V;
};

// kid: KernelId; prec: 0 fp64, 1 mixed; trt/tet: TraceKind of trial/test side.
bool nf_combo_supported(int kid, int trt, int tet);
void launch_nf_regular(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_nf_singular(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_aca(int kid, int prec, const AcaArgs& a, cudaStream_t s);
void launch_projection(int kid, int prec, int trt, int tet, const ProjArgs& a, cudaStream_t s);
int kernel_ncomp(int kid);
int kernel_nterms(int kid);          // kernel terms (factor, component, trial, test)
int kernel_term_comp(int kid, int t);  // the kernel component term t reads
bool kernel_complex(int kid);

// ---- matvec -----------------------------------------------------------------------------
// Item-based matvec pass (see matvec.cu).  pass 0: t = V2 x, 1: y += D x + U2 t,
// 2: t = U2^T x, 3: y += D^T x + V2^T t.  xp holds the permuted input in the pass's
// input form (FP32 hi+lo pairs for fp32 storage), t and yp are FP64 accumulators.
struct MVArgs2 {
  const MVTItem* items;   // seg0/nseg index `pieces`, rng0/nrng index `ranges`
  int nitems;
  const MVPiece* pieces;
  const MVRange* ranges;
  const void* xp;
  void* t;
  const void* tx;    // t converted to the input form (fp32 hi+lo), read by passes 1 and 3
  void* yp;
  int pass;
  int nrhs;
  int compensated;   // fp32 storage: 1 error-free products and sums, 0 plain FP32 FMA
  int in_esz;        // bytes of one staged input value (x or t entry: 8 real, 16 complex)
  int* err;
  int* sched;        // two zeroed counters (items claimed, CTAs finished); left zero after a pass
  int chunked;       // several right-hand sides: items are single-piece chunks (chunk kernel)
  int t_f32;         // plain FP32 arithmetic, single launch: t accumulates in FP32 straight into the
                     // high parts of its input form tx (low parts stay zero), no conversion phase
};
// passes per operator: 0-3 the four-pass pipeline, 4-7 the phases of the single-launch matvec
#define MV_NPASS 8

// Single-launch matvec (one right-hand side): permute x, phase A items (t = V2 x and y += D x),
// t -> input form, phase B items (y += U2 t), un-permute y with alpha/beta; grid barriers
// between the phases (cooperative launch).  a: the shared arguments of the passes (items,
// pieces, ranges, nitems are set per phase from the fields below).
struct MVFusedArgs {
  MVArgs2 a;
  const MVTItem* items[2];
  const MVPiece* pieces[2];
  const MVRange* ranges[2];
  int nitems[2];
  int* ctr[2];          // chunk-claim counters of the two phases (zeroed in the prologue)
  unsigned long long* bar;  // grid barrier: arrival counter (only grows; a multiple of the grid between launches)
  const int* perm_in;   // xp[k] = x[perm_in[k]], k < n_in
  int n_in;
  const void* x;        // FP64 / complex128 input
  const int* perm_out;  // y[perm_out[k]] = alpha yp[k] + beta y[perm_out[k]], k < n_out
  int n_out;
  void* y;
  double alpha[2], beta[2];
  int use_beta;
  long long t_len;
  // bounded waits of the grid barriers: polls before a wait gives up (sets error bit 4 and
  // goes on), and arrivals added to every target (0 normally; 1 makes every barrier wait run
  // out, which a test uses to check that the error is reported without a hang or a fault)
  long long wait_limit;
  unsigned long long bar_extra;
};
// default poll limit of the grid-barrier waits (about a second on a GB300)
#define MV_WAIT_LIMIT (1LL << 24)
// false if the device cannot run it (no cooperative launch or the pipeline does not fit an SM)
bool mv_fused_supported();
cudaError_t launch_mv_fused(int prec, bool cplx, const MVFusedArgs& f, cudaStream_t s);

// Batched single-layer energy E_b = u_b^T V(X_b) u_b, V u and dE/dX (energy.cu)
struct SLEArgs {
  const double* X;        // 3 * nv_total vertex coordinates
  const int4* tri;        // global vertex ids per element
  const double* u;        // P0 densities, one per element
  const double* wprob;    // per-problem factor of the gradient (or null: 1)
  const int* tprob;       // problem of each element
  const int* t0;          // first element of each problem
  const int* nt;          // elements of each problem
  int ntri, dual, nq;
  double rxi[16], reta[16], rw[16];  // regular triangle rule (reference vertices (1,0),(0,1),(0,0))
  // per-element scratch written by the prep kernel
  double* D;              // |J| (1 with the dual mapping)
  double* dD;             // 9 per element: dD/dP_a
  float* cf;              // 6 per element: centroid hi, lo
  float* off;             // nq*3 per element: quadrature points - centroid (float)
  double* q64;            // nq*3 per element: quadrature points
  const int4* units;      // (problem, first test element, first trial element, -)
  int nunits;
  const int2* sing;       // ordered element pairs sharing a vertex (global element ids)
  int nsing;
  const double* ss[3];    // Sauter-Schwab directions x0, x1, y0, y1, w at xi = 1 (identical, edge, vertex)
  int ss_n[3];
  double ss_c1, ss_c2;    // sum over the radial Gauss points of w_xi xi and w_xi xi^2
  int ss_smem;            // 1: stage the three tables in shared memory (they fit 48 KB)
  double* energy;         // nprob (accumulated)
  double* vu;             // ntri (accumulated)
  double* grad;           // 3 * nv_total (accumulated; only with the gradient)
};
int sle_tile_test();
int sle_tile_trial(bool fp64, int nq);
void launch_sle(const SLEArgs& a, bool fp64, bool grad, cudaStream_t s);

// prec 0: fp64 storage, 1: fp32 storage.  cplx: complex operator.
void launch_mv_pass(int prec, bool cplx, const MVArgs2& a, int grid, cudaStream_t s);
// y += D x + U2 t for several right-hand sides, owner computes: one CTA per leaf row cluster
// gathers every dense block and low-rank U2 row slice that touches its rows, adds them up in
// shared memory and stores its rows of y (no global atomics).  entries: {kind (0 dense,
// 1 low rank), block, first local row, rows}; leaves: {first row, end row, first entry, end}.
struct MVRowArgs {
  const int4* leaves;
  int nleaves;
  const int4* ents;
  const MVDense* dense;
  const LRDesc* lr;
  const void* xp;   // permuted x (input form)
  const void* tx;   // t (input form)
  void* yp;         // permuted y (FP64 / complex128), written
  int nrhs;
  int compensated;
};
void launch_mv_rowowner(int prec, bool cplx, const MVRowArgs& a, cudaStream_t s);
int mv_stage_bytes();
int mv_piece_elems();  // target stored elements per piece
// tx = t in the input form (no-op for fp64 storage, where tx aliases t)
void launch_t_to_x(int prec, bool cplx, const void* t, void* tx, long long n, cudaStream_t s);
int mv_max_pieces();   // pieces per work item (descriptors staged with the payload)
int mv_in_bytes();     // staged input bytes per work item
// bytes of one permuted input value (X type) for a storage precision
inline int mv_x_bytes(int prec, bool cplx) { return (prec == 0 ? 8 : 8) * (cplx ? 2 : 1); }
// xp[k*nrhs + r] = (input form) x[r*ld + perm[k]]
void launch_permute_in(int prec, bool cplx, const int* perm, int n, int nrhs, int ld,
                       const void* x, void* xp, cudaStream_t s);
// y[r*ld + perm[k]] = alpha * yp[k*nrhs + r] + beta * y[...]   (fp64 / complex128)
// y[r * ld + rows[i]] = beta y[...] (0 when beta = 0) for i < nrows: the entries of a vector
// in a global numbering that hold no dof of the operator's output space
void launch_scale_rows(bool cplx, const int* rows, int nrows, int nrhs, int ld, const double* beta, void* y,
                       cudaStream_t s);
void launch_permute_out(bool cplx, const int* perm, int n, int nrhs, int ld, const double* alpha,
                        const double* beta, const void* yp, void* y, cudaStream_t s);
// CSR SpMV in fp64: y = alpha*A x + beta*y (A real; vectors real or complex; nrhs columns)
void launch_spmv(bool cplx, bool trans, int nrows, int ncols, const int* rowptr, const int* col,
                 const double* val, const double* alpha, const double* beta, const void* x,
                 void* y, int nrhs, cudaStream_t s);

// ---- BLAS-1/2 helpers for GMRES (fp64 / complex128), column-major basis Q (ld = n) -------
void launch_gemv_ct(bool cplx, int n, int k, const void* Q, const void* w, void* h, cudaStream_t s);
void launch_gemv_sub(bool cplx, int n, int k, const void* Q, const void* h, void* w, cudaStream_t s);
void launch_nrm2(bool cplx, int n, const void* w, double* out, cudaStream_t s);
void launch_scale_copy(bool cplx, int n, const void* w, double inv, void* q, cudaStream_t s);
// x += Q y  (y on device, complex or real)
void launch_axpy_basis(bool cplx, int n, int k, const void* Q, const void* y, void* x, cudaStream_t s);
// r = b - r  (r holds A x on input)
// batched GMRES vectors (gmres_batch.cu): nrhs columns of length n, basis block i at i*nrhs*n
void launch_bgemv_ct(bool cplx, int n, int k, int nrhs, const void* Q, const void* w, void* h, cudaStream_t s);
void launch_bgemv_sub(bool cplx, int n, int k, int nrhs, const void* Q, const void* h, void* w, cudaStream_t s);
void launch_baxpy_basis(bool cplx, int n, int k, int nrhs, const void* Q, const void* y, void* x, cudaStream_t s);
void launch_bnrm2(bool cplx, int n, int nrhs, const void* w, double* out, cudaStream_t s);
void launch_bscale(bool cplx, int n, int nrhs, const void* w, const double* inv, void* q, cudaStream_t s);
void launch_residual(bool cplx, int n, const void* b, void* r, cudaStream_t s);

// ---- potential evaluation (potential.cu) ----------------------------------------------------
struct PotArgs {
  const void* erec;       // ElemRecP<double>[nt]
  const void* qoff;       // QPt<double>[nt * nq]: rule points relative to the centroid, w * |J|
  const double* rq;       // reference points (xi, eta) of the rule
  const void* pgeo;       // PGeo<double>[nt * nq] of curved meshes, else null
  const int* elems;       // the nt source elements (null: elements 0 .. nt-1)
  int nt, nq;
  SpaceDev trial;
  const void* density;    // trial dofs (double or complex128)
  double* src_pos;        // 6 per rule point: y, n_y
  void* src_val;          // trial dimension per rule point: weighted evaluator values
  int npts;
  const double* pts;      // 3 per evaluation point
  const double* normals;  // 3 per evaluation point, or null
  double kappa;
  void* out;              // trial dimension per evaluation point
};
// components of the potential for (kernel, trial trace), 0 if there is none
int potential_dim(int kid, int trt);
int launch_potential(int kid, int trt, const PotArgs& a, cudaStream_t s);

// (kernel, trial trace, test trace) combinations of H1 of order 2, 3 (near field, projection):
// the Laplace single and double layer and the Helmholtz identity-trace operators on H1 x H1,
// the Laplace double layer from H1 of order p to SurfaceL2 of order p - 1 (the pairings of the
// reference's Laplace test, tests/test_Laplace.py:23-45) and the Laplace and Helmholtz
// hypersingular operators on H1
#define BEM_H1P_KERNELS(X, T, TROT, THELM, TL2)                                              \
  X(K_LAPLACE_SL, T, T) X(K_LAPLACE_DL, T, T) X(K_LAPLACE_DL, T, TL2) X(K_LAPLACE_HS, TROT, TROT) \
  X(K_HELMHOLTZ_SL, T, T) X(K_HELMHOLTZ_DL, T, T) X(K_HELMHOLTZ_CF, T, T)                       \
  X(K_HELMHOLTZ_HS, THELM, THELM)
#define BEM_H1P_COMBOS(X)                                              \
  BEM_H1P_KERNELS(X, TR_H1P2, TR_H1P2ROT, TR_H1P2HELM, TR_L2P1)         \
  BEM_H1P_KERNELS(X, TR_H1P3, TR_H1P3ROT, TR_H1P3HELM, TR_L2P2)
// HDivSurface and HCurl of order 1, 2: the Maxwell single layer on either, the Maxwell double
// layer from HCurl to HDivSurface or HCurl (near field, projection)
#define BEM_HDIV_KERNELS(X, D, C)                                                                        \
  X(K_MAXWELL_SL, D##MAX, D##MAX) X(K_MAXWELL_SL, C##MAX, C##MAX) X(K_MAXWELL_DL, C##ROT, D##ID)        \
  X(K_MAXWELL_DL, C##ROT, C##ID)
#define BEM_HDIV_COMBOS(X) BEM_HDIV_KERNELS(X, TR_HDIV1, TR_HCURL1) BEM_HDIV_KERNELS(X, TR_HDIV2, TR_HCURL2)
// order 3, 4 (20, 30 dofs per element): the pairings of the reference's Maxwell tests, the single
// layer on HDivSurface of order 3 and 4 and the double layer from HCurl to HDivSurface of order 3
#define BEM_HDIV34_COMBOS(X)                                                                 \
  X(K_MAXWELL_SL, TR_HDIV3MAX, TR_HDIV3MAX) X(K_MAXWELL_DL, TR_HCURL3ROT, TR_HDIV3ID)         \
  X(K_MAXWELL_SL, TR_HDIV4MAX, TR_HDIV4MAX)

// ---- tensor-core products for several right-hand sides (tc_matvec.cu) ---------------------
// Operand panels are in the canonical K-major, no-swizzle layout of tcgen05 (core matrices of
// 8 rows x 16 bytes), K counted in "cores" of 4 FP32 values:
//   A panel, 128 rows: float4 index kc * 128 + row                     (2048 bytes per core)
//   B panel, N rows, TF32 high and low parts: float4 (2 kc + h) * N + n   (32 N bytes per core)
// Row 4 r + 2 a + h of an A panel is right-hand side r, real (a = 0) or imaginary part, high
// (h = 0) or low TF32 part.
struct TCSeg {
  unsigned long long a, b;  // A and B panels (global addresses, 16-byte aligned)
  int nkc;                  // K cores (even: one MMA takes K = 8)
  int pad[3];
};
struct TCItem {
  int seg0, nseg;  // segments summed into the item's result
  int N;           // MMA N: multiple of 16, 16..256
  int out0, nout;  // pass 0: outputs [out0, out0+nout); pass 1: partial row offset, rows
  int nk2;         // MMA K steps (K = 8) of all its segments
  int pad[2];
};
// The accumulation inside tcgen05.mma rounds toward zero, so its error grows linearly with the
// number of MMAs into one accumulator (about 2.5e-8 relative per MMA, measured on GB300).  An
// item's K steps therefore go round-robin to the A = 256 / round_up(N, 32) accumulators of a
// 256-column tensor-memory buffer, each taking at most TC_CHAIN of them (2 TC_CHAIN MMAs: high
// and low B parts) before the buffer is handed to the epilogue, which adds the accumulators
// into FP32 sums that round to nearest; the other buffer takes the next K steps meanwhile.
#define TC_CHAIN 4
struct TCOut {            // pass 0: one low-rank block of a column tile
  unsigned long long ta;  // its A panel for pass 1 (128 x 2 rpad)
  int col, rpad;          // first accumulator column; rank padded to a multiple of 4
};
// One K range of a segment in a pipeline stage (planned on the host): A at byte `off` of the
// stage, B right after it.  flags: 1 first range of an item, 2 last range of an item, 4 last
// range of the stage.
struct TCChunk {
  unsigned long long a, b;
  unsigned int abytes, bbytes, off;
  unsigned short N, flags;
};
static_assert(sizeof(TCChunk) == 32, "TCChunk is bulk-copied");
#define TC_MAXCH 16  // ranges per stage
struct TCGemmArgs {
  const TCItem* items;
  const TCOut* outs;
  const int4* sched;     // per CTA: first item, items, first stage, stages
  const int2* stages;    // per stage: first range, ranges
  const TCChunk* chunks;
  void* ypart;           // pass 1 output (complex64 rows of 32 right-hand sides)
  int* err;
};
struct TCVJob {  // pack the V2 panel of a column tile
  unsigned long long dst;
  int kc0, nkc, N, cm0;  // first absolute K core, cores, N, column map offset
};
struct TCUJob {  // pack the U2 panel of (row tile, block)
  unsigned long long dst;
  int lr, i0, rows, N, nkc, pad;
};
struct TCDJob {  // pack the panel of (row tile, dense block): K = (column, real/imaginary)
  unsigned long long dst;
  int blk, i0, rows, N, kc0, nkc;
};
// The pipeline ring holds TC_STAGE_BYTES, cut into 2, 3 or 4 stages (the operator's stage plan,
// picked by bem_operator_autotune_tc; 2 by default: fewer, larger stages measured fastest).
// One MMA step of N = 256 takes 20 KB.
#define TC_STAGE_BYTES (192 * 1024)
#define TC_NST_MAX 4
#define TC_NST_DEFAULT 2
__host__ __device__ constexpr int tc_cap(int nst) { return TC_STAGE_BYTES / nst; }
int tc_smem_bytes();
// 1 when the running device executes the tcgen05 kernels (compute capability 10.x)
int tc_supported();
// A panels of x = x[r * ld + perm[j]] (complex128), dof j in cluster order, r < nrhs:
//   xa  (nkc cores): K = dof (4 per core), row (r, a, h) the h part of Re/Im x;
//   xa2 (nkc2 cores): K = (dof, c) (2 dofs per core), row (r, a, h) the h part of
//       a = 0: (Re x, -Im x), a = 1: (Im x, Re x), so that a real product with the
//       (Re D, Im D) columns of a complex block gives Re and Im of D x.
void launch_tc_xprep(const int* perm, int n, int nrhs, int ld, const void* x, void* xa, int nkc, void* xa2, int nkc2,
                     cudaStream_t s);
void launch_tc_pack_v(const TCVJob* jobs, int njobs, const int4* colmap, const LRDesc* lr, cudaStream_t s);
void launch_tc_pack_u(const TCUJob* jobs, int njobs, const LRDesc* lr, cudaStream_t s);
void launch_tc_pack_d(const TCDJob* jobs, int njobs, const MVDense* dense, cudaStream_t s);
// y[r * ld + perm[i]] = alpha * sum_e ypart[(i + delta[e]) * 32 + r] + beta * y[...] over the
// entries [L.z, L.w) of the leaf L = {first row, end row, first entry, end entry} holding row i
void launch_tc_ysum_out(const int4* leaves, int nleaves, const int* deltas, const void* ypart, const int* perm,
                        int nrhs, int ld, const double* alpha, const double* beta, void* y, cudaStream_t s);
// pass 0 (pass = 0): T panels of every low-rank block; pass 1: partial rows of U2 T
cudaError_t launch_tc_gemm(int pass, int nst, const TCGemmArgs& g, int grid, cudaStream_t s);
// one 128 x N x (4 nkc) product D = A B^T on the tensor cores from ready panels (self-test):
// d[row * N + n] (FP32); the B panel holds high and low parts, both are issued
cudaError_t launch_tc_selftest(const void* a, const void* b, int N, int nkc, float* d, int* err, cudaStream_t s);

}  // namespace bem
