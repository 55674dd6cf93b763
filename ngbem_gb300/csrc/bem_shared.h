// Plain-old-data descriptors shared by the host orchestration (C++) and the CUDA kernels.
#pragma once
#include <stdint.h>

namespace bem {

enum KernelId {
  K_LAPLACE_SL = 0, K_LAPLACE_DL = 1, K_LAPLACE_HS = 2, K_HELMHOLTZ_SL = 3,
  K_HELMHOLTZ_DL = 4, K_HELMHOLTZ_HS = 5, K_HELMHOLTZ_CF = 6, K_MAXWELL_SL = 7,
  K_NUM = 8
};

// trace kinds = (space kind, evaluator) combinations the operators use
enum TraceKind { TR_P0 = 0, TR_P1 = 1, TR_ROT = 2, TR_HELM = 3, TR_MAX = 4, TR_RT0ID = 5 };

// Per-element record (FP64): vertices, unit normal, |J|, rotated surface gradients of the
// P1 hat functions (n x grad lambda_a), vertex ids.  128 bytes + 64 bytes, read by the
// singular kernel, the element tables of every precision are built from it on the host.
struct ElemRec64 {
  double p[3][3];     // vertices; reference vertices (1,0),(0,1),(0,0)
  double n[3];
  double detJ;        // |(p0-p2) x (p1-p2)|
  double invdetJ;
  double rot[3][3];   // n x surface-grad(lambda_a)
  double pad[1];
};

// Per-element record in compute precision P: centroid as hi+lo pair (so differences of
// centroids are accurate to P's relative precision), vertex offsets from the centroid.
template <class P>
struct ElemRecP {
  P chi[3], clo[3];
  P n[3];
  P detJ, invdetJ;
  P o[3][3];          // p_k - centroid
  P rot[3][3];
  P pad[3];
};

// A dense (near-field or fallback) block of the H-matrix.
struct DenseDesc {
  long long off;      // offset of the m x n row-major block in the dense pool (elements)
  int r0, m;          // rows [r0, r0+m) in the test cluster permutation
  int c0, n;          // cols [c0, c0+n) in the trial cluster permutation
  int pi0, ni;        // test patch: patch_elems[pi0 .. pi0+ni)
  int pj0, nj;        // trial patch
};

// Work tile of the regular near-field kernel: 128 consecutive element pairs of block b.
struct NFTile {
  int b;              // dense block index
  int k0;             // first flattened pair index (i * nj + j)
};

// Singular element pair found by the regular kernel.
struct SingItem {
  int b, ei, ej;
};

// A far-field (low-rank) block.
struct FarDesc {
  int r0, m, c0, n;   // dof ranges (cluster permutation)
  int pi0, ni, pj0, nj;  // patches
  long long su, sv;   // ACA scratch offsets (elements) of U (kcap x M) and V (kcap x N), per comp
  int kcap;
  int pad;
};

// Low-rank factors after projection: U2 (m x R, column-major) and V2 (R x n, row-major),
// addressed by absolute device pointers (factor pools may be allocated per ACA batch).
struct LRDesc {
  unsigned long long u, v;
  int r0, m, c0, n;
  int R;
  int toff;              // offset of the R-vector of V2*x in the temporary pool
};

// matvec descriptors (absolute device pointers)
struct MVDense {
  unsigned long long ptr;
  int r0, m, c0, n;
};
typedef LRDesc MVLowRank;

struct TermDesc {
  int nterms;
  int kc[4], trc[4], tec[4];
  double fac[4];
};

}  // namespace bem
