// Plain-old-data descriptors shared by the host orchestration (C++) and the CUDA kernels.
#pragma once
#include <stdint.h>

namespace bem {

enum KernelId {
  K_LAPLACE_SL = 0, K_LAPLACE_DL = 1, K_LAPLACE_HS = 2, K_HELMHOLTZ_SL = 3,
  K_HELMHOLTZ_DL = 4, K_HELMHOLTZ_HS = 5, K_HELMHOLTZ_CF = 6, K_MAXWELL_SL = 7,
  K_HELMHOLTZ_SL_DKAPPA = 8,  // d/dkappa of the Helmholtz single layer (no counterpart in the reference)
  K_MAXWELL_DL = 9,
  K_NUM = 10
};

// trace kinds = (space kind, evaluator) combinations the operators use
// TR_NED, TR_NEDROT, TR_NEDMAX: the HCurl (lowest-order Nedelec) traces of the edge dofs:
// the tangential shape n x phi_RT0, the rotated trace n x (n x phi_RT0) = -phi_RT0, and the
// Maxwell trace [-phi_RT0; surface curl] (reference DiffOpRotatedTrace, DiffOpMaxwell,
// src/diffops.hpp:62-255, for the Whitney edge shapes, which are n x the RT0 shapes)
enum TraceKind { TR_P0 = 0, TR_P1 = 1, TR_ROT = 2, TR_HELM = 3, TR_MAX = 4, TR_RT0ID = 5,
                 TR_NED = 6, TR_NEDROT = 7, TR_NEDMAX = 8 };
// traces whose local dofs carry an edge orientation sign
__host__ __device__ constexpr bool edge_trace(int tr) {
  return tr == TR_MAX || tr == TR_RT0ID || tr == TR_NED || tr == TR_NEDROT || tr == TR_NEDMAX;
}

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
  long long off;      // offset of the m x n column-major block in the dense pool (elements, 16-byte aligned)
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

// Low-rank factors after projection, addressed by absolute device pointers (factor pools may
// be allocated per ACA batch).  Chunked layouts so that every chunk is one contiguous,
// 16-byte aligned copy:
//   U2 (m x R): row chunks of cu rows;   U2(i, r) at u + (i/cu)*cu*R + r*cu + i%cu
//   V2 (R x n): column chunks of cv cols; V2(r, j) at v + (j/cv)*cv*R + (j%cv)*R + r
struct LRDesc {
  unsigned long long u, v;
  int r0, m, c0, n;
  int R;
  int toff;              // offset of the R-vector of V2*x in the temporary pool
  int cu, cv;
};
__host__ __device__ inline long long lr_u_index(const LRDesc& L, int i, int r) {
  return (long long)(i / L.cu) * L.cu * L.R + (long long)r * L.cu + (i % L.cu);
}
__host__ __device__ inline long long lr_v_index(const LRDesc& L, int r, int j) {
  return (long long)(j / L.cv) * L.cv * L.R + (long long)(j % L.cv) * L.R + r;
}

// matvec descriptors (absolute device pointers); dense blocks are column-major
struct MVDense {
  unsigned long long ptr;
  int r0, m, c0, n;
};

// A segment of a matvec work item: a (part of a) block whose payload sits at byte offset
// soff of the item.  kind 0: dense columns [k0, k0+cnt); 1: U2 row chunk [k0, k0+cnt);
// 2: V2 column chunk [k0, k0+cnt).
struct MVSeg {
  int kind, blk, k0, cnt, soff, pad;
};
// A work item: one contiguous copy of `bytes` bytes from src (bytes == 0: read in place),
// its pieces [seg0, seg0+nseg) and the input ranges [rng0, rng0+nrng) copied next to it
// (inbytes in total).
struct MVTItem {
  unsigned long long src;
  int bytes, seg0, nseg, rng0, nrng, inbytes;
  int r[8];  // the first two input ranges inline (src, elem, bytes, dst each); others in the range list
  int pad[4];  // 80 bytes: runs of descriptors are bulk-copied (16-byte multiples)
};
static_assert(sizeof(MVTItem) % 16 == 0, "MVTItem is bulk-copied");

// A piece of an item as one pass applies it: out[out_off + o] += sum_k A[o*so + k*sk] *
// in[in_off + k] for o < O, k < Kc, with A at byte soff of the item payload.  flags bit 0:
// the input is the R-vector pool t (else the permuted x); bit 1: the output is t (else y).
// in_soff: byte offset of in[in_off] in the item's staged input area.
struct MVPiece {
  int soff, so, sk, O, Kc, in_off, out_off, flags, in_soff;
  int ow;      // lanes per group: min(O, 32)
  int groups;  // 32 / ow lane groups splitting k
  float inv_ow;  // 1/ow (exact lane -> group mapping for lane < 32)
};

// An input range staged with an item: `bytes` bytes from element `elem` (16-byte aligned
// start) of x (src 0) or t (src 1), to byte `dst` of the input area.
struct MVRange {
  int src, elem, bytes, dst;
};
typedef LRDesc MVLowRank;

struct TermDesc {
  int nterms;
  int kc[4], trc[4], tec[4];
  double fac[4];
};

}  // namespace bem
