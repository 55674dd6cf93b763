// Near-field assembly kernel templates (reference CalcBlockMatrix, src/ngbem.cpp:373-738),
// instantiated by nearfield.cu (the P0 / P1 / edge traces) and nearfield_l2p.cu (SurfaceL2 of
// order 1..3), two translation units so that they compile side by side.
//
// nf_regular : one thread per (test element, trial element) pair of a dense block, 128
//              consecutive pairs per CTA.  Pairs sharing a vertex are appended to the
//              singular work list (binning by singularity class happens in nf_singular).
//              Disjoint pairs use the tensor product of the regular triangle rule
//              (src/ngbem.cpp:680-727) in compute precision P.  Differences x - y are
//              formed from centroid differences (hi+lo pairs) plus local offsets, so that
//              FP32 keeps its relative precision for close panels.
// nf_singular: persistent grid, one warp per singular pair, FP64 Sauter-Schwab quadrature
//              for identical / common-edge / common-vertex pairs (src/ngbem.cpp:535-678)
//              with the vertex permutations of :569-586 and :627-642.  Rule tables are
//              staged in shared memory.
#pragma once
#include <cstdio>

#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

__device__ __forceinline__ int i4c(const int4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

template <class P> struct P2 { P x, y; };

// A curved element's map at (xi, eta): the point, the normal, the rotated gradients, and for
// the traces that read them 1 / |J| and the Piola offsets; returns |J0 x J1|.
template <int TR>
__device__ __forceinline__ double curved_point(int g, const double* nodes, double xi, double eta, double* x,
                                               double* n, double rot[3][3], double& inv, double xp[3][3]) {
  double J0[3], J1[3];
  curved_map(g, nodes, xi, eta, x, J0, J1);
  const double detJ = surface_frame(J0, J1, n, rot);
  if constexpr (piola_trace(TR)) inv = 1.0 / detJ;
  if constexpr (edge_trace(TR)) piola_offsets(J0, J1, xi, eta, xp);
  return detJ;
}

template <int KID, class P, int TRT, int TET>
__global__ void __launch_bounds__(128) nf_regular_kernel(NFArgs a) {
  using G = Green<KID>;
  using V = VT<G::CPLX, P>;
  constexpr int NDI = TraceInfo<TET>::ND, NDJ = TraceInfo<TRT>::ND;
  constexpr int NT = G::NT, NC = G::NC;

  const NFTile tile = a.tiles[blockIdx.x];
  const DenseDesc d = a.blocks[tile.b];
  const int k = tile.k0 + (int)threadIdx.x;
  if (k >= d.ni * d.nj) return;
  const int i = k / d.nj, j = k - i * d.nj;
  const int ei = a.patch_test[d.pi0 + i];
  const int ej = a.patch_trial[d.pj0 + j];
  const int4 vi = a.tri[ei], vj = a.tri[ej];
  const int common = (vi.x == vj.x) + (vi.x == vj.y) + (vi.x == vj.z) + (vi.y == vj.x) + (vi.y == vj.y) +
                     (vi.y == vj.z) + (vi.z == vj.x) + (vi.z == vj.y) + (vi.z == vj.z);
  if (common) {
    int slot = atomicAdd(a.sing_count, 1);
    if (slot < a.sing_cap) a.sing[slot] = SingItem{tile.b, ei, ej};
    else atomicOr(a.err, 1);
    return;
  }
  const ElemRecP<P>* E = (const ElemRecP<P>*)a.erecP;
  const QPt<P>* Q = (const QPt<P>*)a.qoff;
  const P2<P>* RQ = (const P2<P>*)a.rq;
  const ElemRecP<P>& Ei = E[ei];
  const ElemRecP<P>& Ej = E[ej];
  const P Dx = (Ei.chi[0] - Ej.chi[0]) + (Ei.clo[0] - Ej.clo[0]);
  const P Dy = (Ei.chi[1] - Ej.chi[1]) + (Ei.clo[1] - Ej.clo[1]);
  const P Dz = (Ei.chi[2] - Ej.chi[2]) + (Ei.clo[2] - Ej.clo[2]);
  P nx[3], ny[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) { nx[c] = Ei.n[c]; ny[c] = Ej.n[c]; }
  P roti[3][3], rotj[3][3], oi[3][3], oj[3][3];
  P invi = Ei.invdetJ, invj = Ej.invdetJ;
  if (needs_rot(TET)) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) roti[r][c] = Ei.rot[r][c];
  }
  if (needs_rot(TRT)) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) rotj[r][c] = Ej.rot[r][c];
  }
  if (edge_trace(TET)) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) oi[r][c] = Ei.o[r][c];
  }
  if (edge_trace(TRT)) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) oj[r][c] = Ej.o[r][c];
  }
  int sgi[SignSlots<TET>::N], sgj[SignSlots<TRT>::N];
  elem_signs<TET>(a.test.sign, ei, sgi);
  elem_signs<TRT>(a.trial.sign, ej, sgj);
  const bool duali = a.test.dual != 0, dualj = a.trial.dual != 0;
  const P kappa = (P)a.kappa;

  // element matrices above 144 entries (HDivSurface of order 3, 4) keep their rows in rolled
  // loops: the matrix lives in (cached) local memory instead of unrolled spill code
  constexpr int RU = NDI * NDJ > 144 ? 1 : NDI;
  V elmat[NDI][NDJ];
#pragma unroll RU
  for (int r = 0; r < NDI; ++r)
#pragma unroll
    for (int c = 0; c < NDJ; ++c) elmat[r][c] = vzero<V>();

  const int nq = a.nq;
  const QPt<P>* Qi = Q + (size_t)ei * nq;
  const QPt<P>* Qj = Q + (size_t)ej * nq;
  // curved elements: normals and rotated gradients per rule point (flat: per element, above)
  const PGeo<P>* PGi = a.pgeo ? (const PGeo<P>*)a.pgeo + (size_t)ei * nq : nullptr;
  const PGeo<P>* PGj = a.pgeo ? (const PGeo<P>*)a.pgeo + (size_t)ej * nq : nullptr;
  for (int p = 0; p < nq; ++p) {
    const QPt<P> qi = Qi[p];
    const P2<P> rp = RQ[p];
    P xpi[3][3];
    if (edge_trace(TET)) {
#pragma unroll
      for (int r = 0; r < 3; ++r) { xpi[r][0] = qi.x - oi[r][0]; xpi[r][1] = qi.y - oi[r][1]; xpi[r][2] = qi.z - oi[r][2]; }
    }
    if (PGi) pgeo_load<P, G::NEEDS_NX || normal_trace(TET), needs_rot(TET), piola_trace(TET)>(PGi[p], nx, roti, invi, xpi);
    V ks[NT][NDJ];
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
      for (int b = 0; b < NDJ; ++b) ks[t][b] = vzero<V>();
    for (int q = 0; q < nq; ++q) {
      const QPt<P> qj = Qj[q];
      P xpj[3][3];
      if (edge_trace(TRT)) {
#pragma unroll
        for (int r = 0; r < 3; ++r) { xpj[r][0] = qj.x - oj[r][0]; xpj[r][1] = qj.y - oj[r][1]; xpj[r][2] = qj.z - oj[r][2]; }
      }
      if (PGj) pgeo_load<P, G::NEEDS_NY || normal_trace(TRT), needs_rot(TRT), piola_trace(TRT)>(PGj[q], ny, rotj, invj, xpj);
      const P dx = Dx + (qi.x - qj.x), dy = Dy + (qi.y - qj.y), dz = Dz + (qi.z - qj.z);
      V kv[NC];
      G::eval(dx, dy, dz, nx, ny, kappa, kv);
      const P w = qi.w * qj.w;
      const P2<P> rqq = RQ[q];
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        const V kw = kv[G::kc(t)] * w;
#pragma unroll
        for (int b = 0; b < NDJ; ++b) {
          P s = trace_val<TRT, P>(b, G::trc(t), rqq.x, rqq.y, xpj, invj, rotj, sgj[b], dualj, ny);
          ks[t][b] += kw * s;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const P fac = term_fac<G, P>(t, kappa);
#pragma unroll RU
      for (int r = 0; r < NDI; ++r) {
        P s = fac * trace_val<TET, P>(r, G::tec(t), rp.x, rp.y, xpi, invi, roti, sgi[r], duali, nx);
#pragma unroll
        for (int b = 0; b < NDJ; ++b) elmat[r][b] += ks[t][b] * s;
      }
    }
  }
  // scatter into the dense block (src/ngbem.cpp:733-736)
  const int4 dni = a.test.dofs[ei], dnj = a.trial.dofs[ej];
  const int4 xi_ = dof_aux<TET>(a.test.sign, ei), xj_ = dof_aux<TRT>(a.trial.sign, ej);
  int rows[NDI], cols[NDJ];
#pragma unroll
  for (int r = 0; r < NDI; ++r) {
    int pos = a.test.pinv[elem_dof<TET>(dni, xi_, r)] - d.r0;
    rows[r] = (pos >= 0 && pos < d.m) ? pos : -1;
  }
#pragma unroll
  for (int c = 0; c < NDJ; ++c) {
    int pos = a.trial.pinv[elem_dof<TRT>(dnj, xj_, c)] - d.c0;
    cols[c] = (pos >= 0 && pos < d.n) ? pos : -1;
  }
  V* pool = (V*)a.pool + d.off;
#pragma unroll RU
  for (int r = 0; r < NDI; ++r)
#pragma unroll
    for (int c = 0; c < NDJ; ++c)
      if (rows[r] >= 0 && cols[c] >= 0) {
        V* dst = pool + (size_t)cols[c] * d.m + rows[r];  // column-major block
        if (a.atomic_scatter) atomic_add(dst, elmat[r][c]);
        else *dst = elmat[r][c];
      }
}

// CURVED: the elements are curved (a.gnodes): the maps are evaluated per Sauter-Schwab point
template <int KID, class S, int TRT, int TET, bool CURVED>
__global__ void __launch_bounds__(256) nf_singular_kernel(NFArgs a) {
  using G = Green<KID>;
  using V = VT<G::CPLX, double>;
  using VS = VT<G::CPLX, S>;
  constexpr int NDI = TraceInfo<TET>::ND, NDJ = TraceInfo<TRT>::ND;
  constexpr int NT = G::NT, NC = G::NC;
  extern __shared__ double smem[];

  const double* tab[3];
  if (a.ss_smem_bytes > 0) {
    int off = 0;
    for (int c = 0; c < 3; ++c) {
      const int n5 = 5 * a.ss_n[c];
      for (int t = threadIdx.x; t < n5; t += blockDim.x) smem[off + t] = a.ss[c][t];
      tab[c] = smem + off;
      off += n5;
    }
    __syncthreads();
  } else {
    for (int c = 0; c < 3; ++c) tab[c] = a.ss[c];
  }
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int count = min(*a.sing_count, a.sing_cap);
  const double kappa = a.kappa;
  const bool duali = a.test.dual != 0, dualj = a.trial.dual != 0;

  for (int it = warp; it < count; it += nwarps) {
    const SingItem s = a.sing[it];
    const DenseDesc d = a.blocks[s.b];
    const int4 vi4 = a.tri[s.ei], vj4 = a.tri[s.ej];
    const int vi[3] = {vi4.x, vi4.y, vi4.z}, vj[3] = {vj4.x, vj4.y, vj4.z};
    int ncommon = 0;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) ncommon += (vi[p] == vj[q]);
    int cls = ncommon == 3 ? 0 : (ncommon == 2 ? 1 : 2);
    int px[3] = {0, 1, 2}, py[3] = {0, 1, 2};
    if (cls == 1) {
      // edge table (0,1) | (1,2) | (2,0); the common edge comes first, reversed in y
      int cex = 0, cey = 0;
      for (int cx = 0; cx < 3; ++cx)
        for (int cy = 0; cy < 3; ++cy) {
          int a0 = vi[cx], a1 = vi[(cx + 1) % 3], b0 = vj[cy], b1 = vj[(cy + 1) % 3];
          if (min(a0, a1) == min(b0, b1) && max(a0, a1) == max(b0, b1)) { cex = cx; cey = cy; }
        }
      px[0] = cex; px[1] = (cex + 1) % 3; px[2] = 3 - px[0] - px[1];
      py[0] = (cey + 1) % 3; py[1] = cey; py[2] = 3 - py[0] - py[1];
    } else if (cls == 2) {
      int cvx = 0, cvy = 0;
      for (int cx = 0; cx < 3; ++cx)
        for (int cy = 0; cy < 3; ++cy)
          if (vi[cx] == vj[cy]) { cvx = cx; cvy = cy; }
      px[0] = cvx; px[1] = (cvx + 1) % 3; px[2] = (cvx + 2) % 3;
      py[0] = cvy; py[1] = (cvy + 1) % 3; py[2] = (cvy + 2) % 3;
    }
    const ElemRec64& Ei = a.erec64[s.ei];
    const ElemRec64& Ej = a.erec64[s.ej];
    double pi[3][3], pj[3][3], nx[3], ny[3], roti[3][3], rotj[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        pi[r][c] = Ei.p[r][c]; pj[r][c] = Ej.p[r][c];
        roti[r][c] = Ei.rot[r][c]; rotj[r][c] = Ej.rot[r][c];
      }
#pragma unroll
    for (int c = 0; c < 3; ++c) { nx[c] = Ei.n[c]; ny[c] = Ej.n[c]; }
    const double detJ2 = Ei.detJ * Ej.detJ;
    double invi = Ei.invdetJ, invj = Ej.invdetJ;
    int sgi[SignSlots<TET>::N], sgj[SignSlots<TRT>::N];
    elem_signs<TET>(a.test.sign, s.ei, sgi);
    elem_signs<TRT>(a.trial.sign, s.ej, sgj);

    V acc[NDI][NDJ];
#pragma unroll
    for (int r = 0; r < NDI; ++r)
#pragma unroll
      for (int c = 0; c < NDJ; ++c) acc[r][c] = vzero<V>();

    const int npts = a.ss_n[cls];
    const double* T = tab[cls];
    for (int kk = lane; kk < npts; kk += 32) {
      const double x0 = T[kk], x1 = T[npts + kk], y0 = T[2 * npts + kk], y1 = T[3 * npts + kk];
      const double w = T[4 * npts + kk];
      double xi, xe, yi, ye;
      if (cls == 0) {
        xi = x0; xe = x1; yi = y0; ye = y1;
      } else {
        const double lx[3] = {1.0 - x0 - x1, x0, x1};
        const double ly[3] = {1.0 - y0 - y1, y0, y1};
        double plx[3], ply[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) { plx[px[q]] = lx[q]; ply[py[q]] = ly[q]; }
        xi = plx[0]; xe = plx[1]; yi = ply[0]; ye = ply[1];
      }
      double x[3], y[3], xpi[3][3], xpj[3][3];
      double fac;
      if constexpr (CURVED) {
        // curved elements: the maps, normals, rotated gradients and Piola data at the two points
        const int nn = (a.gorder + 1) * (a.gorder + 2) / 2;
        const double dxi = curved_point<TET>(a.gorder, a.gnodes + (size_t)s.ei * nn * 3, xi, xe, x, nx, roti, invi, xpi);
        const double dyj = curved_point<TRT>(a.gorder, a.gnodes + (size_t)s.ej * nn * 3, yi, ye, y, ny, rotj, invj, xpj);
        fac = dxi * dyj * w;
      } else {
        const double l2x = 1.0 - xi - xe, l2y = 1.0 - yi - ye;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          x[c] = xi * pi[0][c] + xe * pi[1][c] + l2x * pi[2][c];
          y[c] = yi * pj[0][c] + ye * pj[1][c] + l2y * pj[2][c];
        }
        fac = detJ2 * w;
      }
      V kv[NC];
      G::eval(x[0] - y[0], x[1] - y[1], x[2] - y[2], nx, ny, kappa, kv);
      if constexpr (!CURVED) {
        if (edge_trace(TET)) {
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) xpi[r][c] = x[c] - pi[r][c];
        }
        if (edge_trace(TRT)) {
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) xpj[r][c] = y[c] - pj[r][c];
        }
      }
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        const V kf = kv[G::kc(t)] * (fac * term_fac<G, double>(t, kappa));
        // the trace values of the point once per side, then their outer product
        V ti[NDI];
        double tj[NDJ];
#pragma unroll
        for (int r = 0; r < NDI; ++r)
          ti[r] = kf * trace_val<TET, double>(r, G::tec(t), xi, xe, xpi, invi, roti, sgi[r], duali, nx);
#pragma unroll
        for (int c = 0; c < NDJ; ++c)
          tj[c] = trace_val<TRT, double>(c, G::trc(t), yi, ye, xpj, invj, rotj, sgj[c], dualj, ny);
        if constexpr (NDI * NDJ > 36) {
          // high-order pairs: the element matrix does not fit the registers; a rolled loop
          // keeps it in (cached) local memory without unrolled spill code
#pragma unroll 1
          for (int r = 0; r < NDI; ++r)
#pragma unroll
            for (int c = 0; c < NDJ; ++c) acc[r][c] += ti[r] * tj[c];
        } else {
#pragma unroll
          for (int r = 0; r < NDI; ++r)
#pragma unroll
            for (int c = 0; c < NDJ; ++c) acc[r][c] += ti[r] * tj[c];
        }
      }
    }
#pragma unroll (NDI * NDJ > 36 ? 1 : NDI)
    for (int r = 0; r < NDI; ++r)
#pragma unroll
      for (int c = 0; c < NDJ; ++c) acc[r][c] = warp_sum(acc[r][c]);
    if (lane == 0) {
      const int4 dni = a.test.dofs[s.ei], dnj = a.trial.dofs[s.ej];
      const int4 xi_ = dof_aux<TET>(a.test.sign, s.ei), xj_ = dof_aux<TRT>(a.trial.sign, s.ej);
      VS* pool = (VS*)a.pool + d.off;
#pragma unroll
      for (int r = 0; r < NDI; ++r) {
        int row = a.test.pinv[elem_dof<TET>(dni, xi_, r)] - d.r0;
        if (row < 0 || row >= d.m) continue;
#pragma unroll
        for (int c = 0; c < NDJ; ++c) {
          int col = a.trial.pinv[elem_dof<TRT>(dnj, xj_, c)] - d.c0;
          if (col < 0 || col >= d.n) continue;
          VS v;
          cvt(v, acc[r][c]);
          VS* dst = pool + (size_t)col * d.m + row;  // column-major block
          if (a.atomic_scatter) atomic_add(dst, v);
          else *dst = v;
        }
      }
    }
  }
}

// ----------------------------------------------------------------------------------------
// SurfaceL2 of order 1..3 on both sides, for the kernels with identity traces (one trace at a
// time: each order compiles in translation units of its own, nearfield_l2p*.cu)
#define BEM_L2P_KERNELS(X, T) \
  X(K_LAPLACE_SL, T, T) X(K_LAPLACE_DL, T, T) X(K_HELMHOLTZ_SL, T, T) X(K_HELMHOLTZ_DL, T, T) X(K_HELMHOLTZ_CF, T, T)
#define BEM_L2P_COMBOS(X) BEM_L2P_KERNELS(X, TR_L2P1) BEM_L2P_KERNELS(X, TR_L2P2) BEM_L2P_KERNELS(X, TR_L2P3)
// H1 of order 2, 3 (BEM_H1P_COMBOS, kernels.h): each order in translation units of its own,
// nearfield_h1p*.cu
void launch_nf_regular_h1p2(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_h1p2(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_nf_regular_h1p3(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_h1p3(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
// HDivSurface and HCurl of order 1, 2 (BEM_HDIV_COMBOS): nearfield_hdiv.cu, nearfield_hdivs.cu
void launch_nf_regular_hdiv(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_hdiv(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
// order 3, 4 (BEM_HDIV34_COMBOS): nearfield_hdiv34r.cu, nearfield_hdiv34s.cu
void launch_nf_regular_hdiv34(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_hdiv34(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s);
// bodies of those launchers: one (kernel, trial trace, test trace) combination
#define BEM_NF_REGULAR_X3(K, A, B)                                                     \
  if (kid == K && trt == A && tet == B) {                                              \
    if (prec == 0) nf_regular_kernel<K, double, A, B><<<a.ntiles, 128, 0, s>>>(a);    \
    else nf_regular_kernel<K, float, A, B><<<a.ntiles, 128, 0, s>>>(a);               \
    return;                                                                            \
  }
#define BEM_NF_SINGULAR_X3(K, A, B)                                                    \
  if (kid == K && trt == A && tet == B) {                                              \
    if (prec == 0) run_singular<K, double, A, B>(a, s);                                \
    else run_singular<K, float, A, B>(a, s);                                           \
    return;                                                                            \
  }
void launch_nf_regular_l2p1(int kid, int prec, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_l2p1(int kid, int prec, const NFArgs& a, cudaStream_t s);
void launch_nf_regular_l2p2(int kid, int prec, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_l2p2(int kid, int prec, const NFArgs& a, cudaStream_t s);
void launch_nf_regular_l2p3(int kid, int prec, const NFArgs& a, cudaStream_t s);
void launch_nf_singular_l2p3(int kid, int prec, const NFArgs& a, cudaStream_t s);
// bodies of those launchers
#define BEM_NF_REGULAR_X(K, A, B)                                                      \
  if (kid == K) {                                                                      \
    if (prec == 0) nf_regular_kernel<K, double, A, B><<<a.ntiles, 128, 0, s>>>(a);    \
    else nf_regular_kernel<K, float, A, B><<<a.ntiles, 128, 0, s>>>(a);               \
    return;                                                                            \
  }
#define BEM_NF_SINGULAR_X(K, A, B)                                                     \
  if (kid == K) {                                                                      \
    if (prec == 0) run_singular<K, double, A, B>(a, s);                                \
    else run_singular<K, float, A, B>(a, s);                                           \
    return;                                                                            \
  }

template <int K, class S, int A, int B>
static void run_singular(const NFArgs& a, cudaStream_t s) {
  auto fn = a.gnodes ? nf_singular_kernel<K, S, A, B, true> : nf_singular_kernel<K, S, A, B, false>;
  int smem = a.ss_smem_bytes > 0 ? a.ss_smem_bytes : 0;
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  fn<<<a.sing_grid, 256, smem, s>>>(a);
}

}  // namespace bem
