// Far-field compression (reference CalcFarFieldBlock, src/ngbem.cpp:743-1163).
//
// aca_warp_kernel / aca_kernel: one warp per small admissible block (at most ACA_WARP_PTS row
//   plus column points; 8 blocks per CTA), one CTA per larger block; both launched over the
//   whole batch, each skipping the other's blocks, on two streams.  Partially
//   pivoted ACA on the point kernel matrix (rows = test quadrature points, cols = trial
//   quadrature points), one pass per kernel component, restating src/ngbem.cpp:902-1049:
//   start row 0, column pivot = argmax |v_j| over j != previous column pivot, symmetric
//   sqrt scaling, row pivot = argmax |u_i| over i != previous row pivot, Frobenius-norm
//   update with the complex inner products, stop when |u_k||v_k| < eps * ||sum u v^T||_F.
//   Pivot searches are warp-shuffle argmax reductions with the lowest-index tie rule of
//   the reference's strict '>' scan.  A block that reaches the rank cap reports status 1
//   and is assembled densely by the host (mirrors the reference's dense fallback).
// aca_project_kernel: weights the point factors by the quadrature weights and projects
//   them onto the dofs through the trace evaluators per KernelTerm (src/ngbem.cpp:1051-1160).
#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

#define ACA_T 256
#define ACA_NW (ACA_T / 32)
#define KCAP_MAX 256
// blocks with at most this many row + column points are compressed by one warp each
// (aca_warp_kernel, 8 blocks per CTA); larger ones by a whole CTA (aca_kernel)
#define ACA_WARP_PTS 1536

template <class V, int N>
__device__ __forceinline__ void block_sum_arr(V (&v)[N], V* sbuf) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) sbuf[w * N + k] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) {
    V s = sbuf[k];
    for (int ww = 1; ww < ACA_NW; ++ww) s += sbuf[ww * N + k];
    v[k] = s;
  }
  __syncthreads();
}

template <class R>
__device__ __forceinline__ void block_argmax(R& v, int& i, R* sv, int* si) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  warp_argmax(v, i);
  if (lane == 0) { sv[w] = v; si[w] = i; }
  __syncthreads();
  v = sv[0]; i = si[0];
  for (int ww = 1; ww < ACA_NW; ++ww) argmax_combine(v, i, sv[ww], si[ww]);
  __syncthreads();
}

template <class P>
struct PtData {
  P h[3], l[3], n[3];
};

template <class P, bool NEEDN>
__device__ __forceinline__ PtData<P> load_pt(const APt<P>* PT, const ElemRecP<P>* E, const PGeo<P>* PG,
                                             const int* patch, int p0, int idx, int nq) {
  const int le = idx / nq;
  const int q = idx - le * nq;
  const int e = patch[p0 + le];
  const APt<P> a = PT[(size_t)e * nq + q];
  PtData<P> r;
  r.h[0] = a.hx; r.h[1] = a.hy; r.h[2] = a.hz;
  r.l[0] = a.lx; r.l[1] = a.ly; r.l[2] = a.lz;
  if (NEEDN) {
    // curved elements: the normal at the point; flat: the element's
    const P* n = PG ? PG[(size_t)e * nq + q].n : E[e].n;
    r.n[0] = n[0]; r.n[1] = n[1]; r.n[2] = n[2];
  }
  else { r.n[0] = r.n[1] = r.n[2] = P(0); }
  return r;
}

template <class G, class P, class V>
__device__ __forceinline__ V kern_entry(const PtData<P>& x, const PtData<P>& y, P kappa, int comp) {
  const P dx = (x.h[0] - y.h[0]) + (x.l[0] - y.l[0]);
  const P dy = (x.h[1] - y.h[1]) + (x.l[1] - y.l[1]);
  const P dz = (x.h[2] - y.h[2]) + (x.l[2] - y.l[2]);
  V kv[G::NC];
  G::eval(dx, dy, dz, x.n, y.n, kappa, kv);
  return G::NC == 1 ? kv[0] : kv[comp];
}

template <int KID, class P>
__global__ void __launch_bounds__(ACA_T, sizeof(P) == 4 ? 4 : 2) aca_kernel(AcaArgs a) {
  using G = Green<KID>;
  using V = VT<G::CPLX, P>;
  constexpr int NC = G::NC;
  __shared__ V s_l[KCAP_MAX];
  __shared__ V s_red[ACA_NW * 16];
  __shared__ P s_redp[ACA_NW * 2];
  __shared__ P s_amv[ACA_NW];
  __shared__ int s_ami[ACA_NW];

  const FarDesc d = a.far[blockIdx.x];
  const int nq = a.nq;
  const int M = d.ni * nq, N = d.nj * nq;
  if (M + N <= ACA_WARP_PTS) return;  // a warp of aca_warp_kernel takes it
  const int p = min(M, N);
  const int kcap = min(d.kcap, KCAP_MAX);
  const APt<P>* PT = (const APt<P>*)a.apts;
  const ElemRecP<P>* E = (const ElemRecP<P>*)a.erecP;
  const PGeo<P>* PG = (const PGeo<P>*)a.pgeo;
  const P kappa = (P)a.kappa;
  const double eps = a.eps;
  int status = 0;

  for (int comp = 0; comp < NC; ++comp) {
    V* U = (V*)a.U + d.su + (size_t)comp * d.kcap * M;
    V* Vm = (V*)a.V + d.sv + (size_t)comp * d.kcap * N;
    int ik = 0, ikm1 = 0, jkm1 = N + 1;
    double norm2 = 0.0;
    int rank = p;
    bool stopped = false;
    const int kmax = min(p, kcap);
    for (int k = 0; k < kmax; ++k) {
      // ---- row ik: v_j = K(x_ik, y_j) - sum_l U(ik,l) V(l,j)
      for (int l = threadIdx.x; l < k; l += ACA_T) s_l[l] = U[(size_t)l * M + ik];
      __syncthreads();
      const PtData<P> x = load_pt<P, G::NEEDS_NX>(PT, E, PG, a.patch_test, d.pi0, ik, nq);
      P best = P(0);
      int bi = -1;
      V* Vk = Vm + (size_t)k * N;
      for (int j = threadIdx.x; j < N; j += ACA_T) {
        const PtData<P> y = load_pt<P, G::NEEDS_NY>(PT, E, PG, a.patch_trial, d.pj0, j, nq);
        V v = kern_entry<G, P, V>(x, y, kappa, comp);
        for (int l = 0; l < k; ++l) v -= s_l[l] * Vm[(size_t)l * N + j];
        Vk[j] = v;
        const P av = absv(v);
        if (j != jkm1 && av > best) { best = av; bi = j; }
      }
      block_argmax(best, bi, s_amv, s_ami);
      if (bi < 0) { rank = k; stopped = true; break; }
      const int jk = bi;
      const P vkj = best;
      const V piv = Vk[jk];
      const V sc = invv(piv) * sqrt_(vkj);
      P nv = P(0);
      for (int j = threadIdx.x; j < N; j += ACA_T) {
        V v = Vk[j] * sc;
        Vk[j] = v;
        nv += norm2v(v);
      }
      // ---- column jk: u_i = (K(x_i, y_jk) - sum_l U(i,l) V(l,jk)) / sqrt(vkj)
      for (int l = threadIdx.x; l < k; l += ACA_T) s_l[l] = Vm[(size_t)l * N + jk];
      __syncthreads();
      const PtData<P> y = load_pt<P, G::NEEDS_NY>(PT, E, PG, a.patch_trial, d.pj0, jk, nq);
      const P isq = P(1) / sqrt_(vkj);
      P nu = P(0), bu = P(0);
      int biu = -1;
      V* Uk = U + (size_t)k * M;
      for (int i = threadIdx.x; i < M; i += ACA_T) {
        const PtData<P> xi = load_pt<P, G::NEEDS_NX>(PT, E, PG, a.patch_test, d.pi0, i, nq);
        V u = kern_entry<G, P, V>(xi, y, kappa, comp);
        for (int l = 0; l < k; ++l) u -= U[(size_t)l * M + i] * s_l[l];
        u *= isq;
        Uk[i] = u;
        nu += norm2v(u);
        const P au = absv(u);
        if (i != ikm1 && au > bu) { bu = au; biu = i; }
      }
      block_argmax(bu, biu, s_amv, s_ami);
      P sums[2] = {nv, nu};
      block_sum_arr<P, 2>(sums, s_redp);
      const int iknew = biu >= 0 ? biu : ik;
      const double norm_k = sqrt((double)sums[0]) * sqrt((double)sums[1]);
      norm2 += norm_k * norm_k;
      // ---- cross terms 2 Re(conj(<V_k, V_l>) <U_k, U_l>) for l < k, 8 at a time
      for (int l0 = 0; l0 < k; l0 += 8) {
        V dd[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) dd[c] = vzero<V>();
        const int nl = min(8, k - l0);
        for (int j = threadIdx.x; j < N; j += ACA_T) {
          const V vk = Vk[j];
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nl) dd[c] += vk * conjv(Vm[(size_t)(l0 + c) * N + j]);
        }
        for (int i = threadIdx.x; i < M; i += ACA_T) {
          const V uk = Uk[i];
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nl) dd[8 + c] += uk * conjv(U[(size_t)(l0 + c) * M + i]);
        }
        block_sum_arr<V, 16>(dd, s_red);
        for (int c = 0; c < nl; ++c) norm2 += 2.0 * (double)realv(conjv(dd[c]) * dd[8 + c]);
      }
      ikm1 = iknew;
      jkm1 = jk;
      ik = iknew;
      // FP32 residuals carry rounding noise of about u32*sqrt(k)*||A||; an update at that
      // level carries no information, so the FP32 path also stops there (FP64: no change).
      const double noise = sizeof(P) == 4 ? 4.0 * 5.9604644775390625e-8 * sqrt((double)(k + 1)) : 0.0;
      if (norm_k < fmax(eps, noise) * sqrt(norm2)) { rank = k + 1; stopped = true; break; }
    }
    if (!stopped) {
      if (kmax < p) { status = 1; rank = kmax; }
      else rank = p;
    }
    if (threadIdx.x == 0) a.ranks[blockIdx.x * NC + comp] = rank;
    __syncthreads();
  }
  if (threadIdx.x == 0) a.status[blockIdx.x] = status;
}

// The same partially pivoted ACA as aca_kernel (identical steps, pivot and stopping rules),
// one warp per block: the reductions are warp shuffles and no CTA barrier is needed, so the
// many small admissible blocks (a few hundred points a side) run 64 to an SM instead of 4.
template <int KID, class P>
__global__ void __launch_bounds__(256, 4) aca_warp_kernel(AcaArgs a) {
  using G = Green<KID>;
  using V = VT<G::CPLX, P>;
  constexpr int NC = G::NC;
  __shared__ V s_lw[8][KCAP_MAX];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int b = blockIdx.x * 8 + wid;
  if (b >= a.nfar) return;
  const FarDesc d = a.far[b];
  const int nq = a.nq;
  const int M = d.ni * nq, N = d.nj * nq;
  if (M + N > ACA_WARP_PTS) return;  // aca_kernel takes it
  V* s_l = s_lw[wid];
  const int p = min(M, N);
  const int kcap = min(d.kcap, KCAP_MAX);
  const APt<P>* PT = (const APt<P>*)a.apts;
  const ElemRecP<P>* E = (const ElemRecP<P>*)a.erecP;
  const PGeo<P>* PG = (const PGeo<P>*)a.pgeo;
  const P kappa = (P)a.kappa;
  const double eps = a.eps;
  int status = 0;

  for (int comp = 0; comp < NC; ++comp) {
    V* U = (V*)a.U + d.su + (size_t)comp * d.kcap * M;
    V* Vm = (V*)a.V + d.sv + (size_t)comp * d.kcap * N;
    int ik = 0, ikm1 = 0, jkm1 = N + 1;
    double norm2 = 0.0;
    int rank = p;
    bool stopped = false;
    const int kmax = min(p, kcap);
    for (int k = 0; k < kmax; ++k) {
      // ---- row ik: v_j = K(x_ik, y_j) - sum_l U(ik,l) V(l,j)
      for (int l = lane; l < k; l += 32) s_l[l] = U[(size_t)l * M + ik];
      __syncwarp();
      const PtData<P> x = load_pt<P, G::NEEDS_NX>(PT, E, PG, a.patch_test, d.pi0, ik, nq);
      P best = P(0);
      int bi = -1;
      V* Vk = Vm + (size_t)k * N;
      for (int j = lane; j < N; j += 32) {
        const PtData<P> y = load_pt<P, G::NEEDS_NY>(PT, E, PG, a.patch_trial, d.pj0, j, nq);
        V v = kern_entry<G, P, V>(x, y, kappa, comp);
        for (int l = 0; l < k; ++l) v -= s_l[l] * Vm[(size_t)l * N + j];
        Vk[j] = v;
        const P av = absv(v);
        if (j != jkm1 && av > best) { best = av; bi = j; }
      }
      warp_argmax(best, bi);
      if (bi < 0) { rank = k; stopped = true; break; }
      const int jk = bi;
      const P vkj = best;
      __syncwarp();
      const V piv = Vk[jk];
      const V sc = invv(piv) * sqrt_(vkj);
      P nv = P(0);
      for (int j = lane; j < N; j += 32) {
        V v = Vk[j] * sc;
        Vk[j] = v;
        nv += norm2v(v);
      }
      // ---- column jk: u_i = (K(x_i, y_jk) - sum_l U(i,l) V(l,jk)) / sqrt(vkj)
      __syncwarp();
      for (int l = lane; l < k; l += 32) s_l[l] = Vm[(size_t)l * N + jk];
      __syncwarp();
      const PtData<P> y = load_pt<P, G::NEEDS_NY>(PT, E, PG, a.patch_trial, d.pj0, jk, nq);
      const P isq = P(1) / sqrt_(vkj);
      P nu = P(0), bu = P(0);
      int biu = -1;
      V* Uk = U + (size_t)k * M;
      for (int i = lane; i < M; i += 32) {
        const PtData<P> xi = load_pt<P, G::NEEDS_NX>(PT, E, PG, a.patch_test, d.pi0, i, nq);
        V u = kern_entry<G, P, V>(xi, y, kappa, comp);
        for (int l = 0; l < k; ++l) u -= U[(size_t)l * M + i] * s_l[l];
        u *= isq;
        Uk[i] = u;
        nu += norm2v(u);
        const P au = absv(u);
        if (i != ikm1 && au > bu) { bu = au; biu = i; }
      }
      warp_argmax(bu, biu);
      nv = warp_sum(nv);
      nu = warp_sum(nu);
      const int iknew = biu >= 0 ? biu : ik;
      const double norm_k = sqrt((double)nv) * sqrt((double)nu);
      norm2 += norm_k * norm_k;
      __syncwarp();
      // ---- cross terms 2 Re(conj(<V_k, V_l>) <U_k, U_l>) for l < k, 8 at a time
      for (int l0 = 0; l0 < k; l0 += 8) {
        V dd[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) dd[c] = vzero<V>();
        const int nl = min(8, k - l0);
        for (int j = lane; j < N; j += 32) {
          const V vk = Vk[j];
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nl) dd[c] += vk * conjv(Vm[(size_t)(l0 + c) * N + j]);
        }
        for (int i = lane; i < M; i += 32) {
          const V uk = Uk[i];
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nl) dd[8 + c] += uk * conjv(U[(size_t)(l0 + c) * M + i]);
        }
#pragma unroll
        for (int c = 0; c < 16; ++c) dd[c] = warp_sum(dd[c]);
        for (int c = 0; c < nl; ++c) norm2 += 2.0 * (double)realv(conjv(dd[c]) * dd[8 + c]);
      }
      ikm1 = iknew;
      jkm1 = jk;
      ik = iknew;
      const double noise = sizeof(P) == 4 ? 4.0 * 5.9604644775390625e-8 * sqrt((double)(k + 1)) : 0.0;
      if (norm_k < fmax(eps, noise) * sqrt(norm2)) { rank = k + 1; stopped = true; break; }
    }
    if (!stopped) {
      if (kmax < p) { status = 1; rank = kmax; }
      else rank = p;
    }
    if (lane == 0) a.ranks[b * NC + comp] = rank;
    __syncwarp();
  }
  if (lane == 0) a.status[b] = status;
}

__device__ __forceinline__ int i4c_(const int4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
template <class P> struct P2_ { P x, y; };

template <int KID, class P, int TRT, int TET>
__global__ void __launch_bounds__(256) aca_project_kernel(ProjArgs a) {
  using G = Green<KID>;
  using V = VT<G::CPLX, P>;
  constexpr int NDI = TraceInfo<TET>::ND, NDJ = TraceInfo<TRT>::ND;
  constexpr int NT = G::NT, NC = G::NC;
  const FarDesc d = a.far[blockIdx.x];
  const LRDesc L = a.lr[blockIdx.x];
  const int nq = a.nq;
  const int M = d.ni * nq, N = d.nj * nq;
  const ElemRecP<P>* E = (const ElemRecP<P>*)a.erecP;
  const PGeo<P>* PG = (const PGeo<P>*)a.pgeo;
  const QPt<P>* Q = (const QPt<P>*)a.qoff;
  const P2_<P>* RQ = (const P2_<P>*)a.rq;
  const P kappa = (P)a.kappa;
  V* U2 = (V*)L.u;
  V* V2 = (V*)L.v;
  int rk[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) rk[c] = a.ranks[blockIdx.x * NC + c];
  int off = 0;
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const int kc = G::kc(t);
    const int r = rk[kc];
    const P fac = term_fac<G, P>(t, kappa);
    const V* Us = (const V*)a.U + d.su + (size_t)kc * d.kcap * M;
    const V* Vs = (const V*)a.V + d.sv + (size_t)kc * d.kcap * N;
    for (int idx = threadIdx.x; idx < d.ni * r; idx += blockDim.x) {
      const int kk = idx / d.ni, ie = idx - kk * d.ni;
      const int e = a.patch_test[d.pi0 + ie];
      const ElemRecP<P>& Ee = E[e];
      P rot[3][3], o[3][3];
      for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) { rot[x][y] = Ee.rot[x][y]; o[x][y] = Ee.o[x][y]; }
      P nrm[3] = {Ee.n[0], Ee.n[1], Ee.n[2]};
      int sg[SignSlots<TET>::N];
      elem_signs<TET>(a.test.sign, e, sg);
      V acc[NDI];
#pragma unroll
      for (int x = 0; x < NDI; ++x) acc[x] = vzero<V>();
      for (int q = 0; q < nq; ++q) {
        const QPt<P> qo = Q[(size_t)e * nq + q];
        const P2_<P> rp = RQ[q];
        P xp[3][3];
        for (int x = 0; x < 3; ++x) { xp[x][0] = qo.x - o[x][0]; xp[x][1] = qo.y - o[x][1]; xp[x][2] = qo.z - o[x][2]; }
        P inv = Ee.invdetJ;
        if (PG) point_geo<P>(PG[(size_t)e * nq + q], nrm, rot, inv, xp);
        const V u = Us[(size_t)kk * M + ie * nq + q] * qo.w;
#pragma unroll
        for (int x = 0; x < NDI; ++x)
          acc[x] += u * trace_val<TET, P>(x, G::tec(t), rp.x, rp.y, xp, inv, rot, sg[x], a.test.dual != 0, nrm);
      }
      const int4 dn = a.test.dofs[e], dx = dof_aux<TET>(a.test.sign, e);
#pragma unroll
      for (int x = 0; x < NDI; ++x) {
        const int li = a.test.pinv[elem_dof<TET>(dn, dx, x)] - L.r0;
        if (li >= 0 && li < L.m) atomic_add(&U2[lr_u_index(L, li, off + kk)], acc[x] * fac);
      }
    }
    for (int idx = threadIdx.x; idx < d.nj * r; idx += blockDim.x) {
      const int kk = idx / d.nj, je = idx - kk * d.nj;
      const int e = a.patch_trial[d.pj0 + je];
      const ElemRecP<P>& Ee = E[e];
      P rot[3][3], o[3][3];
      for (int x = 0; x < 3; ++x)
        for (int y = 0; y < 3; ++y) { rot[x][y] = Ee.rot[x][y]; o[x][y] = Ee.o[x][y]; }
      P nrm[3] = {Ee.n[0], Ee.n[1], Ee.n[2]};
      int sg[SignSlots<TRT>::N];
      elem_signs<TRT>(a.trial.sign, e, sg);
      V acc[NDJ];
#pragma unroll
      for (int x = 0; x < NDJ; ++x) acc[x] = vzero<V>();
      for (int q = 0; q < nq; ++q) {
        const QPt<P> qo = Q[(size_t)e * nq + q];
        const P2_<P> rp = RQ[q];
        P xp[3][3];
        for (int x = 0; x < 3; ++x) { xp[x][0] = qo.x - o[x][0]; xp[x][1] = qo.y - o[x][1]; xp[x][2] = qo.z - o[x][2]; }
        P inv = Ee.invdetJ;
        if (PG) point_geo<P>(PG[(size_t)e * nq + q], nrm, rot, inv, xp);
        const V v = Vs[(size_t)kk * N + je * nq + q] * qo.w;
#pragma unroll
        for (int x = 0; x < NDJ; ++x)
          acc[x] += v * trace_val<TRT, P>(x, G::trc(t), rp.x, rp.y, xp, inv, rot, sg[x], a.trial.dual != 0, nrm);
      }
      const int4 dn = a.trial.dofs[e], dx = dof_aux<TRT>(a.trial.sign, e);
#pragma unroll
      for (int x = 0; x < NDJ; ++x) {
        const int lj = a.trial.pinv[elem_dof<TRT>(dn, dx, x)] - L.c0;
        if (lj >= 0 && lj < L.n) atomic_add(&V2[lr_v_index(L, off + kk, lj)], acc[x]);
      }
    }
    off += r;
  }
}

void launch_aca(int kid, int prec, const AcaArgs& a, cudaStream_t s) {
  if (a.nfar <= 0) return;
  // small blocks (a warp each) on the caller's stream, large blocks (a CTA each) beside them
  // on a second stream, joined before returning
  cudaStream_t s2 = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess) s2 = s;
  if (s2 != s) {
    cudaEventCreateWithFlags(&e0, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&e1, cudaEventDisableTiming);
    cudaEventRecord(e0, s);
    cudaStreamWaitEvent(s2, e0, 0);
  }
  auto join = [&]() {
    if (s2 == s) return;
    cudaEventRecord(e1, s2);
    cudaStreamWaitEvent(s, e1, 0);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s2);
  };
#define X(K)                                                                   \
  if (kid == K) {                                                              \
    if (prec == 0) {                                                           \
      aca_kernel<K, double><<<a.nfar, ACA_T, 0, s2>>>(a);                      \
      aca_warp_kernel<K, double><<<(a.nfar + 7) / 8, 256, 0, s>>>(a);          \
    } else {                                                                   \
      aca_kernel<K, float><<<a.nfar, ACA_T, 0, s2>>>(a);                       \
      aca_warp_kernel<K, float><<<(a.nfar + 7) / 8, 256, 0, s>>>(a);           \
    }                                                                          \
    join();                                                                    \
    return;                                                                    \
  }
  X(K_LAPLACE_SL) X(K_LAPLACE_DL) X(K_LAPLACE_HS) X(K_HELMHOLTZ_SL) X(K_HELMHOLTZ_DL)
  X(K_HELMHOLTZ_HS) X(K_HELMHOLTZ_CF) X(K_MAXWELL_SL) X(K_HELMHOLTZ_SL_DKAPPA)
  X(K_MAXWELL_DL)
#undef X
  join();
}

// SurfaceL2 of order 1..3 on both sides, for the kernels with identity traces
#define BEM_L2P_COMBOS(X)                                                                      \
  X(K_LAPLACE_SL, TR_L2P1, TR_L2P1) X(K_LAPLACE_SL, TR_L2P2, TR_L2P2) X(K_LAPLACE_SL, TR_L2P3, TR_L2P3) \
  X(K_LAPLACE_DL, TR_L2P1, TR_L2P1) X(K_LAPLACE_DL, TR_L2P2, TR_L2P2) X(K_LAPLACE_DL, TR_L2P3, TR_L2P3) \
  X(K_HELMHOLTZ_SL, TR_L2P1, TR_L2P1) X(K_HELMHOLTZ_SL, TR_L2P2, TR_L2P2)                        \
  X(K_HELMHOLTZ_SL, TR_L2P3, TR_L2P3) X(K_HELMHOLTZ_DL, TR_L2P1, TR_L2P1)                        \
  X(K_HELMHOLTZ_DL, TR_L2P2, TR_L2P2) X(K_HELMHOLTZ_DL, TR_L2P3, TR_L2P3)                        \
  X(K_HELMHOLTZ_CF, TR_L2P1, TR_L2P1) X(K_HELMHOLTZ_CF, TR_L2P2, TR_L2P2)                        \
  X(K_HELMHOLTZ_CF, TR_L2P3, TR_L2P3)
#define BEM_PJ_COMBOS(X)                                                              \
  X(K_LAPLACE_SL, TR_P0, TR_P0) X(K_LAPLACE_SL, TR_P1, TR_P1)                         \
  X(K_LAPLACE_SL, TR_P1, TR_P0) X(K_LAPLACE_SL, TR_P0, TR_P1)                         \
  X(K_LAPLACE_DL, TR_P0, TR_P0) X(K_LAPLACE_DL, TR_P1, TR_P1)                         \
  X(K_LAPLACE_DL, TR_P1, TR_P0) X(K_LAPLACE_DL, TR_P0, TR_P1)                         \
  X(K_LAPLACE_HS, TR_ROT, TR_ROT)                                                     \
  X(K_HELMHOLTZ_SL, TR_P0, TR_P0) X(K_HELMHOLTZ_SL, TR_P1, TR_P1)                     \
  X(K_HELMHOLTZ_SL, TR_P1, TR_P0) X(K_HELMHOLTZ_SL, TR_P0, TR_P1)                     \
  X(K_HELMHOLTZ_SL_DKAPPA, TR_P0, TR_P0) X(K_HELMHOLTZ_SL_DKAPPA, TR_P1, TR_P1)       \
  X(K_HELMHOLTZ_SL_DKAPPA, TR_P1, TR_P0) X(K_HELMHOLTZ_SL_DKAPPA, TR_P0, TR_P1)       \
  X(K_HELMHOLTZ_DL, TR_P0, TR_P0) X(K_HELMHOLTZ_DL, TR_P1, TR_P1)                     \
  X(K_HELMHOLTZ_DL, TR_P1, TR_P0) X(K_HELMHOLTZ_DL, TR_P0, TR_P1)                     \
  X(K_HELMHOLTZ_CF, TR_P0, TR_P0) X(K_HELMHOLTZ_CF, TR_P1, TR_P1)                     \
  X(K_HELMHOLTZ_CF, TR_P1, TR_P0) X(K_HELMHOLTZ_CF, TR_P0, TR_P1)                     \
  X(K_HELMHOLTZ_HS, TR_HELM, TR_HELM)                                                 \
  X(K_MAXWELL_SL, TR_MAX, TR_MAX) X(K_MAXWELL_SL, TR_NEDMAX, TR_NEDMAX)                \
  X(K_MAXWELL_DL, TR_NEDROT, TR_NED) X(K_MAXWELL_DL, TR_NEDROT, TR_RT0ID)  \
  BEM_L2P_COMBOS(X) BEM_H1P_COMBOS(X) BEM_HDIV_COMBOS(X) BEM_HDIV34_COMBOS(X)

void launch_projection(int kid, int prec, int trt, int tet, const ProjArgs& a, cudaStream_t s) {
  if (a.nfar <= 0) return;
#define X(K, A, B)                                                                    \
  if (kid == K && trt == A && tet == B) {                                             \
    if (prec == 0) aca_project_kernel<K, double, A, B><<<a.nfar, 256, 0, s>>>(a);    \
    else aca_project_kernel<K, float, A, B><<<a.nfar, 256, 0, s>>>(a);               \
    return;                                                                           \
  }
  BEM_PJ_COMBOS(X)
#undef X
}

}  // namespace bem
