// Potential evaluation: the field of a density at arbitrary points (reference
// GenericIntegralOperator::GetPotential / PotentialCF::T_Evaluate, src/ngbem.cpp:1166-1301).
//
// The reference evaluates, for every point x, a loop over all trial elements, the regular
// rule's points y on each, the trial evaluator applied to the element vector, and the kernel
// terms: u(x)_tec += w_y K_kc(x, y, n_x, n_y) (evaluator . density)_trc (term factors are not
// applied there).  Here that sum is an all-pairs reduction:
//   pot_sources_kernel  one thread per (element, rule point): the point, its normal and the
//                       trial evaluator values weighted by w_y, once per density;
//   pot_eval_kernel     one thread per evaluation point, tiles of sources staged in shared
//                       memory, FP64 like the reference.
#include <algorithm>

#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

#define POT_TILE 128
#define POT_THREADS 256

// sources: y, n_y and the DIM weighted trial-evaluator values of every rule point
template <int TRT, class V>
__global__ void pot_sources_kernel(PotArgs a) {
  constexpr int ND = TraceInfo<TRT>::ND, DIM = TraceInfo<TRT>::DIM;
  const ElemRecP<double>* E = (const ElemRecP<double>*)a.erec;
  const QPt<double>* Q = (const QPt<double>*)a.qoff;
  const double* RQ = a.rq;
  const V* dens = (const V*)a.density;
  const long long total = (long long)a.nt * a.nq;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / a.nq), q = (int)(t - (long long)k * a.nq);
    const int e = a.elems ? a.elems[k] : k;
    const ElemRecP<double>& Ee = E[e];
    const QPt<double> qo = Q[(size_t)e * a.nq + q];
    double rot[3][3], xp[3][3];
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y) {
        rot[x][y] = Ee.rot[x][y];
        xp[x][y] = (y == 0 ? qo.x : (y == 1 ? qo.y : qo.z)) - Ee.o[x][y];
      }
    double nrm[3] = {Ee.n[0], Ee.n[1], Ee.n[2]};
    double inv = Ee.invdetJ;
    // curved elements: the normal, rotated gradients and Piola data at the rule point
    if (a.pgeo) point_geo<double>(((const PGeo<double>*)a.pgeo)[(size_t)e * a.nq + q], nrm, rot, inv, xp);
    int sg[SignSlots<TRT>::N];
    elem_signs<TRT>(a.trial.sign, e, sg);
    const int4 dn = a.trial.dofs[e], dx = dof_aux<TRT>(a.trial.sign, e);
    V val[DIM];
#pragma unroll
    for (int c = 0; c < DIM; ++c) val[c] = vzero<V>();
#pragma unroll
    for (int x = 0; x < ND; ++x) {
      const V dv = dens[elem_dof<TRT>(dn, dx, x)];
#pragma unroll
      for (int c = 0; c < DIM; ++c)
        val[c] += dv * trace_val<TRT, double>(x, c, RQ[2 * q], RQ[2 * q + 1], xp, inv, rot, sg[x],
                                               a.trial.dual != 0, nrm);
    }
    double* py = a.src_pos + 6 * t;
    py[0] = Ee.chi[0] + Ee.clo[0] + qo.x;
    py[1] = Ee.chi[1] + Ee.clo[1] + qo.y;
    py[2] = Ee.chi[2] + Ee.clo[2] + qo.z;
    py[3] = nrm[0];
    py[4] = nrm[1];
    py[5] = nrm[2];
    V* sv = (V*)a.src_val + (size_t)DIM * t;
#pragma unroll
    for (int c = 0; c < DIM; ++c) sv[c] = val[c] * qo.w;
  }
}

// u(x_p)_tec = sum over sources and kernel terms of K_kc(x_p - y, n_x, n_y) s_trc
template <int KID, int TRT, class V>
__global__ void __launch_bounds__(POT_THREADS) pot_eval_kernel(PotArgs a) {
  using G = Green<KID>;
  constexpr int DIM = TraceInfo<TRT>::DIM, NC = G::NC, NT = G::NT;
  __shared__ double sp[POT_TILE][6];
  __shared__ V sv[POT_TILE][DIM];
  const int p = blockIdx.x * POT_THREADS + threadIdx.x;
  const bool live = p < a.npts;
  double x[3] = {0.0, 0.0, 0.0}, nx[3] = {0.0, 0.0, 0.0};
  if (live) {
    for (int k = 0; k < 3; ++k) x[k] = a.pts[3 * (size_t)p + k];
    if (a.normals)
      for (int k = 0; k < 3; ++k) nx[k] = a.normals[3 * (size_t)p + k];
  }
  V acc[DIM];
#pragma unroll
  for (int c = 0; c < DIM; ++c) acc[c] = vzero<V>();
  const long long nsrc = (long long)a.nt * a.nq;
  for (long long s0 = 0; s0 < nsrc; s0 += POT_TILE) {
    const int ns = (int)min((long long)POT_TILE, nsrc - s0);
    __syncthreads();
    for (int i = threadIdx.x; i < ns * 6; i += POT_THREADS) sp[i / 6][i % 6] = a.src_pos[6 * s0 + i];
    for (int i = threadIdx.x; i < ns * DIM; i += POT_THREADS)
      sv[i / DIM][i % DIM] = ((const V*)a.src_val)[DIM * s0 + i];
    __syncthreads();
    if (!live) continue;
    for (int j = 0; j < ns; ++j) {
      V kv[NC];
      G::eval(x[0] - sp[j][0], x[1] - sp[j][1], x[2] - sp[j][2], nx, &sp[j][3], a.kappa, kv);
#pragma unroll
      for (int t = 0; t < NT; ++t) acc[G::tec(t)] += kv[G::kc(t)] * sv[j][G::trc(t)];
    }
  }
  if (live) {
    V* out = (V*)a.out + (size_t)DIM * p;
#pragma unroll
    for (int c = 0; c < DIM; ++c) out[c] = acc[c];
  }
}

// (kernel, trial trace) pairs of the operators: the scalar kernels with P0 / P1 (SurfaceL2 of
// order 1..3, H1 of order 2, 3) identity traces, the hypersingular kernels with their curl
// traces, the Maxwell single layer with RT0 (and HDivSurface of order 1, 2) and in its curl
// form with HCurl (of order 0-2), and the Maxwell
// double layer with the rotated trace of HCurl.  The sum leaves out the kernel terms' factors,
// as the reference's PotentialCF does (src/ngbem.cpp:1228-1232); for the double layer's six
// cross-product terms (factors +-1) that is the reference's field, not the signed one.
#define BEM_POT_COMBOS(X)                                                                        \
  X(K_LAPLACE_SL, TR_P0, double) X(K_LAPLACE_SL, TR_P1, double) X(K_LAPLACE_DL, TR_P0, double)  \
  X(K_LAPLACE_DL, TR_P1, double) X(K_LAPLACE_HS, TR_ROT, double)                                 \
  X(K_HELMHOLTZ_SL, TR_P0, cpx<double>) X(K_HELMHOLTZ_SL, TR_P1, cpx<double>)                   \
  X(K_HELMHOLTZ_DL, TR_P0, cpx<double>) X(K_HELMHOLTZ_DL, TR_P1, cpx<double>)                   \
  X(K_HELMHOLTZ_CF, TR_P0, cpx<double>) X(K_HELMHOLTZ_CF, TR_P1, cpx<double>)                   \
  X(K_HELMHOLTZ_HS, TR_HELM, cpx<double>) X(K_MAXWELL_SL, TR_MAX, cpx<double>)                  \
  X(K_MAXWELL_SL, TR_NEDMAX, cpx<double>)                                                        \
  X(K_HELMHOLTZ_SL_DKAPPA, TR_P0, cpx<double>) X(K_HELMHOLTZ_SL_DKAPPA, TR_P1, cpx<double>)      \
  X(K_LAPLACE_SL, TR_L2P1, double) X(K_LAPLACE_SL, TR_L2P2, double) X(K_LAPLACE_SL, TR_L2P3, double) \
  X(K_LAPLACE_DL, TR_L2P1, double) X(K_LAPLACE_DL, TR_L2P2, double) X(K_LAPLACE_DL, TR_L2P3, double) \
  X(K_HELMHOLTZ_SL, TR_L2P1, cpx<double>) X(K_HELMHOLTZ_SL, TR_L2P2, cpx<double>)               \
  X(K_HELMHOLTZ_SL, TR_L2P3, cpx<double>)                                                       \
  X(K_LAPLACE_SL, TR_H1P2, double) X(K_LAPLACE_SL, TR_H1P3, double) X(K_LAPLACE_DL, TR_H1P2, double) \
  X(K_LAPLACE_DL, TR_H1P3, double) X(K_HELMHOLTZ_SL, TR_H1P2, cpx<double>)                          \
  X(K_HELMHOLTZ_SL, TR_H1P3, cpx<double>) X(K_MAXWELL_DL, TR_NEDROT, cpx<double>)                \
  X(K_HELMHOLTZ_DL, TR_L2P1, cpx<double>) X(K_HELMHOLTZ_DL, TR_L2P2, cpx<double>)               \
  X(K_HELMHOLTZ_DL, TR_L2P3, cpx<double>) X(K_HELMHOLTZ_DL, TR_H1P2, cpx<double>)               \
  X(K_HELMHOLTZ_DL, TR_H1P3, cpx<double>) X(K_HELMHOLTZ_CF, TR_L2P1, cpx<double>)               \
  X(K_HELMHOLTZ_CF, TR_L2P2, cpx<double>) X(K_HELMHOLTZ_CF, TR_L2P3, cpx<double>)               \
  X(K_HELMHOLTZ_CF, TR_H1P2, cpx<double>) X(K_HELMHOLTZ_CF, TR_H1P3, cpx<double>)               \
  X(K_MAXWELL_SL, TR_HDIV1MAX, cpx<double>) X(K_MAXWELL_SL, TR_HDIV2MAX, cpx<double>)               \
  X(K_MAXWELL_SL, TR_HCURL1MAX, cpx<double>) X(K_MAXWELL_SL, TR_HCURL2MAX, cpx<double>)             \
  X(K_MAXWELL_DL, TR_HCURL1ROT, cpx<double>) X(K_MAXWELL_DL, TR_HCURL2ROT, cpx<double>)             \
  X(K_MAXWELL_SL, TR_HDIV3MAX, cpx<double>) X(K_MAXWELL_SL, TR_HDIV4MAX, cpx<double>)               \
  X(K_MAXWELL_DL, TR_HCURL3ROT, cpx<double>)

int potential_dim(int kid, int trt) {
#define X(K, T, V) \
  if (kid == K && trt == T) return TraceInfo<T>::DIM;
  BEM_POT_COMBOS(X)
#undef X
  return 0;
}

int launch_potential(int kid, int trt, const PotArgs& a, cudaStream_t s) {
  const long long nsrc = (long long)a.nt * a.nq;
  const int gs = (int)std::max<long long>(1, std::min<long long>((nsrc + 255) / 256, 152 * 16));
  const int ge = (a.npts + POT_THREADS - 1) / POT_THREADS;
#define X(K, T, V)                                                            \
  if (kid == K && trt == T) {                                                 \
    pot_sources_kernel<T, V><<<gs, 256, 0, s>>>(a);                           \
    if (ge > 0) pot_eval_kernel<K, T, V><<<ge, POT_THREADS, 0, s>>>(a);       \
    return 1;                                                                 \
  }
  BEM_POT_COMBOS(X)
#undef X
  return 0;
}

}  // namespace bem
