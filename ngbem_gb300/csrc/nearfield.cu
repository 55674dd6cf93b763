// Near-field assembly (reference CalcBlockMatrix, src/ngbem.cpp:373-738): the P0 / P1 and
// edge-trace combinations of the kernel templates in nearfield_kernels.cuh and the dispatch.
#include "nearfield_kernels.cuh"

namespace bem {

// dispatch over the (kernel, trial trace, test trace) combinations the operators use
// ----------------------------------------------------------------------------------------
#define BEM_NF_COMBOS(X)                                                              \
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
  X(K_MAXWELL_DL, TR_NEDROT, TR_NED) X(K_MAXWELL_DL, TR_NEDROT, TR_RT0ID)

bool nf_combo_supported(int kid, int trt, int tet) {
#define X(K, A, B) if (kid == K && trt == A && tet == B) return true;
  BEM_NF_COMBOS(X)
  BEM_L2P_COMBOS(X)
  BEM_H1P_COMBOS(X)
  BEM_HDIV_COMBOS(X)
  BEM_HDIV34_COMBOS(X)
#undef X
  return false;
}

void launch_nf_regular(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s) {
  if (a.ntiles <= 0) return;
  if (l2p_trace(trt)) {
    if (trt != tet) return;
    if (trt == TR_L2P1) launch_nf_regular_l2p1(kid, prec, a, s);
    if (trt == TR_L2P2) launch_nf_regular_l2p2(kid, prec, a, s);
    if (trt == TR_L2P3) launch_nf_regular_l2p3(kid, prec, a, s);
    return;
  }
  if (h1p_trace(trt)) {
    if (h1p_order(trt) == 2) launch_nf_regular_h1p2(kid, prec, trt, tet, a, s);
    else launch_nf_regular_h1p3(kid, prec, trt, tet, a, s);
    return;
  }
  if (hdiv_trace(trt)) {
    if (hdiv_order(trt) <= 2) launch_nf_regular_hdiv(kid, prec, trt, tet, a, s);
    else launch_nf_regular_hdiv34(kid, prec, trt, tet, a, s);
    return;
  }
#define X(K, A, B)                                                                    \
  if (kid == K && trt == A && tet == B) {                                             \
    if (prec == 0) nf_regular_kernel<K, double, A, B><<<a.ntiles, 128, 0, s>>>(a);   \
    else nf_regular_kernel<K, float, A, B><<<a.ntiles, 128, 0, s>>>(a);              \
    return;                                                                           \
  }
  BEM_NF_COMBOS(X)
#undef X
}

void launch_nf_singular(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s) {
  if (l2p_trace(trt)) {
    if (trt != tet) return;
    if (trt == TR_L2P1) launch_nf_singular_l2p1(kid, prec, a, s);
    if (trt == TR_L2P2) launch_nf_singular_l2p2(kid, prec, a, s);
    if (trt == TR_L2P3) launch_nf_singular_l2p3(kid, prec, a, s);
    return;
  }
  if (h1p_trace(trt)) {
    if (h1p_order(trt) == 2) launch_nf_singular_h1p2(kid, prec, trt, tet, a, s);
    else launch_nf_singular_h1p3(kid, prec, trt, tet, a, s);
    return;
  }
  if (hdiv_trace(trt)) {
    if (hdiv_order(trt) <= 2) launch_nf_singular_hdiv(kid, prec, trt, tet, a, s);
    else launch_nf_singular_hdiv34(kid, prec, trt, tet, a, s);
    return;
  }
#define X(K, A, B)                                                          \
  if (kid == K && trt == A && tet == B) {                                   \
    if (prec == 0) run_singular<K, double, A, B>(a, s);                     \
    else run_singular<K, float, A, B>(a, s);                                \
    return;                                                                 \
  }
  BEM_NF_COMBOS(X)
#undef X
}

#define BEM_ALL_KERNELS(X)                                                                     \
  X(K_LAPLACE_SL) X(K_LAPLACE_DL) X(K_LAPLACE_HS) X(K_HELMHOLTZ_SL) X(K_HELMHOLTZ_DL)          \
  X(K_HELMHOLTZ_HS) X(K_HELMHOLTZ_CF) X(K_MAXWELL_SL) X(K_HELMHOLTZ_SL_DKAPPA) X(K_MAXWELL_DL)

int kernel_ncomp(int kid) {
#define X(K) if (kid == K) return Green<K>::NC;
  BEM_ALL_KERNELS(X)
#undef X
  return 1;
}
int kernel_nterms(int kid) {
#define X(K) if (kid == K) return Green<K>::NT;
  BEM_ALL_KERNELS(X)
#undef X
  return 1;
}
int kernel_term_comp(int kid, int t) {
#define X(K) if (kid == K) return Green<K>::kc(t);
  BEM_ALL_KERNELS(X)
#undef X
  return 0;
}
bool kernel_complex(int kid) { return kid >= K_HELMHOLTZ_SL; }

}  // namespace bem
