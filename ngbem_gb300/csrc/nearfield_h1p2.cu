// Near-field assembly of H1 of order 2 (the kernel templates of nearfield_kernels.cuh, the
// combinations of BEM_H1P_COMBOS), a translation unit of its own so that the instances
// compile in parallel.
#include "nearfield_kernels.cuh"

namespace bem {

void launch_nf_regular_h1p2(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s) {
  BEM_H1P_KERNELS(BEM_NF_REGULAR_X3, TR_H1P2, TR_H1P2ROT, TR_H1P2HELM, TR_L2P1)
}

void launch_nf_singular_h1p2(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s) {
  BEM_H1P_KERNELS(BEM_NF_SINGULAR_X3, TR_H1P2, TR_H1P2ROT, TR_H1P2HELM, TR_L2P1)
}

}  // namespace bem
