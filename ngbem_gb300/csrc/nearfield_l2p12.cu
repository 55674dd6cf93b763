// Near-field assembly of SurfaceL2 spaces, orders 1 and 2 (the kernel templates of
// nearfield_kernels.cuh), a translation unit of its own so that the instances compile in
// parallel.
#include "nearfield_kernels.cuh"

namespace bem {

void launch_nf_regular_l2p1(int kid, int prec, const NFArgs& a, cudaStream_t s) {
  BEM_L2P_KERNELS(BEM_NF_REGULAR_X, TR_L2P1)
}

void launch_nf_singular_l2p1(int kid, int prec, const NFArgs& a, cudaStream_t s) {
  BEM_L2P_KERNELS(BEM_NF_SINGULAR_X, TR_L2P1)
}

void launch_nf_regular_l2p2(int kid, int prec, const NFArgs& a, cudaStream_t s) {
  BEM_L2P_KERNELS(BEM_NF_REGULAR_X, TR_L2P2)
}

void launch_nf_singular_l2p2(int kid, int prec, const NFArgs& a, cudaStream_t s) {
  BEM_L2P_KERNELS(BEM_NF_SINGULAR_X, TR_L2P2)
}

}  // namespace bem
