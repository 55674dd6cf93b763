// Near-field assembly of SurfaceL2 spaces, order 3, regular pairs (the kernel templates of
// nearfield_kernels.cuh), a translation unit of its own so that the instances compile in
// parallel.
#include "nearfield_kernels.cuh"

namespace bem {

void launch_nf_regular_l2p3(int kid, int prec, const NFArgs& a, cudaStream_t s) {
  BEM_L2P_KERNELS(BEM_NF_REGULAR_X, TR_L2P3)
}

}  // namespace bem
