// Near-field assembly of H1 of order 3, Sauter-Schwab pairs (the kernel templates of
// nearfield_kernels.cuh), a translation unit of its own so that the instances compile in
// parallel.
#include "nearfield_kernels.cuh"

namespace bem {

void launch_nf_singular_h1p3(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s) {
  BEM_H1P_KERNELS(BEM_NF_SINGULAR_X3, TR_H1P3, TR_H1P3ROT, TR_H1P3HELM, TR_L2P2)
}

}  // namespace bem
