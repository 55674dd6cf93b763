// Near-field assembly of HDivSurface and HCurl of order 3, 4, Sauter-Schwab pairs (the
// combinations of BEM_HDIV34_COMBOS), a translation unit of its own so that the instances
// compile in parallel.
#include "nearfield_kernels.cuh"

namespace bem {

void launch_nf_singular_hdiv34(int kid, int prec, int trt, int tet, const NFArgs& a, cudaStream_t s) {
  BEM_HDIV34_COMBOS(BEM_NF_SINGULAR_X3)
}

}  // namespace bem
