// H-matrix application (reference BEMBlock::MultAdd / LowRankMatrix::Mult / HMatrix::MultAdd,
// src/hmat.cpp:473-515, 527-565, 647-666).
//
// Vectors are permuted once into cluster order, where every block is a contiguous row range
// [r0, r0+m) x column range [c0, c0+n): the gather/scatter of the reference becomes a slice.
// Stage 1 computes t = V2 x for every low-rank block (column chunks, atomics into t);
// the apply pass computes y += D x (dense) and y += U2 t (low rank) over row chunks,
// accumulating into an FP64 (complex128) permuted vector with atomics; a final kernel
// un-permutes and applies alpha/beta.  Storage precision S is fp64 or fp32; products are
// formed in S and block partial sums are added in FP64.
#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

template <class A> struct acc_of;
template <> struct acc_of<float> { using type = double; };
template <> struct acc_of<double> { using type = double; };
template <> struct acc_of<cpx<float>> { using type = cpx<double>; };
template <> struct acc_of<cpx<double>> { using type = cpx<double>; };

__device__ __forceinline__ double to_acc(float v) { return (double)v; }
__device__ __forceinline__ double to_acc(double v) { return v; }
__device__ __forceinline__ cpx<double> to_acc(cpx<float> v) { return {(double)v.x, (double)v.y}; }
__device__ __forceinline__ cpx<double> to_acc(cpx<double> v) { return v; }

// ---------------------------------------------------------------------------------------
template <class VS>
__global__ void permute_in_kernel(const int* perm, int n, int nrhs, int ld, const void* xv, VS* xp) {
  using VD = typename acc_of<VS>::type;
  const VD* x = (const VD*)xv;
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / nrhs), r = (int)(t - (long long)k * nrhs);
    VS v;
    cvt(v, x[(size_t)r * ld + perm[k]]);
    xp[t] = v;
  }
}

template <class VD>
__global__ void permute_out_kernel(const int* perm, int n, int nrhs, int ld, VD alpha, VD beta, int use_beta,
                                   const VD* yp, VD* y) {
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / nrhs), r = (int)(t - (long long)k * nrhs);
    VD* dst = y + (size_t)r * ld + perm[k];
    VD v = alpha * yp[t];
    if (use_beta) v += beta * (*dst);
    *dst = v;
  }
}

__device__ __forceinline__ double scal_mul(double a, double b) { return a * b; }

// ---------------------------------------------------------------------------------------
// stage 1: t = V2 x (non-transposed) over column chunks; transposed: t = U2^T x over row chunks
template <class VS>
__global__ void __launch_bounds__(256) mv_stage1_kernel(MVArgs a, int trans) {
  const MVItem it = a.items[blockIdx.x];
  const LRDesc L = a.lr[it.idx];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const VS* xp = (const VS*)a.xp;
  VS* t = (VS*)a.t;
  const int nrhs = a.nrhs;
  if (!trans) {
    const VS* V2 = (const VS*)L.v;
    for (int r = w; r < L.R; r += nw) {
      const VS* row = V2 + (size_t)r * L.n;
      if (nrhs == 1) {
        VS s = vzero<VS>();
        for (int j = it.start + lane; j < it.start + it.count; j += 32) s += row[j] * xp[L.c0 + j];
        s = warp_sum(s);
        if (lane == 0) atomic_add(&t[L.toff + r], s);
      } else {
        for (int g = 0; g < nrhs; g += 32) {
          const int rh = g + lane;
          if (rh >= nrhs) continue;
          VS s = vzero<VS>();
          for (int j = it.start; j < it.start + it.count; ++j) s += row[j] * xp[(size_t)(L.c0 + j) * nrhs + rh];
          atomic_add(&t[(size_t)(L.toff + r) * nrhs + rh], s);
        }
      }
    }
  } else {
    const VS* U2 = (const VS*)L.u;
    for (int r = w; r < L.R; r += nw) {
      const VS* col = U2 + (size_t)r * L.m;
      if (nrhs == 1) {
        VS s = vzero<VS>();
        for (int i = it.start + lane; i < it.start + it.count; i += 32) s += col[i] * xp[L.r0 + i];
        s = warp_sum(s);
        if (lane == 0) atomic_add(&t[L.toff + r], s);
      } else {
        for (int g = 0; g < nrhs; g += 32) {
          const int rh = g + lane;
          if (rh >= nrhs) continue;
          VS s = vzero<VS>();
          for (int i = it.start; i < it.start + it.count; ++i) s += col[i] * xp[(size_t)(L.r0 + i) * nrhs + rh];
          atomic_add(&t[(size_t)(L.toff + r) * nrhs + rh], s);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// apply: y += D x (dense) and y += U2 t (low rank), row chunks; transposed over column chunks
template <class VS>
__global__ void __launch_bounds__(256) mv_apply_kernel(MVArgs a, int trans) {
  using VD = typename acc_of<VS>::type;
  const MVItem it = a.items[blockIdx.x];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const VS* xp = (const VS*)a.xp;
  const VS* t = (const VS*)a.t;
  VD* yp = (VD*)a.yp;
  const int nrhs = a.nrhs;
  if (it.kind == 0) {
    const MVDense D = a.dense[it.idx];
    const VS* M = (const VS*)D.ptr;
    if (!trans) {
      for (int i = it.start + w; i < it.start + it.count; i += nw) {
        const VS* row = M + (size_t)i * D.n;
        if (nrhs == 1) {
          VS s = vzero<VS>();
          for (int j = lane; j < D.n; j += 32) s += row[j] * xp[D.c0 + j];
          s = warp_sum(s);
          if (lane == 0) atomic_add(&yp[D.r0 + i], to_acc(s));
        } else {
          for (int g = 0; g < nrhs; g += 32) {
            const int rh = g + lane;
            if (rh >= nrhs) continue;
            VS s = vzero<VS>();
            for (int j = 0; j < D.n; ++j) s += row[j] * xp[(size_t)(D.c0 + j) * nrhs + rh];
            atomic_add(&yp[(size_t)(D.r0 + i) * nrhs + rh], to_acc(s));
          }
        }
      }
    } else {
      // columns [start, start+count) of the block; thread per (column, rhs)
      for (int jj = threadIdx.x; jj < it.count * nrhs; jj += blockDim.x) {
        const int j = it.start + jj / nrhs, rh = jj - (jj / nrhs) * nrhs;
        VS s = vzero<VS>();
        for (int i = 0; i < D.m; ++i) s += M[(size_t)i * D.n + j] * xp[(size_t)(D.r0 + i) * nrhs + rh];
        atomic_add(&yp[(size_t)(D.c0 + j) * nrhs + rh], to_acc(s));
      }
    }
  } else {
    const LRDesc L = a.lr[it.idx];
    if (!trans) {
      const VS* U2 = (const VS*)L.u;
      for (int ii = threadIdx.x; ii < it.count * nrhs; ii += blockDim.x) {
        const int i = it.start + ii / nrhs, rh = ii - (ii / nrhs) * nrhs;
        VS s = vzero<VS>();
        for (int r = 0; r < L.R; ++r) s += U2[(size_t)r * L.m + i] * t[(size_t)(L.toff + r) * nrhs + rh];
        atomic_add(&yp[(size_t)(L.r0 + i) * nrhs + rh], to_acc(s));
      }
    } else {
      const VS* V2 = (const VS*)L.v;
      for (int jj = threadIdx.x; jj < it.count * nrhs; jj += blockDim.x) {
        const int j = it.start + jj / nrhs, rh = jj - (jj / nrhs) * nrhs;
        VS s = vzero<VS>();
        for (int r = 0; r < L.R; ++r) s += V2[(size_t)r * L.n + j] * t[(size_t)(L.toff + r) * nrhs + rh];
        atomic_add(&yp[(size_t)(L.c0 + j) * nrhs + rh], to_acc(s));
      }
    }
  }
  (void)lane;
}

template <class VS>
static void stage1_t(const MVArgs& a, bool trans, cudaStream_t s) {
  if (a.nitems > 0) mv_stage1_kernel<VS><<<a.nitems, 256, 0, s>>>(a, trans ? 1 : 0);
}
template <class VS>
static void apply_t(const MVArgs& a, bool trans, cudaStream_t s) {
  if (a.nitems > 0) mv_apply_kernel<VS><<<a.nitems, 256, 0, s>>>(a, trans ? 1 : 0);
}

void launch_mv_stage1(int prec, bool cplx, bool trans, const MVArgs& a, cudaStream_t s) {
  if (prec == 0) { if (cplx) stage1_t<cpx<double>>(a, trans, s); else stage1_t<double>(a, trans, s); }
  else { if (cplx) stage1_t<cpx<float>>(a, trans, s); else stage1_t<float>(a, trans, s); }
}
void launch_mv_apply(int prec, bool cplx, bool trans, const MVArgs& a, cudaStream_t s) {
  if (prec == 0) { if (cplx) apply_t<cpx<double>>(a, trans, s); else apply_t<double>(a, trans, s); }
  else { if (cplx) apply_t<cpx<float>>(a, trans, s); else apply_t<float>(a, trans, s); }
}

static int grid_for(long long total) {
  long long g = (total + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

void launch_permute_in(int prec, bool cplx, const int* perm, int n, int nrhs, int ld, const void* x, void* xp,
                       cudaStream_t s) {
  int g = grid_for((long long)n * nrhs);
  if (prec == 0) {
    if (cplx) permute_in_kernel<cpx<double>><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, (cpx<double>*)xp);
    else permute_in_kernel<double><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, (double*)xp);
  } else {
    if (cplx) permute_in_kernel<cpx<float>><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, (cpx<float>*)xp);
    else permute_in_kernel<float><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, (float*)xp);
  }
}

void launch_permute_out(bool cplx, const int* perm, int n, int nrhs, int ld, const double* alpha, const double* beta,
                        const void* yp, void* y, cudaStream_t s) {
  int g = grid_for((long long)n * nrhs);
  int use_beta = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
  if (cplx)
    permute_out_kernel<cpx<double>><<<g, 256, 0, s>>>(perm, n, nrhs, ld, mkc(alpha[0], alpha[1]), mkc(beta[0], beta[1]),
                                                      use_beta, (const cpx<double>*)yp, (cpx<double>*)y);
  else
    permute_out_kernel<double><<<g, 256, 0, s>>>(perm, n, nrhs, ld, alpha[0], beta[0], use_beta, (const double*)yp,
                                                 (double*)y);
}

// ---------------------------------------------------------------------------------------
// CSR SpMV (mass matrices).  trans: y = alpha A^T x + beta y via atomics into y after scaling.
template <class VD>
__global__ void spmv_kernel(int nrows, const int* rowptr, const int* col, const double* val, VD alpha, VD beta,
                            int use_beta, const VD* x, VD* y, int nrhs, int ldx, int ldy) {
  const long long total = (long long)nrows * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nrows), r = (int)(t / nrows);
    VD s = vzero<VD>();
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += x[(size_t)r * ldx + col[k]] * val[k];
    VD* dst = y + (size_t)r * ldy + i;
    VD v = alpha * s;
    if (use_beta) v += beta * (*dst);
    *dst = v;
  }
}
template <class VD>
__global__ void scale_kernel(VD* y, long long n, VD beta, int zero) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    y[t] = zero ? vzero<VD>() : beta * y[t];
}
template <class VD>
__global__ void spmv_t_kernel(int nrows, const int* rowptr, const int* col, const double* val, VD alpha, const VD* x,
                              VD* y, int nrhs, int ldx, int ldy) {
  const long long total = (long long)nrows * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nrows), r = (int)(t / nrows);
    const VD xi = alpha * x[(size_t)r * ldx + i];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) atomic_add(&y[(size_t)r * ldy + col[k]], xi * val[k]);
  }
}

void launch_spmv(bool cplx, bool trans, int nrows, int ncols, const int* rowptr, const int* col, const double* val,
                 const double* alpha, const double* beta, const void* x, void* y, int nrhs, cudaStream_t s) {
  int use_beta = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
  if (!trans) {
    int g = grid_for((long long)nrows * nrhs);
    if (cplx)
      spmv_kernel<cpx<double>><<<g, 256, 0, s>>>(nrows, rowptr, col, val, mkc(alpha[0], alpha[1]), mkc(beta[0], beta[1]),
                                                 use_beta, (const cpx<double>*)x, (cpx<double>*)y, nrhs, ncols, nrows);
    else
      spmv_kernel<double><<<g, 256, 0, s>>>(nrows, rowptr, col, val, alpha[0], beta[0], use_beta, (const double*)x,
                                            (double*)y, nrhs, ncols, nrows);
  } else {
    long long ny = (long long)ncols * nrhs;
    int g1 = grid_for(ny), g2 = grid_for((long long)nrows * nrhs);
    if (cplx) {
      scale_kernel<cpx<double>><<<g1, 256, 0, s>>>((cpx<double>*)y, ny, mkc(beta[0], beta[1]), use_beta ? 0 : 1);
      spmv_t_kernel<cpx<double>><<<g2, 256, 0, s>>>(nrows, rowptr, col, val, mkc(alpha[0], alpha[1]),
                                                    (const cpx<double>*)x, (cpx<double>*)y, nrhs, nrows, ncols);
    } else {
      scale_kernel<double><<<g1, 256, 0, s>>>((double*)y, ny, beta[0], use_beta ? 0 : 1);
      spmv_t_kernel<double><<<g2, 256, 0, s>>>(nrows, rowptr, col, val, alpha[0], (const double*)x, (double*)y, nrhs,
                                               nrows, ncols);
    }
  }
}

// ---------------------------------------------------------------------------------------
// GMRES helpers (fp64 / complex128): h = Q^H w, w -= Q h, ||w||, q = w / ||w||, x += Q y
template <class VD>
__global__ void __launch_bounds__(256) gemv_ct_kernel(int n, const VD* Q, const VD* w, VD* h) {
  __shared__ VD sb[8];
  const int c = blockIdx.x;
  const VD* q = Q + (size_t)c * n;
  VD s = vzero<VD>();
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += conjv(q[i]) * w[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    VD t = sb[0];
    for (int k = 1; k < 8; ++k) t += sb[k];
    h[c] = t;
  }
}
template <class VD>
__global__ void gemv_sub_kernel(int n, int k, const VD* Q, const VD* h, VD* w, int sign) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    VD s = vzero<VD>();
    for (int c = 0; c < k; ++c) s += Q[(size_t)c * n + i] * h[c];
    if (sign < 0) w[i] -= s;
    else w[i] += s;
  }
}
template <class VD>
__global__ void __launch_bounds__(256) nrm2_kernel(int n, const VD* w, double* out) {
  __shared__ double sb[8];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += norm2v(w[i]);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < 8; ++k) t += sb[k];
    *out = sqrt(t);
  }
}
template <class VD>
__global__ void scale_copy_kernel(int n, const VD* w, double inv, VD* q) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) q[i] = w[i] * inv;
}
template <class VD>
__global__ void residual_kernel(int n, const VD* b, VD* r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r[i] = b[i] - r[i];
}

void launch_gemv_ct(bool cplx, int n, int k, const void* Q, const void* w, void* h, cudaStream_t s) {
  if (k <= 0) return;
  if (cplx) gemv_ct_kernel<cpx<double>><<<k, 256, 0, s>>>(n, (const cpx<double>*)Q, (const cpx<double>*)w, (cpx<double>*)h);
  else gemv_ct_kernel<double><<<k, 256, 0, s>>>(n, (const double*)Q, (const double*)w, (double*)h);
}
void launch_gemv_sub(bool cplx, int n, int k, const void* Q, const void* h, void* w, cudaStream_t s) {
  if (k <= 0) return;
  int g = grid_for(n);
  if (cplx) gemv_sub_kernel<cpx<double>><<<g, 256, 0, s>>>(n, k, (const cpx<double>*)Q, (const cpx<double>*)h, (cpx<double>*)w, -1);
  else gemv_sub_kernel<double><<<g, 256, 0, s>>>(n, k, (const double*)Q, (const double*)h, (double*)w, -1);
}
void launch_axpy_basis(bool cplx, int n, int k, const void* Q, const void* y, void* x, cudaStream_t s) {
  if (k <= 0) return;
  int g = grid_for(n);
  if (cplx) gemv_sub_kernel<cpx<double>><<<g, 256, 0, s>>>(n, k, (const cpx<double>*)Q, (const cpx<double>*)y, (cpx<double>*)x, 1);
  else gemv_sub_kernel<double><<<g, 256, 0, s>>>(n, k, (const double*)Q, (const double*)y, (double*)x, 1);
}
void launch_nrm2(bool cplx, int n, const void* w, double* out, cudaStream_t s) {
  if (cplx) nrm2_kernel<cpx<double>><<<1, 256, 0, s>>>(n, (const cpx<double>*)w, out);
  else nrm2_kernel<double><<<1, 256, 0, s>>>(n, (const double*)w, out);
}
void launch_scale_copy(bool cplx, int n, const void* w, double inv, void* q, cudaStream_t s) {
  int g = grid_for(n);
  if (cplx) scale_copy_kernel<cpx<double>><<<g, 256, 0, s>>>(n, (const cpx<double>*)w, inv, (cpx<double>*)q);
  else scale_copy_kernel<double><<<g, 256, 0, s>>>(n, (const double*)w, inv, (double*)q);
}
void launch_residual(bool cplx, int n, const void* b, void* r, cudaStream_t s) {
  int g = grid_for(n);
  if (cplx) residual_kernel<cpx<double>><<<g, 256, 0, s>>>(n, (const cpx<double>*)b, (cpx<double>*)r);
  else residual_kernel<double><<<g, 256, 0, s>>>(n, (const double*)b, (double*)r);
}

}  // namespace bem
