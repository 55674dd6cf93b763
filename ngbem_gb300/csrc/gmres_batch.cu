// Vector kernels of the batched GMRES (nrhs independent systems advanced in lockstep, so that
// every Arnoldi step applies the operator once to all right-hand sides).  Vectors are FP64 /
// complex128, column r of a block at offset r * n; the Krylov basis holds k blocks of nrhs
// columns (basis vector i of column r at (i * nrhs + r) * n).
#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

template <class V> __device__ __forceinline__ V conj_(V v) { return v; }
template <> __device__ __forceinline__ cpx<double> conj_(cpx<double> v) { return {v.x, -v.y}; }

template <class V>
__device__ __forceinline__ V block_reduce(V v, V* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  V s = vzero<V>();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : vzero<V>();
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

// h[i * nrhs + r] = Q_{i,r}^H w_r for i < k (one block per (i, r))
template <class V>
__global__ void bgemv_ct_kernel(int n, int k, int nrhs, const V* Q, const V* w, V* h) {
  __shared__ V sh[32];
  const int i = blockIdx.x / nrhs, r = blockIdx.x % nrhs;
  const V* q = Q + ((size_t)i * nrhs + r) * n;
  const V* x = w + (size_t)r * n;
  V acc = vzero<V>();
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc += conj_(q[t]) * x[t];
  acc = block_reduce(acc, sh);
  if (threadIdx.x == 0) h[(size_t)i * nrhs + r] = acc;
}

// w_r -= sum_{i<k} Q_{i,r} h[i * nrhs + r]
template <class V>
__global__ void bgemv_sub_kernel(int n, int k, int nrhs, const V* Q, const V* h, V* w) {
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / n), e = (int)(t - (long long)r * n);
    V acc = w[t];
    for (int i = 0; i < k; ++i) acc -= Q[((size_t)i * nrhs + r) * n + e] * h[(size_t)i * nrhs + r];
    w[t] = acc;
  }
}

// x_r += sum_{i<k} Q_{i,r} y[i * nrhs + r]
template <class V>
__global__ void baxpy_basis_kernel(int n, int k, int nrhs, const V* Q, const V* y, V* x) {
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / n), e = (int)(t - (long long)r * n);
    V acc = x[t];
    for (int i = 0; i < k; ++i) acc += Q[((size_t)i * nrhs + r) * n + e] * y[(size_t)i * nrhs + r];
    x[t] = acc;
  }
}

__device__ __forceinline__ double sqnorm(double v) { return v * v; }
__device__ __forceinline__ double sqnorm(cpx<double> v) { return v.x * v.x + v.y * v.y; }

// out[r] = ||w_r||_2
template <class V>
__global__ void bnrm2_kernel(int n, int nrhs, const V* w, double* out) {
  __shared__ double sh[32];
  const int r = blockIdx.x;
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc += sqnorm(w[(size_t)r * n + t]);
  acc = block_reduce(acc, sh);
  if (threadIdx.x == 0) out[r] = sqrt(acc);
}

// q_r = w_r * inv[r]
template <class V>
__global__ void bscale_kernel(int n, int nrhs, const V* w, const double* inv, V* q) {
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / n);
    q[t] = w[t] * inv[r];
  }
}

static int bgrid(long long total) {
  long long g = (total + 255) / 256;
  return (int)std::max(1ll, std::min(g, 152ll * 16));
}

void launch_bgemv_ct(bool cplx, int n, int k, int nrhs, const void* Q, const void* w, void* h, cudaStream_t s) {
  if (cplx) bgemv_ct_kernel<cpx<double>><<<k * nrhs, 256, 0, s>>>(n, k, nrhs, (const cpx<double>*)Q, (const cpx<double>*)w, (cpx<double>*)h);
  else bgemv_ct_kernel<double><<<k * nrhs, 256, 0, s>>>(n, k, nrhs, (const double*)Q, (const double*)w, (double*)h);
}
void launch_bgemv_sub(bool cplx, int n, int k, int nrhs, const void* Q, const void* h, void* w, cudaStream_t s) {
  const int g = bgrid((long long)n * nrhs);
  if (cplx) bgemv_sub_kernel<cpx<double>><<<g, 256, 0, s>>>(n, k, nrhs, (const cpx<double>*)Q, (const cpx<double>*)h, (cpx<double>*)w);
  else bgemv_sub_kernel<double><<<g, 256, 0, s>>>(n, k, nrhs, (const double*)Q, (const double*)h, (double*)w);
}
void launch_baxpy_basis(bool cplx, int n, int k, int nrhs, const void* Q, const void* y, void* x, cudaStream_t s) {
  const int g = bgrid((long long)n * nrhs);
  if (cplx) baxpy_basis_kernel<cpx<double>><<<g, 256, 0, s>>>(n, k, nrhs, (const cpx<double>*)Q, (const cpx<double>*)y, (cpx<double>*)x);
  else baxpy_basis_kernel<double><<<g, 256, 0, s>>>(n, k, nrhs, (const double*)Q, (const double*)y, (double*)x);
}
void launch_bnrm2(bool cplx, int n, int nrhs, const void* w, double* out, cudaStream_t s) {
  if (cplx) bnrm2_kernel<cpx<double>><<<nrhs, 256, 0, s>>>(n, nrhs, (const cpx<double>*)w, out);
  else bnrm2_kernel<double><<<nrhs, 256, 0, s>>>(n, nrhs, (const double*)w, out);
}
void launch_bscale(bool cplx, int n, int nrhs, const void* w, const double* inv, void* q, cudaStream_t s) {
  const int g = bgrid((long long)n * nrhs);
  if (cplx) bscale_kernel<cpx<double>><<<g, 256, 0, s>>>(n, nrhs, (const cpx<double>*)w, inv, (cpx<double>*)q);
  else bscale_kernel<double><<<g, 256, 0, s>>>(n, nrhs, (const double*)w, inv, (double*)q);
}

}  // namespace bem
