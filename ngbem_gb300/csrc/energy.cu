// Batched Laplace single-layer energy and its derivatives (shape gradient).
//
// For a batch of closed triangle meshes X_b with piecewise-constant densities u_b:
//   E_b = u_b^T V(X_b) u_b,   V_ij = D_i D_j sum_k w_k G(x_k - y_k),   G(d) = 1/(4 pi |d|),
// where V is the Galerkin single-layer matrix of the P0 space as the near-field kernels
// assemble it (reference CalcBlockMatrix, src/ngbem.cpp:373-738, with the Laplace kernel of
// src/ngbem.hpp:215-260): the tensor Gauss rule on element pairs that share no vertex, the
// Sauter-Schwab rules on pairs that do.  D = |J| (D = 1 with the dual mapping, whose basis
// 1/|J| cancels the measure).  Outputs: E_b, (V u)_i and dE/dX.
//
// The derivative is the exact derivative of this discrete energy (the quadrature points are
// fixed in reference coordinates, so the rule moves with the mesh):
//   dG(x - y)/dP_a = lambda_a(x) grad G,  dG/dQ_b = -mu_b(y) grad G,  grad G(d) = -d/(4 pi |d|^3),
//   dD/dP_0 = e1 x n^,  dD/dP_1 = n^ x e0,  dD/dP_2 = -(dD/dP_0 + dD/dP_1)   (e_a = P_a - P_2).
// Regular pairs: V_ij and V_ji are the same function of X (same rule on both sides) and the
// set of regular pairs is symmetric, so sum_ij u_i u_j (d_test + d_trial) V_ij =
// 2 sum_ij u_i u_j d_test V_ij: one thread per test element accumulates its derivative over
// all trial elements in registers and writes 9 numbers per work unit.  Singular pairs take
// the full derivative of both elements.  The backward pass recomputes the quadrature; nothing
// is stored between the energy and the gradient.
#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

#define SLE_TI 128  // test elements per work unit (threads per CTA)

// trial elements per work unit (staged in shared memory): 256 while the points fit ~32 KB
__host__ __device__ constexpr int sle_tj(int rbytes, int nq) {
  return rbytes * nq * 4 * 256 <= 32768 ? 256 : (rbytes * nq * 4 * 128 <= 32768 ? 128 : 64);
}

__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Per element: D, dD/dP (9), centroid as hi+lo floats, quadrature-point offsets from the
// centroid (float, mixed precision) and quadrature points (double).
__global__ void sle_prep_kernel(SLEArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.ntri) return;
  const int4 t = a.tri[i];
  const int id[3] = {t.x, t.y, t.z};
  double P[3][3];
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int c = 0; c < 3; ++c) P[v][c] = a.X[3 * id[v] + c];
  double e0[3], e1[3], n[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    e0[c] = P[0][c] - P[2][c];
    e1[c] = P[1][c] - P[2][c];
  }
  cross3(e0, e1, n);
  const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  double* dD = a.dD + 9 * (size_t)i;
  if (a.dual) {
    a.D[i] = 1.0;
    for (int k = 0; k < 9; ++k) dD[k] = 0.0;
  } else {
    a.D[i] = nn;
    const double nh[3] = {n[0] / nn, n[1] / nn, n[2] / nn};
    double g0[3], g1[3];
    cross3(e1, nh, g0);
    cross3(nh, e0, g1);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dD[c] = g0[c];
      dD[3 + c] = g1[c];
      dD[6 + c] = -(g0[c] + g1[c]);
    }
  }
  double cen[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) cen[c] = (P[0][c] + P[1][c] + P[2][c]) / 3.0;
  float* cf = a.cf + 6 * (size_t)i;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float h = __double2float_rn(cen[c]);
    cf[c] = h;
    cf[3 + c] = __double2float_rn(cen[c] - (double)h);
  }
  for (int q = 0; q < a.nq; ++q) {
    const double xi = a.rxi[q], et = a.reta[q], l2 = 1.0 - xi - et;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double x = xi * P[0][c] + et * P[1][c] + l2 * P[2][c];
      a.q64[((size_t)i * a.nq + q) * 3 + c] = x;
      a.off[((size_t)i * a.nq + q) * 3 + c] = __double2float_rn(x - cen[c]);
    }
  }
}

// 1/sqrt(x) for x > 0 in FP64: the FP32 hardware estimate refined by one Newton-Raphson step
// for f(y) = 1/y^2 - x (y <- y (3 - x y^2) / 2), which squares the relative error of the
// estimate (about 1e-7) to about 1e-14 -- far below the quadrature error -- for a handful of
// FP64 operations instead of a full-precision FP64 reciprocal square root.
__device__ __forceinline__ double rsqrt_nr(double x) {
  const double y = (double)rsqrtf((float)x);
  return y * fma(-0.5 * x, y * y, 1.5);
}

template <class R> __device__ __forceinline__ R rsq(R x);
template <> __device__ __forceinline__ float rsq<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double rsq<double>(double x) { return rsqrt(x); }

__device__ __forceinline__ double block_sum128(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < SLE_TI / 32; ++k) s += red[k];
  return s;
}

// Regular pairs.  Work unit = (problem, SLE_TI test elements, SLE_TJ trial elements); one thread
// per test element.  R = float: differences of centroids from hi+lo pairs plus float offsets
// (relative precision of FP32 kept for close elements); R = double: FP64 points.
template <class R, bool GRAD, int NQ>
__global__ void __launch_bounds__(SLE_TI) sle_regular_kernel(SLEArgs a) {
  constexpr int SLE_TJ = sle_tj(sizeof(R), NQ);
  __shared__ int4 s_id[SLE_TJ];
  __shared__ R s_x[SLE_TJ][NQ * 3];  // float: offsets from the centroid; double: points
  __shared__ R s_wc[SLE_TJ][NQ];     // w_q * u_j * D_j
  __shared__ float4 s_ch[SLE_TJ], s_cl[SLE_TJ];
  __shared__ double red[SLE_TI / 32];
  constexpr bool F32 = sizeof(R) == 4;
  const double inv4pi = 0.25 / 3.14159265358979323846;
  for (int unit = blockIdx.x; unit < a.nunits; unit += gridDim.x) {
    const int4 U = a.units[unit];
    const int b = U.x, tb = a.t0[b], nt = a.nt[b];
    const int jn = min(SLE_TJ, nt - U.z);
    __syncthreads();  // the previous unit is done with shared memory
    for (int jj = threadIdx.x; jj < jn; jj += SLE_TI) {
      const int j = tb + U.z + jj;
      s_id[jj] = a.tri[j];
      const double cj = a.u[j] * a.D[j];
#pragma unroll
      for (int q = 0; q < NQ; ++q) s_wc[jj][q] = (R)(a.rw[q] * cj);
      if (F32) {
        const float* cf = a.cf + 6 * (size_t)j;
        s_ch[jj] = make_float4(cf[0], cf[1], cf[2], 0.f);
        s_cl[jj] = make_float4(cf[3], cf[4], cf[5], 0.f);
#pragma unroll
        for (int k = 0; k < NQ * 3; ++k) s_x[jj][k] = (R)a.off[(size_t)j * NQ * 3 + k];
      } else {
#pragma unroll
        for (int k = 0; k < NQ * 3; ++k) s_x[jj][k] = (R)a.q64[(size_t)j * NQ * 3 + k];
      }
    }
    __syncthreads();
    const int il = U.y + threadIdx.x;
    const bool valid = il < nt;
    const int i = tb + (valid ? il : 0);
    const int4 ti = a.tri[i];
    R xo[NQ][3];
    float chi[3], clo[3];
    if (F32) {
      const float* cf = a.cf + 6 * (size_t)i;
#pragma unroll
      for (int c = 0; c < 3; ++c) { chi[c] = cf[c]; clo[c] = cf[3 + c]; }
#pragma unroll
      for (int q = 0; q < NQ; ++q)
#pragma unroll
        for (int c = 0; c < 3; ++c) xo[q][c] = (R)a.off[((size_t)i * NQ + q) * 3 + c];
    } else {
#pragma unroll
      for (int q = 0; q < NQ; ++q)
#pragma unroll
        for (int c = 0; c < 3; ++c) xo[q][c] = (R)a.q64[((size_t)i * NQ + q) * 3 + c];
    }
    R A = 0;
    R B[NQ][3];
#pragma unroll
    for (int p = 0; p < NQ; ++p) B[p][0] = B[p][1] = B[p][2] = 0;
    if (valid) {
      for (int jj = 0; jj < jn; ++jj) {
        const int4 tj = s_id[jj];
        const bool shared = ti.x == tj.x || ti.x == tj.y || ti.x == tj.z || ti.y == tj.x || ti.y == tj.y ||
                            ti.y == tj.z || ti.z == tj.x || ti.z == tj.y || ti.z == tj.z;
        if (shared) continue;  // singular pair (Sauter-Schwab kernel)
        R dc[3] = {0, 0, 0};
        if (F32) {
          const float4 h = s_ch[jj], l = s_cl[jj];
          dc[0] = (R)((chi[0] - h.x) + (clo[0] - l.x));
          dc[1] = (R)((chi[1] - h.y) + (clo[1] - l.y));
          dc[2] = (R)((chi[2] - h.z) + (clo[2] - l.z));
        }
#pragma unroll
        for (int p = 0; p < NQ; ++p) {
          const R ex = dc[0] + xo[p][0], ey = dc[1] + xo[p][1], ez = dc[2] + xo[p][2];
          R Ap = 0;
#pragma unroll
          for (int q = 0; q < NQ; ++q) {
            const R dx = ex - s_x[jj][3 * q], dy = ey - s_x[jj][3 * q + 1], dz = ez - s_x[jj][3 * q + 2];
            const R rinv = rsq<R>(dx * dx + dy * dy + dz * dz);
            const R g = s_wc[jj][q] * rinv;
            Ap += g;
            if (GRAD) {
              const R h = g * rinv * rinv;
              B[p][0] += h * dx;
              B[p][1] += h * dy;
              B[p][2] += h * dz;
            }
          }
          A += (R)a.rw[p] * Ap;
        }
      }
    }
    double e = 0.0;
    if (valid) {
      const double Di = a.D[i];
      const double vu = Di * (double)A * inv4pi;
      atomicAdd(&a.vu[i], vu);
      e = a.u[i] * vu;
      if (GRAD) {
        const double wb = a.wprob ? a.wprob[b] : 1.0;
        const double s = 2.0 * a.u[i] * wb * inv4pi;
        const double* dD = a.dD + 9 * (size_t)i;
        const int id[3] = {ti.x, ti.y, ti.z};
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          double gp[3] = {0.0, 0.0, 0.0};
#pragma unroll
          for (int p = 0; p < NQ; ++p) {
            const double lam = v == 0 ? a.rxi[p] : (v == 1 ? a.reta[p] : 1.0 - a.rxi[p] - a.reta[p]);
            const double wl = a.rw[p] * lam;
            gp[0] += wl * (double)B[p][0];
            gp[1] += wl * (double)B[p][1];
            gp[2] += wl * (double)B[p][2];
          }
#pragma unroll
          for (int c = 0; c < 3; ++c)
            atomicAdd(&a.grad[3 * (size_t)id[v] + c], s * (dD[3 * v + c] * (double)A - Di * gp[c]));
        }
      }
    }
    const double es = block_sum128(e, red);
    if (threadIdx.x == 0 && es != 0.0) atomicAdd(&a.energy[b], es);
  }
}

// Singular pairs (sharing a vertex, an edge or identical): one warp per ordered pair, FP64
// Sauter-Schwab rules.  The tables hold one point per Duffy direction (xi = 1): 1/|d| is
// homogeneous of degree -1 and the points of a direction are xi times its xi = 1 point, so the
// radial sum is ss_c2 times the direction's term (ss_c1 for the degree -2 gradient moment M,
// ss_c2 for the moments that carry one more factor xi through s_k or t_k).  The vertices are permuted once per pair so that the rule's barycentric
// coordinates (1 - s0 - s1, s0, s1) belong to (P'0, P'1, P'2) -- the same assignment as the
// near-field kernel's vertex permutations -- and P'0 is the common vertex (identical pairs:
// P'0 = P2).  Then d = x - y = s0 E1 + s1 E2 - t0 F1 - t1 F2 with edge vectors from P'0, and the
// position derivative needs only the moments M = sum w h d, sum s_k w h d, sum t_k w h d
// (h = 1/|d|^3), mapped back to the three vertices once per pair.
template <bool GRAD>
__global__ void __launch_bounds__(256) sle_singular_kernel(SLEArgs a) {
  extern __shared__ double s_tab[];
  const double* tab[3];
  {
    int off = 0;
    for (int c = 0; c < 3; ++c) {
      const int n5 = 5 * a.ss_n[c];
      if (a.ss_smem) {
        for (int t = threadIdx.x; t < n5; t += blockDim.x) s_tab[off + t] = a.ss[c][t];
        tab[c] = s_tab + off;
      } else {
        tab[c] = a.ss[c];
      }
      off += n5;
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const double inv4pi = 0.25 / 3.14159265358979323846;
  for (int it = warp; it < a.nsing; it += nwarps) {
    const int2 pr = a.sing[it];
    const int4 vi4 = a.tri[pr.x], vj4 = a.tri[pr.y];
    const int vi[3] = {vi4.x, vi4.y, vi4.z}, vj[3] = {vj4.x, vj4.y, vj4.z};
    int ncommon = 0;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 3; ++q) ncommon += (vi[p] == vj[q]);
    const int cls = ncommon == 3 ? 0 : (ncommon == 2 ? 1 : 2);
    int px[3] = {2, 0, 1}, py[3] = {2, 0, 1};
    if (cls == 1) {
      // edge table (0,1) | (1,2) | (2,0); the common edge comes first, reversed in y
      int cex = 0, cey = 0;
      for (int cx = 0; cx < 3; ++cx)
        for (int cy = 0; cy < 3; ++cy) {
          const int a0 = vi[cx], a1 = vi[(cx + 1) % 3], b0 = vj[cy], b1 = vj[(cy + 1) % 3];
          if (min(a0, a1) == min(b0, b1) && max(a0, a1) == max(b0, b1)) { cex = cx; cey = cy; }
        }
      px[0] = cex; px[1] = (cex + 1) % 3; px[2] = 3 - px[0] - px[1];
      py[0] = (cey + 1) % 3; py[1] = cey; py[2] = 3 - py[0] - py[1];
    } else if (cls == 2) {
      int cvx = 0, cvy = 0;
      for (int cx = 0; cx < 3; ++cx)
        for (int cy = 0; cy < 3; ++cy)
          if (vi[cx] == vj[cy]) { cvx = cx; cvy = cy; }
      px[0] = cvx; px[1] = (cvx + 1) % 3; px[2] = (cvx + 2) % 3;
      py[0] = cvy; py[1] = (cvy + 1) % 3; py[2] = (cvy + 2) % 3;
    }
    int gi[3], gj[3];  // global vertex ids in permuted order
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      gi[k] = px[k] == 0 ? vi[0] : (px[k] == 1 ? vi[1] : vi[2]);
      gj[k] = py[k] == 0 ? vj[0] : (py[k] == 1 ? vj[1] : vj[2]);
    }
    double E1[3], E2[3], F1[3], F2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double pi0 = a.X[3 * gi[0] + c], pj0 = a.X[3 * gj[0] + c];
      E1[c] = a.X[3 * gi[1] + c] - pi0;
      E2[c] = a.X[3 * gi[2] + c] - pi0;
      F1[c] = a.X[3 * gj[1] + c] - pj0;
      F2[c] = a.X[3 * gj[2] + c] - pj0;
    }
    const int npts = a.ss_n[cls];
    const double* T = tab[cls];
    double S = 0.0, M[3] = {0, 0, 0}, Ms0[3] = {0, 0, 0}, Ms1[3] = {0, 0, 0}, Mt0[3] = {0, 0, 0},
           Mt1[3] = {0, 0, 0};
    for (int k = lane; k < npts; k += 32) {
      const double s0 = T[k], s1 = T[npts + k], t0 = T[2 * npts + k], t1 = T[3 * npts + k], w = T[4 * npts + k];
      double d[3];
      if (cls == 0) {
        const double u0 = s0 - t0, u1 = s1 - t1;
#pragma unroll
        for (int c = 0; c < 3; ++c) d[c] = u0 * E1[c] + u1 * E2[c];
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) d[c] = (s0 * E1[c] + s1 * E2[c]) - (t0 * F1[c] + t1 * F2[c]);
      }
      const double rinv = rsqrt_nr(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      const double g = w * rinv;
      S += g;
      if (GRAD) {
        const double h = g * rinv * rinv;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double hd = h * d[c];
          M[c] += hd;
          Ms0[c] += s0 * hd;
          Ms1[c] += s1 * hd;
          Mt0[c] += t0 * hd;
          Mt1[c] += t1 * hd;
        }
      }
    }
    S = warp_sum(S);
    if (GRAD) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        M[c] = warp_sum(M[c]);
        Ms0[c] = warp_sum(Ms0[c]);
        Ms1[c] = warp_sum(Ms1[c]);
        Mt0[c] = warp_sum(Mt0[c]);
        Mt1[c] = warp_sum(Mt1[c]);
      }
    }
    if (lane == 0) {
      S *= a.ss_c2;
      if (GRAD) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          M[c] *= a.ss_c1;
          Ms0[c] *= a.ss_c2;
          Ms1[c] *= a.ss_c2;
          Mt0[c] *= a.ss_c2;
          Mt1[c] *= a.ss_c2;
        }
      }
      const int b = a.tprob[pr.x];
      const double Di = a.D[pr.x], Dj = a.D[pr.y], ui = a.u[pr.x], uj = a.u[pr.y];
      const double v = Di * Dj * S * inv4pi;
      atomicAdd(&a.vu[pr.x], uj * v);
      atomicAdd(&a.energy[b], ui * uj * v);
      if (GRAD) {
        const double c0 = ui * uj * (a.wprob ? a.wprob[b] : 1.0) * inv4pi, DD = Di * Dj;
        const double* dDi = a.dD + 9 * (size_t)pr.x;
        const double* dDj = a.dD + 9 * (size_t)pr.y;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          // sum w lambda'_k h d for the permuted vertices: lambda' = (1 - s0 - s1, s0, s1)
          const double bx[3] = {M[c] - Ms0[c] - Ms1[c], Ms0[c], Ms1[c]};
          const double by[3] = {M[c] - Mt0[c] - Mt1[c], Mt0[c], Mt1[c]};
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            atomicAdd(&a.grad[3 * (size_t)gi[k] + c], c0 * (Dj * dDi[3 * px[k] + c] * S - DD * bx[k]));
            atomicAdd(&a.grad[3 * (size_t)gj[k] + c], c0 * (Di * dDj[3 * py[k] + c] * S + DD * by[k]));
          }
        }
      }
    }
  }
}

template <class R, bool GRAD>
static void launch_reg(const SLEArgs& a, int grid, cudaStream_t s) {
  switch (a.nq) {
    case 1: sle_regular_kernel<R, GRAD, 1><<<grid, SLE_TI, 0, s>>>(a); break;
    case 4: sle_regular_kernel<R, GRAD, 4><<<grid, SLE_TI, 0, s>>>(a); break;
    case 9: sle_regular_kernel<R, GRAD, 9><<<grid, SLE_TI, 0, s>>>(a); break;
    default: break;
  }
}

int sle_tile_test() { return SLE_TI; }
int sle_tile_trial(bool fp64, int nq) { return sle_tj(fp64 ? 8 : 4, nq); }

void launch_sle(const SLEArgs& a, bool fp64, bool grad, cudaStream_t s) {
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (a.ntri > 0) sle_prep_kernel<<<(a.ntri + 127) / 128, 128, 0, s>>>(a);
  if (a.nunits > 0) {
    const int grid = std::min(a.nunits, nsm * 8);
    if (fp64) {
      if (grad) launch_reg<double, true>(a, grid, s);
      else launch_reg<double, false>(a, grid, s);
    } else {
      if (grad) launch_reg<float, true>(a, grid, s);
      else launch_reg<float, false>(a, grid, s);
    }
  }
  if (a.nsing > 0) {
    const int grid = std::min((a.nsing + 7) / 8, nsm * 8);
    const int smem = a.ss_smem ? 40 * (a.ss_n[0] + a.ss_n[1] + a.ss_n[2]) : 0;
    if (grad) sle_singular_kernel<true><<<grid, 256, smem, s>>>(a);
    else sle_singular_kernel<false><<<grid, 256, smem, s>>>(a);
  }
}

}  // namespace bem
