// Plain-old-data descriptors shared by the host orchestration (C++) and the CUDA kernels.
#pragma once
#include <math.h>
#include <stdint.h>

namespace bem {

enum KernelId {
  K_LAPLACE_SL = 0, K_LAPLACE_DL = 1, K_LAPLACE_HS = 2, K_HELMHOLTZ_SL = 3,
  K_HELMHOLTZ_DL = 4, K_HELMHOLTZ_HS = 5, K_HELMHOLTZ_CF = 6, K_MAXWELL_SL = 7,
  K_HELMHOLTZ_SL_DKAPPA = 8,  // d/dkappa of the Helmholtz single layer (no counterpart in the reference)
  K_MAXWELL_DL = 9,
  K_NUM = 10
};

// trace kinds = (space kind, evaluator) combinations the operators use
// TR_NED, TR_NEDROT, TR_NEDMAX: the HCurl (lowest-order Nedelec) traces of the edge dofs:
// the tangential shape n x phi_RT0, the rotated trace n x (n x phi_RT0) = -phi_RT0, and the
// Maxwell trace [-phi_RT0; surface curl] (reference DiffOpRotatedTrace, DiffOpMaxwell,
// src/diffops.hpp:62-255, for the Whitney edge shapes, which are n x the RT0 shapes)
// TR_L2P1..3: SurfaceL2 of order 1..3 (the identity trace of the Dubiner basis)
// TR_H1P2, TR_H1P3: H1 of order 2, 3 (identity trace); TR_H1P2ROT, TR_H1P3ROT: their surface
// curl n x grad_Gamma phi (DiffOpBoundaryRot, src/diffops.hpp:12-60, for the hierarchical basis
// h1p_shape below); TR_H1P2HELM, TR_H1P3HELM: [n x grad_Gamma phi; phi] (DiffOpHelmholtz)
// TR_HDIVkID: HDivSurface of order k = 1..4 (identity trace, the Piola-mapped shape psi);
// TR_HDIVkMAX: [psi; surface divergence] (DiffOpMaxwellNew) for hdiv_shape below
// TR_HCURLk*: HCurl of order k, whose shapes are n x the HDivSurface shapes of the same order and
// dofs: ID n x psi, ROT (DiffOpRotatedTrace) n x (n x psi) = -psi, MAX (DiffOpMaxwell)
// [-psi; surface curl = surface divergence of psi]
enum TraceKind { TR_P0 = 0, TR_P1 = 1, TR_ROT = 2, TR_HELM = 3, TR_MAX = 4, TR_RT0ID = 5,
                 TR_NED = 6, TR_NEDROT = 7, TR_NEDMAX = 8, TR_L2P1 = 9, TR_L2P2 = 10, TR_L2P3 = 11,
                 TR_H1P2 = 12, TR_H1P3 = 13, TR_H1P2ROT = 14, TR_H1P3ROT = 15, TR_H1P2HELM = 16,
                 TR_H1P3HELM = 17,
                 // HDivSurface / HCurl of order K = 1..4: TR_BDM + 5 (K - 1) + variant
                 TR_BDM = 18,
                 TR_HDIV1ID = 18, TR_HDIV1MAX = 19, TR_HCURL1ID = 20, TR_HCURL1ROT = 21, TR_HCURL1MAX = 22,
                 TR_HDIV2ID = 23, TR_HDIV2MAX = 24, TR_HCURL2ID = 25, TR_HCURL2ROT = 26, TR_HCURL2MAX = 27,
                 TR_HDIV3ID = 28, TR_HDIV3MAX = 29, TR_HCURL3ID = 30, TR_HCURL3ROT = 31, TR_HCURL3MAX = 32,
                 TR_HDIV4ID = 33, TR_HDIV4MAX = 34, TR_HCURL4ID = 35, TR_HCURL4ROT = 36, TR_HCURL4MAX = 37 };
// traces of a discontinuous space of order >= 1: the element's dofs are consecutive
// (first dof + local index) and its "signs" hold the order of its vertices by global number
__host__ __device__ constexpr bool l2p_trace(int tr) { return tr >= TR_L2P1 && tr <= TR_L2P3; }
__host__ __device__ constexpr int l2p_order(int tr) { return tr - TR_L2P1 + 1; }
// traces of H1 of order 2, 3: vertex dofs, then the p - 1 dofs of each local edge (0,1),
// (1,2), (2,0), then the (p - 1)(p - 2) / 2 face dofs
__host__ __device__ constexpr bool h1p_trace(int tr) { return tr >= TR_H1P2 && tr <= TR_H1P3HELM; }
__host__ __device__ constexpr int h1p_order(int tr) {
  return tr == TR_H1P2 || tr == TR_H1P2ROT || tr == TR_H1P2HELM ? 2 : 3;
}
// the traces with the surface curl in components 0..2 (and, HELM, the value in 3)
__host__ __device__ constexpr bool h1p_rot(int tr) { return tr >= TR_H1P2ROT && tr <= TR_H1P3HELM; }
__host__ __device__ constexpr bool h1p_helm(int tr) { return tr == TR_H1P2HELM || tr == TR_H1P3HELM; }

// traces of HDivSurface (and HCurl) of order K = 1..4: per local edge k (vertices k, k + 1 mod 3)
// K + 1 dofs, then (K + 1)(K - 1) interior dofs
// (also the HCurl traces of order 1..4: the same dofs and reference fields)
__host__ __device__ constexpr bool hdiv_trace(int tr) { return tr >= TR_BDM && tr <= TR_HCURL4MAX; }
__host__ __device__ constexpr int hdiv_order(int tr) { return (tr - TR_BDM) / 5 + 1; }
__host__ __device__ constexpr int bdm_variant(int tr) { return (tr - TR_BDM) % 5; }
__host__ __device__ constexpr bool hcurl_hi_trace(int tr) { return hdiv_trace(tr) && bdm_variant(tr) >= 2; }
// traces that read the unit normal of the point (n x the HDiv shape)
__host__ __device__ constexpr bool normal_trace(int tr) { return tr == TR_NED || (hdiv_trace(tr) && bdm_variant(tr) == 2); }
// the trace kind of HDivSurface (curl = false) or HCurl of order k with an evaluator variant:
// HDivSurface 0 ID, 1 MAXWELL; HCurl 0 ID, 1 ROTATED_TRACE, 2 MAXWELL_CURL
__host__ __device__ constexpr int bdm_trace(int k, bool curl, int v) { return TR_BDM + 5 * (k - 1) + (curl ? 2 : 0) + v; }

// Hierarchical basis of HDivSurface of order K = 1..4 (BDM_K: all vector polynomials of degree
// K; our own choice of basis, spanning the space of NGSolve's HDivSurface(order=K)) as reference
// fields (vx, vy) on the triangle with vertices (1,0), (0,1), (0,0), in barycentrics
// l = (xi, eta, 1 - xi - eta); the physical shape is the Piola map J (vx, vy) / |J| and the
// surface divergence the returned reference divergence / |J|.  rot f = (df/deta, -df/dxi).
// Local dof a:
//   a < 3 (K + 1)  edge k = a / (K + 1) between local vertices i = k, j = k + 1 (mod 3),
//                  m = a % (K + 1):
//                  m = 0   sg (xhat - vhat_o), o the vertex opposite (the RT0 shape);
//                  m >= 1  sg^(m-1) rot(l_i l_j (l_j - l_i)^(m-1))
//                  with sg the edge's orientation (+1 when its first vertex has the lower global
//                  number): the surface curls of the global H1 edge bubbles (curls of continuous
//                  functions are normal-continuous)
//   a >= 3 (K + 1) interior, zero normal trace on every edge: for i = 0, 1, 2 and the monomials
//                  xi^p eta^q (p + q <= K - 2; p outer, q inner; for i = 2 only p = 0):
//                  l_j l_k xi^p eta^q rot(l_i), (j, k) the other two vertices;
//                  (K + 1)(K - 1) of them
template <class R>
__host__ __device__ inline R hdiv_shape(int K, int a, R xi, R eta, int sg, R& vx, R& vy) {
  const R l[3] = {xi, eta, R(1) - xi - eta};
  const R rx[3] = {R(0), R(1), R(-1)}, ry[3] = {R(-1), R(0), R(1)};   // rot l_i
  const R gx[3] = {R(1), R(0), R(-1)}, gy[3] = {R(0), R(1), R(-1)};   // grad l_i
  if (a < 3 * (K + 1)) {
    const int k = a / (K + 1), m = a % (K + 1);
    const int i = k, j = (k + 1) % 3, o = (k + 2) % 3;
    if (m == 0) {
      const R ox = o == 0 ? R(1) : R(0), oy = o == 1 ? R(1) : R(0);
      vx = R(sg) * (xi - ox);
      vy = R(sg) * (eta - oy);
      return R(2 * sg);
    }
    // d phi / d l_i and d phi / d l_j of the edge bubble phi = l_i l_j s^e, s = l_j - l_i
    const int e = m - 1;
    const R sd = l[j] - l[i];
    R se = R(1), se1 = R(0);  // s^e, e s^(e-1)
    for (int t = 0; t < e; ++t) {
      se1 = se1 * sd + se;
      se = se * sd;
    }
    const R q = l[i] * l[j], f = (e & 1) ? R(sg) : R(1);
    const R di = f * (l[j] * se - q * se1), dj = f * (l[i] * se + q * se1);
    vx = di * rx[i] + dj * rx[j];
    vy = di * ry[i] + dj * ry[j];
    return R(0);
  }
  // interior: find (i, p, q) of index t
  int t = a - 3 * (K + 1), i = 0, p = 0, q = 0;
  for (i = 0; i < 3; ++i) {
    const int cnt = i < 2 ? K * (K - 1) / 2 : K - 1;
    if (t < cnt) break;
    t -= cnt;
  }
  if (i < 2) {
    while (t >= K - 1 - p) {
      t -= K - 1 - p;
      ++p;
    }
    q = t;
  } else {
    q = t;
  }
  const int j = (i + 1) % 3, k = (i + 2) % 3;
  R h = R(1), hx = R(0), hy = R(0);  // xi^p eta^q and its derivatives
  for (int u = 0; u < p; ++u) {
    hx = hx * xi + h;
    h = h * xi;
  }
  R hq = R(1), hqy = R(0);
  for (int u = 0; u < q; ++u) {
    hqy = hqy * eta + hq;
    hq = hq * eta;
  }
  hy = h * hqy;
  hx = hx * hq;
  h = h * hq;
  const R g = l[j] * l[k], gxv = l[k] * gx[j] + l[j] * gx[k], gyv = l[k] * gy[j] + l[j] * gy[k];
  const R f = g * h;
  vx = f * rx[i];
  vy = f * ry[i];
  return (gxv * h + g * hx) * rx[i] + (gyv * h + g * hy) * ry[i];
}

// Hierarchical H1 basis of order P <= 3 on a triangle in barycentric coordinates l[3] (our own
// choice of basis; the reference takes NGSolve's H1 element, whose shapes differ but span
// the same space): local dof a
//   a < 3               vertex:  l_a
//   3 <= a < 3 + 3(P-1) edge k = (a - 3) / (P - 1) between local vertices i = k, j = k + 1
//                       (mod 3), degree m + 2 with m = (a - 3) % (P - 1):
//                       l_i l_j (l_j - l_i)^m, in the element's local orientation; the
//                       global one (i the vertex of the lower global number) multiplies it
//                       by the edge's orientation sign to the power m (passed by the caller)
//   a = 9 (P = 3)       face:    l_0 l_1 l_2
// Returns the value and, in d[3], its partial derivatives in l_0, l_1, l_2 (as if the three
// were independent: the surface gradient is sum_i d_i grad l_i, and sum_i grad l_i = 0).
template <class R>
__host__ __device__ inline R h1p_shape(int P, int a, const R* l, R* d) {
  d[0] = d[1] = d[2] = R(0);
  if (a < 3) {
    d[a] = R(1);
    return l[a];
  }
  const int ne = 3 * (P - 1);
  if (a < 3 + ne) {
    const int k = (a - 3) / (P - 1), m = (a - 3) % (P - 1);
    const int i = k, j = (k + 1) % 3;
    if (m == 0) {
      d[i] = l[j];
      d[j] = l[i];
      return l[i] * l[j];
    }
    const R s = l[j] - l[i];  // m == 1
    d[i] = l[j] * s - l[i] * l[j];
    d[j] = l[i] * s + l[i] * l[j];
    return l[i] * l[j] * s;
  }
  d[0] = l[1] * l[2];
  d[1] = l[0] * l[2];
  d[2] = l[0] * l[1];
  return l[0] * l[1] * l[2];
}

// Dubiner basis function a of order P on a triangle (Dubiner 1991; Karniadakis and Sherwin,
// Spectral/hp Element Methods, ch. 3), in the form NGSolve's L2 triangle element uses it:
// with x = lambda_f0, y = lambda_f1 (f0, f1 the element's vertices of the lowest and the next
// global number), s = 2x + y - 1, t = 1 - y, z = 2y - 1,
//   phi_ij = t^i P_i(s / t) * P_j^(2i+1, 0)(z),   i = 0..P, j = 0..P-i,
// numbered with i outer and j inner.  P_i: Legendre (scaled by t^i through its recurrence),
// P_j^(alpha, 0): Jacobi.  code = f0 + 3 f1.
template <class R>
__host__ __device__ inline R dubiner(int P, int a, R xi, R eta, int code) {
  const int f0 = code % 3, f1 = code / 3;
  const R l2 = R(1) - xi - eta;
  const R x = f0 == 0 ? xi : (f0 == 1 ? eta : l2);
  const R y = f1 == 0 ? xi : (f1 == 1 ? eta : l2);
  int i = 0, first = 0;
  while (a >= first + (P - i + 1)) {
    first += P - i + 1;
    ++i;
  }
  const int j = a - first;
  const R s = R(2) * x + y - R(1), t = R(1) - y, z = R(2) * y - R(1);
  // scaled Legendre: L_0 = 1, L_1 = s, (n+1) L_{n+1} = (2n+1) s L_n - n t^2 L_{n-1}
  R l0 = R(1), l1 = s;
  R L = i == 0 ? l0 : l1;
  for (int n = 1; n < i; ++n) {
    const R ln = (R(2 * n + 1) * s * l1 - R(n) * t * t * l0) / R(n + 1);
    l0 = l1;
    l1 = ln;
    L = ln;
  }
  // Jacobi P^(al, 0): P_0 = 1, P_1 = ((al + 2) z + al) / 2,
  // 2n(n+al)(2n+al-2) P_n = (2n+al-1)((2n+al)(2n+al-2) z + al^2) P_{n-1} - 2(n+al-1)(n-1)(2n+al) P_{n-2}
  const int al = 2 * i + 1;
  R j0 = R(1), j1 = (R(al + 2) * z + R(al)) * R(0.5);
  R J = j == 0 ? j0 : j1;
  for (int n = 2; n <= j; ++n) {
    const R c1 = R((2 * n + al - 1) * (2 * n + al) * (2 * n + al - 2));
    const R c0 = R((2 * n + al - 1) * al * al);
    const R cm = R(2 * (n + al - 1) * (n - 1) * (2 * n + al));
    const R jn = ((c1 * z + c0) * j1 - cm * j0) / R(2 * n * (n + al) * (2 * n + al - 2));
    j0 = j1;
    j1 = jn;
    J = jn;
  }
  return L * J;
}

// traces whose local dofs carry an edge orientation sign
__host__ __device__ constexpr bool edge_trace(int tr) {
  return tr == TR_MAX || tr == TR_RT0ID || tr == TR_NED || tr == TR_NEDROT || tr == TR_NEDMAX || hdiv_trace(tr);
}

// Per-element record (FP64): vertices, unit normal, |J|, rotated surface gradients of the
// P1 hat functions (n x grad lambda_a), vertex ids.  128 bytes + 64 bytes, read by the
// singular kernel, the element tables of every precision are built from it on the host.
struct ElemRec64 {
  double p[3][3];     // vertices; reference vertices (1,0),(0,1),(0,0)
  double n[3];
  double detJ;        // |(p0-p2) x (p1-p2)|
  double invdetJ;
  double rot[3][3];   // n x surface-grad(lambda_a)
  double pad[1];
};

// Per-element record in compute precision P: centroid as hi+lo pair (so differences of
// centroids are accurate to P's relative precision), vertex offsets from the centroid.
template <class P>
struct ElemRecP {
  P chi[3], clo[3];
  P n[3];
  P detJ, invdetJ;
  P o[3][3];          // p_k - centroid
  P rot[3][3];
  P pad[3];
};

// Geometry of one regular-rule point of a curved element (flat elements keep it per element,
// in ElemRecP): the unit normal, the rotated surface gradients n x grad_Gamma(lambda_a) of the
// barycentrics, 1 / |J|, and per local vertex o the vector J (xhat - vhat_o), which the RT0
// shape of the edge opposite o scales by its sign / |J| (the Piola map; on a flat element it is
// x - p_o).
template <class P>
struct PGeo {
  P n[3];
  P rot[3][3];
  P invdetJ;
  P xp[3][3];
};

// J (xhat - vhat_o) for the reference vertices vhat = (1,0), (0,1), (0,0)
__host__ __device__ inline void piola_offsets(const double* J0, const double* J1, double xi, double eta,
                                              double xp[3][3]) {
  const double vx[3] = {1.0, 0.0, 0.0}, vy[3] = {0.0, 1.0, 0.0};
  for (int o = 0; o < 3; ++o)
    for (int c = 0; c < 3; ++c) xp[o][c] = J0[c] * (xi - vx[o]) + J1[c] * (eta - vy[o]);
}

// Curved (isoparametric Lagrange) element map of order g at (xi, eta): the point and its
// derivatives J0 = dx/dxi, J1 = dx/deta from the element's (g+1)(g+2)/2 nodes P (3 doubles
// each).  Node (i, j, k), i + j + k = g, sits at barycentric (i, j, k) / g of the vertices
// (v0, v1, v2) and the nodes are listed for i = g..0, j = g-i..0; its shape function is
// L_i(l0) L_j(l1) L_k(l2) with (l0, l1, l2) = (xi, eta, 1 - xi - eta) and
// L_i(t) = prod_{m<i} (g t - m) / (m + 1).
__host__ __device__ inline void curved_map(int g, const double* P, double xi, double eta, double* x, double* J0,
                                           double* J1) {
  const double l[3] = {xi, eta, 1.0 - xi - eta};
  double L[3][5], D[3][5];
  for (int s = 0; s < 3; ++s)
    for (int i = 0; i <= g; ++i) {
      double v = 1.0, d = 0.0;
      for (int m = 0; m < i; ++m) {
        const double f = (g * l[s] - m) / (m + 1);
        d = d * f + v * g / (m + 1);
        v = v * f;
      }
      L[s][i] = v;
      D[s][i] = d;
    }
  for (int c = 0; c < 3; ++c) x[c] = J0[c] = J1[c] = 0.0;
  int n = 0;
  for (int i = g; i >= 0; --i)
    for (int j = g - i; j >= 0; --j, ++n) {
      const int k = g - i - j;
      const double N = L[0][i] * L[1][j] * L[2][k];
      const double dxi = D[0][i] * L[1][j] * L[2][k] - L[0][i] * L[1][j] * D[2][k];
      const double deta = L[0][i] * D[1][j] * L[2][k] - L[0][i] * L[1][j] * D[2][k];
      for (int c = 0; c < 3; ++c) {
        x[c] += N * P[3 * n + c];
        J0[c] += dxi * P[3 * n + c];
        J1[c] += deta * P[3 * n + c];
      }
    }
}

// |J0 x J1|, the unit normal and the rotated surface gradients n x grad_Gamma(lambda_a) of the
// barycentrics (lambda_0 = xi, lambda_1 = eta): grad_Gamma = J (J^T J)^{-1} grad_ref.
__host__ __device__ inline double surface_frame(const double* J0, const double* J1, double* n, double rot[3][3]) {
  const double cr[3] = {J0[1] * J1[2] - J0[2] * J1[1], J0[2] * J1[0] - J0[0] * J1[2], J0[0] * J1[1] - J0[1] * J1[0]};
  const double detJ = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  for (int c = 0; c < 3; ++c) n[c] = cr[c] / detJ;
  const double g00 = J0[0] * J0[0] + J0[1] * J0[1] + J0[2] * J0[2];
  const double g01 = J0[0] * J1[0] + J0[1] * J1[1] + J0[2] * J1[2];
  const double g11 = J1[0] * J1[0] + J1[1] * J1[1] + J1[2] * J1[2];
  const double det = g00 * g11 - g01 * g01;
  const double gh[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {-1.0, -1.0}};
  for (int a = 0; a < 3; ++a) {
    const double c0 = (g11 * gh[a][0] - g01 * gh[a][1]) / det;
    const double c1 = (-g01 * gh[a][0] + g00 * gh[a][1]) / det;
    double gv[3];
    for (int c = 0; c < 3; ++c) gv[c] = J0[c] * c0 + J1[c] * c1;
    rot[a][0] = n[1] * gv[2] - n[2] * gv[1];
    rot[a][1] = n[2] * gv[0] - n[0] * gv[2];
    rot[a][2] = n[0] * gv[1] - n[1] * gv[0];
  }
  return detJ;
}

// A dense (near-field or fallback) block of the H-matrix.
struct DenseDesc {
  long long off;      // offset of the m x n column-major block in the dense pool (elements, 16-byte aligned)
  int r0, m;          // rows [r0, r0+m) in the test cluster permutation
  int c0, n;          // cols [c0, c0+n) in the trial cluster permutation
  int pi0, ni;        // test patch: patch_elems[pi0 .. pi0+ni)
  int pj0, nj;        // trial patch
};

// Work tile of the regular near-field kernel: 128 consecutive element pairs of block b.
struct NFTile {
  int b;              // dense block index
  int k0;             // first flattened pair index (i * nj + j)
};

// Singular element pair found by the regular kernel.
struct SingItem {
  int b, ei, ej;
};

// A far-field (low-rank) block.
struct FarDesc {
  int r0, m, c0, n;   // dof ranges (cluster permutation)
  int pi0, ni, pj0, nj;  // patches
  long long su, sv;   // ACA scratch offsets (elements) of U (kcap x M) and V (kcap x N), per comp
  int kcap;
  int pad;
};

// Low-rank factors after projection, addressed by absolute device pointers (factor pools may
// be allocated per ACA batch).  Chunked layouts so that every chunk is one contiguous,
// 16-byte aligned copy:
//   U2 (m x R): row chunks of cu rows;   U2(i, r) at u + (i/cu)*cu*R + r*cu + i%cu
//   V2 (R x n): column chunks of cv cols; V2(r, j) at v + (j/cv)*cv*R + (j%cv)*R + r
struct LRDesc {
  unsigned long long u, v;
  int r0, m, c0, n;
  int R;
  int toff;              // offset of the R-vector of V2*x in the temporary pool
  int cu, cv;
};
__host__ __device__ inline long long lr_u_index(const LRDesc& L, int i, int r) {
  return (long long)(i / L.cu) * L.cu * L.R + (long long)r * L.cu + (i % L.cu);
}
__host__ __device__ inline long long lr_v_index(const LRDesc& L, int r, int j) {
  return (long long)(j / L.cv) * L.cv * L.R + (long long)(j % L.cv) * L.R + r;
}

// matvec descriptors (absolute device pointers); dense blocks are column-major
struct MVDense {
  unsigned long long ptr;
  int r0, m, c0, n;
};

// A segment of a matvec work item: a (part of a) block whose payload sits at byte offset
// soff of the item.  kind 0: dense columns [k0, k0+cnt); 1: U2 row chunk [k0, k0+cnt);
// 2: V2 column chunk [k0, k0+cnt).
struct MVSeg {
  int kind, blk, k0, cnt, soff, pad;
};
// A work item: one contiguous copy of `bytes` bytes from src (bytes == 0: read in place),
// its pieces [seg0, seg0+nseg) and the input ranges [rng0, rng0+nrng) copied next to it
// (inbytes in total).
struct MVTItem {
  unsigned long long src;
  int bytes, seg0, nseg, rng0, nrng, inbytes;
  int r[8];  // the first two input ranges inline (src, elem, bytes, dst each); others in the range list
  int pad[4];  // 80 bytes: runs of descriptors are bulk-copied (16-byte multiples)
};
static_assert(sizeof(MVTItem) % 16 == 0, "MVTItem is bulk-copied");

// A piece of an item as one pass applies it: out[out_off + o] += sum_k A[o*so + k*sk] *
// in[in_off + k] for o < O, k < Kc, with A at byte soff of the item payload.  flags bit 0:
// the input is the R-vector pool t (else the permuted x); bit 1: the output is t (else y).
// in_soff: byte offset of in[in_off] in the item's staged input area.
struct MVPiece {
  int soff, so, sk, O, Kc, in_off, out_off, flags, in_soff;
  int ow;      // lanes per group: min(O, 32)
  int groups;  // 32 / ow lane groups splitting k
  float inv_ow;  // 1/ow (exact lane -> group mapping for lane < 32)
};

// An input range staged with an item: `bytes` bytes from element `elem` (16-byte aligned
// start) of x (src 0) or t (src 1), to byte `dst` of the input area.
struct MVRange {
  int src, elem, bytes, dst;
};
typedef LRDesc MVLowRank;

struct TermDesc {
  int nterms;
  int kc[4], trc[4], tec[4];
  double fac[4];
};

}  // namespace bem
