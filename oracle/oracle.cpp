// FP64 CPU oracle: a restatement of the reference's operator path (TEST INFRASTRUCTURE).
// See oracle.hpp for the list of reference files followed and for the parity status.
#include "oracle.hpp"

#include <algorithm>
#include <array>
#include <atomic>
#include <climits>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <thread>
#include <vector>

namespace orc {

using cplx = std::complex<double>;
static const double PI = 3.14159265358979323846;

// ---------------------------------------------------------------------------------------
// Symmetric eigen solver (cyclic Jacobi).  Stands in for LapackEigenValuesSymmetric
// (reference src/hmat.cpp:203).  Eigenvalues ascending; row k of evecs is the eigenvector
// of eigenvalue k; each eigenvector has its largest-magnitude component positive (first
// index on ties).  Uses only + - * / sqrt so that it is bit-reproducible across hosts.
// ---------------------------------------------------------------------------------------
static void jacobi_eigen(int n, std::vector<double> A, std::vector<double>& evals,
                         std::vector<double>& evecs) {
  std::vector<double> V(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p * n + q];
        if (apq == 0.0) continue;
        double tau = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double c = 1.0 / std::sqrt(1.0 + t * t);
        double s = t * c;
        for (int r = 0; r < n; ++r) {
          if (r == p || r == q) continue;
          double arp = A[r * n + p], arq = A[r * n + q];
          double nrp = c * arp - s * arq;
          double nrq = s * arp + c * arq;
          A[r * n + p] = nrp; A[p * n + r] = nrp;
          A[r * n + q] = nrq; A[q * n + r] = nrq;
        }
        A[p * n + p] = A[p * n + p] - t * apq;
        A[q * n + q] = A[q * n + q] + t * apq;
        A[p * n + q] = 0.0; A[q * n + p] = 0.0;
        for (int r = 0; r < n; ++r) {
          double vrp = V[r * n + p], vrq = V[r * n + q];
          V[r * n + p] = c * vrp - s * vrq;
          V[r * n + q] = s * vrp + c * vrq;
        }
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(),
                   [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
  evals.assign(n, 0.0);
  evecs.assign(n * n, 0.0);
  for (int k = 0; k < n; ++k) {
    int j = idx[k];
    evals[k] = A[j * n + j];
    int imax = 0;
    for (int r = 1; r < n; ++r)
      if (std::fabs(V[r * n + j]) > std::fabs(V[imax * n + j])) imax = r;
    double sgn = V[imax * n + j] < 0.0 ? -1.0 : 1.0;
    for (int r = 0; r < n; ++r) evecs[k * n + r] = sgn * V[r * n + j];
  }
}

// Gauss-Jacobi nodes/weights on [0,1] for weight (1-u)^alpha u^beta (Golub-Welsch).
static void gauss_jacobi01(int n, double alpha, double beta, std::vector<double>& x,
                           std::vector<double>& w) {
  std::vector<double> J(n * n, 0.0);
  for (int k = 0; k < n; ++k) {
    double s = 2.0 * k + alpha + beta;
    double a = (k == 0) ? (beta - alpha) / (alpha + beta + 2.0)
                        : (beta * beta - alpha * alpha) / (s * (s + 2.0));
    J[k * n + k] = a;
    if (k >= 1) {
      double num = 4.0 * k * (k + alpha) * (k + beta) * (k + alpha + beta);
      double den = s * s * (s + 1.0) * (s - 1.0);
      double b = std::sqrt(num / den);
      J[k * n + k - 1] = b; J[(k - 1) * n + k] = b;
    }
  }
  double mu0 = std::pow(2.0, alpha + beta + 1.0) * std::tgamma(alpha + 1.0) *
               std::tgamma(beta + 1.0) / std::tgamma(alpha + beta + 2.0);
  std::vector<double> ev, evec;
  jacobi_eigen(n, J, ev, evec);
  x.resize(n); w.resize(n);
  double scale = std::pow(2.0, alpha + beta + 1.0);
  for (int k = 0; k < n; ++k) {
    double v0 = evec[k * n + 0];
    x[k] = 0.5 * (1.0 + ev[k]);
    w[k] = mu0 * v0 * v0 / scale;
  }
}

// Segment rule of NGSolve-style "order": n = order/2 + 1 Gauss-Legendre points on [0,1].
static void segm_rule(int order, std::vector<double>& x, std::vector<double>& w) {
  gauss_jacobi01(order / 2 + 1, 0.0, 0.0, x, w);
}

// Triangle rule on the reference triangle {xi>=0, eta>=0, xi+eta<=1}: collapsed
// (Stroud conical) product of Gauss-Jacobi(1,0) and Gauss-Legendre, n = order/2+1 each.
struct TrigRule { std::vector<double> xi, eta, w; };
static TrigRule trig_rule(int order) {
  int n = order / 2 + 1;
  std::vector<double> u, wu, v, wv;
  gauss_jacobi01(n, 1.0, 0.0, u, wu);
  gauss_jacobi01(n, 0.0, 0.0, v, wv);
  TrigRule r;
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      r.xi.push_back(u[a]);
      r.eta.push_back(v[b] * (1.0 - u[a]));
      r.w.push_back(wu[a] * wv[b]);
    }
  return r;
}

// Sauter-Schwab rules (reference src/intrules.cpp:13-136).  Points on the triangle
// [(0,0),(1,0),(0,1)]; Duffy 4-vectors mapped to (p0-p1, p1), (p2-p3, p3).
struct SSRule { std::vector<double> x0, x1, y0, y1, w; };
static SSRule ss_rule(int cls, int order) {
  std::vector<double> s, ws;
  segm_rule(order, s, ws);
  int n = (int)s.size();
  std::vector<std::array<double, 4>> duff;
  std::vector<double> wts;
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int i3 = 0; i3 < n; ++i3) {
        double e1 = s[i1], e2 = s[i2], e3 = s[i3];
        double weta = ws[i1] * ws[i2] * ws[i3];
        for (int ix = 0; ix < n; ++ix) {
          double xi = s[ix];
          double wbase = weta * ws[ix];
          auto push = [&](double a, double b, double c, double d) {
            duff.push_back({xi * a, xi * b, xi * c, xi * d});
          };
          if (cls == 0) {  // identical panel, intrules.cpp:24-39
            push(1, 1 - e1 + e1 * e2, 1 - e1 * e2 * e3, 1 - e1);
            push(1 - e1 * e2 * e3, 1 - e1, 1, 1 - e1 + e1 * e2);
            push(1, e1 * (1 - e2 + e2 * e3), 1 - e1 * e2, e1 * (1 - e2));
            push(1 - e1 * e2, e1 * (1 - e2), 1, e1 * (1 - e2 + e2 * e3));
            push(1 - e1 * e2 * e3, e1 * (1 - e2 * e3), 1, e1 * (1 - e2));
            push(1, e1 * (1 - e2), 1 - e1 * e2 * e3, e1 * (1 - e2 * e3));
            for (int j = 0; j < 6; ++j) wts.push_back(xi * xi * xi * e1 * e1 * e2 * wbase);
          } else if (cls == 1) {  // common edge, intrules.cpp:110-123
            push(1, e1 * e3, 1 - e1 * e2, e1 * (1 - e2));
            push(1, e1, 1 - e1 * e2 * e3, e1 * e2 * (1 - e3));
            push(1 - e1 * e2, e1 * (1 - e2), 1, e1 * e2 * e3);
            push(1 - e1 * e2 * e3, e1 * e2 * (1 - e3), 1, e1);
            push(1 - e1 * e2 * e3, e1 * (1 - e2 * e3), 1, e1 * e2);
            wts.push_back(xi * xi * xi * e1 * e1 * wbase);
            for (int j = 0; j < 4; ++j) wts.push_back(xi * xi * xi * e1 * e1 * e2 * wbase);
          } else {  // common vertex, intrules.cpp:75-79
            push(1, e1, e2, e2 * e3);
            push(e2, e2 * e3, 1, e1);
            for (int j = 0; j < 2; ++j) wts.push_back(xi * xi * xi * e2 * wbase);
          }
        }
      }
  SSRule r;
  for (size_t k = 0; k < duff.size(); ++k) {
    r.x0.push_back(duff[k][0] - duff[k][1]);
    r.x1.push_back(duff[k][1]);
    r.y0.push_back(duff[k][2] - duff[k][3]);
    r.y1.push_back(duff[k][3]);
    r.w.push_back(wts[k]);
  }
  return r;
}

// ---------------------------------------------------------------------------------------
// Mesh, element transformation, spaces
// ---------------------------------------------------------------------------------------
struct Geo {
  double p[3][3];      // vertices (reference vertices (1,0),(0,1),(0,0))
  double J0[3], J1[3]; // p0-p2, p1-p2
  double detJ;         // |J0 x J1| (= 2 * area)
  double n[3];         // unit normal (J0 x J1)/detJ
};

// The element map at one reference point (the reference's MappedIntegrationPoint, through
// mesh->GetTrafo): the point, the derivatives J0 = dx/dxi, J1 = dx/deta, |J0 x J1| and the
// unit normal.
struct MP {
  double x[3], J0[3], J1[3], detJ, n[3];
};

// Curved elements (NGSolve's Mesh.Curve(order), third-party code the reference's tests call;
// restated as isoparametric Lagrange triangles): element e of order g holds (g+1)(g+2)/2
// nodes; node (i, j, k), i + j + k = g, sits at barycentric (i, j, k) / g of the element's
// vertices (v0, v1, v2), and the nodes are listed for i = g..0, j = g-i..0.  The map is
// x(xi, eta) = sum N_ijk X_ijk with N_ijk = L_i(l0) L_j(l1) L_k(l2), (l0, l1, l2) =
// (xi, eta, 1 - xi - eta), L_i(t) = prod_{m<i} (g t - m) / (m + 1).
static int g_geo_order = 1, g_geo_nt = 0;
static std::vector<double> g_geo_nodes;

static void lagrange_1d(int g, int i, double t, double& v, double& d) {
  v = 1.0;
  d = 0.0;
  for (int m = 0; m < i; ++m) {
    const double f = (g * t - m) / (m + 1);
    d = d * f + v * g / (m + 1);
    v = v * f;
  }
}

struct Mesh {
  int nv = 0, nt = 0, ne = 0;
  int gorder = 1;            // geometry order (1: flat triangles)
  std::vector<double> X;
  std::vector<int> T, E, TE;
  std::vector<Geo> geo;
  std::vector<double> G;     // gorder > 1: the nodes, 3 (gorder+1)(gorder+2)/2 per element
  void build(int nv_, const double* xyz, int nt_, const int* tri) {
    nv = nv_; nt = nt_;
    X.assign(xyz, xyz + 3 * nv);
    T.assign(tri, tri + 3 * nt);
    E.resize(6 * nt); TE.resize(3 * nt);
    ne = orc_mesh_edges(nv, nt, tri, E.data(), TE.data());
    E.resize(2 * ne);
    geo.resize(nt);
    for (int e = 0; e < nt; ++e) {
      Geo& g = geo[e];
      for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) g.p[k][c] = X[3 * T[3 * e + k] + c];
      for (int c = 0; c < 3; ++c) {
        g.J0[c] = g.p[0][c] - g.p[2][c];
        g.J1[c] = g.p[1][c] - g.p[2][c];
      }
      double cr[3] = {g.J0[1] * g.J1[2] - g.J0[2] * g.J1[1],
                      g.J0[2] * g.J1[0] - g.J0[0] * g.J1[2],
                      g.J0[0] * g.J1[1] - g.J0[1] * g.J1[0]};
      g.detJ = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      for (int c = 0; c < 3; ++c) g.n[c] = cr[c] / g.detJ;
    }
    if (g_geo_order > 1 && g_geo_nt == nt) {
      gorder = g_geo_order;
      G = g_geo_nodes;
    }
  }
  // the curved map and its derivatives (the sums in node order)
  void curved(int e, double xi, double eta, double* x, double* J0, double* J1) const {
    const int g = gorder, nn = (g + 1) * (g + 2) / 2;
    const double l[3] = {xi, eta, 1.0 - xi - eta};
    double L[3][5], D[3][5];
    for (int s = 0; s < 3; ++s)
      for (int i = 0; i <= g; ++i) lagrange_1d(g, i, l[s], L[s][i], D[s][i]);
    for (int c = 0; c < 3; ++c) x[c] = J0[c] = J1[c] = 0.0;
    const double* P = &G[(size_t)e * nn * 3];
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
  // flat: x = xi*p0 + eta*p1 + (1-xi-eta)*p2 (shape-function form of the affine map)
  void map(int e, double xi, double eta, double* x) const {
    if (gorder > 1) {
      double J0[3], J1[3];
      curved(e, xi, eta, x, J0, J1);
      return;
    }
    const Geo& g = geo[e];
    double l2 = 1.0 - xi - eta;
    for (int c = 0; c < 3; ++c) x[c] = xi * g.p[0][c] + eta * g.p[1][c] + l2 * g.p[2][c];
  }
  MP mp(int e, double xi, double eta) const {
    MP r;
    if (gorder == 1) {
      const Geo& g = geo[e];
      map(e, xi, eta, r.x);
      for (int c = 0; c < 3; ++c) { r.J0[c] = g.J0[c]; r.J1[c] = g.J1[c]; r.n[c] = g.n[c]; }
      r.detJ = g.detJ;
      return r;
    }
    curved(e, xi, eta, r.x, r.J0, r.J1);
    const double cr[3] = {r.J0[1] * r.J1[2] - r.J0[2] * r.J1[1], r.J0[2] * r.J1[0] - r.J0[0] * r.J1[2],
                          r.J0[0] * r.J1[1] - r.J0[1] * r.J1[0]};
    r.detJ = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    for (int c = 0; c < 3; ++c) r.n[c] = cr[c] / r.detJ;
    return r;
  }
  // the element's weight in the cluster data (the reference's SurfaceElementVolume): the
  // flat area, or for curved elements |J0 x J1| / 2 at the centroid
  double area(int e) const { return gorder > 1 ? 0.5 * mp(e, 1. / 3, 1. / 3).detJ : 0.5 * geo[e].detJ; }
};

// SurfaceL2 of order p >= 1 has (p+1)(p+2)/2 dofs per element (at most 10 for p = 3),
// HDivSurface of order K (K+1)(K+2) (30 for K = 4)
constexpr int ORC_MAXND = 30;

// Dubiner basis function a of order P on a triangle (Dubiner 1991; Karniadakis and Sherwin,
// Spectral/hp Element Methods, ch. 3), as NGSolve's L2 triangle element uses it (third-party
// code the reference calls through SurfaceL2; restated): x = lambda_f0, y = lambda_f1 with f0,
// f1 the element's vertices of the lowest and the next global number; s = 2x + y - 1,
// t = 1 - y, z = 2y - 1;  phi_ij = t^i P_i(s / t) P_j^(2i+1, 0)(z), i = 0..P, j = 0..P-i,
// numbered with i outer.  Legendre by its three-term recurrence (scaled by t^i), Jacobi by
// the recurrence of P_n^(alpha, 0).
static double dubiner(int P, int a, double xi, double eta, int f0, int f1) {
  const double lam[3] = {xi, eta, 1.0 - xi - eta};
  const double x = lam[f0], y = lam[f1];
  int i = 0, first = 0;
  while (a >= first + (P - i + 1)) { first += P - i + 1; ++i; }
  const int j = a - first;
  const double s = 2.0 * x + y - 1.0, t = 1.0 - y, z = 2.0 * y - 1.0;
  double l0 = 1.0, l1 = s, L = i == 0 ? 1.0 : s;
  for (int n = 1; n < i; ++n) {
    const double ln = ((2 * n + 1) * s * l1 - n * t * t * l0) / (n + 1);
    l0 = l1; l1 = ln; L = ln;
  }
  const int al = 2 * i + 1;
  double j0 = 1.0, j1 = 0.5 * ((al + 2) * z + al), J = j == 0 ? 1.0 : j1;
  for (int n = 2; n <= j; ++n) {
    const double jn = ((2.0 * n + al - 1) * ((2.0 * n + al) * (2.0 * n + al - 2) * z + (double)al * al) * j1 -
                       2.0 * (n + al - 1) * (n - 1) * (2.0 * n + al) * j0) /
                      (2.0 * n * (n + al) * (2.0 * n + al - 2));
    j0 = j1; j1 = jn; J = jn;
  }
  return L * J;
}

// HDivSurface / HCurl of order K >= 1: K, else 0
static int bdm_order(int kind) {
  if (kind == ORC_HDIV1 || kind == ORC_HCURL1) return 1;
  if (kind == ORC_HDIV2 || kind == ORC_HCURL2) return 2;
  if (kind == ORC_HDIV3 || kind == ORC_HCURL3) return 3;
  if (kind == ORC_HDIV4 || kind == ORC_HCURL4) return 4;
  return 0;
}
static bool bdm_curl(int kind) {
  return kind == ORC_HCURL1 || kind == ORC_HCURL2 || kind == ORC_HCURL3 || kind == ORC_HCURL4;
}

struct Space {
  int kind = ORC_P0, ndof = 0, nd = 1;
  bool dual = false;
  std::vector<int> dofs;   // nd per element
  std::vector<int> sign;   // RT0 orientation per element-local dof
  void build(const Mesh& m, int kind_, bool dual_) {
    kind = kind_; dual = dual_;
    if (kind == ORC_P0) {
      nd = 1; ndof = m.nt; dofs.resize(m.nt);
      for (int e = 0; e < m.nt; ++e) dofs[e] = e;
    } else if (kind == ORC_P1) {
      nd = 3; ndof = m.nv; dofs = m.T;
    } else if (kind >= ORC_L2P1 && kind <= ORC_L2P3) {
      // SurfaceL2 of order p: consecutive dofs per element; sign holds the element's local
      // vertices in the order of their global numbers (the Dubiner basis is built on it)
      const int pp = kind - ORC_L2P1 + 1;
      nd = (pp + 1) * (pp + 2) / 2; ndof = m.nt * nd; dofs.resize((size_t)m.nt * nd); sign.resize(3 * m.nt);
      for (int e = 0; e < m.nt; ++e) {
        for (int a = 0; a < nd; ++a) dofs[(size_t)e * nd + a] = e * nd + a;
        int f[3] = {0, 1, 2};
        std::sort(f, f + 3, [&](int x, int y) { return m.T[3 * e + x] < m.T[3 * e + y]; });
        for (int k = 0; k < 3; ++k) sign[3 * e + k] = f[k];
      }
    } else if (kind == ORC_H1P2 || kind == ORC_H1P3) {
      // H1 of order p: vertex dofs = vertex ids, then p - 1 dofs per edge, then the face dofs
      const int pp = kind == ORC_H1P2 ? 2 : 3, pe = pp - 1, pf = (pp - 1) * (pp - 2) / 2;
      nd = (pp + 1) * (pp + 2) / 2;
      ndof = m.nv + m.ne * pe + m.nt * pf;
      dofs.resize((size_t)m.nt * nd);
      for (int e = 0; e < m.nt; ++e) {
        int* d = &dofs[(size_t)e * nd];
        for (int k = 0; k < 3; ++k) {
          d[k] = m.T[3 * e + k];
          for (int j = 0; j < pe; ++j) d[3 + k * pe + j] = m.nv + m.TE[3 * e + k] * pe + j;
        }
        for (int j = 0; j < pf; ++j) d[3 + 3 * pe + j] = m.nv + m.ne * pe + e * pf + j;
      }
    } else if (kind >= ORC_HDIV1) {
      // HDivSurface (and HCurl) of order K: per local edge K + 1 dofs (the edge's lowest-order
      // dof = the edge id, then ne + edge K + m - 1), then (K + 1)(K - 1) interior dofs per element
      const int K = bdm_order(kind), nin = (K + 1) * (K - 1);
      nd = (K + 1) * (K + 2);
      ndof = m.ne * (K + 1) + m.nt * nin;
      dofs.resize((size_t)m.nt * nd);
      sign.resize(3 * m.nt);
      for (int e = 0; e < m.nt; ++e) {
        int* d = &dofs[(size_t)e * nd];
        for (int k = 0; k < 3; ++k) {
          const int g = m.TE[3 * e + k];
          d[k * (K + 1)] = g;
          for (int j = 0; j < K; ++j) d[k * (K + 1) + 1 + j] = m.ne + g * K + j;
          sign[3 * e + k] = m.T[3 * e + k] < m.T[3 * e + (k + 1) % 3] ? 1 : -1;
        }
        for (int j = 0; j < nin; ++j) d[3 * (K + 1) + j] = m.ne * (K + 1) + e * nin + j;
      }
    } else {
      nd = 3; ndof = m.ne; dofs = m.TE; sign.resize(3 * m.nt);
      for (int e = 0; e < m.nt; ++e)
        for (int k = 0; k < 3; ++k) {
          int a = m.T[3 * e + k], b = m.T[3 * e + (k + 1) % 3];
          sign[3 * e + k] = a < b ? 1 : -1;
        }
    }
  }
  const int* el_dofs(int e) const { return &dofs[nd * e]; }
};

static int trace_dim(int kind, int ev) {
  if (ev == ORC_EV_ID) return (kind == ORC_RT0 || kind == ORC_HCURL || kind >= ORC_HDIV1) ? 3 : 1;
  if (ev == ORC_EV_ROT || ev == ORC_EV_ROTATED_TRACE) return 3;
  return 4;  // HELM, MAXWELL, MAXWELL_CURL
}

static void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Trace evaluator values S[a][c] at reference point (xi, eta) of element e.
// P1: lambda_0 = xi, lambda_1 = eta, lambda_2 = 1-xi-eta.  ROT: n x surface gradient
// (reference DiffOpBoundaryRot, src/diffops.hpp:12-57); HELM: [n x grad; value]
// (DiffOpHelmholtz :110-165); MAXWELL: [Piola shape; surface div] (DiffOpMaxwellNew
// :263-338) with RT0 shapes sigma*(xhat - vhat_opposite) on the reference triangle.
// HCURL: shape phi = n x psi (psi the RT0 shape of the same edge and sign); ID is phi,
// ROTATED_TRACE n x phi (DiffOpRotatedTrace :62-104), MAXWELL_CURL [n x phi; curl phi]
// (DiffOpMaxwell :172-255) with the surface curl of phi = div psi = 2 sigma / |J|.
static void eval_trace(const Mesh& m, const Space& sp, int ev, int e, double xi, double eta,
                       double S[ORC_MAXND][4]) {
  const MP g = m.mp(e, xi, eta);
  if (sp.kind == ORC_P0) {
    S[0][0] = sp.dual ? 1.0 / g.detJ : 1.0;
    return;
  }
  if (sp.kind >= ORC_L2P1 && sp.kind <= ORC_L2P3) {
    for (int a = 0; a < sp.nd; ++a)
      S[a][0] = dubiner(sp.kind - ORC_L2P1 + 1, a, xi, eta, sp.sign[3 * e], sp.sign[3 * e + 1]);
    return;
  }
  if (bdm_order(sp.kind) > 0) {
    // HDivSurface of order K (DiffOpMaxwellNew on NGSolve's HDivSurface element, restated for
    // a hierarchical BDM_K basis of our own): reference fields v on the triangle with vertices
    // (1,0), (0,1), (0,0), Piola-mapped J v / |J|, surface divergence (div v) / |J|.  Per local
    // edge k (vertices i = k, j = k+1; orientation s): m = 0 the RT0 shape s (xhat - vhat_o);
    // m >= 1 the curl (d/deta, -d/dxi) of s^(m-1) l_i l_j (l_j - l_i)^(m-1).  Interior: for
    // i = 0, 1, 2 and the monomials xi^p eta^q (p + q <= K - 2, p outer; only p = 0 for i = 2),
    // l_j l_k xi^p eta^q curl(l_i).  HCurl of order K: phi = n x those shapes, traces as on the
    // lowest-order HCurl below (ID phi, ROTATED_TRACE n x phi, MAXWELL_CURL
    // [n x phi; the divergence of the HDiv shape]).
    const int K = bdm_order(sp.kind);
    const bool hcurl = bdm_curl(sp.kind);
    // the interior functions' (i, p, q)
    std::vector<std::array<int, 3>> inner;
    for (int i = 0; i < 3; ++i)
      for (int p = 0; p <= K - 2; ++p)
        for (int q = 0; p + q <= K - 2; ++q)
          if (i < 2 || p == 0) inner.push_back({i, p, q});
    const double lam[3] = {xi, eta, 1.0 - xi - eta};
    const double dxi[3] = {1.0, 0.0, -1.0}, deta[3] = {0.0, 1.0, -1.0};  // d lambda / d(xi, eta)
    const double vh[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {0.0, 0.0}};
    for (int a = 0; a < sp.nd; ++a) {
      double vx, vy, dv;
      if (a < 3 * (K + 1)) {
        const int k = a / (K + 1), mm = a % (K + 1), i = k, j = (k + 1) % 3, o = (k + 2) % 3;
        const double sg = sp.sign[3 * e + k];
        if (mm == 0) {
          vx = sg * (xi - vh[o][0]);
          vy = sg * (eta - vh[o][1]);
          dv = 2.0 * sg;
        } else {
          double d[3] = {0.0, 0.0, 0.0};  // d phi / d lambda
          const int ex = mm - 1;
          const double sd = lam[j] - lam[i], o = (ex % 2) ? sg : 1.0;
          const double pw = std::pow(sd, ex), pw1 = ex > 0 ? ex * std::pow(sd, ex - 1) : 0.0;
          d[i] = o * (lam[j] * pw - lam[i] * lam[j] * pw1);
          d[j] = o * (lam[i] * pw + lam[i] * lam[j] * pw1);
          double px = 0.0, py = 0.0;  // d phi / d xi, d phi / d eta
          for (int t = 0; t < 3; ++t) { px += d[t] * dxi[t]; py += d[t] * deta[t]; }
          vx = py;
          vy = -px;
          dv = 0.0;
        }
      } else {
        const auto& ipq = inner[a - 3 * (K + 1)];
        const int i = ipq[0], j = (i + 1) % 3, k = (i + 2) % 3, p = ipq[1], q = ipq[2];
        const double mon = std::pow(xi, p) * std::pow(eta, q);
        const double mx = p > 0 ? p * std::pow(xi, p - 1) * std::pow(eta, q) : 0.0;
        const double my = q > 0 ? q * std::pow(xi, p) * std::pow(eta, q - 1) : 0.0;
        const double b = lam[j] * lam[k];
        const double bx = lam[k] * dxi[j] + lam[j] * dxi[k], by = lam[k] * deta[j] + lam[j] * deta[k];
        const double cx = deta[i], cy = -dxi[i];  // curl lambda_i
        vx = b * mon * cx;
        vy = b * mon * cy;
        dv = (bx * mon + b * mx) * cx + (by * mon + b * my) * cy;
      }
      double psi[3];
      for (int c = 0; c < 3; ++c) psi[c] = (g.J0[c] * vx + g.J1[c] * vy) / g.detJ;
      if (!hcurl) {
        for (int c = 0; c < 3; ++c) S[a][c] = psi[c];
        if (ev == ORC_EV_MAXWELL) S[a][3] = dv / g.detJ;
        continue;
      }
      double phi[3], rot[3];
      cross3(g.n, psi, phi);
      if (ev == ORC_EV_ID) {
        for (int c = 0; c < 3; ++c) S[a][c] = phi[c];
        continue;
      }
      cross3(g.n, phi, rot);
      for (int c = 0; c < 3; ++c) S[a][c] = rot[c];
      if (ev == ORC_EV_MAXWELL_CURL) S[a][3] = dv / g.detJ;
    }
    return;
  }
  if (sp.kind == ORC_H1P2 || sp.kind == ORC_H1P3) {
    // values, and surface curls n x sum_i (dphi / dl_i) grad_Gamma l_i (the surface gradients
    // of the barycentrics through the metric of the element map)
    const int pp = sp.kind == ORC_H1P2 ? 2 : 3, pe = pp - 1;
    const double lam[3] = {xi, eta, 1.0 - xi - eta};
    double gl[3][3];
    {
      double g00 = g.J0[0] * g.J0[0] + g.J0[1] * g.J0[1] + g.J0[2] * g.J0[2];
      double g01 = g.J0[0] * g.J1[0] + g.J0[1] * g.J1[1] + g.J0[2] * g.J1[2];
      double g11 = g.J1[0] * g.J1[0] + g.J1[1] * g.J1[1] + g.J1[2] * g.J1[2];
      double det = g00 * g11 - g01 * g01;
      const double gh[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {-1.0, -1.0}};
      for (int a = 0; a < 3; ++a) {
        double c0 = (g11 * gh[a][0] - g01 * gh[a][1]) / det;
        double c1 = (-g01 * gh[a][0] + g00 * gh[a][1]) / det;
        for (int c = 0; c < 3; ++c) gl[a][c] = g.J0[c] * c0 + g.J1[c] * c1;
      }
    }
    for (int a = 0; a < sp.nd; ++a) {
      double phi = 0.0, dl[3] = {0.0, 0.0, 0.0};
      if (a < 3) {
        phi = lam[a];
        dl[a] = 1.0;
      } else if (a < 3 + 3 * pe) {
        const int k = (a - 3) / pe, mm = (a - 3) % pe;
        int lo = k, hi = (k + 1) % 3;  // the edge's local vertices by global number
        if (m.T[3 * e + lo] > m.T[3 * e + hi]) std::swap(lo, hi);
        const double s = lam[hi] - lam[lo], q = lam[lo] * lam[hi];
        const double sm = mm == 0 ? 1.0 : s;
        phi = q * sm;
        dl[lo] = lam[hi] * sm - (mm == 0 ? 0.0 : q);
        dl[hi] = lam[lo] * sm + (mm == 0 ? 0.0 : q);
      } else {
        phi = lam[0] * lam[1] * lam[2];
        dl[0] = lam[1] * lam[2];
        dl[1] = lam[0] * lam[2];
        dl[2] = lam[0] * lam[1];
      }
      if (ev == ORC_EV_ID) {
        S[a][0] = phi;
        continue;
      }
      double grad[3], rot[3];
      for (int c = 0; c < 3; ++c) grad[c] = dl[0] * gl[0][c] + dl[1] * gl[1][c] + dl[2] * gl[2][c];
      cross3(g.n, grad, rot);
      for (int c = 0; c < 3; ++c) S[a][c] = rot[c];
      if (ev == ORC_EV_HELM) S[a][3] = phi;  // DiffOpHelmholtz: [n x grad phi; phi]
    }
    return;
  }
  if (sp.kind == ORC_P1) {
    double lam[3] = {xi, eta, 1.0 - xi - eta};
    if (ev == ORC_EV_ID) {
      for (int a = 0; a < 3; ++a) S[a][0] = lam[a];
      return;
    }
    double g00 = g.J0[0] * g.J0[0] + g.J0[1] * g.J0[1] + g.J0[2] * g.J0[2];
    double g01 = g.J0[0] * g.J1[0] + g.J0[1] * g.J1[1] + g.J0[2] * g.J1[2];
    double g11 = g.J1[0] * g.J1[0] + g.J1[1] * g.J1[1] + g.J1[2] * g.J1[2];
    double det = g00 * g11 - g01 * g01;
    const double gh[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {-1.0, -1.0}};
    for (int a = 0; a < 3; ++a) {
      double c0 = (g11 * gh[a][0] - g01 * gh[a][1]) / det;
      double c1 = (-g01 * gh[a][0] + g00 * gh[a][1]) / det;
      double grad[3], rot[3];
      for (int c = 0; c < 3; ++c) grad[c] = g.J0[c] * c0 + g.J1[c] * c1;
      cross3(g.n, grad, rot);
      for (int c = 0; c < 3; ++c) S[a][c] = rot[c];
      if (ev == ORC_EV_HELM) S[a][3] = lam[a];
    }
    return;
  }
  // RT0
  const double vh[3][2] = {{1.0, 0.0}, {0.0, 1.0}, {0.0, 0.0}};
  for (int k = 0; k < 3; ++k) {
    int o = (k + 2) % 3;
    double sg = sp.sign[3 * e + k];
    double ph0 = sg * (xi - vh[o][0]), ph1 = sg * (eta - vh[o][1]);
    for (int c = 0; c < 3; ++c) S[k][c] = (g.J0[c] * ph0 + g.J1[c] * ph1) / g.detJ;
    if (sp.kind == ORC_RT0) {
      if (ev == ORC_EV_MAXWELL) S[k][3] = 2.0 * sg / g.detJ;
      continue;
    }
    double phi[3], rot[3];
    cross3(g.n, S[k], phi);
    if (ev == ORC_EV_ID) {
      for (int c = 0; c < 3; ++c) S[k][c] = phi[c];
    } else {
      cross3(g.n, phi, rot);
      for (int c = 0; c < 3; ++c) S[k][c] = rot[c];
      if (ev == ORC_EV_MAXWELL_CURL) S[k][3] = 2.0 * sg / g.detJ;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Kernels (reference src/ngbem.hpp:215-510)
// ---------------------------------------------------------------------------------------
struct Term { double fac; int kc, trc, tec; };
struct Kernel {
  int id; double kappa; int ncomp; bool complex_valued;
  std::vector<Term> terms;
  Kernel(int id_, double kappa_) : id(id_), kappa(kappa_) {
    complex_valued = id >= ORC_HELMHOLTZ_SL;
    ncomp = (id == ORC_HELMHOLTZ_HS) ? 2 : (id == ORC_MAXWELL_DL ? 3 : 1);
    switch (id) {
      case ORC_LAPLACE_HS:
        terms = {{1.0, 0, 0, 0}, {1.0, 0, 1, 1}, {1.0, 0, 2, 2}};
        break;
      case ORC_HELMHOLTZ_HS:
        terms = {{1.0, 0, 0, 0}, {1.0, 0, 1, 1}, {1.0, 0, 2, 2}, {1.0, 1, 3, 3}};
        break;
      case ORC_MAXWELL_SL:
        for (int i = 0; i < 3; ++i) terms.push_back({kappa, 0, i, i});
        terms.push_back({-1.0 / kappa, 0, 3, 3});
        break;
      case ORC_MAXWELL_DL:  // {factor, component, trial, test}: the cross product of curl
        terms = {{1.0, 0, 1, 2}, {-1.0, 0, 2, 1}, {1.0, 1, 2, 0}, {-1.0, 1, 0, 2}, {1.0, 2, 0, 1}, {-1.0, 2, 1, 0}};
        break;
      default:
        terms = {{1.0, 0, 0, 0}};
    }
  }
  template <class T>
  void eval(const double* x, const double* y, const double* nx, const double* ny, T* out) const;
};

template <>
void Kernel::eval<double>(const double* x, const double* y, const double* nx, const double* ny,
                          double* out) const {
  double d[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
  double norm = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (id == ORC_LAPLACE_DL) {
    double nxy = ny[0] * d[0] + ny[1] * d[1] + ny[2] * d[2];
    out[0] = nxy / (4 * PI * norm * norm * norm);
  } else {
    out[0] = 1.0 / (4 * PI * norm);
  }
}

template <>
void Kernel::eval<cplx>(const double* x, const double* y, const double* nx, const double* ny,
                        cplx* out) const {
  double d[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
  double norm = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const cplx I(0.0, 1.0);
  cplx ex = std::exp(cplx(0.0, kappa) * norm);
  switch (id) {
    case ORC_HELMHOLTZ_DL: {
      double nxy = ny[0] * d[0] + ny[1] * d[1] + ny[2] * d[2];
      out[0] = ex / (4 * PI * norm * norm * norm) * nxy * (cplx(1.0, 0.0) - cplx(0.0, kappa) * norm);
      break;
    }
    case ORC_HELMHOLTZ_HS: {
      double nxny = nx[0] * ny[0] + nx[1] * ny[1] + nx[2] * ny[2];
      cplx kern = ex / (4 * PI * norm);
      out[0] = kern;
      out[1] = -kappa * kappa * kern * nxny;
      break;
    }
    case ORC_HELMHOLTZ_CF: {
      double nxy = ny[0] * d[0] + ny[1] * d[1] + ny[2] * d[2];
      out[0] = ex / (4 * PI * norm * norm * norm) *
               (nxy * (cplx(1.0, 0.0) - cplx(0.0, kappa) * norm) - cplx(0.0, kappa) * norm * norm);
      break;
    }
    case ORC_HELMHOLTZ_SL_DKAPPA:
      out[0] = cplx(0.0, 1.0) * ex / (4 * PI);
      break;
    case ORC_MAXWELL_DL: {
      const cplx g = ex / (4 * PI * norm * norm * norm) * (cplx(0.0, kappa) * norm - 1.0);
      for (int c = 0; c < 3; ++c) out[c] = g * d[c];
      break;
    }
    default:  // HELMHOLTZ_SL, MAXWELL_SL
      out[0] = ex / (4 * PI * norm);
  }
  (void)I;
}

template <class T> static inline T conj_(T v);
template <> inline double conj_(double v) { return v; }
template <> inline cplx conj_(cplx v) { return std::conj(v); }
static inline double re_(double v) { return v; }
static inline double re_(cplx v) { return v.real(); }

// ---------------------------------------------------------------------------------------
// Cluster tree (reference src/hmat.cpp:13-453)
// ---------------------------------------------------------------------------------------
struct Cluster {
  long Level = 0, Parent = -1, Child1 = -1, Child2 = -1, Number = 0, PermuPos = 0, BasisElement = 0;
  double Radius = 0, EVec[9] = {0}, EVal[3] = {0}, XMin[3] = {0}, XMax[3] = {0}, Centre[3] = {0};
  double DiagLength = 0;
};

// ComputeClusterData, src/hmat.cpp:13-150 (all dofs of a surface space are boundary dofs)
static void compute_cluster_data(const Mesh& m, const Space& sp, std::vector<double>& G,
                                 std::vector<std::array<double, 3>>& X) {
  int ndof = sp.ndof;
  G.assign(ndof, 0.0);
  X.assign(ndof, {0.0, 0.0, 0.0});
  std::vector<int> cnt(ndof, 0);
  for (int e = 0; e < m.nt; ++e)
    for (int a = 0; a < sp.nd; ++a) {
      int d = sp.el_dofs(e)[a];
      G[d] += m.area(e);
      cnt[d] += 1;
    }
  const double xhat[7][2] = {{1, 0}, {0, 1}, {0, 0}, {0.5, 0.5}, {0, 0.5}, {0.5, 0}, {1. / 3, 1. / 3}};
  for (int e = 0; e < m.nt; ++e) {
    double mip[7][3];
    for (int j = 0; j < 7; ++j) m.map(e, xhat[j][0], xhat[j][1], mip[j]);
    const int* dn = sp.el_dofs(e);
    int vertcounter = 0, edgecounter = 0;
    for (int ii = 0; ii < sp.nd; ++ii) {
      int clc = cnt[dn[ii]];
      if (clc > 2) { X[dn[ii]] = {mip[vertcounter][0], mip[vertcounter][1], mip[vertcounter][2]}; vertcounter++; }
      if (clc == 2) edgecounter++;
      if (clc == 1) X[dn[ii]] = {mip[6][0], mip[6][1], mip[6][2]};
    }
    // An element with one or two two-element dofs (at the border of an open surface or of a
    // region) takes each as its own edge: with edgeoffset 0 the reference's loop below would
    // not advance (src/hmat.cpp:122-138).  Closed surfaces never get there.
    int edgeoffset = std::max(1, edgecounter / 3);
    edgecounter = 0;
    for (int ii = 0; ii < sp.nd; ++ii) {
      int clc = cnt[dn[ii]];
      if (clc == 2) {
        for (int off = 0; off < edgeoffset; ++off)
          X[dn[ii + off]] = {mip[3 + edgecounter][0], mip[3 + edgecounter][1], mip[3 + edgecounter][2]};
        edgecounter++;
        ii += edgeoffset - 1;
      }
    }
  }
  for (int i = 0; i < ndof; ++i) G[i] /= (double)cnt[i];
}

// Rja_DivideCluster, src/hmat.cpp:155-374
static void divide_cluster(const std::vector<double>& G, const std::vector<std::array<double, 3>>& X,
                           int* NClusters, int IClu, std::vector<Cluster>& Clusters,
                           std::vector<int>& Permu, int leafsize) {
  int NClu = (int)Clusters[IClu].Number;
  int ClBegin = (int)Clusters[IClu].PermuPos;
  int ClEnd = ClBegin + NClu - 1;
  double Mom[10] = {0.};
  for (int i = ClBegin; i <= ClEnd; i++) {
    int j = Permu[i];
    Mom[0] += G[j];
    Mom[1] += G[j] * X[j][0];
    Mom[2] += G[j] * X[j][1];
    Mom[3] += G[j] * X[j][2];
    Mom[4] += G[j] * X[j][0] * X[j][0];
    Mom[5] += G[j] * X[j][0] * X[j][1];
    Mom[6] += G[j] * X[j][0] * X[j][2];
    Mom[7] += G[j] * X[j][1] * X[j][1];
    Mom[8] += G[j] * X[j][1] * X[j][2];
    Mom[9] += G[j] * X[j][2] * X[j][2];
  }
  double Centre[3] = {Mom[1] / Mom[0], Mom[2] / Mom[0], Mom[3] / Mom[0]};
  double A[9];
  A[0] = Mom[4] - Centre[0] * Mom[1];
  A[1] = Mom[5] - Centre[0] * Mom[2];
  A[2] = Mom[6] - Centre[0] * Mom[3];
  A[3] = A[1];
  A[4] = Mom[7] - Centre[1] * Mom[2];
  A[5] = Mom[8] - Centre[1] * Mom[3];
  A[6] = A[2];
  A[7] = A[5];
  A[8] = Mom[9] - Centre[2] * Mom[3];
  std::vector<double> W, evecs;
  jacobi_eigen(3, std::vector<double>(A, A + 9), W, evecs);
  for (int k = 0; k < 9; ++k) A[k] = evecs[k];

  int jMin = 0;
  double XMin[3] = {0, 0, 0}, XMax[3] = {0, 0, 0};
  double Radius = 0., DistMin = 0.;
  for (int i = ClBegin; i <= ClEnd; i++) {
    int j = Permu[i];
    double Diff[3] = {X[j][0] - Centre[0], X[j][1] - Centre[1], X[j][2] - Centre[2]};
    double Dist = std::sqrt(Diff[0] * Diff[0] + Diff[1] * Diff[1] + Diff[2] * Diff[2]);
    if (i == ClBegin || Dist < DistMin) { jMin = j; DistMin = Dist; }
    double XT[3];
    for (int r = 0; r < 3; ++r) XT[r] = A[3 * r + 0] * Diff[0] + A[3 * r + 1] * Diff[1] + A[3 * r + 2] * Diff[2];
    Radius = std::fmax(Radius, std::sqrt(XT[0] * XT[0] + XT[1] * XT[1] + XT[2] * XT[2]));
    if (i == ClBegin) {
      for (int r = 0; r < 3; ++r) { XMin[r] = XT[r]; XMax[r] = XT[r]; }
    } else {
      for (int r = 0; r < 3; ++r) { XMin[r] = std::fmin(XMin[r], XT[r]); XMax[r] = std::fmax(XMax[r], XT[r]); }
    }
  }
  double Diag[3] = {XMax[0] - XMin[0], XMax[1] - XMin[1], XMax[2] - XMin[2]};
  double DiagLength = std::sqrt(Diag[0] * Diag[0] + Diag[1] * Diag[1] + Diag[2] * Diag[2]);

  Cluster& C = Clusters[IClu];
  C.BasisElement = jMin;
  C.Radius = Radius;
  C.DiagLength = DiagLength;
  for (int k = 0; k < 3; k++) {
    C.EVal[k] = W[k]; C.XMin[k] = XMin[k]; C.XMax[k] = XMax[k]; C.Centre[k] = Centre[k];
  }
  for (int k = 0; k < 9; k++) C.EVec[k] = A[k];

  if (NClu <= leafsize) { C.Child1 = -1; C.Child2 = -1; return; }
  int Num1 = 0, Num2 = 0;
  int ICheck = ClBegin, IEnd = ClEnd;
  double Crit = Centre[0] * A[6] + Centre[1] * A[7] + Centre[2] * A[8];
  for (int i = 0; i < NClu; i++) {
    int j = Permu[ICheck];
    if (X[j][0] * A[6] + X[j][1] * A[7] + X[j][2] * A[8] >= Crit) { Num1 += 1; ICheck += 1; }
    else { Num2 += 1; Permu[ICheck] = Permu[IEnd]; Permu[IEnd] = j; IEnd -= 1; }
  }
  if (Num1 == 0 || Num2 == 0) { Clusters[IClu].Child1 = -1; Clusters[IClu].Child2 = -1; return; }
  Cluster cl1, cl2;
  int IClu1 = *NClusters;
  Clusters[IClu].Child1 = IClu1;
  cl1.Level = Clusters[IClu].Level + 1; cl1.Parent = IClu; cl1.Number = Num1; cl1.PermuPos = ClBegin;
  Clusters.push_back(cl1);
  int IClu2 = *NClusters + 1;
  Clusters[IClu].Child2 = IClu2;
  cl2.Level = Clusters[IClu].Level + 1; cl2.Parent = IClu; cl2.Number = Num2; cl2.PermuPos = ClBegin + Num1;
  Clusters.push_back(cl2);
  *NClusters += 2;
}

struct ClusterTree {
  std::vector<int> perm;  // mapcluster2glob
  std::vector<Cluster> cl;
  void build(const Mesh& m, const Space& sp, int leafsize) {
    std::vector<double> G;
    std::vector<std::array<double, 3>> X;
    compute_cluster_data(m, sp, G, X);
    int n = sp.ndof;
    perm.resize(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    Cluster c0; c0.Level = 0; c0.Parent = -1; c0.Number = n; c0.PermuPos = 0;
    cl.push_back(c0);
    int NClusters = 1, IClu = 0;
    do { divide_cluster(G, X, &NClusters, IClu, cl, perm, leafsize); IClu += 1; } while (IClu < NClusters);
  }
  int begin(long c) const { return (int)cl[c].PermuPos; }
  int size(long c) const { return (int)cl[c].Number; }
};

// Rja_AdmissiblePair, src/hmat.cpp:457-471
static bool admissible(const Cluster& c1, const Cluster& c2, double eta) {
  double diff[3] = {c1.Centre[0] - c2.Centre[0], c1.Centre[1] - c2.Centre[1], c1.Centre[2] - c2.Centre[2]};
  double dist = std::sqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
  dist = std::fmax(0., dist - c1.Radius - c2.Radius);
  return std::fmin(c1.Radius, c2.Radius) < eta * dist;
}

// ---------------------------------------------------------------------------------------
// H-matrix blocks
// ---------------------------------------------------------------------------------------
template <class T>
struct Block {
  long rowcl = 0, colcl = 0;
  bool near = true, fallback = false;
  std::vector<int> testdofs, trialdofs;
  std::vector<T> D;        // dense m x n row-major
  std::vector<T> U, V;     // U: m x R row-major, V: R x n row-major
  int rank = -1;
};

// HMatrix_help, src/hmat.cpp:587-612
template <class T>
static void partition(const ClusterTree& row, const ClusterTree& col, long i, long j, double eta,
                      std::vector<Block<T>>& out) {
  const Cluster& rc = row.cl[i];
  const Cluster& cc = col.cl[j];
  bool near;
  if (rc.Child1 == -1 || cc.Child1 == -1) near = true;
  else if (admissible(rc, cc, eta)) near = false;
  else {
    partition(row, col, rc.Child1, cc.Child1, eta, out);
    partition(row, col, rc.Child1, cc.Child2, eta, out);
    partition(row, col, rc.Child2, cc.Child1, eta, out);
    partition(row, col, rc.Child2, cc.Child2, eta, out);
    return;
  }
  Block<T> b;
  b.rowcl = i; b.colcl = j; b.near = near;
  b.testdofs.assign(row.perm.begin() + row.begin(i), row.perm.begin() + row.begin(i) + row.size(i));
  b.trialdofs.assign(col.perm.begin() + col.begin(j), col.perm.begin() + col.begin(j) + col.size(j));
  out.push_back(std::move(b));
}

struct FarFieldFailure {};

// ---------------------------------------------------------------------------------------
// Operator
// ---------------------------------------------------------------------------------------
template <class T>
struct Operator {
  Mesh mesh;
  Space trial, test;
  int trial_ev, test_ev;
  Kernel kernel;
  orc_params_t p;
  ClusterTree trial_ct, test_ct_own;
  const ClusterTree* test_ct = nullptr;
  std::vector<std::vector<int>> elems4dof, elems4dof2;
  std::vector<Block<T>> blocks;
  TrigRule irtrig;
  SSRule ss[3];

  Operator(int kid, double kappa) : kernel(kid, kappa) {}

  void setup(const orc_params_t& prm, bool same_space) {
    p = prm;
    trial_ct.build(mesh, trial, p.leafsize);
    if (same_space) test_ct = &trial_ct;
    else { test_ct_own.build(mesh, test, p.leafsize); test_ct = &test_ct_own; }
    elems4dof.assign(trial.ndof, {});
    for (int e = 0; e < mesh.nt; ++e)
      for (int a = 0; a < trial.nd; ++a) elems4dof[trial.el_dofs(e)[a]].push_back(e);
    elems4dof2.assign(test.ndof, {});
    for (int e = 0; e < mesh.nt; ++e)
      for (int a = 0; a < test.nd; ++a) elems4dof2[test.el_dofs(e)[a]].push_back(e);
    irtrig = trig_rule(p.intorder_regular);
    for (int c = 0; c < 3; ++c) ss[c] = ss_rule(c, p.intorder_singular);
  }

  void patches(const std::vector<int>& dofs, const std::vector<std::vector<int>>& e4d,
               std::vector<int>& patch) const {
    std::vector<int> tmp;
    for (int d : dofs) tmp.insert(tmp.end(), e4d[d].begin(), e4d[d].end());
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    patch.swap(tmp);
  }

  // singular-pair integration, the Integrate4D lambda (src/ngbem.cpp:451-497)
  void integrate4d(int ei, int ej, const SSRule& r, const int* vpermx, const int* vpermy,
                   bool identic, T* elmat) const {
    int di = trace_dim(test.kind, test_ev), dj = trace_dim(trial.kind, trial_ev);
    int ndi = test.nd, ndj = trial.nd;
    (void)di; (void)dj;
    const size_t npts = r.w.size();
    for (size_t k = 0; k < npts; ++k) {
      double xi, xe, yi, ye;
      if (identic) { xi = r.x0[k]; xe = r.x1[k]; yi = r.y0[k]; ye = r.y1[k]; }
      else {
        double lamx[3] = {1 - r.x0[k] - r.x1[k], r.x0[k], r.x1[k]};
        double lamy[3] = {1 - r.y0[k] - r.y1[k], r.y0[k], r.y1[k]};
        double plamx[3], plamy[3];
        for (int q = 0; q < 3; ++q) { plamx[vpermx[q]] = lamx[q]; plamy[vpermy[q]] = lamy[q]; }
        xi = plamx[0]; xe = plamx[1]; yi = plamy[0]; ye = plamy[1];
      }
      const MP gi = mesh.mp(ei, xi, xe), gj = mesh.mp(ej, yi, ye);
      T kv[3];
      kernel.eval<T>(gi.x, gj.x, gi.n, gj.n, kv);
      double fac = gi.detJ * gj.detJ * r.w[k];
      for (int c = 0; c < kernel.ncomp; ++c) kv[c] = fac * kv[c];
      double Si[ORC_MAXND][4], Sj[ORC_MAXND][4];
      eval_trace(mesh, test, test_ev, ei, xi, xe, Si);
      eval_trace(mesh, trial, trial_ev, ej, yi, ye, Sj);
      for (const Term& t : kernel.terms) {
        T kf = t.fac * kv[t.kc];
        for (int a = 0; a < ndi; ++a) {
          T ka = kf * Si[a][t.tec];
          for (int b = 0; b < ndj; ++b) elmat[a * ndj + b] += ka * Sj[b][t.trc];
        }
      }
    }
  }

  // CalcBlockMatrix, src/ngbem.cpp:373-738
  void calc_block(const std::vector<int>& trialdofs, const std::vector<int>& testdofs, T* matrix,
                  std::vector<int>& trialinv, std::vector<int>& testinv) const {
    int m = (int)testdofs.size(), n = (int)trialdofs.size();
    std::fill(matrix, matrix + (size_t)m * n, T(0.0));
    std::vector<int> patchi, patchj;
    for (int i = 0; i < m; ++i) testinv[testdofs[i]] = i;
    patches(testdofs, elems4dof2, patchi);
    for (int j = 0; j < n; ++j) trialinv[trialdofs[j]] = j;
    patches(trialdofs, elems4dof, patchj);

    const int ndi = test.nd, ndj = trial.nd;
    const int nq = (int)irtrig.w.size();
    // shapes of the regular rule per patch element
    std::vector<double> shi((size_t)patchi.size() * nq * 4 * ORC_MAXND), shj((size_t)patchj.size() * nq * 4 * ORC_MAXND);
    for (size_t i = 0; i < patchi.size(); ++i)
      for (int q = 0; q < nq; ++q)
        eval_trace(mesh, test, test_ev, patchi[i], irtrig.xi[q], irtrig.eta[q],
                   reinterpret_cast<double(*)[4]>(&shi[(i * nq + q) * 4 * ORC_MAXND]));
    for (size_t j = 0; j < patchj.size(); ++j)
      for (int q = 0; q < nq; ++q)
        eval_trace(mesh, trial, trial_ev, patchj[j], irtrig.xi[q], irtrig.eta[q],
                   reinterpret_cast<double(*)[4]>(&shj[(j * nq + q) * 4 * ORC_MAXND]));
    // per rule point: x, w |J|, the unit normal
    std::vector<double> pxi((size_t)patchi.size() * nq * 7), pyj((size_t)patchj.size() * nq * 7);
    auto point = [&](int e, int q, double* P) {
      const MP g = mesh.mp(e, irtrig.xi[q], irtrig.eta[q]);
      for (int c = 0; c < 3; ++c) { P[c] = g.x[c]; P[4 + c] = g.n[c]; }
      P[3] = irtrig.w[q] * g.detJ;
    };
    for (size_t i = 0; i < patchi.size(); ++i)
      for (int q = 0; q < nq; ++q) point(patchi[i], q, &pxi[(i * nq + q) * 7]);
    for (size_t j = 0; j < patchj.size(); ++j)
      for (int q = 0; q < nq; ++q) point(patchj[j], q, &pyj[(j * nq + q) * 7]);
    std::vector<T> kern((size_t)nq * nq), ks((size_t)nq * ndj);
    T elmat[ORC_MAXND * ORC_MAXND];
    for (size_t i = 0; i < patchi.size(); ++i)
      for (size_t j = 0; j < patchj.size(); ++j) {
        int ei = patchi[i], ej = patchj[j];
        const int* vi = &mesh.T[3 * ei];
        const int* vj = &mesh.T[3 * ej];
        for (int k = 0; k < ndi * ndj; ++k) elmat[k] = T(0.0);
        int ncommon = 0;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b)
            if (vi[a] == vj[b]) ncommon++;
        if (ncommon == 3) {
          int id[3] = {0, 1, 2};
          integrate4d(ei, ej, ss[0], id, id, true, elmat);
        } else if (ncommon == 2) {
          // edge table 0 1 | 1 2 | 2 0 (src/ngbem.cpp:569)
          const int edges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
          int cex = 0, cey = 0;
          bool found = false;
          for (int cx = 0; cx < 3 && !found; cx++)
            for (int cy = 0; cy < 3; cy++) {
              int ex0 = vi[edges[cx][0]], ex1 = vi[edges[cx][1]];
              int ey0 = vj[edges[cy][0]], ey1 = vj[edges[cy][1]];
              if (std::min(ex0, ex1) == std::min(ey0, ey1) && std::max(ex0, ex1) == std::max(ey0, ey1)) {
                cex = cx; cey = cy; found = true; break;
              }
            }
          int vpermx[3] = {edges[cex][0], edges[cex][1], -1};
          vpermx[2] = 3 - vpermx[0] - vpermx[1];
          int vpermy[3] = {edges[cey][1], edges[cey][0], -1};
          vpermy[2] = 3 - vpermy[0] - vpermy[1];
          integrate4d(ei, ej, ss[1], vpermx, vpermy, false, elmat);
        } else if (ncommon == 1) {
          int cvx = -1, cvy = -1;
          for (int cx = 0; cx < 3 && cvx < 0; cx++)
            for (int cy = 0; cy < 3; cy++)
              if (vi[cx] == vj[cy]) { cvx = cx; cvy = cy; break; }
          int vpermx[3] = {cvx, (cvx + 1) % 3, (cvx + 2) % 3};
          int vpermy[3] = {cvy, (cvy + 1) % 3, (cvy + 2) % 3};
          integrate4d(ei, ej, ss[2], vpermx, vpermy, false, elmat);
        } else {
          // disjoint panels, src/ngbem.cpp:680-727
          for (const Term& t : kernel.terms) {
            for (int ix = 0; ix < nq; ++ix)
              for (int iy = 0; iy < nq; ++iy) {
                const double* X = &pxi[(i * nq + ix) * 7];
                const double* Y = &pyj[(j * nq + iy) * 7];
                T kv[3];
                kernel.eval<T>(X, Y, X + 4, Y + 4, kv);
                double fac = X[3] * Y[3];
                kern[ix * nq + iy] = t.fac * fac * kv[t.kc];
              }
            // kernel_shapesj = kernel_ixiy * Trans(shapesj1); elmat += shapesi1 * kernel_shapesj
            for (int ix = 0; ix < nq; ++ix)
              for (int b = 0; b < ndj; ++b) {
                T s = T(0.0);
                for (int iy = 0; iy < nq; ++iy) s += kern[ix * nq + iy] * shj[(j * nq + iy) * 4 * ORC_MAXND + b * 4 + t.trc];
                ks[ix * ndj + b] = s;
              }
            for (int a = 0; a < ndi; ++a)
              for (int b = 0; b < ndj; ++b) {
                T s = T(0.0);
                for (int ix = 0; ix < nq; ++ix) s += shi[(i * nq + ix) * 4 * ORC_MAXND + a * 4 + t.tec] * ks[ix * ndj + b];
                elmat[a * ndj + b] += s;
              }
          }
        }
        const int* dni = test.el_dofs(ei);
        const int* dnj = trial.el_dofs(ej);
        for (int ii = 0; ii < ndi; ++ii)
          for (int jj = 0; jj < ndj; ++jj)
            if (trialinv[dnj[jj]] != -1 && testinv[dni[ii]] != -1)
              matrix[(size_t)testinv[dni[ii]] * n + trialinv[dnj[jj]]] += elmat[ii * ndj + jj];
      }
    for (int i = 0; i < m; ++i) testinv[testdofs[i]] = -1;
    for (int j = 0; j < n; ++j) trialinv[trialdofs[j]] = -1;
  }

  // CalcFarFieldBlock, src/ngbem.cpp:743-1163
  void calc_farfield(Block<T>& blk, std::vector<int>& trialinv, std::vector<int>& testinv,
                     std::vector<char>& vmark) const {
    const auto& trialdofs = blk.trialdofs;
    const auto& testdofs = blk.testdofs;
    std::vector<int> patchi, patchj;
    patches(testdofs, elems4dof2, patchi);
    patches(trialdofs, elems4dof, patchj);
    const int nq = (int)irtrig.w.size();
    // common-vertex test (src/ngbem.cpp:839-842); trial and test live on one mesh here
    for (int e : patchi)
      for (int k = 0; k < 3; ++k) vmark[mesh.T[3 * e + k]] = 1;
    bool shared = false;
    for (int e : patchj)
      for (int k = 0; k < 3; ++k)
        if (vmark[mesh.T[3 * e + k]]) shared = true;
    for (int e : patchi)
      for (int k = 0; k < 3; ++k) vmark[mesh.T[3 * e + k]] = 0;
    if (shared) throw FarFieldFailure();

    const size_t M = patchi.size() * nq, N = patchj.size() * nq;
    std::vector<double> xi(3 * M), yj(3 * N), nxi(3 * M), nyj(3 * N), wxi(M), wyj(N);
    for (size_t i = 0; i < patchi.size(); ++i)
      for (int q = 0; q < nq; ++q) {
        size_t r = i * nq + q;
        const MP g = mesh.mp(patchi[i], irtrig.xi[q], irtrig.eta[q]);
        for (int c = 0; c < 3; ++c) { xi[3 * r + c] = g.x[c]; nxi[3 * r + c] = g.n[c]; }
        wxi[r] = irtrig.w[q] * g.detJ;
      }
    for (size_t j = 0; j < patchj.size(); ++j)
      for (int q = 0; q < nq; ++q) {
        size_t r = j * nq + q;
        const MP g = mesh.mp(patchj[j], irtrig.xi[q], irtrig.eta[q]);
        for (int c = 0; c < 3; ++c) { yj[3 * r + c] = g.x[c]; nyj[3 * r + c] = g.n[c]; }
        wyj[r] = irtrig.w[q] * g.detJ;
      }
    const size_t p = std::min(M, N);
    auto getrow = [&](size_t i, T* row, int comp) {
      T kv[3];
      for (size_t j = 0; j < N; ++j) { kernel.eval<T>(&xi[3 * i], &yj[3 * j], &nxi[3 * i], &nyj[3 * j], kv); row[j] = kv[comp]; }
    };
    auto getcol = [&](size_t j, T* col, int comp) {
      T kv[3];
      for (size_t i = 0; i < M; ++i) { kernel.eval<T>(&xi[3 * i], &yj[3 * j], &nxi[3 * i], &nyj[3 * j], kv); col[i] = kv[comp]; }
    };
    int ncomp = 0;
    for (const Term& t : kernel.terms) ncomp = std::max(ncomp, t.kc + 1);
    // Us[c]: M x rank (stored column-wise: col k contiguous), Vs[c]: rank x N row-wise
    std::vector<std::vector<T>> Us(ncomp), Vs(ncomp);
    std::vector<size_t> ranks(ncomp);
    for (int comp = 0; comp < ncomp; ++comp) {
      std::vector<T> U, V;  // U col-major (k*M + i), V row-major (k*N + j)
      size_t ik = 0, jk = 0, ikm1 = 0, jkm1 = N + 1, rank = p;
      const double eps = p_eps();
      double norm2 = 0.;
      for (size_t k = 0; k < p; k++) {
        if ((k % 20) == 0) { U.resize((k + 20) * M); V.resize((k + 20) * N); }
        T* Vk = &V[k * N];
        getrow(ik, Vk, comp);
        for (size_t l = 0; l < k; ++l) {
          T u = U[l * M + ik];
          const T* Vl = &V[l * N];
          for (size_t j = 0; j < N; ++j) Vk[j] -= Vl[j] * u;
        }
        double vkj = 0.;
        for (size_t j = 0; j < N; j++)
          if (std::abs(Vk[j]) > vkj && j != jkm1) { vkj = std::abs(Vk[j]); jk = j; }
        if (vkj == 0.) { rank = k; break; }
        T sc = std::sqrt(vkj) / Vk[jk];
        for (size_t j = 0; j < N; ++j) Vk[j] *= sc;
        T* Uk = &U[k * M];
        getcol(jk, Uk, comp);
        for (size_t l = 0; l < k; ++l) {
          T v = V[l * N + jk];
          const T* Ul = &U[l * M];
          for (size_t i = 0; i < M; ++i) Uk[i] -= Ul[i] * v;
        }
        double isq = 1. / std::sqrt(vkj);
        for (size_t i = 0; i < M; ++i) Uk[i] *= isq;
        double uik = 0.;
        for (size_t i = 0; i < M; i++)
          if (std::abs(Uk[i]) > uik && i != ikm1) { uik = std::abs(Uk[i]); ik = i; }
        double nv = 0., nu = 0.;
        for (size_t j = 0; j < N; ++j) nv += std::norm(Vk[j]);
        for (size_t i = 0; i < M; ++i) nu += std::norm(Uk[i]);
        double norm_k = std::sqrt(nv) * std::sqrt(nu);
        norm2 += norm_k * norm_k;
        for (size_t l = 0; l < k; l++) {
          T dv = T(0.0), du = T(0.0);
          const T* Vl = &V[l * N];
          const T* Ul = &U[l * M];
          for (size_t j = 0; j < N; ++j) dv += Vk[j] * conj_(Vl[j]);
          for (size_t i = 0; i < M; ++i) du += Uk[i] * conj_(Ul[i]);
          norm2 += 2. * re_(conj_(dv) * du);
        }
        ikm1 = ik;
        jkm1 = jk;
        if (norm_k < eps * std::sqrt(norm2)) { rank = k + 1; break; }
      }
      U.resize(rank * M); V.resize(rank * N);
      for (size_t k = 0; k < rank; ++k) {
        for (size_t i = 0; i < M; ++i) U[k * M + i] *= wxi[i];
        for (size_t j = 0; j < N; ++j) V[k * N + j] *= wyj[j];
      }
      Us[comp].swap(U); Vs[comp].swap(V); ranks[comp] = rank;
    }
    // projection onto dofs, src/ngbem.cpp:1051-1160
    std::vector<size_t> off;
    size_t R = 0;
    for (const Term& t : kernel.terms) { off.push_back(R); R += ranks[t.kc]; }
    const int m = (int)testdofs.size(), n = (int)trialdofs.size();
    blk.U.assign((size_t)m * R, T(0.0));
    blk.V.assign(R * (size_t)n, T(0.0));
    blk.rank = (int)R;
    for (int i = 0; i < m; ++i) testinv[testdofs[i]] = i;
    for (int j = 0; j < n; ++j) trialinv[trialdofs[j]] = j;
    for (size_t ie = 0; ie < patchi.size(); ++ie) {
      int e = patchi[ie];
      const int* dn = test.el_dofs(e);
      for (int q = 0; q < nq; ++q) {
        double S[ORC_MAXND][4];
        eval_trace(mesh, test, test_ev, e, irtrig.xi[q], irtrig.eta[q], S);
        size_t row = ie * nq + q;
        for (size_t t = 0; t < kernel.terms.size(); ++t) {
          const Term& tm = kernel.terms[t];
          size_t rk = ranks[tm.kc];
          for (int a = 0; a < test.nd; ++a) {
            int li = testinv[dn[a]];
            if (li == -1) continue;
            for (size_t k = 0; k < rk; ++k)
              blk.U[(size_t)li * R + off[t] + k] += tm.fac * (S[a][tm.tec] * Us[tm.kc][k * M + row]);
          }
        }
      }
    }
    for (size_t je = 0; je < patchj.size(); ++je) {
      int e = patchj[je];
      const int* dn = trial.el_dofs(e);
      for (int q = 0; q < nq; ++q) {
        double S[ORC_MAXND][4];
        eval_trace(mesh, trial, trial_ev, e, irtrig.xi[q], irtrig.eta[q], S);
        size_t col = je * nq + q;
        for (size_t t = 0; t < kernel.terms.size(); ++t) {
          const Term& tm = kernel.terms[t];
          size_t rk = ranks[tm.kc];
          for (int b = 0; b < trial.nd; ++b) {
            int lj = trialinv[dn[b]];
            if (lj == -1) continue;
            for (size_t k = 0; k < rk; ++k)
              blk.V[(off[t] + k) * n + lj] += S[b][tm.trc] * Vs[tm.kc][k * N + col];
          }
        }
      }
    }
    for (int i = 0; i < m; ++i) testinv[testdofs[i]] = -1;
    for (int j = 0; j < n; ++j) trialinv[trialdofs[j]] = -1;
  }
  double p_eps() const { return p.eps; }

  int nthreads() const {
    int nt = p.nthreads > 0 ? p.nthreads : (int)std::thread::hardware_concurrency();
    return std::max(1, nt);
  }

  // CalcHMatrix, src/ngbem.cpp:118-157 (dynamic chunks, ~TasksPerThread(4))
  void assemble() {
    blocks.clear();
    partition<T>(*test_ct, trial_ct, 0, 0, p.eta, blocks);
    int nth = nthreads();
    size_t nb = blocks.size();
    size_t chunk = std::max<size_t>(1, nb / (4 * (size_t)nth));
    std::atomic<size_t> next(0);
    auto worker = [&]() {
      std::vector<int> trialinv(trial.ndof, -1), testinv(test.ndof, -1);
      std::vector<char> vmark(mesh.nv, 0);
      for (;;) {
        size_t s = next.fetch_add(chunk);
        if (s >= nb) break;
        size_t e = std::min(nb, s + chunk);
        for (size_t k = s; k < e; ++k) {
          Block<T>& b = blocks[k];
          if (!b.near) {
            try { calc_farfield(b, trialinv, testinv, vmark); continue; }
            catch (FarFieldFailure&) { b.fallback = true; }
          }
          b.D.resize(b.testdofs.size() * b.trialdofs.size());
          calc_block(b.trialdofs, b.testdofs, b.D.data(), trialinv, testinv);
        }
      }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) th.emplace_back(worker);
    for (auto& t : th) t.join();
  }

  // HMatrix::MultAdd / MultTransAdd (src/hmat.cpp:473-515, 527-565, 647-666)
  void mult(bool trans, const T* x, T* y) const {
    size_t H = trans ? trial.ndof : test.ndof;
    int nth = nthreads();
    size_t nb = blocks.size();
    std::vector<std::vector<T>> ys(nth, std::vector<T>(H, T(0.0)));
    auto worker = [&](int t) {
      std::vector<T> xp, yp, tmp;
      size_t s = nb * t / nth, e = nb * (t + 1) / nth;
      T* Y = ys[t].data();
      for (size_t k = s; k < e; ++k) {
        const Block<T>& b = blocks[k];
        const auto& in = trans ? b.testdofs : b.trialdofs;
        const auto& out = trans ? b.trialdofs : b.testdofs;
        size_t m = b.testdofs.size(), n = b.trialdofs.size();
        xp.resize(in.size()); yp.assign(out.size(), T(0.0));
        for (size_t i = 0; i < in.size(); ++i) xp[i] = x[in[i]];
        if (b.rank < 0) {
          if (!trans) {
            for (size_t i = 0; i < m; ++i) { T s2 = T(0.0); const T* row = &b.D[i * n]; for (size_t j = 0; j < n; ++j) s2 += row[j] * xp[j]; yp[i] = s2; }
          } else {
            for (size_t i = 0; i < m; ++i) { const T* row = &b.D[i * n]; for (size_t j = 0; j < n; ++j) yp[j] += row[j] * xp[i]; }
          }
        } else {
          size_t R = b.rank;
          tmp.assign(R, T(0.0));
          if (!trans) {
            for (size_t r = 0; r < R; ++r) { T s2 = T(0.0); for (size_t j = 0; j < n; ++j) s2 += b.V[r * n + j] * xp[j]; tmp[r] = s2; }
            for (size_t i = 0; i < m; ++i) { T s2 = T(0.0); for (size_t r = 0; r < R; ++r) s2 += b.U[i * R + r] * tmp[r]; yp[i] = s2; }
          } else {
            for (size_t i = 0; i < m; ++i) for (size_t r = 0; r < R; ++r) tmp[r] += b.U[i * R + r] * xp[i];
            for (size_t r = 0; r < R; ++r) for (size_t j = 0; j < n; ++j) yp[j] += b.V[r * n + j] * tmp[r];
          }
        }
        for (size_t i = 0; i < out.size(); ++i) Y[out[i]] += yp[i];
      }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) th.emplace_back(worker, t);
    for (auto& t : th) t.join();
    for (size_t i = 0; i < H; ++i) {
      T s2 = T(0.0);
      for (int t = 0; t < nth; ++t) s2 += ys[t][i];
      y[i] = s2;
    }
  }
};

struct OpHandle {
  bool complex_valued;
  void* op;
};

template <class T>
static Operator<T>* make_op(int kernel, double kappa, int nv, const double* xyz, int nt, const int* tri,
                            int trial_kind, int trial_eval, int trial_dual, int test_kind, int test_eval,
                            int test_dual, const orc_params_t* params) {
  auto* op = new Operator<T>(kernel, kappa);
  op->mesh.build(nv, xyz, nt, tri);
  op->trial.build(op->mesh, trial_kind, trial_dual != 0);
  op->test.build(op->mesh, test_kind, test_dual != 0);
  op->trial_ev = trial_eval;
  op->test_ev = test_eval;
  bool same = trial_kind == test_kind && trial_dual == test_dual;
  op->setup(*params, same);
  return op;
}

}  // namespace orc

using namespace orc;

extern "C" {

int orc_mesh_edges(int nv, int nt, const int* tri, int* edges, int* tri_edges) {
  // edge key (min,max) -> id, assigned by first appearance
  std::vector<std::vector<std::pair<int, int>>> adj(nv);
  int ne = 0;
  for (int e = 0; e < nt; ++e)
    for (int k = 0; k < 3; ++k) {
      int a = tri[3 * e + k], b = tri[3 * e + (k + 1) % 3];
      int lo = std::min(a, b), hi = std::max(a, b);
      int id = -1;
      for (auto& pr : adj[lo]) if (pr.first == hi) { id = pr.second; break; }
      if (id < 0) {
        id = ne++;
        adj[lo].push_back({hi, id});
        edges[2 * id] = lo; edges[2 * id + 1] = hi;
      }
      tri_edges[3 * e + k] = id;
    }
  return ne;
}

int orc_trig_rule(int order, double* xi, double* eta, double* w) {
  TrigRule r = trig_rule(order);
  for (size_t k = 0; k < r.w.size(); ++k) { xi[k] = r.xi[k]; eta[k] = r.eta[k]; w[k] = r.w[k]; }
  return (int)r.w.size();
}

int orc_ss_rule(int cls, int order, double* x0, double* x1, double* y0, double* y1, double* w) {
  SSRule r = ss_rule(cls, order);
  for (size_t k = 0; k < r.w.size(); ++k) { x0[k] = r.x0[k]; x1[k] = r.x1[k]; y0[k] = r.y0[k]; y1[k] = r.y1[k]; w[k] = r.w[k]; }
  return (int)r.w.size();
}

int orc_cluster_tree(int nv, const double* xyz, int nt, const int* tri, int kind, int leafsize,
                     int* perm, int max_clusters, long* ci, double* cd) {
  Mesh m; m.build(nv, xyz, nt, tri);
  Space sp; sp.build(m, kind, false);
  ClusterTree ct; ct.build(m, sp, leafsize);
  for (int i = 0; i < sp.ndof; ++i) perm[i] = ct.perm[i];
  int nc = (int)ct.cl.size();
  if (nc > max_clusters) return -1;
  for (int c = 0; c < nc; ++c) {
    const Cluster& C = ct.cl[c];
    long* I = ci + 7 * c;
    I[0] = C.Level; I[1] = C.Parent; I[2] = C.Child1; I[3] = C.Child2; I[4] = C.Number; I[5] = C.PermuPos; I[6] = C.BasisElement;
    double* D = cd + 23 * c;
    D[0] = C.Radius;
    for (int k = 0; k < 9; ++k) D[1 + k] = C.EVec[k];
    for (int k = 0; k < 3; ++k) { D[10 + k] = C.EVal[k]; D[13 + k] = C.XMin[k]; D[16 + k] = C.XMax[k]; D[19 + k] = C.Centre[k]; }
    D[22] = C.DiagLength;
  }
  return nc;
}

void* orc_operator_create(int kernel, double kappa, int nv, const double* xyz, int nt, const int* tri,
                          int trial_kind, int trial_eval, int trial_dual, int test_kind, int test_eval,
                          int test_dual, const orc_params_t* params) {
  try {
    auto* h = new OpHandle;
    h->complex_valued = kernel >= ORC_HELMHOLTZ_SL;
    if (h->complex_valued) {
      auto* op = make_op<cplx>(kernel, kappa, nv, xyz, nt, tri, trial_kind, trial_eval, trial_dual, test_kind, test_eval, test_dual, params);
      op->assemble();
      h->op = op;
    } else {
      auto* op = make_op<double>(kernel, kappa, nv, xyz, nt, tri, trial_kind, trial_eval, trial_dual, test_kind, test_eval, test_dual, params);
      op->assemble();
      h->op = op;
    }
    return h;
  } catch (...) {
    return nullptr;
  }
}

extern "C++" {
template <class T>
static void fill_info(Operator<T>* op, long* info) {
  long nnear = 0, nfar = 0, nze = 0, nfb = 0, maxr = 0, sumr = 0;
  for (auto& b : op->blocks) {
    long m = (long)b.testdofs.size(), n = (long)b.trialdofs.size();
    if (b.rank < 0) { nnear += b.near ? 1 : 0; nze += m * n; nfb += b.fallback ? 1 : 0; }
    else { nfar++; nze += (long)b.rank * (m + n); maxr = std::max<long>(maxr, b.rank); sumr += b.rank; }
  }
  info[0] = std::is_same<T, cplx>::value;
  info[1] = op->test.ndof; info[2] = op->trial.ndof;
  info[3] = (long)op->blocks.size(); info[4] = nnear; info[5] = nfar; info[6] = nze;
  info[7] = nfb; info[8] = maxr; info[9] = sumr;
}
}  // extern "C++"

int orc_operator_info(void* h_, long* info) {
  auto* h = (OpHandle*)h_;
  if (h->complex_valued) fill_info((Operator<cplx>*)h->op, info);
  else fill_info((Operator<double>*)h->op, info);
  return 0;
}

int orc_operator_mult(void* h_, int trans, const double* x, double* y) {
  auto* h = (OpHandle*)h_;
  if (h->complex_valued) ((Operator<cplx>*)h->op)->mult(trans != 0, (const cplx*)x, (cplx*)y);
  else ((Operator<double>*)h->op)->mult(trans != 0, x, y);
  return 0;
}

int orc_operator_mult_multi(void* h_, int nrhs, const double* x, double* y) {
  auto* h = (OpHandle*)h_;
  long info[10];
  orc_operator_info(h_, info);
  long H = info[1], W = info[2];
  int s = h->complex_valued ? 2 : 1;
  for (int r = 0; r < nrhs; ++r) orc_operator_mult(h_, 0, x + (size_t)r * W * s, y + (size_t)r * H * s);
  return 0;
}

int orc_operator_blocks(void* h_, int* rowcl, int* colcl, int* near, int* rank, int* fallback) {
  auto* h = (OpHandle*)h_;
  auto fill = [&](auto* op) {
    size_t k = 0;
    for (auto& b : op->blocks) {
      rowcl[k] = (int)b.rowcl; colcl[k] = (int)b.colcl; near[k] = b.near ? 1 : 0;
      rank[k] = b.rank; fallback[k] = b.fallback ? 1 : 0; ++k;
    }
  };
  if (h->complex_valued) fill((Operator<cplx>*)h->op);
  else fill((Operator<double>*)h->op);
  return 0;
}

extern "C++" {
template <class T>
static void to_dense(Operator<T>* op, T* out) {
  size_t H = op->test.ndof, W = op->trial.ndof;
  std::fill(out, out + H * W, T(0.0));
  for (auto& b : op->blocks) {
    size_t m = b.testdofs.size(), n = b.trialdofs.size();
    for (size_t i = 0; i < m; ++i)
      for (size_t j = 0; j < n; ++j) {
        T v;
        if (b.rank < 0) v = b.D[i * n + j];
        else { v = T(0.0); for (int r = 0; r < b.rank; ++r) v += b.U[i * b.rank + r] * b.V[r * n + j]; }
        out[(size_t)b.testdofs[i] * W + b.trialdofs[j]] += v;
      }
  }
}
}  // extern "C++"

int orc_operator_to_dense(void* h_, double* out) {
  auto* h = (OpHandle*)h_;
  if (h->complex_valued) to_dense((Operator<cplx>*)h->op, (cplx*)out);
  else to_dense((Operator<double>*)h->op, out);
  return 0;
}

extern "C++" {
template <class T>
static void dense_all(Operator<T>* op, T* out) {
  std::vector<int> trialdofs(op->trial.ndof), testdofs(op->test.ndof);
  for (int i = 0; i < op->trial.ndof; ++i) trialdofs[i] = i;
  for (int i = 0; i < op->test.ndof; ++i) testdofs[i] = i;
  std::vector<int> ti(op->trial.ndof, -1), si(op->test.ndof, -1);
  op->calc_block(trialdofs, testdofs, out, ti, si);
  delete op;
}
}  // extern "C++"

int orc_dense_matrix(int kernel, double kappa, int nv, const double* xyz, int nt, const int* tri,
                     int trial_kind, int trial_eval, int trial_dual, int test_kind, int test_eval,
                     int test_dual, const orc_params_t* params, double* out) {
  orc_params_t p = *params;
  p.leafsize = INT_MAX; p.eta = 0.0;
  if (kernel >= ORC_HELMHOLTZ_SL)
    dense_all(make_op<cplx>(kernel, kappa, nv, xyz, nt, tri, trial_kind, trial_eval, trial_dual, test_kind, test_eval, test_dual, &p), (cplx*)out);
  else
    dense_all(make_op<double>(kernel, kappa, nv, xyz, nt, tri, trial_kind, trial_eval, trial_dual, test_kind, test_eval, test_dual, &p), out);
  return 0;
}

void orc_operator_destroy(void* h_) {
  auto* h = (OpHandle*)h_;
  if (!h) return;
  if (h->complex_valued) delete (Operator<cplx>*)h->op;
  else delete (Operator<double>*)h->op;
  delete h;
}

extern "C++" {
// PotentialCF::T_Evaluate (src/ngbem.cpp:1187-1238): for each point, every element of the trial
// space, the evaluator applied to the element vector at the regular rule's points, and the
// kernel terms (term factors are not applied there, as in the reference)
template <class T>
static void potential_t(int kernel, double kappa, const Mesh& m, const Space& sp, int ev, int intorder,
                        const T* density, int npts, const double* pts, const double* normals, T* out) {
  Kernel K(kernel, kappa);
  TrigRule r = trig_rule(intorder);
  const int dim = trace_dim(sp.kind, ev);
  std::fill(out, out + (size_t)npts * dim, T(0));
  const double nz[3] = {0.0, 0.0, 0.0};
  for (int p = 0; p < npts; ++p) {
    const double* x = pts + 3 * (size_t)p;
    const double* nx = normals ? normals + 3 * (size_t)p : nz;
    for (int e = 0; e < m.nt; ++e) {
      for (size_t q = 0; q < r.w.size(); ++q) {
        double S[ORC_MAXND][4] = {{0}};
        eval_trace(m, sp, ev, e, r.xi[q], r.eta[q], S);
        T vals[4] = {T(0), T(0), T(0), T(0)};
        for (int a = 0; a < sp.nd; ++a)
          for (int c = 0; c < dim; ++c) vals[c] += density[sp.el_dofs(e)[a]] * S[a][c];
        const MP g = m.mp(e, r.xi[q], r.eta[q]);
        const double w = r.w[q] * g.detJ;
        T kv[3];
        K.eval<T>(x, g.x, nx, g.n, kv);
        for (const Term& t : K.terms) out[(size_t)p * dim + t.tec] += w * kv[t.kc] * vals[t.trc];
      }
    }
  }
}
}

int orc_potential(int kernel, double kappa, int nv, const double* xyz, int nt, const int* tri, int trial_kind,
                  int trial_eval, int trial_dual, int intorder, const double* density, int npts, const double* pts,
                  const double* normals, double* out) {
  Mesh m;
  m.build(nv, xyz, nt, tri);
  Space sp;
  sp.build(m, trial_kind, trial_dual != 0);
  if (kernel >= ORC_HELMHOLTZ_SL)
    potential_t<cplx>(kernel, kappa, m, sp, trial_eval, intorder, (const cplx*)density, npts, pts, normals,
                      (cplx*)out);
  else
    potential_t<double>(kernel, kappa, m, sp, trial_eval, intorder, density, npts, pts, normals, out);
  return 0;
}

int orc_set_geometry(int order, int nt, const double* nodes) {
  if (order < 1 || order > 4 || nt < 0 || (order > 1 && !nodes)) return -1;
  g_geo_order = order;
  g_geo_nt = nt;
  if (order == 1) g_geo_nodes.clear();
  else g_geo_nodes.assign(nodes, nodes + (size_t)nt * 3 * (order + 1) * (order + 2) / 2);
  return 0;
}

int orc_eval_trace(int nv, const double* xyz, int nt, const int* tri, int kind, int ev, int e, double xi,
                   double eta, double* out, int* dofs) {
  Mesh m; m.build(nv, xyz, nt, tri);
  Space sp; sp.build(m, kind, false);
  double S[ORC_MAXND][4] = {{0.0}};
  eval_trace(m, sp, ev, e, xi, eta, S);
  for (int a = 0; a < ORC_MAXND; ++a)
    for (int c = 0; c < 4; ++c) out[4 * a + c] = a < sp.nd ? S[a][c] : 0.0;
  for (int a = 0; a < sp.nd; ++a) dofs[a] = sp.el_dofs(e)[a];
  return sp.nd;
}

int orc_mass_matrix(int nv, const double* xyz, int nt, const int* tri, int trial_kind, int test_kind,
                    int order, double* out) {
  Mesh m; m.build(nv, xyz, nt, tri);
  Space tr, te; tr.build(m, trial_kind, false); te.build(m, test_kind, false);
  TrigRule r = trig_rule(order);
  std::fill(out, out + (size_t)te.ndof * tr.ndof, 0.0);
  int evtr = ORC_EV_ID, evte = ORC_EV_ID;
  int dim = trace_dim(tr.kind, evtr);
  for (int e = 0; e < m.nt; ++e)
    for (size_t q = 0; q < r.w.size(); ++q) {
      double Si[ORC_MAXND][4], Sj[ORC_MAXND][4];
      eval_trace(m, te, evte, e, r.xi[q], r.eta[q], Si);
      eval_trace(m, tr, evtr, e, r.xi[q], r.eta[q], Sj);
      double w = r.w[q] * m.mp(e, r.xi[q], r.eta[q]).detJ;
      for (int a = 0; a < te.nd; ++a)
        for (int b = 0; b < tr.nd; ++b) {
          double s = 0;
          for (int c = 0; c < dim; ++c) s += Si[a][c] * Sj[b][c];
          out[(size_t)te.el_dofs(e)[a] * tr.ndof + tr.el_dofs(e)[b]] += w * s;
        }
    }
  return 0;
}

}  // extern "C"
