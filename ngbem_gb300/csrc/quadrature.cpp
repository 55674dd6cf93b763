// Quadrature rules of the operator path.
//  - Gauss-Legendre / Gauss-Jacobi rules by the Golub-Welsch method (eigen-decomposition
//    of the Jacobi matrix of the orthogonal polynomials).
//  - "order p" segment rule: n = p/2 + 1 points (exact to degree 2n-1 >= p), as the
//    reference's IntegrationRule(ET_SEGM, p) calls expect (src/intrules.cpp:15-16).
//  - triangle rule: collapsed (Stroud conical) product of Gauss-Jacobi(1,0) and
//    Gauss-Legendre, n = p/2 + 1 each, stands in for IntegrationRule(ET_TRIG, p)
//    (src/ngbem.cpp:391); n*n points, exact to degree p.
//  - Sauter-Schwab rules for identical panels, common edges and common vertices
//    (src/intrules.cpp:13-136): the Duffy maps of Sauter & Schwab, "Boundary Element
//    Methods", section 5.2, on the hexahedron tensor rule times the segment rule.
#include <algorithm>
#include <cmath>

#include "host.hpp"

namespace bem {

// Cyclic Jacobi eigen solver for small symmetric matrices.  Eigenvalues ascending; row k
// of evecs is the eigenvector of eigenvalue k, normalised so that its largest-magnitude
// component (first index on ties) is positive.  Only + - * / sqrt are used, so results are
// reproducible bit for bit on any IEEE host compiled without FMA contraction.
void sym_eigen(int n, std::vector<double> A, std::vector<double>& evals, std::vector<double>& evecs) {
  std::vector<double> Vm(n * n, 0.0);
  for (int i = 0; i < n; ++i) Vm[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off == 0.0) break;
    for (int p = 0; p < n - 1; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (apq == 0.0) continue;
        const double tau = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t);
        const double s = t * c;
        for (int r = 0; r < n; ++r) {
          if (r == p || r == q) continue;
          const double arp = A[r * n + p], arq = A[r * n + q];
          const double nrp = c * arp - s * arq;
          const double nrq = s * arp + c * arq;
          A[r * n + p] = nrp;
          A[p * n + r] = nrp;
          A[r * n + q] = nrq;
          A[q * n + r] = nrq;
        }
        A[p * n + p] = A[p * n + p] - t * apq;
        A[q * n + q] = A[q * n + q] + t * apq;
        A[p * n + q] = 0.0;
        A[q * n + p] = 0.0;
        for (int r = 0; r < n; ++r) {
          const double vrp = Vm[r * n + p], vrq = Vm[r * n + q];
          Vm[r * n + p] = c * vrp - s * vrq;
          Vm[r * n + q] = s * vrp + c * vrq;
        }
      }
    }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
  evals.assign(n, 0.0);
  evecs.assign(n * n, 0.0);
  for (int k = 0; k < n; ++k) {
    const int col = order[k];
    evals[k] = A[col * n + col];
    int big = 0;
    for (int r = 1; r < n; ++r)
      if (std::fabs(Vm[r * n + col]) > std::fabs(Vm[big * n + col])) big = r;
    const double sg = Vm[big * n + col] < 0.0 ? -1.0 : 1.0;
    for (int r = 0; r < n; ++r) evecs[k * n + r] = sg * Vm[r * n + col];
  }
}

// The same cyclic Jacobi iteration for n = 3 on stack arrays (the cluster tree calls it once
// per cluster): identical operations in the identical order, so identical bits, without the
// heap traffic of the general version.
void sym_eigen3(const double* A0, double* evals, double* evecs) {
  double A[9], Vm[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int k = 0; k < 9; ++k) A[k] = A0[k];
  for (int sweep = 0; sweep < 64; ++sweep) {
    const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    if (off == 0.0) break;
    for (int p = 0; p < 2; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        const double apq = A[p * 3 + q];
        if (apq == 0.0) continue;
        const double tau = (A[q * 3 + q] - A[p * 3 + p]) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t);
        const double s = t * c;
        const int r = 3 - p - q;  // the one row that is neither p nor q
        const double arp = A[r * 3 + p], arq = A[r * 3 + q];
        const double nrp = c * arp - s * arq;
        const double nrq = s * arp + c * arq;
        A[r * 3 + p] = nrp;
        A[p * 3 + r] = nrp;
        A[r * 3 + q] = nrq;
        A[q * 3 + r] = nrq;
        A[p * 3 + p] = A[p * 3 + p] - t * apq;
        A[q * 3 + q] = A[q * 3 + q] + t * apq;
        A[p * 3 + q] = 0.0;
        A[q * 3 + p] = 0.0;
        for (int k = 0; k < 3; ++k) {
          const double vrp = Vm[k * 3 + p], vrq = Vm[k * 3 + q];
          Vm[k * 3 + p] = c * vrp - s * vrq;
          Vm[k * 3 + q] = s * vrp + c * vrq;
        }
      }
    }
  }
  // stable ascending order of the diagonal (insertion sort moves only on a strict <)
  int order[3] = {0, 1, 2};
  for (int i = 1; i < 3; ++i)
    for (int j = i; j > 0 && A[order[j] * 3 + order[j]] < A[order[j - 1] * 3 + order[j - 1]]; --j)
      std::swap(order[j], order[j - 1]);
  for (int k = 0; k < 3; ++k) {
    const int col = order[k];
    evals[k] = A[col * 3 + col];
    int big = 0;
    for (int r = 1; r < 3; ++r)
      if (std::fabs(Vm[r * 3 + col]) > std::fabs(Vm[big * 3 + col])) big = r;
    const double sg = Vm[big * 3 + col] < 0.0 ? -1.0 : 1.0;
    for (int r = 0; r < 3; ++r) evecs[k * 3 + r] = sg * Vm[r * 3 + col];
  }
}

// Gauss-Jacobi nodes and weights on [0,1] for the weight (1-u)^alpha u^beta.
static void gauss_jacobi_unit(int n, double alpha, double beta, std::vector<double>& x, std::vector<double>& w) {
  std::vector<double> J(n * n, 0.0);
  for (int k = 0; k < n; ++k) {
    const double s = 2.0 * k + alpha + beta;
    J[k * n + k] = (k == 0) ? (beta - alpha) / (alpha + beta + 2.0) : (beta * beta - alpha * alpha) / (s * (s + 2.0));
    if (k > 0) {
      const double num = 4.0 * k * (k + alpha) * (k + beta) * (k + alpha + beta);
      const double den = s * s * (s + 1.0) * (s - 1.0);
      const double b = std::sqrt(num / den);
      J[k * n + k - 1] = b;
      J[(k - 1) * n + k] = b;
    }
  }
  const double mu0 = std::pow(2.0, alpha + beta + 1.0) * std::tgamma(alpha + 1.0) * std::tgamma(beta + 1.0) /
                     std::tgamma(alpha + beta + 2.0);
  std::vector<double> ev, vecs;
  sym_eigen(n, J, ev, vecs);
  const double scale = std::pow(2.0, alpha + beta + 1.0);
  x.resize(n);
  w.resize(n);
  for (int k = 0; k < n; ++k) {
    const double v0 = vecs[k * n];
    x[k] = 0.5 * (1.0 + ev[k]);
    w[k] = mu0 * v0 * v0 / scale;
  }
}

TrigRule make_trig_rule(int order) {
  const int n = order / 2 + 1;
  std::vector<double> u, wu, v, wv;
  gauss_jacobi_unit(n, 1.0, 0.0, u, wu);
  gauss_jacobi_unit(n, 0.0, 0.0, v, wv);
  TrigRule r;
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      r.xi.push_back(u[a]);
      r.eta.push_back(v[b] * (1.0 - u[a]));
      r.w.push_back(wu[a] * wv[b]);
    }
  return r;
}

SSRule make_ss_rule(int cls, int order, bool radial) {
  std::vector<double> s, ws;
  gauss_jacobi_unit(order / 2 + 1, 0.0, 0.0, s, ws);
  const int n = (int)s.size();
  SSRule r;
  for (int ix = 0; ix < n; ++ix) {
    r.c1 += ws[ix] * s[ix];
    r.c2 += ws[ix] * s[ix] * s[ix];
  }
  auto add = [&](double xi, double a, double b, double c, double d, double w) {
    const double p0 = xi * a, p1 = xi * b, p2 = xi * c, p3 = xi * d;
    r.x0.push_back(p0 - p1);
    r.x1.push_back(p1);
    r.y0.push_back(p2 - p3);
    r.y1.push_back(p3);
    r.w.push_back(w);
  };
  for (int i1 = 0; i1 < n; ++i1)
    for (int i2 = 0; i2 < n; ++i2)
      for (int i3 = 0; i3 < n; ++i3) {
        const double e1 = s[i1], e2 = s[i2], e3 = s[i3];
        const double whex = ws[i1] * ws[i2] * ws[i3];
        for (int ix = 0; ix < (radial ? 1 : n); ++ix) {
          // radial: one point per direction at xi = 1, weight without xi^3 and the xi weight
          const double xi = radial ? 1.0 : s[ix];
          const double wb = radial ? whex : whex * ws[ix];
          const double x3 = xi * xi * xi;
          if (cls == 0) {
            const double w = x3 * e1 * e1 * e2 * wb;
            add(xi, 1, 1 - e1 + e1 * e2, 1 - e1 * e2 * e3, 1 - e1, w);
            add(xi, 1 - e1 * e2 * e3, 1 - e1, 1, 1 - e1 + e1 * e2, w);
            add(xi, 1, e1 * (1 - e2 + e2 * e3), 1 - e1 * e2, e1 * (1 - e2), w);
            add(xi, 1 - e1 * e2, e1 * (1 - e2), 1, e1 * (1 - e2 + e2 * e3), w);
            add(xi, 1 - e1 * e2 * e3, e1 * (1 - e2 * e3), 1, e1 * (1 - e2), w);
            add(xi, 1, e1 * (1 - e2), 1 - e1 * e2 * e3, e1 * (1 - e2 * e3), w);
          } else if (cls == 1) {
            const double w0 = x3 * e1 * e1 * wb;
            const double w1 = x3 * e1 * e1 * e2 * wb;
            add(xi, 1, e1 * e3, 1 - e1 * e2, e1 * (1 - e2), w0);
            add(xi, 1, e1, 1 - e1 * e2 * e3, e1 * e2 * (1 - e3), w1);
            add(xi, 1 - e1 * e2, e1 * (1 - e2), 1, e1 * e2 * e3, w1);
            add(xi, 1 - e1 * e2 * e3, e1 * e2 * (1 - e3), 1, e1, w1);
            add(xi, 1 - e1 * e2 * e3, e1 * (1 - e2 * e3), 1, e1 * e2, w1);
          } else {
            const double w = x3 * e2 * wb;
            add(xi, 1, e1, e2, e2 * e3, w);
            add(xi, e2, e2 * e3, 1, e1, w);
          }
        }
      }
  return r;
}

}  // namespace bem
