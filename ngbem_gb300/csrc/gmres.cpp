// Krylov solvers on the GPU operators (the role of ngsolve.krylovspace.GMRes as the
// reference's tests use it, tests/test_Laplace.py:51-60): GMRES(restart) with the operator
// application captured in a CUDA graph, and a batched GMRES for many right-hand sides.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "host.hpp"

namespace bem {

// ---------------------------------------------------------------------------------------------
// GMRES(restart) with CGS2 Arnoldi in fp64; the operator application is a CUDA graph.
static int gmres_impl(int nterms, OperatorBase* const* ops, const double* coef, const void* b, void* x, int maxiter,
                      int restart, double tol, int* iters, double* resid, cudaStream_t s);

// GMRES runs on a private stream (the legacy default stream cannot be captured into a graph),
// ordered after the caller's stream on entry and before it on exit.
int gmres_solve(int nterms, OperatorBase* const* ops, const double* coef, const void* b, void* x, int maxiter,
                int restart, double tol, int* iters, double* resid, cudaStream_t caller) {
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct Guard {
    cudaStream_t& s; cudaEvent_t& a; cudaEvent_t& b;
    ~Guard() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); if (s) cudaStreamDestroy(s); }
  } guard{s, e0, e1};
  BEM_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
  BEM_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
  BEM_CUDA(cudaEventRecord(e0, caller));
  BEM_CUDA(cudaStreamWaitEvent(s, e0, 0));
  int rc = gmres_impl(nterms, ops, coef, b, x, maxiter, restart, tol, iters, resid, s);
  BEM_CUDA(cudaEventRecord(e1, s));
  BEM_CUDA(cudaStreamWaitEvent(caller, e1, 0));
  BEM_CUDA(cudaStreamSynchronize(s));
  return rc;
}

// One restarted GMRES(restart) run on the operator replayed by `exec` (input gin, output
// gout): x is the initial guess and the result; stops at ||b - A x|| <= tol * scale.
struct GmresWS {
  bool cplx = false;
  int n = 0, restart = 0;
  size_t esz = 8;
  DevBuf Q, gin, gout, hdev, nrm, one;
  cudaStream_t s = nullptr;
  double dnorm(const void* v) {
    launch_nrm2(cplx, n, v, nrm.as<double>(), s);
    double h;
    BEM_CUDA(cudaMemcpyAsync(&h, nrm.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    BEM_CUDA(cudaStreamSynchronize(s));
    return h;
  }
  // r = b - A x into gout; returns ||r||
  double residual(cudaGraphExec_t exec, const void* b, const void* x) {
    BEM_CUDA(cudaMemcpyAsync(gin.p, x, (size_t)n * esz, cudaMemcpyDeviceToDevice, s));
    BEM_CUDA(cudaGraphLaunch(exec, s));
    launch_residual(cplx, n, b, gout.p, s);
    return dnorm(gout.p);
  }
};

static void gmres_run(GmresWS& w, cudaGraphExec_t exec, const void* b, void* x, int maxiter, double tol, double scale,
                      int& it, double& rel) {
  using C = std::complex<double>;
  const int n = w.n, restart = w.restart;
  const size_t esz = w.esz;
  const bool cplx = w.cplx;
  cudaStream_t s = w.s;
  char* Qp = (char*)w.Q.p;
  it = 0;
  rel = 0.0;
  for (;;) {
    const double beta = w.residual(exec, b, x);
    rel = beta / scale;
    if (rel <= tol || it >= maxiter || beta == 0.0) break;
    launch_scale_copy(cplx, n, w.gout.p, 1.0 / beta, Qp, s);
    std::vector<C> H((size_t)(restart + 1) * restart, C(0)), cs(restart), sn(restart), g(restart + 1, C(0));
    g[0] = beta;
    int j = 0;
    for (; j < restart && it < maxiter; ++j, ++it) {
      BEM_CUDA(cudaMemcpyAsync(w.gin.p, Qp + (size_t)j * n * esz, (size_t)n * esz, cudaMemcpyDeviceToDevice, s));
      BEM_CUDA(cudaGraphLaunch(exec, s));
      std::vector<C> h(j + 1, C(0));
      for (int pass = 0; pass < 2; ++pass) {
        launch_gemv_ct(cplx, n, j + 1, w.Q.p, w.gout.p, w.hdev.p, s);
        launch_gemv_sub(cplx, n, j + 1, w.Q.p, w.hdev.p, w.gout.p, s);
        std::vector<double> hh((size_t)(j + 1) * (cplx ? 2 : 1));
        BEM_CUDA(cudaMemcpyAsync(hh.data(), w.hdev.p, hh.size() * 8, cudaMemcpyDeviceToHost, s));
        BEM_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i <= j; ++i) h[i] += cplx ? C(hh[2 * i], hh[2 * i + 1]) : C(hh[i], 0.0);
      }
      const double hn = w.dnorm(w.gout.p);
      if (hn > 0.0) launch_scale_copy(cplx, n, w.gout.p, 1.0 / hn, Qp + (size_t)(j + 1) * n * esz, s);
      for (int i = 0; i <= j; ++i) H[(size_t)i * restart + j] = h[i];
      H[(size_t)(j + 1) * restart + j] = hn;
      for (int i = 0; i < j; ++i) {
        C a = H[(size_t)i * restart + j], c2 = H[(size_t)(i + 1) * restart + j];
        H[(size_t)i * restart + j] = std::conj(cs[i]) * a + std::conj(sn[i]) * c2;
        H[(size_t)(i + 1) * restart + j] = -sn[i] * a + cs[i] * c2;
      }
      C a = H[(size_t)j * restart + j], c2 = H[(size_t)(j + 1) * restart + j];
      const double den = std::sqrt(std::norm(a) + std::norm(c2));
      if (den == 0.0) { cs[j] = 1.0; sn[j] = 0.0; }
      else { cs[j] = a / den; sn[j] = c2 / den; }
      H[(size_t)j * restart + j] = std::conj(cs[j]) * a + std::conj(sn[j]) * c2;
      H[(size_t)(j + 1) * restart + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = std::conj(cs[j]) * g[j];
      rel = std::abs(g[j + 1]) / scale;
      if (rel <= tol || hn == 0.0) { ++j; ++it; break; }
    }
    const int k = j;
    std::vector<C> yv(k, C(0));
    for (int i = k - 1; i >= 0; --i) {
      C sacc = g[i];
      for (int l = i + 1; l < k; ++l) sacc -= H[(size_t)i * restart + l] * yv[l];
      yv[i] = sacc / H[(size_t)i * restart + i];
    }
    std::vector<double> yh((size_t)k * (cplx ? 2 : 1));
    for (int i = 0; i < k; ++i) {
      if (cplx) { yh[2 * i] = yv[i].real(); yh[2 * i + 1] = yv[i].imag(); }
      else yh[i] = yv[i].real();
    }
    BEM_CUDA(cudaMemcpyAsync(w.hdev.p, yh.data(), yh.size() * 8, cudaMemcpyHostToDevice, s));
    launch_axpy_basis(cplx, n, k, w.Q.p, w.hdev.p, x, s);
    BEM_CUDA(cudaStreamSynchronize(s));
    if (rel <= tol || it >= maxiter) {
      rel = w.residual(exec, b, x) / scale;
      break;
    }
  }
}

// GMRES for sum_k coef[k] ops[k].  When an operator stores its blocks in FP32, the solve is a
// GMRES-based iterative refinement: the Krylov iterations apply the plain FP32 matvec, each
// outer step recomputes the residual with the error-free (compensated) matvec and corrects x,
// so the final residual reaches the tolerance for the stored operator.
static int gmres_impl(int nterms, OperatorBase* const* ops, const double* coef, const void* b, void* x, int maxiter,
                      int restart, double tol, int* iters, double* resid, cudaStream_t s) {
  if (nterms < 1) throw Error(BEM_ERR_ARG, "gmres needs at least one operator");
  const int n = ops[0]->height;
  bool cplx = false, mixed = false;
  std::vector<HOperator*> hops;
  for (int k = 0; k < nterms; ++k) {
    if (ops[k]->height != n || ops[k]->width != n) throw Error(BEM_ERR_ARG, "gmres operators must be square and equal-sized");
    cplx = cplx || ops[k]->cplx || coef[2 * k + 1] != 0.0;
    if (auto* h = dynamic_cast<HOperator*>(ops[k])) {
      hops.push_back(h);
      mixed = mixed || h->prec == 1;
    }
  }
  for (int k = 0; k < nterms; ++k)
    if (ops[k]->cplx != cplx)
      throw Error(BEM_ERR_ARG, "gmres operators must all act on real or all on complex vectors");
  restart = std::max(1, std::min(restart, maxiter > 0 ? maxiter : restart));
  GmresWS w;
  w.cplx = cplx;
  w.n = n;
  w.restart = restart;
  w.esz = cplx ? 16 : 8;
  w.s = s;
  w.Q.alloc((size_t)n * (restart + 1) * w.esz);
  w.gin.alloc((size_t)n * w.esz);
  w.gout.alloc((size_t)n * w.esz);
  w.hdev.alloc((size_t)(restart + 2) * w.esz);
  w.nrm.alloc(sizeof(double));
  const double onev[2] = {1.0, 0.0};
  w.one.alloc(16);
  BEM_CUDA(cudaMemcpy(w.one.p, onev, 16, cudaMemcpyHostToDevice));
  const double zero[2] = {0.0, 0.0}, one[2] = {1.0, 0.0};
  std::vector<int> saved;
  for (auto* h : hops) saved.push_back(h->mv_compensated);
  struct Restore {
    std::vector<HOperator*>& h;
    std::vector<int>& v;
    ~Restore() { for (size_t i = 0; i < h.size(); ++i) h[i]->mv_compensated = v[i]; }
  } restore{hops, saved};
  auto capture = [&](int compensated, cudaGraph_t& g, cudaGraphExec_t& e) {
    for (auto* h : hops) h->mv_compensated = compensated;
    auto apply = [&]() {
      for (int k = 0; k < nterms; ++k) ops[k]->mult(0, coef + 2 * k, w.gin.p, k == 0 ? zero : one, w.gout.p, 1, s);
    };
    apply();  // allocates the operators' workspaces outside the capture
    BEM_CUDA(cudaStreamSynchronize(s));
    BEM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    apply();
    BEM_CUDA(cudaStreamEndCapture(s, &g));
    BEM_CUDA(cudaGraphInstantiate(&e, g, 0));
  };
  struct GraphGuard {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    ~GraphGuard() { if (e) cudaGraphExecDestroy(e); if (g) cudaGraphDestroy(g); }
  } acc, fast;
  capture(1, acc.g, acc.e);
  const double bnorm = w.dnorm(b);
  const double scale = bnorm > 0.0 ? bnorm : 1.0;
  int it = 0;
  double rel = 0.0;
  if (!mixed) {
    gmres_run(w, acc.e, b, x, maxiter, tol, scale, it, rel);
  } else {
    capture(0, fast.g, fast.e);
    DevBuf r, e;
    r.alloc((size_t)n * w.esz);
    e.alloc((size_t)n * w.esz);
    for (int outer = 0; outer < 50; ++outer) {
      rel = w.residual(acc.e, b, x) / scale;
      if (rel <= tol || it >= maxiter) break;
      BEM_CUDA(cudaMemcpyAsync(r.p, w.gout.p, (size_t)n * w.esz, cudaMemcpyDeviceToDevice, s));
      BEM_CUDA(cudaMemsetAsync(e.p, 0, (size_t)n * w.esz, s));
      // the inner solve reduces the residual to what the outer step still needs, but not
      // below the rounding level of the FP32 matvec
      const double inner_tol = std::max(0.5 * tol / rel, 1e-6);
      int iit = 0;
      double irel = 0.0;
      gmres_run(w, fast.e, r.p, e.p, maxiter - it, inner_tol, rel * scale, iit, irel);
      it += std::max(iit, 1);
      launch_axpy_basis(cplx, n, 1, e.p, w.one.p, x, s);  // x += e
    }
  }
  BEM_CUDA(cudaStreamSynchronize(s));
  if (iters) *iters = it;
  if (resid) *resid = rel;
  return BEM_OK;
}


// ---------------------------------------------------------------------------------------------
// Batched GMRES: nrhs independent systems sum_k coef[k] ops[k] x_r = b_r advanced in lockstep,
// so that each Arnoldi step applies the operators once to all right-hand sides (the H-matrix is
// streamed once per step for all of them).  FP64 CGS2 Arnoldi per column, Givens rotations and
// least squares per column on the host; a column stops extending its Krylov space once it has
// converged.  With FP32-stored operators: iterative refinement as in gmres_impl.
struct BGmresWS {
  bool cplx = false;
  int n = 0, nrhs = 0, restart = 0;
  size_t esz = 8;
  DevBuf Q, gin, gout, hdev, nrm, inv;
  cudaStream_t s = nullptr;
  size_t block() const { return (size_t)n * nrhs * esz; }
  std::vector<double> norms(const void* v) {
    launch_bnrm2(cplx, n, nrhs, v, nrm.as<double>(), s);
    std::vector<double> h(nrhs);
    BEM_CUDA(cudaMemcpyAsync(h.data(), nrm.p, nrhs * sizeof(double), cudaMemcpyDeviceToHost, s));
    BEM_CUDA(cudaStreamSynchronize(s));
    return h;
  }
  std::vector<double> residual(cudaGraphExec_t exec, const void* b, const void* x) {
    BEM_CUDA(cudaMemcpyAsync(gin.p, x, block(), cudaMemcpyDeviceToDevice, s));
    BEM_CUDA(cudaGraphLaunch(exec, s));
    launch_residual(cplx, n * nrhs, b, gout.p, s);
    return norms(gout.p);
  }
  void scale_into(const void* w, const std::vector<double>& f, void* q) {
    BEM_CUDA(cudaMemcpyAsync(inv.p, f.data(), nrhs * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_bscale(cplx, n, nrhs, w, inv.as<double>(), q, s);
  }
};

static void bgmres_run(BGmresWS& w, cudaGraphExec_t exec, const void* b, void* x, int maxiter, double tol,
                       const std::vector<double>& scale, int& it, std::vector<double>& rel) {
  using C = std::complex<double>;
  const int n = w.n, R = w.nrhs, restart = w.restart;
  const bool cplx = w.cplx;
  cudaStream_t s = w.s;
  char* Qp = (char*)w.Q.p;
  it = 0;
  rel.assign(R, 0.0);
  for (;;) {
    std::vector<double> beta = w.residual(exec, b, x);
    bool done = true;
    for (int r = 0; r < R; ++r) {
      rel[r] = beta[r] / scale[r];
      if (rel[r] > tol && beta[r] > 0.0) done = false;
    }
    if (done || it >= maxiter) break;
    std::vector<double> f(R);
    for (int r = 0; r < R; ++r) f[r] = beta[r] > 0.0 ? 1.0 / beta[r] : 0.0;
    w.scale_into(w.gout.p, f, Qp);
    std::vector<C> H((size_t)R * (restart + 1) * restart, C(0)), cs((size_t)R * restart), sn((size_t)R * restart),
        g((size_t)R * (restart + 1), C(0));
    std::vector<int> kr(R, 0);
    std::vector<char> active(R, 0);
    for (int r = 0; r < R; ++r) {
      g[(size_t)r * (restart + 1)] = beta[r];
      active[r] = rel[r] > tol && beta[r] > 0.0;
    }
    auto Hs = [&](int r, int i, int j) -> C& { return H[((size_t)r * (restart + 1) + i) * restart + j]; };
    int j = 0;
    for (; j < restart && it < maxiter; ++j, ++it) {
      BEM_CUDA(cudaMemcpyAsync(w.gin.p, Qp + (size_t)j * w.block(), w.block(), cudaMemcpyDeviceToDevice, s));
      BEM_CUDA(cudaGraphLaunch(exec, s));
      std::vector<C> h((size_t)(j + 1) * R, C(0));
      for (int pass = 0; pass < 2; ++pass) {
        launch_bgemv_ct(cplx, n, j + 1, R, w.Q.p, w.gout.p, w.hdev.p, s);
        launch_bgemv_sub(cplx, n, j + 1, R, w.Q.p, w.hdev.p, w.gout.p, s);
        std::vector<double> hh((size_t)(j + 1) * R * (cplx ? 2 : 1));
        BEM_CUDA(cudaMemcpyAsync(hh.data(), w.hdev.p, hh.size() * 8, cudaMemcpyDeviceToHost, s));
        BEM_CUDA(cudaStreamSynchronize(s));
        for (size_t q = 0; q < h.size(); ++q) h[q] += cplx ? C(hh[2 * q], hh[2 * q + 1]) : C(hh[q], 0.0);
      }
      const std::vector<double> hn = w.norms(w.gout.p);
      std::vector<double> fi(R);
      for (int r = 0; r < R; ++r) fi[r] = hn[r] > 0.0 ? 1.0 / hn[r] : 0.0;
      w.scale_into(w.gout.p, fi, Qp + (size_t)(j + 1) * w.block());
      bool any = false;
      for (int r = 0; r < R; ++r) {
        if (!active[r]) continue;
        for (int i = 0; i <= j; ++i) Hs(r, i, j) = h[(size_t)i * R + r];
        Hs(r, j + 1, j) = hn[r];
        C* csr = &cs[(size_t)r * restart];
        C* snr = &sn[(size_t)r * restart];
        C* gr = &g[(size_t)r * (restart + 1)];
        for (int i = 0; i < j; ++i) {
          const C a = Hs(r, i, j), c2 = Hs(r, i + 1, j);
          Hs(r, i, j) = std::conj(csr[i]) * a + std::conj(snr[i]) * c2;
          Hs(r, i + 1, j) = -snr[i] * a + csr[i] * c2;
        }
        const C a = Hs(r, j, j), c2 = Hs(r, j + 1, j);
        const double den = std::sqrt(std::norm(a) + std::norm(c2));
        if (den == 0.0) { csr[j] = 1.0; snr[j] = 0.0; }
        else { csr[j] = a / den; snr[j] = c2 / den; }
        Hs(r, j, j) = std::conj(csr[j]) * a + std::conj(snr[j]) * c2;
        Hs(r, j + 1, j) = 0.0;
        gr[j + 1] = -snr[j] * gr[j];
        gr[j] = std::conj(csr[j]) * gr[j];
        kr[r] = j + 1;
        rel[r] = std::abs(gr[j + 1]) / scale[r];
        if (rel[r] <= tol || hn[r] == 0.0) active[r] = 0;
        any = any || active[r];
      }
      if (!any) { ++j; ++it; break; }
    }
    // per-column least squares over its own Krylov dimension
    const int kmax = *std::max_element(kr.begin(), kr.end());
    std::vector<double> yh((size_t)kmax * R * (cplx ? 2 : 1), 0.0);
    for (int r = 0; r < R; ++r) {
      const int k = kr[r];
      std::vector<C> yv(k, C(0));
      for (int i = k - 1; i >= 0; --i) {
        C sacc = g[(size_t)r * (restart + 1) + i];
        for (int l = i + 1; l < k; ++l) sacc -= Hs(r, i, l) * yv[l];
        yv[i] = sacc / Hs(r, i, i);
      }
      for (int i = 0; i < k; ++i) {
        const size_t q = (size_t)i * R + r;
        if (cplx) { yh[2 * q] = yv[i].real(); yh[2 * q + 1] = yv[i].imag(); }
        else yh[q] = yv[i].real();
      }
    }
    if (kmax > 0) {
      BEM_CUDA(cudaMemcpyAsync(w.hdev.p, yh.data(), yh.size() * 8, cudaMemcpyHostToDevice, s));
      launch_baxpy_basis(cplx, n, kmax, R, w.Q.p, w.hdev.p, x, s);
    }
    BEM_CUDA(cudaStreamSynchronize(s));
    bool conv = true;
    for (int r = 0; r < R; ++r) conv = conv && rel[r] <= tol;
    if (conv || it >= maxiter) {
      const std::vector<double> fin = w.residual(exec, b, x);
      for (int r = 0; r < R; ++r) rel[r] = fin[r] / scale[r];
      break;
    }
  }
}

int gmres_batched_solve(int nterms, OperatorBase* const* ops, const double* coef, int nrhs, const void* b, void* x,
                        int maxiter, int restart, double tol, int* iters, double* resid, cudaStream_t caller) {
  if (nterms < 1) throw Error(BEM_ERR_ARG, "gmres needs at least one operator");
  if (nrhs < 1) throw Error(BEM_ERR_ARG, "nrhs must be >= 1");
  const int n = ops[0]->height;
  bool cplx = false, mixed = false;
  std::vector<HOperator*> hops;
  for (int k = 0; k < nterms; ++k) {
    if (ops[k]->height != n || ops[k]->width != n) throw Error(BEM_ERR_ARG, "gmres operators must be square and equal-sized");
    cplx = cplx || ops[k]->cplx || coef[2 * k + 1] != 0.0;
    if (auto* h = dynamic_cast<HOperator*>(ops[k])) {
      hops.push_back(h);
      mixed = mixed || h->prec == 1;
    }
  }
  for (int k = 0; k < nterms; ++k)
    if (ops[k]->cplx != cplx) throw Error(BEM_ERR_ARG, "gmres operators must all act on real or all on complex vectors");
  restart = std::max(1, std::min(restart, maxiter > 0 ? maxiter : restart));
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct Guard {
    cudaStream_t& s; cudaEvent_t& a; cudaEvent_t& b;
    ~Guard() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); if (s) cudaStreamDestroy(s); }
  } guard{s, e0, e1};
  BEM_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
  BEM_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
  BEM_CUDA(cudaEventRecord(e0, caller));
  BEM_CUDA(cudaStreamWaitEvent(s, e0, 0));
  BGmresWS w;
  w.cplx = cplx;
  w.n = n;
  w.nrhs = nrhs;
  w.restart = restart;
  w.esz = cplx ? 16 : 8;
  w.s = s;
  w.Q.alloc(w.block() * (restart + 1));
  w.gin.alloc(w.block());
  w.gout.alloc(w.block());
  w.hdev.alloc((size_t)(restart + 2) * nrhs * w.esz);
  w.nrm.alloc(nrhs * sizeof(double));
  w.inv.alloc(nrhs * sizeof(double));
  const double zero[2] = {0.0, 0.0}, one[2] = {1.0, 0.0};
  std::vector<int> saved;
  for (auto* h : hops) saved.push_back(h->mv_compensated);
  struct Restore {
    std::vector<HOperator*>& h;
    std::vector<int>& v;
    ~Restore() { for (size_t i = 0; i < h.size(); ++i) h[i]->mv_compensated = v[i]; }
  } restore{hops, saved};
  struct GraphGuard {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    ~GraphGuard() { if (e) cudaGraphExecDestroy(e); if (g) cudaGraphDestroy(g); }
  } acc, fast;
  auto capture = [&](int compensated, GraphGuard& gg) {
    for (auto* h : hops) h->mv_compensated = compensated;
    auto apply = [&]() {
      for (int k = 0; k < nterms; ++k)
        ops[k]->mult(0, coef + 2 * k, w.gin.p, k == 0 ? zero : one, w.gout.p, nrhs, s);
    };
    apply();  // allocates the operators' workspaces outside the capture
    BEM_CUDA(cudaStreamSynchronize(s));
    BEM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    apply();
    BEM_CUDA(cudaStreamEndCapture(s, &gg.g));
    BEM_CUDA(cudaGraphInstantiate(&gg.e, gg.g, 0));
  };
  capture(1, acc);
  std::vector<double> scale = w.norms(b);
  for (double& v : scale) v = v > 0.0 ? v : 1.0;
  int it = 0;
  std::vector<double> rel(nrhs, 0.0);
  if (!mixed) {
    bgmres_run(w, acc.e, b, x, maxiter, tol, scale, it, rel);
  } else {
    capture(0, fast);
    DevBuf r, e, onev;
    r.alloc(w.block());
    e.alloc(w.block());
    std::vector<double> ones((size_t)nrhs * (cplx ? 2 : 1), 0.0);
    for (int q = 0; q < nrhs; ++q) ones[(size_t)q * (cplx ? 2 : 1)] = 1.0;
    onev.upload(ones, s);
    for (int outer = 0; outer < 50; ++outer) {
      const std::vector<double> res = w.residual(acc.e, b, x);
      double worst = 0.0;
      std::vector<double> inner_scale(nrhs);
      for (int q = 0; q < nrhs; ++q) {
        rel[q] = res[q] / scale[q];
        worst = std::max(worst, rel[q]);
        inner_scale[q] = res[q] > 0.0 ? res[q] : 1.0;
      }
      if (worst <= tol || it >= maxiter) break;
      BEM_CUDA(cudaMemcpyAsync(r.p, w.gout.p, w.block(), cudaMemcpyDeviceToDevice, s));
      BEM_CUDA(cudaMemsetAsync(e.p, 0, w.block(), s));
      const double inner_tol = std::max(0.5 * tol / worst, 1e-6);
      int iit = 0;
      std::vector<double> irel;
      bgmres_run(w, fast.e, r.p, e.p, maxiter - it, inner_tol, inner_scale, iit, irel);
      it += std::max(iit, 1);
      launch_baxpy_basis(cplx, n, 1, nrhs, e.p, onev.p, x, s);  // x += e (column-wise weight 1)
    }
  }
  BEM_CUDA(cudaStreamSynchronize(s));
  BEM_CUDA(cudaEventRecord(e1, s));
  BEM_CUDA(cudaStreamWaitEvent(caller, e1, 0));
  if (iters) *iters = it;
  if (resid)
    for (int q = 0; q < nrhs; ++q) resid[q] = rel[q];
  return BEM_OK;
}

}  // namespace bem
