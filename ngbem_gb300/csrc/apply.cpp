// Application of the assembled operators: the H-matrix products (single launch, four-pass
// pipeline, several right-hand sides, tensor cores; reference HMatrix::Mult / MultAdd /
// MultTrans, src/hmat.cpp:623-681), the potential (PotentialCF, src/ngbem.cpp:1166-1301), the
// dense copy, the mass matrix and the autotuner.
#include <algorithm>
#include <cstring>
#include <vector>

#include "host.hpp"

namespace bem {

HOperator::VecMap HOperator::vec_map(int trans) const {
  const bool shared = ttest == ttrial;
  const int* p_trial = d_perm_trial.as<int>();
  const int* p_test = shared ? d_perm_trial.as<int>() : d_perm_test.as<int>();
  VecMap m{};
  const bool gt = apply_gmap && gn_trial > 0, ge = apply_gmap && gn_test > 0;
  const int* g_trial = gt ? d_gperm_trial.as<int>() : p_trial;
  const int* g_test = ge ? d_gperm_test.as<int>() : p_test;
  const int l_trial = gt ? gn_trial : width, l_test = ge ? gn_test : height;
  if (!trans) {
    m.pin = g_trial;
    m.pout = g_test;
    m.ld_in = l_trial;
    m.ld_out = l_test;
    m.free_out = ge ? d_gfree_test.as<int>() : nullptr;
    m.n_free_out = ge ? n_gfree_test : 0;
  } else {
    m.pin = g_test;
    m.pout = g_trial;
    m.ld_in = l_test;
    m.ld_out = l_trial;
    m.free_out = gt ? d_gfree_trial.as<int>() : nullptr;
    m.n_free_out = gt ? n_gfree_trial : 0;
  }
  return m;
}

void HOperator::set_global_dofs(int trial_n, const int* trial_map, int test_n, const int* test_map) {
  auto build = [&](const SpaceH* sp, const ClusterTreeH* t, int n, const int* map, int& gn, int& nfree, DevBuf& gperm,
                   DevBuf& gfree) {
    if (!map) {
      gn = 0;
      nfree = 0;
      gperm.release();
      gfree.release();
      return;
    }
    if (n < sp->ndof) throw Error(BEM_ERR_ARG, "a global numbering has fewer entries than the space has dofs");
    std::vector<char> hit((size_t)n, 0);
    for (int d = 0; d < sp->ndof; ++d) {
      if (map[d] < 0 || map[d] >= n) throw Error(BEM_ERR_ARG, "global dof out of range");
      if (hit[(size_t)map[d]]) throw Error(BEM_ERR_ARG, "two dofs map to the same global dof");
      hit[(size_t)map[d]] = 1;
    }
    std::vector<int> gp(t->perm.size()), fr;
    for (size_t k = 0; k < t->perm.size(); ++k) gp[k] = map[t->perm[k]];
    for (int i = 0; i < n; ++i)
      if (!hit[(size_t)i]) fr.push_back(i);
    gperm.upload(gp);
    if (fr.empty()) gfree.release();
    else gfree.upload(fr);
    gn = n;
    nfree = (int)fr.size();
  };
  build(trial, ttrial, trial_n, trial_map, gn_trial, n_gfree_trial, d_gperm_trial, d_gfree_trial);
  build(test, ttest, test_n, test_map, gn_test, n_gfree_test, d_gperm_test, d_gfree_test);
  BEM_CUDA(cudaDeviceSynchronize());
}

void HOperator::mult(int trans, const double* alpha, const void* x, const double* beta, void* y, int nrhs,
                     cudaStream_t s) {
  if (nrhs < 1) throw Error(BEM_ERR_ARG, "nrhs must be >= 1");
  const int in_n = trans ? height : width;
  const int out_n = trans ? width : height;
  const int nmax = std::max(height, width);
  const size_t dsz = cplx ? 16 : 8;                 // FP64 accumulators
  const size_t xsz = (size_t)mv_x_bytes(prec, cplx);  // permuted input values
  if (ws_nrhs < nrhs) {
    d_xp.alloc((size_t)nmax * nrhs * xsz + 32);
    d_yp.alloc((size_t)nmax * nrhs * dsz + 32);
    d_t.alloc((size_t)std::max(t_len, 1) * nrhs * dsz + 32);
    d_tx.alloc((size_t)std::max(t_len, 1) * nrhs * xsz + 32);
    ws_nrhs = nrhs;
    // the accumulators are zero between matvecs (see the single-launch kernel)
    BEM_CUDA(cudaMemsetAsync(d_yp.p, 0, d_yp.bytes, s));
    BEM_CUDA(cudaMemsetAsync(d_t.p, 0, d_t.bytes, s));
    BEM_CUDA(cudaMemsetAsync(d_tx.p, 0, d_tx.bytes, s));
  }
  const VecMap vm = vec_map(trans);
  const int* pin = vm.pin;
  const int* pout = vm.pout;
  if (vm.n_free_out > 0) {
    // entries of a globally numbered output that hold no dof: y = beta y there (Mult: 0)
    launch_scale_rows(cplx, vm.free_out, vm.n_free_out, nrhs, vm.ld_out, beta, y, s);
  }
  if (tc_eligible(trans, nrhs, s)) {
    mult_tc(alpha, x, beta, y, nrhs, s);  // records its own profiling events
    return;
  }
  std::array<cudaEvent_t, 5> ev{};
  if (profiling) {
    for (auto& e : ev) BEM_CUDA(cudaEventCreate(&e));
    BEM_CUDA(cudaEventRecord(ev[0], s));
  }
  if (mv_fused && nrhs == 1) ensure_mv(trans ? 0xC0u : 0x30u, false, s);
  else if (nrhs > 1 && !trans) ensure_mv(prec == 0 ? 0u : 0u, true, s);
  else ensure_mv(trans ? 0x0Cu : 0x03u, false, s);
  if (mv_fused && nrhs == 1) {
    // one cooperative launch: permute, phase A, t -> input form, phase B, un-permute
    MVFusedArgs f{};
    f.a.xp = d_xp.p;
    f.a.t = d_t.p;
    f.a.tx = prec == 0 ? d_t.p : d_tx.p;
    f.a.yp = d_yp.p;
    f.a.nrhs = 1;
    f.a.compensated = mv_compensated;
    f.a.in_esz = cplx ? 16 : 8;
    f.a.err = d_err.as<int>();
    // plain FP32 arithmetic: t accumulates in FP32 in the high parts of its input form
    f.a.t_f32 = (prec == 1 && !mv_compensated) ? 1 : 0;
    const int p0 = trans ? 6 : 4;
    for (int ph = 0; ph < 2; ++ph) {
      f.items[ph] = d_items[p0 + ph].as<MVTItem>();
      f.pieces[ph] = d_pieces[p0 + ph].as<MVPiece>();
      f.ranges[ph] = d_ranges[p0 + ph].as<MVRange>();
      f.nitems[ph] = n_items[p0 + ph];
      f.ctr[ph] = d_sched.as<int>() + 2 + ph;
    }
    f.bar = (unsigned long long*)(d_sched.as<int>() + 4);
    f.perm_in = pin;
    f.n_in = in_n;
    f.x = x;
    f.perm_out = pout;
    f.n_out = out_n;
    f.y = y;
    f.alpha[0] = alpha[0];
    f.alpha[1] = alpha[1];
    f.beta[0] = beta[0];
    f.beta[1] = beta[1];
    f.use_beta = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
    f.t_len = t_len;
    f.wait_limit = wait_limit;
    f.bar_extra = bar_extra;
    if (profiling) {
      BEM_CUDA(cudaEventRecord(ev[1], s));
      BEM_CUDA(cudaEventRecord(ev[2], s));
    }
    BEM_CUDA(launch_mv_fused(prec, cplx, f, s));
    if (profiling) {
      BEM_CUDA(cudaEventRecord(ev[3], s));
      BEM_CUDA(cudaEventRecord(ev[4], s));
      pending.push_back(ev);
      pending_fused.push_back(true);
    }
    return;
  }
  launch_permute_in(prec, cplx, pin, in_n, nrhs, vm.ld_in, x, d_xp.p, s);
  BEM_CUDA(cudaMemsetAsync(d_yp.p, 0, (size_t)out_n * nrhs * dsz, s));
  if (profiling) BEM_CUDA(cudaEventRecord(ev[1], s));
  MVArgs2 a{};
  a.xp = d_xp.p;
  a.t = d_t.p;
  a.tx = prec == 0 ? d_t.p : d_tx.p;
  a.yp = d_yp.p;
  a.nrhs = nrhs;
  a.compensated = mv_compensated;
  a.in_esz = cplx ? 16 : 8;
  a.err = d_err.as<int>();
  a.sched = d_sched.as<int>();
  if (t_len > 0) {
    BEM_CUDA(cudaMemsetAsync(d_t.p, 0, (size_t)t_len * nrhs * dsz, s));
    a.pass = trans ? 2 : 0;
    a.items = d_items[a.pass].as<MVTItem>();
    a.pieces = d_pieces[a.pass].as<MVPiece>();
    a.ranges = d_ranges[a.pass].as<MVRange>();
    a.nitems = n_items[a.pass];
    if (nrhs > 1 && !trans) {
      a.items = d_mr_items[0].as<MVTItem>();
      a.pieces = d_mr_pieces[0].as<MVPiece>();
      a.nitems = n_mr_items[0];
      a.chunked = 1;
    }
    launch_mv_pass(prec, cplx, a, mv_grid, s);
    launch_t_to_x(prec, cplx, d_t.p, d_tx.p, (long long)t_len * nrhs, s);
  }
  if (profiling) BEM_CUDA(cudaEventRecord(ev[2], s));
  a.pass = trans ? 3 : 1;
  a.items = d_items[a.pass].as<MVTItem>();
  a.pieces = d_pieces[a.pass].as<MVPiece>();
  a.ranges = d_ranges[a.pass].as<MVRange>();
  a.nitems = n_items[a.pass];
  a.chunked = 0;
  if (nrhs > 1 && !trans && prec == 0) {
    a.items = d_mr_items[1].as<MVTItem>();
    a.pieces = d_mr_pieces[1].as<MVPiece>();
    a.nitems = n_mr_items[1];
    a.chunked = 1;
    launch_mv_pass(prec, cplx, a, mv_grid, s);
  } else if (nrhs > 1 && !trans) {
    // FP32 storage, owner computes: each leaf row cluster sums its dense and U2 contributions
    // and stores y (FP64 storage keeps the chunk pass: its wider accumulators favour it)
    MVRowArgs ra{};
    ra.leaves = d_ro_leaves.as<int4>();
    ra.nleaves = n_ro_leaves;
    ra.ents = d_ro_ents.as<int4>();
    ra.dense = d_mvdense.as<MVDense>();
    ra.lr = d_mvlr.as<LRDesc>();
    ra.xp = d_xp.p;
    ra.tx = prec == 0 ? d_t.p : d_tx.p;
    ra.yp = d_yp.p;
    ra.nrhs = nrhs;
    ra.compensated = mv_compensated;
    launch_mv_rowowner(prec, cplx, ra, s);
  } else {
    launch_mv_pass(prec, cplx, a, mv_grid, s);
  }
  if (profiling) BEM_CUDA(cudaEventRecord(ev[3], s));
  launch_permute_out(cplx, pout, out_n, nrhs, vm.ld_out, alpha, beta, d_yp.p, y, s);
  // leave the accumulators zero for the single-launch kernel
  BEM_CUDA(cudaMemsetAsync(d_yp.p, 0, (size_t)out_n * nrhs * dsz, s));
  if (t_len > 0) {
    BEM_CUDA(cudaMemsetAsync(d_t.p, 0, (size_t)t_len * nrhs * dsz, s));
    if (prec == 1) BEM_CUDA(cudaMemsetAsync(d_tx.p, 0, (size_t)t_len * nrhs * xsz, s));
  }
  if (profiling) {
    BEM_CUDA(cudaEventRecord(ev[4], s));
    pending.push_back(ev);
    pending_fused.push_back(false);
  }
  BEM_CUDA(cudaGetLastError());
}

void HOperator::potential(const void* density, int npts, const double* pts, const double* normals, void* out,
                          cudaStream_t s) {
  const int dim = potential_dim(kid, trt);
  if (dim == 0) throw Error(BEM_ERR_ARG, "no potential for this kernel and trial space");
  if (npts < 0) throw Error(BEM_ERR_ARG, "npts must be >= 0");
  if (kid == K_HELMHOLTZ_HS && !normals) throw Error(BEM_ERR_ARG, "this kernel needs the normals at the points");
  MeshH& mesh = *trial->mesh;
  mesh.ensure_device();
  trial->ensure_device();
  const int order_r = prm.intorder_regular > 0 ? prm.intorder_regular : prm.intorder;
  MeshH::RuleTables& rt = mesh.rule_tables(order_r);
  // source elements: the trial space's, within the trial definedon region when there is one
  // (PotentialCF skips the elements outside it, src/ngbem.cpp:1205)
  std::vector<int> el;
  for (int e : trial->elems)
    if (def_trial.empty() || def_trial[e]) el.push_back(e);
  const bool all = (int)el.size() == mesh.nt;
  DevBuf d_el;
  if (!all && !el.empty()) d_el.upload(el, s);
  const size_t nsrc = std::max<size_t>(1, el.size() * (size_t)rt.nq);
  DevBuf src_pos, src_val;
  src_pos.alloc(nsrc * 6 * sizeof(double));
  src_val.alloc(nsrc * dim * (cplx ? 16 : 8));
  PotArgs a{};
  a.erec = rt.rec[0].p;
  a.qoff = rt.qoff[0].p;
  a.rq = rt.rq[0].as<double>();
  a.pgeo = rt.pgeo[0].p;
  a.elems = all ? nullptr : d_el.as<int>();
  a.nt = (int)el.size();
  a.nq = rt.nq;
  a.trial = space_dev(*trial, trt, d_pinv_trial);
  a.density = density;
  a.src_pos = src_pos.as<double>();
  a.src_val = src_val.p;
  a.npts = npts;
  a.pts = pts;
  a.normals = normals;
  a.kappa = kappa;
  a.out = out;
  if (!launch_potential(kid, trt, a, s)) throw Error(BEM_ERR_ARG, "no potential for this kernel and trial space");
  BEM_CUDA(cudaGetLastError());
  BEM_CUDA(cudaStreamSynchronize(s));
}

int HOperator::device_status() {
  int e = 0;
  if (!d_err.p) return 0;
  BEM_CUDA(cudaDeviceSynchronize());
  BEM_CUDA(cudaMemcpy(&e, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  return e;
}

void HOperator::reset_device_state() {
  BEM_CUDA(cudaDeviceSynchronize());
  if (d_err.p) BEM_CUDA(cudaMemset(d_err.p, 0, d_err.bytes));
  if (d_sched.p) BEM_CUDA(cudaMemset(d_sched.p, 0, d_sched.bytes));
  for (DevBuf* b : {&d_yp, &d_t, &d_tx})
    if (b->p) BEM_CUDA(cudaMemset(b->p, 0, b->bytes));
  BEM_CUDA(cudaDeviceSynchronize());
}

void HOperator::collect_profile() {
  for (size_t i = 0; i < pending.size(); ++i) {
    auto& ev = pending[i];
    BEM_CUDA(cudaEventSynchronize(ev[4]));
    for (int k = 0; k < 4; ++k) {
      if (pending_fused[i] && k != 2) continue;  // one launch: its time is the apply slot
      float t = 0.f;
      BEM_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      kms[k] += t;
      kcount[k] += 1;
    }
    for (auto& e : ev) cudaEventDestroy(e);
  }
  pending.clear();
  pending_fused.clear();
}

HOperator::~HOperator() {
  for (auto& ev : pending)
    for (auto& e : ev) cudaEventDestroy(e);
  if (h_status) cudaFreeHost(h_status);
}

void HOperator::queue_status(cudaStream_t s) {
  if (!d_err.p) return;
  if (!h_status) {
    BEM_CUDA(cudaHostAlloc((void**)&h_status, sizeof(int), cudaHostAllocDefault));
    *h_status = 0;
  }
  BEM_CUDA(cudaMemcpyAsync(h_status, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
}

void HOperator::to_dense(void* out) {
  const size_t esz = cplx ? 16 : 8;
  const int chunk = std::min(width, 32);
  DevBuf X, Y;
  X.alloc((size_t)width * chunk * esz);
  Y.alloc((size_t)height * chunk * esz);
  std::vector<char> hx((size_t)width * chunk * esz), hy((size_t)height * chunk * esz);
  const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
  for (int c0 = 0; c0 < width; c0 += chunk) {
    const int nc = std::min(chunk, width - c0);
    std::fill(hx.begin(), hx.end(), 0);
    for (int c = 0; c < nc; ++c) {
      double* col = (double*)(hx.data() + (size_t)c * width * esz);
      col[(size_t)(c0 + c) * (cplx ? 2 : 1)] = 1.0;
    }
    BEM_CUDA(cudaMemcpy(X.p, hx.data(), (size_t)width * nc * esz, cudaMemcpyHostToDevice));
    mult(0, one, X.p, zero, Y.p, nc, 0);
    BEM_CUDA(cudaMemcpy(hy.data(), Y.p, (size_t)height * nc * esz, cudaMemcpyDeviceToHost));
    for (int c = 0; c < nc; ++c)
      for (int r = 0; r < height; ++r)
        std::memcpy((char*)out + ((size_t)r * width + c0 + c) * esz, hy.data() + ((size_t)c * height + r) * esz, esz);
  }
}

// ---------------------------------------------------------------------------------------------
// mass matrix <u, v> of identity traces, CSR in fp64 (rows = test dofs)
void MassOperator::build(SpaceH* trial, SpaceH* test, bool complex_vectors) {
  if (trial->mesh != test->mesh) throw Error(BEM_ERR_ARG, "mass matrix needs one mesh");
  MeshH& m = *trial->mesh;
  cplx = complex_vectors;
  nrows = test->ndof;
  ncols = trial->ndof;
  height = nrows;
  width = ncols;
  // a rule exact for the product of the two spaces' polynomials (at least order 4)
  auto degree = [](const SpaceH& sp) {
    if (sp.kind == BEM_P0) return 0;
    if (sp.kind >= BEM_L2P1 && sp.kind <= BEM_L2P3) return sp.kind - BEM_L2P1 + 1;
    if (sp.kind == BEM_H1P2) return 2;
    if (sp.kind == BEM_H1P3) return 3;
    if (bdm_kind_order(sp.kind) > 0) return bdm_kind_order(sp.kind);
    return 1;
  };
  TrigRule r = make_trig_rule(std::max(4, degree(*trial) + degree(*test)));
  const int nq = (int)r.w.size();
  std::vector<std::vector<std::pair<int, double>>> rows(nrows);
  // curved elements: 1 / |J|, the normal and the Piola offsets at the point (flat: per element)
  auto piola = [&](int e, double xi, double eta, double& inv, double* n, double xp[3][3]) {
    const ElemRec64& g = m.rec[e];
    if (!m.curved()) {
      double x[3];
      m.map(e, xi, eta, x);
      inv = g.invdetJ;
      for (int c = 0; c < 3; ++c) {
        n[c] = g.n[c];
        for (int o = 0; o < 3; ++o) xp[o][c] = x[c] - g.p[o][c];
      }
      return;
    }
    double x[3], rt[3][3], J0[3], J1[3];
    inv = 1.0 / m.frame(e, xi, eta, x, n, rt, J0, J1);
    piola_offsets(J0, J1, xi, eta, xp);
  };
  auto shape = [&](const SpaceH& sp, int e, double xi, double eta, double S[30][3], int& dim) {
    double inv, n[3], xp[3][3];
    if (sp.kind == BEM_P0) {
      if (sp.dual) piola(e, xi, eta, inv, n, xp);
      S[0][0] = sp.dual ? inv : 1.0;
      dim = 1;
      return;
    }
    if (bdm_kind_order(sp.kind) > 0) {
      // the Piola map of the reference fields (hdiv_shape), J = (xp_2 - xp_0, xp_2 - xp_1);
      // HCurl: n x it
      const int K = bdm_kind_order(sp.kind);
      const bool curl = bdm_kind_curl(sp.kind);
      piola(e, xi, eta, inv, n, xp);
      for (int a = 0; a < sp.nd; ++a) {
        const int sg = a < 3 * (K + 1) ? sp.sign[3 * e + a / (K + 1)] : 1;
        double vx, vy, v[3];
        hdiv_shape<double>(K, a, xi, eta, sg, vx, vy);
        for (int c = 0; c < 3; ++c) v[c] = ((xp[2][c] - xp[0][c]) * vx + (xp[2][c] - xp[1][c]) * vy) * inv;
        for (int c = 0; c < 3; ++c)
          S[a][c] = curl ? n[(c + 1) % 3] * v[(c + 2) % 3] - n[(c + 2) % 3] * v[(c + 1) % 3] : v[c];
      }
      dim = 3;
      return;
    }
    if (sp.kind == BEM_H1P2 || sp.kind == BEM_H1P3) {
      // vertex hats, edge bubbles (orientation sign to the power m), face bubble
      const int P = sp.kind == BEM_H1P2 ? 2 : 3;
      const double l[3] = {xi, eta, 1.0 - xi - eta};
      for (int a = 0; a < sp.nd; ++a) {
        double d[3];
        double v = h1p_shape<double>(P, a, l, d);
        if (a >= 3 && a < 3 + 3 * (P - 1) && (a - 3) % (P - 1) == 1) v *= sp.sign[3 * e + (a - 3) / (P - 1)];
        S[a][0] = v;
      }
      dim = 1;
      return;
    }
    if (sp.kind >= BEM_L2P1) {
      const int code = sp.sign[3 * e] + 3 * sp.sign[3 * e + 1];
      for (int a = 0; a < sp.nd; ++a) S[a][0] = dubiner<double>(sp.kind - BEM_L2P1 + 1, a, xi, eta, code);
      dim = 1;
      return;
    }
    if (sp.kind == BEM_P1) { S[0][0] = xi; S[1][0] = eta; S[2][0] = 1.0 - xi - eta; dim = 1; return; }
    piola(e, xi, eta, inv, n, xp);
    for (int a = 0; a < 3; ++a) {
      const int o = (a + 2) % 3;
      double v[3];
      for (int c = 0; c < 3; ++c) v[c] = sp.sign[3 * e + a] * xp[o][c] * inv;
      // HCurl trace: n x the RT0 shape of the same edge
      for (int c = 0; c < 3; ++c)
        S[a][c] = sp.kind == BEM_HCURL ? n[(c + 1) % 3] * v[(c + 2) % 3] - n[(c + 2) % 3] * v[(c + 1) % 3] : v[c];
    }
    dim = 3;
  };
  for (int e = 0; e < m.nt; ++e)
    for (int q = 0; q < nq && trial->on(e) && test->on(e); ++q) {
      double Si[30][3], Sj[30][3];
      int di, dj;
      shape(*test, e, r.xi[q], r.eta[q], Si, di);
      shape(*trial, e, r.xi[q], r.eta[q], Sj, dj);
      if (di != dj) throw Error(BEM_ERR_ARG, "mass matrix of scalar and vector spaces");
      double x[3], nrm[3], rt[3][3];
      const double w = r.w[q] * m.frame(e, r.xi[q], r.eta[q], x, nrm, rt);
      for (int a = 0; a < test->nd; ++a)
        for (int b = 0; b < trial->nd; ++b) {
          double s = 0.0;
          for (int c = 0; c < di; ++c) s += Si[a][c] * Sj[b][c];
          rows[test->dof(e, a)].push_back({trial->dof(e, b), w * s});
        }
    }
  h_rowptr.assign(nrows + 1, 0);
  h_col.clear();
  h_val.clear();
  for (int i = 0; i < nrows; ++i) {
    auto& rw = rows[i];
    std::sort(rw.begin(), rw.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (size_t k = 0; k < rw.size();) {
      size_t l = k;
      double s = 0.0;
      while (l < rw.size() && rw[l].first == rw[k].first) s += rw[l++].second;
      h_col.push_back(rw[k].first);
      h_val.push_back(s);
      k = l;
    }
    h_rowptr[i + 1] = (int)h_col.size();
  }
  rowptr.upload(h_rowptr);
  col.upload(h_col);
  val.upload(h_val);
  BEM_CUDA(cudaDeviceSynchronize());
}

void MassOperator::mult(int trans, const double* alpha, const void* x, const double* beta, void* y, int nrhs,
                        cudaStream_t s) {
  launch_spmv(cplx, trans != 0, nrows, ncols, rowptr.as<int>(), col.as<int>(), val.as<double>(), alpha, beta,
              x, y, nrhs, s);
  BEM_CUDA(cudaGetLastError());
}


// Picks the matvec work decomposition for this operator by timing it: the piece size (stored
// elements per consumer-warp task, which also shapes the work items) and the schedule (one
// cooperative launch, or the four-pass pipeline).  Each candidate is timed over `reps`
// matvecs with CUDA events after a warm-up; the fastest is kept.
double HOperator::autotune(int reps, int* best_piece, int* best_fused) {
  if (reps < 1) reps = 1;
  const int cand[] = {256, 384, 512, 768, 1024, 1536, 2048};
  const size_t esz = cplx ? 16 : 8;
  DevBuf x, y;
  x.alloc((size_t)width * esz);
  y.alloc((size_t)height * esz);
  BEM_CUDA(cudaMemset(x.p, 0, (size_t)width * esz));
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct Guard {
    cudaStream_t& s; cudaEvent_t& a; cudaEvent_t& b;
    ~Guard() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); if (s) cudaStreamDestroy(s); }
  } guard{s, e0, e1};
  BEM_CUDA(cudaEventCreate(&e0));
  BEM_CUDA(cudaEventCreate(&e1));
  const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
  const bool fused_ok = mv_fused_supported();
  const bool was_profiling = profiling;
  profiling = false;
  double best = 1e300;
  int bp = mv_piece > 0 ? mv_piece : mv_piece_elems(), bf = mv_fused ? 1 : 0;
  for (int pc : cand) {
    mv_piece = pc;
    build_mv_items(fused_ok ? 0x33u : 0x03u, false, false);
    for (int f = fused_ok ? 1 : 0; f >= 0; --f) {
      mv_fused = f != 0;
      for (int w = 0; w < 2; ++w) mult(0, one, x.p, zero, y.p, 1, s);
      BEM_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < reps; ++r) mult(0, one, x.p, zero, y.p, 1, s);
      BEM_CUDA(cudaEventRecord(e1, s));
      BEM_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      BEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      const double per = ms / reps;
      if (per < best) {
        best = per;
        bp = pc;
        bf = f;
      }
    }
  }
  mv_piece = bp;
  mv_fused = bf != 0;
  build_mv_items(mv_fused ? 0x30u : 0x03u, false, false);
  BEM_CUDA(cudaStreamSynchronize(s));
  profiling = was_profiling;
  if (best_piece) *best_piece = bp;
  if (best_fused) *best_fused = bf;
  return best;
}

}  // namespace bem
