// Assembly and application of the H-matrix on the GPU (reference GenericIntegralOperator
// ctor src/ngbem.cpp:314-330, CalcHMatrix :118-157, HMatrix src/hmat.cpp:614-681).
//
// Assembly pipeline (one operator, two CUDA streams):
//   host : cluster trees, element patches per cluster, partition, far blocks whose patches
//          share a vertex are re-binned to dense (the reference throws and falls back,
//          src/ngbem.cpp:839-842 / :143-153)
//   sA   : batched ACA over the admissible blocks, then projection onto the dofs
//   sN   : regular near-field kernel over all dense blocks (bins singular pairs), then the
//          persistent FP64 Sauter-Schwab kernel over the binned singular pairs
//   host : blocks whose ACA hit the rank cap are assembled densely in a second near pass
#include <algorithm>
#include <atomic>
#include <chrono>
#include <exception>
#include <thread>
#include <cmath>
#include <complex>
#include <cstring>

#include "host.hpp"

namespace bem {

using clk = std::chrono::steady_clock;
static double ms_since(clk::time_point t0) {
  return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
}

struct StreamPair {
  cudaStream_t a = nullptr, n = nullptr;
  StreamPair() {
    BEM_CUDA(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
    BEM_CUDA(cudaStreamCreateWithFlags(&n, cudaStreamNonBlocking));
  }
  ~StreamPair() {
    if (a) cudaStreamDestroy(a);
    if (n) cudaStreamDestroy(n);
  }
};

static SpaceDev space_dev(const SpaceH& s, int tr, const DevBuf& pinv) {
  SpaceDev d;
  d.tr = tr;
  d.nd = s.nd;
  d.dual = s.dual;
  d.dofs = s.d_dofs.as<int4>();
  d.sign = s.d_sign.as<int4>();
  d.pinv = pinv.as<int>();
  return d;
}

// Dense near-field pass over a list of blocks (pool owned by the caller).
struct NearPass {
  std::vector<DenseDesc> desc;
  std::vector<int> block_ids;  // index into HOperator::blocks
  DevBuf d_desc, d_tiles, d_sing, d_count, d_err;
  long long npairs = 0;
  int ntiles = 0;
  int sing_cap = 0;
};

void HOperator::merge_meshes() {
  if (own_mesh) return;  // already merged: trial / test are the merged-mesh spaces
  trial_nt0 = trial->mesh->nt;
  test_nt0 = test->mesh->nt;
  if (trial->mesh == test->mesh) return;
  const MeshH& a = *test->mesh;
  const MeshH& b = *trial->mesh;
  std::vector<double> X(a.X);
  X.insert(X.end(), b.X.begin(), b.X.end());
  std::vector<int> T(a.T);
  for (int v : b.T) T.push_back(v + a.nv);
  own_mesh = std::make_unique<MeshH>();
  own_mesh->build(a.nv + b.nv, X.data(), a.nt + b.nt, T.data());
  std::vector<unsigned char> on_test(own_mesh->nt, 0), on_trial(own_mesh->nt, 0);
  for (int e = 0; e < a.nt; ++e) on_test[e] = test->on(e);
  for (int e = 0; e < b.nt; ++e) on_trial[a.nt + e] = trial->on(e);
  own_test_space = std::make_unique<SpaceH>();
  own_test_space->build(own_mesh.get(), test->kind, test->dual, on_test.data());
  own_trial_space = std::make_unique<SpaceH>();
  own_trial_space->build(own_mesh.get(), trial->kind, trial->dual, on_trial.data());
  if (own_test_space->ndof != test->ndof || own_trial_space->ndof != trial->ndof)
    throw Error(BEM_ERR_INTERNAL, "merged-mesh spaces differ from the caller's spaces");
  test = own_test_space.get();
  trial = own_trial_space.get();
  trial_e0 = a.nt;
}

void HOperator::assemble() {
  const auto t_start = clk::now();
  merge_meshes();
  trt = trace_kind(trial->kind, trial_ev);
  tet = trace_kind(test->kind, test_ev);
  if (trt < 0 || tet < 0) throw Error(BEM_ERR_ARG, "evaluator not available for this space");
  if (!nf_combo_supported(kid, trt, tet)) throw Error(BEM_ERR_ARG, "kernel / trace combination not supported");
  cplx = kernel_complex(kid);
  const int NC = kernel_ncomp(kid);
  prec = prm.precision == BEM_MIXED ? 1 : 0;
  const size_t rsz = prec == 0 ? 8 : 4;
  vsize = rsz * (cplx ? 2 : 1);
  const int order_s = prm.intorder_singular > 0 ? prm.intorder_singular : prm.intorder;
  const int order_r = prm.intorder_regular > 0 ? prm.intorder_regular : prm.intorder;
  if (order_s < 0 || order_r < 0 || order_s > 40 || order_r > 40) throw Error(BEM_ERR_ARG, "intorder out of range");
  const bool dense_method = prm.method == BEM_METHOD_DENSE;
  const int leaf = dense_method ? INT_MAX : prm.leafsize;
  const double eta = dense_method ? 0.0 : prm.eta;
  if (leaf < 1) throw Error(BEM_ERR_ARG, "leafsize must be positive");
  int kcap = prm.max_rank > 0 ? prm.max_rank : 128;
  kcap = std::min(kcap, 256);
  double eps = prm.eps;
  if (prec == 1) eps = std::max(eps, prm.aca_eps_floor > 0 ? prm.aca_eps_floor : 2e-7);
  // ACA scratch budget: the parameter, else an eighth of the device memory up to 16 GiB
  long long budget = prm.scratch_bytes;
  if (budget <= 0) {
    size_t freeb = 0, totalb = 0;
    BEM_CUDA(cudaMemGetInfo(&freeb, &totalb));
    budget = std::min<long long>(16LL << 30, (long long)(totalb / 8));
    budget = std::max<long long>(budget, 1LL << 30);
  }
  MeshH& mesh = *trial->mesh;
  height = test->ndof;
  width = trial->ndof;

  // ---- trees, patches, partition (host) ------------------------------------------------
  own_trial = trial->tree(leaf);
  ttrial = own_trial.get();
  if (test == trial) {
    ttest = ttrial;
  } else {
    own_test = test->tree(leaf);
    ttest = own_test.get();
  }
  partition_blocks(*ttest, *ttrial, eta, blocks);
  const int nb = (int)blocks.size();
  block_rank.assign(nb, -1);
  block_fallback.assign(nb, 0);

  // far blocks whose patches share a vertex -> dense (reference fallback)
  std::vector<int> stamp(mesh.nv, -1);
  std::vector<int> far_ids, dense_ids;
  for (int b = 0; b < nb; ++b) {
    const BlockH& B = blocks[b];
    if (B.near) { dense_ids.push_back(b); continue; }
    const ClusterH& ci = ttest->cl[B.rowcl];
    const ClusterH& cj = ttrial->cl[B.colcl];
    const double dx = ci.Centre[0] - cj.Centre[0], dy = ci.Centre[1] - cj.Centre[1], dz = ci.Centre[2] - cj.Centre[2];
    const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
    bool shared = false;
    if (dist <= ttest->patch_rad[B.rowcl] + ttrial->patch_rad[B.colcl] + 1e-12 * (1.0 + dist)) {
      for (int k = ttest->patch_ptr[B.rowcl]; k < ttest->patch_ptr[B.rowcl + 1]; ++k) {
        const int e = ttest->patch[k];
        for (int v = 0; v < 3; ++v) stamp[mesh.T[3 * e + v]] = b;
      }
      for (int k = ttrial->patch_ptr[B.colcl]; k < ttrial->patch_ptr[B.colcl + 1] && !shared; ++k) {
        const int e = ttrial->patch[k];
        for (int v = 0; v < 3; ++v)
          if (stamp[mesh.T[3 * e + v]] == b) shared = true;
      }
    }
    if (shared) { block_fallback[b] = 1; dense_ids.push_back(b); }
    else far_ids.push_back(b);
  }

  // ---- device tables ---------------------------------------------------------------------
  mesh.ensure_device();
  trial->ensure_device();
  test->ensure_device();
  MeshH::RuleTables& rt = mesh.rule_tables(order_r);
  const int nq = rt.nq;
  d_perm_trial.upload(ttrial->perm);
  d_pinv_trial.upload(ttrial->pinv);
  DevBuf d_patch_trial, d_patch_test;
  d_patch_trial.upload(ttrial->patch);
  if (ttest != ttrial) {
    d_perm_test.upload(ttest->perm);
    d_pinv_test.upload(ttest->pinv);
    d_patch_test.upload(ttest->patch);
  }
  const DevBuf& pinv_test = ttest != ttrial ? d_pinv_test : d_pinv_trial;
  const int* patch_test_dev = ttest != ttrial ? d_patch_test.as<int>() : d_patch_trial.as<int>();
  SpaceDev sd_trial = space_dev(*trial, trt, d_pinv_trial);
  SpaceDev sd_test = space_dev(*test, tet, pinv_test);
  // Sauter-Schwab tables
  DevBuf d_ss[3];
  int ss_n[3];
  long long ss_bytes = 0;
  for (int c = 0; c < 3; ++c) {
    SSRule r = make_ss_rule(c, order_s);
    ss_n[c] = (int)r.w.size();
    std::vector<double> tab;
    tab.reserve(5 * r.w.size());
    tab.insert(tab.end(), r.x0.begin(), r.x0.end());
    tab.insert(tab.end(), r.x1.begin(), r.x1.end());
    tab.insert(tab.end(), r.y0.begin(), r.y0.end());
    tab.insert(tab.end(), r.y1.begin(), r.y1.end());
    tab.insert(tab.end(), r.w.begin(), r.w.end());
    d_ss[c].upload(tab);
    ss_bytes += (long long)tab.size() * 8;
  }
  // max number of elements sharing a vertex with one element (bound for singular pairs)
  std::vector<int> valence(mesh.nv, 0);
  for (int k = 0; k < 3 * mesh.nt; ++k) valence[mesh.T[k]]++;
  int maxnb = 1;
  for (int e = 0; e < mesh.nt; ++e)
    maxnb = std::max(maxnb, valence[mesh.T[3 * e]] + valence[mesh.T[3 * e + 1]] + valence[mesh.T[3 * e + 2]]);
  BEM_CUDA(cudaDeviceSynchronize());
  info.ms_setup = ms_since(t_start);

  StreamPair sp;
  cudaEvent_t evA0, evA1, evN0, evN1, evP0, evP1;
  BEM_CUDA(cudaEventCreate(&evA0)); BEM_CUDA(cudaEventCreate(&evA1));
  BEM_CUDA(cudaEventCreate(&evN0)); BEM_CUDA(cudaEventCreate(&evN1));
  BEM_CUDA(cudaEventCreate(&evP0)); BEM_CUDA(cudaEventCreate(&evP1));
  struct EvGuard {
    cudaEvent_t* e; int n;
    ~EvGuard() { for (int i = 0; i < n; ++i) cudaEventDestroy(e[i]); }
  };
  cudaEvent_t evs[6] = {evA0, evA1, evN0, evN1, evP0, evP1};
  EvGuard eg{evs, 6};

  // ---- near field (dense blocks) ----------------------------------------------------------
  const long long align_el = (long long)std::max<size_t>(1, 16 / vsize);
  auto run_near = [&](NearPass& np, const std::vector<int>& ids, cudaStream_t s) {
    np.block_ids = ids;
    np.desc.clear();
    long long off = 0;
    std::vector<NFTile> tiles;
    long long cap = 0;
    for (int b : ids) {
      const BlockH& B = blocks[b];
      const ClusterH& ci = ttest->cl[B.rowcl];
      const ClusterH& cj = ttrial->cl[B.colcl];
      DenseDesc d;
      d.off = off;
      d.r0 = (int)ci.PermuPos;
      d.m = (int)ci.Number;
      d.c0 = (int)cj.PermuPos;
      d.n = (int)cj.Number;
      d.pi0 = ttest->patch_ptr[B.rowcl];
      d.ni = ttest->patch_ptr[B.rowcl + 1] - d.pi0;
      d.pj0 = ttrial->patch_ptr[B.colcl];
      d.nj = ttrial->patch_ptr[B.colcl + 1] - d.pj0;
      off += ((long long)d.m * d.n + align_el - 1) / align_el * align_el;  // 16-byte aligned blocks
      const long long pairs = (long long)d.ni * d.nj;
      np.npairs += pairs;
      const int bi = (int)np.desc.size();
      for (long long k0 = 0; k0 < pairs; k0 += 128) tiles.push_back(NFTile{bi, (int)k0});
      // bound on singular pairs of this block
      const double dx = ci.Centre[0] - cj.Centre[0], dy = ci.Centre[1] - cj.Centre[1], dz = ci.Centre[2] - cj.Centre[2];
      const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (dist <= ttest->patch_rad[B.rowcl] + ttrial->patch_rad[B.colcl] + 1e-12 * (1.0 + dist))
        cap += std::min(pairs, (long long)std::min(d.ni, d.nj) * maxnb);
      np.desc.push_back(d);
    }
    if (np.desc.empty()) return std::unique_ptr<DevBuf>();
    if (np.npairs > (long long)INT_MAX || pairs_overflow(tiles.size())) throw Error(BEM_ERR_ARG, "too many near-field tiles");
    if (cap > (1LL << 31) - 1) throw Error(BEM_ERR_ALLOC, "singular pair list too large");
    np.ntiles = (int)tiles.size();
    np.sing_cap = (int)std::max<long long>(cap, 1);
    auto pool = std::make_unique<DevBuf>();
    pool->alloc((size_t)(off + align_el) * vsize);
    BEM_CUDA(cudaMemsetAsync(pool->p, 0, pool->bytes, s));
    np.d_desc.upload(np.desc, s);
    np.d_tiles.upload(tiles, s);
    np.d_sing.alloc((size_t)np.sing_cap * sizeof(SingItem));
    np.d_count.alloc(sizeof(int));
    np.d_err.alloc(sizeof(int));
    BEM_CUDA(cudaMemsetAsync(np.d_count.p, 0, sizeof(int), s));
    BEM_CUDA(cudaMemsetAsync(np.d_err.p, 0, sizeof(int), s));
    NFArgs a{};
    a.tiles = np.d_tiles.as<NFTile>();
    a.ntiles = np.ntiles;
    a.blocks = np.d_desc.as<DenseDesc>();
    a.patch_test = patch_test_dev;
    a.patch_trial = d_patch_trial.as<int>();
    a.tri = mesh.d_tri.as<int4>();
    a.test = sd_test;
    a.trial = sd_trial;
    a.erecP = rt.rec[prec].p;
    a.qoff = rt.qoff[prec].p;
    a.rq = rt.rq[prec].p;
    a.nq = nq;
    a.kappa = kappa;
    a.pool = pool->p;
    a.atomic_scatter = (trt == TR_P0 && tet == TR_P0) ? 0 : 1;
    a.sing = np.d_sing.as<SingItem>();
    a.sing_count = np.d_count.as<int>();
    a.sing_cap = np.sing_cap;
    a.err = np.d_err.as<int>();
    a.erec64 = mesh.d_rec64.as<ElemRec64>();
    for (int c = 0; c < 3; ++c) { a.ss[c] = d_ss[c].as<double>(); a.ss_n[c] = ss_n[c]; }
    a.ss_smem_bytes = ss_bytes <= 160 * 1024 ? (int)ss_bytes : 0;
    a.sing_grid = 152 * 4;
    launch_nf_regular(kid, prec, trt, tet, a, s);
    BEM_CUDA(cudaGetLastError());
    launch_nf_singular(kid, prec, trt, tet, a, s);
    BEM_CUDA(cudaGetLastError());
    return pool;
  };

  NearPass np1;
  BEM_CUDA(cudaEventRecord(evN0, sp.n));
  auto pool1 = run_near(np1, dense_ids, sp.n);
  BEM_CUDA(cudaEventRecord(evN1, sp.n));

  // ---- ACA (batched by scratch budget) + projection ----------------------------------------
  const size_t psz = rsz * (cplx ? 2 : 1);  // ACA value size (compute precision = storage precision)
  std::vector<int> overflow_ids;
  std::vector<LRDesc> lr_all;
  std::vector<int> lr_block;
  float ms_aca = 0.f, ms_proj = 0.f;
  // rows (cols) per U2 (V2) chunk: a multiple of 4, one chunk at most one matvec stage
  auto chunk_len = [&](int dim, int R) {
    const int full = (dim + 3) / 4 * 4;
    if (R <= 0) return 4;
    const int maxc = (int)(mv_stage_bytes() / ((size_t)R * vsize)) / 4 * 4;
    if (maxc < 4) return full;  // too wide for a stage: one chunk, read in place
    return std::min(full, maxc);
  };
  // ACA in rounds: every block first with a provisional rank cap; blocks that reach it while
  // the operator's cap is larger run again from the start with that cap.  ACA is deterministic,
  // so a block gets the factors it would get with the full cap in one round, while the scratch
  // (cap x points per block) of the first round is a fraction of the full-cap one and fits in
  // few batches (each batch waits for the host between its ACA and its projection).
  std::vector<std::unique_ptr<DevBuf>> keep;
  auto newbuf = [&]() { keep.push_back(std::make_unique<DevBuf>()); return keep.back().get(); };
  auto aca_round = [&](const std::vector<int>& ids, int cap, std::vector<int>* retry) {
  // plan the batches first so that the scratch is allocated once per round: cudaFree would
  // synchronise the device and serialise the near-field stream with the ACA stream
  std::vector<std::vector<FarDesc>> batches;
  std::vector<size_t> batch_first;
  long long max_su = 0, max_sv = 0;
  {
    size_t f0 = 0;
    while (f0 < ids.size()) {
    std::vector<FarDesc> fd;
    long long su = 0, sv = 0;
    size_t f1 = f0;
    while (f1 < ids.size()) {
      const BlockH& B = blocks[ids[f1]];
      FarDesc d;
      const ClusterH& ci = ttest->cl[B.rowcl];
      const ClusterH& cj = ttrial->cl[B.colcl];
      d.r0 = (int)ci.PermuPos; d.m = (int)ci.Number; d.c0 = (int)cj.PermuPos; d.n = (int)cj.Number;
      d.pi0 = ttest->patch_ptr[B.rowcl];
      d.ni = ttest->patch_ptr[B.rowcl + 1] - d.pi0;
      d.pj0 = ttrial->patch_ptr[B.colcl];
      d.nj = ttrial->patch_ptr[B.colcl + 1] - d.pj0;
      const long long M = (long long)d.ni * nq, N = (long long)d.nj * nq;
      d.kcap = (int)std::min<long long>(cap, std::min(M, N));
      d.pad = 0;
      const long long need = (long long)NC * d.kcap * (M + N) * (long long)psz;
      if (f1 > f0 && (su + sv) * (long long)psz + need > budget) break;
      d.su = su;
      d.sv = sv;
      su += (long long)NC * d.kcap * M;
      sv += (long long)NC * d.kcap * N;
      fd.push_back(d);
      ++f1;
    }
    max_su = std::max(max_su, su);
    max_sv = std::max(max_sv, sv);
    batches.push_back(std::move(fd));
    batch_first.push_back(f0);
    f0 = f1;
    }
  }
  DevBuf& d_U = *newbuf();
  DevBuf& d_V = *newbuf();
  if (!batches.empty()) {
    d_U.alloc((size_t)max_su * psz);
    d_V.alloc((size_t)max_sv * psz);
  }
  for (size_t bi = 0; bi < batches.size(); ++bi) {
    const std::vector<FarDesc>& fd = batches[bi];
    const size_t f0 = batch_first[bi];
    const int nf = (int)fd.size();
    DevBuf& d_fd = *newbuf();
    DevBuf& d_ranks = *newbuf();
    DevBuf& d_status = *newbuf();
    d_fd.upload(fd, sp.a);
    d_ranks.alloc((size_t)nf * NC * sizeof(int));
    d_status.alloc((size_t)nf * sizeof(int));
    AcaArgs aa{};
    aa.far = d_fd.as<FarDesc>();
    aa.nfar = nf;
    aa.patch_test = patch_test_dev;
    aa.patch_trial = d_patch_trial.as<int>();
    aa.apts = rt.apts[prec].p;
    aa.erecP = rt.rec[prec].p;
    aa.nq = nq;
    aa.kappa = kappa;
    aa.eps = eps;
    aa.U = d_U.p;
    aa.V = d_V.p;
    aa.ranks = d_ranks.as<int>();
    aa.status = d_status.as<int>();
    BEM_CUDA(cudaEventRecord(evA0, sp.a));
    launch_aca(kid, prec, aa, sp.a);
    BEM_CUDA(cudaGetLastError());
    BEM_CUDA(cudaEventRecord(evA1, sp.a));
    std::vector<int> ranks((size_t)nf * NC), status(nf);
    BEM_CUDA(cudaMemcpyAsync(ranks.data(), d_ranks.p, ranks.size() * sizeof(int), cudaMemcpyDeviceToHost, sp.a));
    BEM_CUDA(cudaMemcpyAsync(status.data(), d_status.p, status.size() * sizeof(int), cudaMemcpyDeviceToHost, sp.a));
    BEM_CUDA(cudaStreamSynchronize(sp.a));
    float t;
    BEM_CUDA(cudaEventElapsedTime(&t, evA0, evA1));
    ms_aca += t;
    // factor pool for this batch
    std::vector<LRDesc> lr(nf);
    std::vector<int> pranks((size_t)nf * NC, 0);
    long long usz = 0, vsz = 0;
    for (int f = 0; f < nf; ++f) {
      const int b = ids[f0 + f];
      LRDesc& L = lr[f];
      L.r0 = fd[f].r0; L.m = fd[f].m; L.c0 = fd[f].c0; L.n = fd[f].n;
      L.R = 0; L.toff = 0; L.u = 0; L.v = 0; L.cu = 4; L.cv = 4;
      if (status[f]) {
        if (retry && fd[f].kcap < kcap) retry->push_back(b);  // the full cap may still converge
        else { overflow_ids.push_back(b); block_fallback[b] = 2; }
        continue;
      }
      int R = 0;
      for (int tt = 0; tt < kernel_nterms(kid); ++tt) R += ranks[(size_t)f * NC + kernel_term_comp(kid, tt)];
      for (int c = 0; c < NC; ++c) pranks[(size_t)f * NC + c] = ranks[(size_t)f * NC + c];
      L.R = R;
      L.cu = chunk_len(L.m, R);
      L.cv = chunk_len(L.n, R);
      L.u = (unsigned long long)usz;  // offsets for now
      L.v = (unsigned long long)vsz;
      usz += (long long)((L.m + L.cu - 1) / L.cu) * L.cu * R;
      vsz += (long long)((L.n + L.cv - 1) / L.cv) * L.cv * R;
    }
    auto upool = std::make_unique<DevBuf>(), vpool = std::make_unique<DevBuf>();
    upool->alloc((size_t)std::max<long long>(usz, 1) * vsize);
    vpool->alloc((size_t)std::max<long long>(vsz, 1) * vsize);
    BEM_CUDA(cudaMemsetAsync(upool->p, 0, upool->bytes, sp.a));
    BEM_CUDA(cudaMemsetAsync(vpool->p, 0, vpool->bytes, sp.a));
    for (int f = 0; f < nf; ++f) {
      if (status[f]) continue;
      lr[f].u = (unsigned long long)((char*)upool->p + lr[f].u * vsize);
      lr[f].v = (unsigned long long)((char*)vpool->p + lr[f].v * vsize);
    }
    DevBuf& d_lr = *newbuf();
    DevBuf& d_pr = *newbuf();
    d_lr.upload(lr, sp.a);
    d_pr.upload(pranks, sp.a);
    ProjArgs pa{};
    pa.far = d_fd.as<FarDesc>();
    pa.lr = d_lr.as<LRDesc>();
    pa.nfar = nf;
    pa.ranks = d_pr.as<int>();
    pa.patch_test = patch_test_dev;
    pa.patch_trial = d_patch_trial.as<int>();
    pa.erecP = rt.rec[prec].p;
    pa.qoff = rt.qoff[prec].p;
    pa.rq = rt.rq[prec].p;
    pa.nq = nq;
    pa.kappa = kappa;
    pa.test = sd_test;
    pa.trial = sd_trial;
    pa.U = d_U.p;
    pa.V = d_V.p;
    BEM_CUDA(cudaEventRecord(evP0, sp.a));
    launch_projection(kid, prec, trt, tet, pa, sp.a);
    BEM_CUDA(cudaGetLastError());
    BEM_CUDA(cudaEventRecord(evP1, sp.a));
    BEM_CUDA(cudaStreamSynchronize(sp.a));
    BEM_CUDA(cudaEventElapsedTime(&t, evP0, evP1));
    ms_proj += t;
    for (int f = 0; f < nf; ++f) {
      if (status[f]) continue;
      const int b = ids[f0 + f];
      block_rank[b] = lr[f].R;
      lr_all.push_back(lr[f]);
      lr_block.push_back(b);
    }
    pools.push_back(std::move(upool));
    pools.push_back(std::move(vpool));
  }
  };
  {
    const int cap1 = std::min(kcap, 48);
    std::vector<int> retry;
    aca_round(far_ids, cap1, cap1 < kcap ? &retry : nullptr);
    if (!retry.empty()) aca_round(retry, kcap, nullptr);
  }

  // ---- near-field pass 1 done; pass 2 for ACA rank-cap blocks ------------------------------
  BEM_CUDA(cudaStreamSynchronize(sp.n));
  float ms_near = 0.f;
  if (!np1.desc.empty()) BEM_CUDA(cudaEventElapsedTime(&ms_near, evN0, evN1));
  auto check_pass = [&](NearPass& np) {
    if (np.desc.empty()) return;
    int err = 0, cnt = 0;
    BEM_CUDA(cudaMemcpy(&err, np.d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    BEM_CUDA(cudaMemcpy(&cnt, np.d_count.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err || cnt > np.sing_cap) throw Error(BEM_ERR_INTERNAL, "singular pair list overflow");
    info.n_singular_pairs += cnt;
    info.n_regular_pairs += np.npairs - cnt;
  };
  check_pass(np1);
  NearPass np2;
  std::unique_ptr<DevBuf> pool2;
  if (!overflow_ids.empty()) {
    BEM_CUDA(cudaEventRecord(evN0, sp.n));
    pool2 = run_near(np2, overflow_ids, sp.n);
    BEM_CUDA(cudaEventRecord(evN1, sp.n));
    BEM_CUDA(cudaStreamSynchronize(sp.n));
    float t2 = 0.f;
    BEM_CUDA(cudaEventElapsedTime(&t2, evN0, evN1));
    ms_near += t2;
    check_pass(np2);
  }

  // ---- matvec descriptors -------------------------------------------------------------------
  mvdense.clear();
  auto add_dense = [&](NearPass& np, DevBuf* pool) {
    for (size_t k = 0; k < np.desc.size(); ++k) {
      const DenseDesc& d = np.desc[k];
      MVDense m;
      m.ptr = (unsigned long long)((char*)pool->p + (size_t)d.off * vsize);
      m.r0 = d.r0; m.m = d.m; m.c0 = d.c0; m.n = d.n;
      mvdense.push_back(m);
      info.bytes_dense += (long long)d.m * d.n * (long long)vsize;
    }
  };
  if (pool1) add_dense(np1, pool1.get());
  if (pool2) add_dense(np2, pool2.get());
  if (pool1) pools.push_back(std::move(pool1));
  if (pool2) pools.push_back(std::move(pool2));
  mvlr = lr_all;
  t_len = 0;
  for (auto& L : mvlr) {
    L.toff = t_len;
    t_len += L.R;
    info.bytes_lowrank += (long long)L.R * (L.m + L.n) * (long long)vsize;
    info.bytes_lowrank_u += (long long)L.R * L.m * (long long)vsize;
  }
  const auto t_items = clk::now();
  mv_fused = mv_fused_supported();
  // the lists of the single right-hand-side matvec; the others on first use
  build_mv_items(mv_fused ? 0x30u : 0x03u, false, false);
  info.ms_mvitems = ms_since(t_items);
  BEM_CUDA(cudaDeviceSynchronize());
  keep.clear();

  // ---- info -----------------------------------------------------------------------------------
  info.is_complex = cplx ? 1 : 0;
  info.height = height;
  info.width = width;
  info.nblocks = nb;
  info.nnear = 0;
  info.nfar = (int)mvlr.size();
  info.nfallback = 0;
  info.nze = 0;
  info.max_rank = 0;
  info.sum_rank = 0;
  for (int b = 0; b < nb; ++b) {
    const ClusterH& ci = ttest->cl[blocks[b].rowcl];
    const ClusterH& cj = ttrial->cl[blocks[b].colcl];
    if (blocks[b].near) info.nnear++;
    if (block_fallback[b]) info.nfallback++;
    if (block_rank[b] >= 0) {
      info.nze += (long long)block_rank[b] * (ci.Number + cj.Number);
      info.max_rank = std::max(info.max_rank, block_rank[b]);
      info.sum_rank += block_rank[b];
    } else {
      info.nze += (long long)ci.Number * cj.Number;
    }
  }
  info.ms_aca = ms_aca;
  info.ms_projection = ms_proj;
  info.ms_nearfield = ms_near;
  info.ms_total = ms_since(t_start);
}

bool pairs_overflow(size_t ntiles) { return ntiles > (size_t)INT_MAX; }

// ---------------------------------------------------------------------------------------------
// Groups the payload (dense blocks, U2 chunks, V2 chunks) into work items of at most one
// matvec stage: consecutive segments whose bytes are contiguous share one bulk copy.
void HOperator::ensure_mv(unsigned mask, bool multi, cudaStream_t s) {
  const unsigned miss = mask & ~mv_built;
  const bool mmiss = multi && !mv_multi_built;
  if (!miss && !mmiss) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  BEM_CUDA(cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone)
    throw Error(BEM_ERR_STATE, "this matvec form has not run before: apply it once outside the stream capture");
  build_mv_items(miss, mmiss, true);
}

void HOperator::build_mv_items(unsigned mask, bool multi, bool keep) {
  if (!keep) {
    mv_built = 0;
    mv_multi_built = false;
    for (int p = 0; p < MV_NPASS; ++p) n_items[p] = 0;
    n_mr_items[0] = n_mr_items[1] = 0;
    n_ro_leaves = 0;
  }
  const size_t stage = (size_t)mv_stage_bytes();
  const int piece = mv_piece > 0 ? mv_piece : mv_piece_elems();  // target elements per piece (one warp's task)
  // A span is one contiguous payload range (a block, or a chunk of one) with its generic
  // pieces (kind, block, first row/col, count, byte offset from the span start).
  struct GPiece { int kind, blk, k0, cnt, soff; };
  // spans and items keep their pieces in flat pools (first piece, count): no allocation per span
  struct Span { unsigned long long src; size_t bytes; bool direct; int p0, np; };
  struct GItem { unsigned long long src; int bytes; int p0, np; };
  auto group = [&](const std::vector<Span>& spans, const std::vector<GPiece>& spool, std::vector<GItem>& items,
                   std::vector<GPiece>& ipool) {
    ipool.reserve(spool.size());
    GItem cur{0, 0, 0, 0};
    bool open = false;
    for (const Span& sp : spans) {
      if (sp.direct) {
        if (open) { items.push_back(cur); open = false; }
        items.push_back(GItem{sp.src, 0, (int)ipool.size(), sp.np});
        ipool.insert(ipool.end(), spool.begin() + sp.p0, spool.begin() + sp.p0 + sp.np);
        continue;
      }
      if (!(open && sp.src == cur.src + (unsigned long long)cur.bytes && cur.bytes + sp.bytes <= stage &&
            (size_t)cur.np + sp.np <= (size_t)mv_max_pieces())) {
        if (open) items.push_back(cur);
        cur = GItem{sp.src, 0, (int)ipool.size(), 0};
        open = true;
      }
      for (int q = 0; q < sp.np; ++q) {
        GPiece g = spool[sp.p0 + q];
        g.soff += cur.bytes;
        ipool.push_back(g);
      }
      cur.np += sp.np;
      cur.bytes += (int)sp.bytes;
    }
    if (open) items.push_back(cur);
  };
  auto pad16 = [](size_t b) { return (b + 15) / 16 * 16; };
  // appends the pieces of one span to pool; returns the count
  auto pieces = [&](std::vector<GPiece>& pool, int kind, int blk, int k0, int cnt, int per, size_t step) {
    int pc = std::max(1, piece / std::max(1, per));
    const int cap = mv_max_pieces();
    if ((cnt + pc - 1) / pc > cap) pc = (cnt + cap - 1) / cap;
    int np = 0;
    for (int a = 0; a < cnt; a += pc, ++np) pool.push_back(GPiece{kind, blk, k0 + a, std::min(pc, cnt - a), (int)(a * step)});
    return np;
  };
  // dense blocks (column-major): column chunks with 16-byte aligned starts
  std::vector<Span> sd;
  std::vector<GPiece> pd;
  sd.reserve(mvdense.size());
  for (int k = 0; k < (int)mvdense.size(); ++k) {
    const MVDense& D = mvdense[k];
    const size_t colb = (size_t)D.m * vsize;
    const size_t total = pad16(colb * D.n);
    if (total <= stage) {
      const int p0 = (int)pd.size();
      sd.push_back({D.ptr, total, false, p0, pieces(pd, 0, k, 0, D.n, D.m, colb)});
      continue;
    }
    size_t q = 1;
    while ((colb * q) % 16) ++q;
    const size_t cc = stage / colb / q * q;
    if (cc == 0) {  // one column exceeds a stage: read in place
      const int p0 = (int)pd.size();
      sd.push_back({D.ptr, 0, true, p0, pieces(pd, 0, k, 0, D.n, D.m, colb)});
      continue;
    }
    for (int j0 = 0; j0 < D.n; j0 += (int)cc) {
      const int cnt = std::min((int)cc, D.n - j0);
      const size_t b0 = (size_t)j0 * colb;
      const size_t b1 = (j0 + cnt == D.n) ? total : (size_t)(j0 + cnt) * colb;
      const int p0 = (int)pd.size();
      sd.push_back({D.ptr + b0, b1 - b0, false, p0, pieces(pd, 0, k, j0, cnt, D.m, colb)});
    }
  }
  // low-rank factors: U2 row chunks (pieces of rows), V2 column chunks (pieces of columns)
  std::vector<Span> su, sv;
  std::vector<GPiece> pu, pv;
  for (int f = 0; f < (int)mvlr.size(); ++f) {
    const LRDesc& L = mvlr[f];
    if (L.R == 0) continue;
    const size_t cub = (size_t)L.cu * L.R * vsize, cvb = (size_t)L.cv * L.R * vsize;
    for (int i0 = 0, c = 0; i0 < L.m; i0 += L.cu, ++c) {
      const int p0 = (int)pu.size();
      su.push_back({L.u + c * cub, cub, cub > stage, p0, pieces(pu, 1, f, i0, std::min(L.cu, L.m - i0), L.R, vsize)});
    }
    for (int j0 = 0, c = 0; j0 < L.n; j0 += L.cv, ++c) {
      const int p0 = (int)pv.size();
      sv.push_back({L.v + c * cvb, cvb, cvb > stage, p0,
                    pieces(pv, 2, f, j0, std::min(L.cv, L.n - j0), L.R, (size_t)L.R * vsize)});
    }
  }
  std::vector<GItem> id, iu, iv;
  std::vector<GPiece> qd, qu, qv;
  group(sd, pd, id, qd);
  group(su, pu, iu, qu);
  group(sv, pv, iv, qv);
  // per pass: 0 t = V2 x, 1 y += D x + U2 t, 2 t = U2^T x, 3 y += D^T x + V2^T t
  auto piece_raw = [&](int pass, const GPiece& g) {
    MVPiece p{};
    p.soff = g.soff;
    if (g.kind == 0) {
      const MVDense& D = mvdense[g.blk];
      if (pass == 1) p = MVPiece{g.soff, 1, D.m, D.m, g.cnt, D.c0 + g.k0, D.r0, 0};
      else p = MVPiece{g.soff, D.m, 1, g.cnt, D.m, D.r0, D.c0 + g.k0, 0};
    } else if (g.kind == 1) {
      const LRDesc& L = mvlr[g.blk];
      if (pass == 1) p = MVPiece{g.soff, 1, L.cu, g.cnt, L.R, L.toff, L.r0 + g.k0, 1};
      else p = MVPiece{g.soff, L.cu, 1, L.R, g.cnt, L.r0 + g.k0, L.toff, 2};
    } else {
      const LRDesc& L = mvlr[g.blk];
      if (pass == 0) p = MVPiece{g.soff, 1, L.R, L.R, g.cnt, L.c0 + g.k0, L.toff, 2};
      else p = MVPiece{g.soff, L.R, 1, g.cnt, L.R, L.toff, L.c0 + g.k0, 1};
    }
    return p;
  };
  auto piece_for = [&](int pass, const GPiece& g) {
    MVPiece p = piece_raw(pass, g);
    p.ow = std::min(p.O, 32);
    p.groups = 32 / p.ow;
    p.inv_ow = 1.0f / (float)p.ow;
    return p;
  };
  // passes 0-3 as above; 4-7 are the phases of the single-launch matvec: 4 = t = V2 x with
  // y += D x (no dependence on t), 5 = y += U2 t; 6 = t = U2^T x with y += D^T x, 7 = y += V2^T t.
  // Each list is applied with the piece semantics of pass `sem`.
  struct LS { const std::vector<GItem>* L; const std::vector<GPiece>* P; int sem; };
  const std::vector<LS> lists[MV_NPASS] = {
      {{&iv, &qv, 0}},                   {{&id, &qd, 1}, {&iu, &qu, 1}}, {{&iu, &qu, 2}}, {{&id, &qd, 3}, {&iv, &qv, 3}},
      {{&iv, &qv, 0}, {&id, &qd, 1}},   {{&iu, &qu, 1}},                {{&iu, &qu, 2}, {&id, &qd, 3}}, {{&iv, &qv, 3}}};
  long long npieces = 0;
  const int esz = cplx ? 16 : 8;          // one x or t entry as staged (x: FP32 hi+lo or FP64)
  const int per16 = 16 / esz;             // entries per 16 bytes
  const int inarea = mv_in_bytes();
  // the passes are independent: build their host tables on parallel threads, upload after
  std::vector<MVTItem> pass_items[MV_NPASS];
  std::vector<MVPiece> pass_pcs[MV_NPASS];
  std::vector<MVRange> pass_rngs[MV_NPASS];
  // tasks: a pass's item lists cut into chunks; each chunk builds its own tables with local
  // offsets, and the chunks are concatenated in order afterwards
  struct Task {
    int pass;
    const LS* ls;
    size_t i0, i1;
    std::vector<MVTItem> items;
    std::vector<MVPiece> pcs;
    std::vector<MVRange> rngs;
  };
  std::vector<Task> tasks;
  for (int pass = 0; pass < MV_NPASS; ++pass)
    for (const LS& ls : lists[pass]) {
      if (!(mask & (1u << pass))) continue;
      const size_t n = ls.L->size(), chunk = std::max<size_t>(128, (n + 7) / 8);
      for (size_t i0 = 0; i0 < n; i0 += chunk) tasks.push_back(Task{pass, &ls, i0, std::min(n, i0 + chunk), {}, {}, {}});
    }
  auto build_task = [&](Task& tk) {
    std::vector<MVTItem>& items = tk.items;
    std::vector<MVPiece>& pcs = tk.pcs;
    std::vector<MVRange>& rngs = tk.rngs;
    struct Iv { int src, e0, e1; };
    std::vector<Iv> raw, ivs, merged;  // per-item scratch, reused
    std::vector<int> piv, dst;
    {
      const LS& ls = *tk.ls;
      const int sem = ls.sem;
      for (size_t ii = tk.i0; ii < tk.i1; ++ii) {
        const GItem& gi = (*ls.L)[ii];
        const GPiece* gp = ls.P->data() + gi.p0;
        MVTItem it{};
        it.src = gi.src;
        it.bytes = gi.bytes;
        it.seg0 = (int)pcs.size();
        it.nseg = gi.np;
        it.rng0 = (int)rngs.size();
        // input intervals of the pieces, merged into 16-byte aligned ranges of x or t.  Nearby
        // ranges are merged further (smallest gap first) while the staged bytes still fit the
        // input area: the producer issues the first two ranges from the descriptor and has to
        // load the others, so staging a few unused entries of x or t (L2 resident) is cheaper.
        raw.clear();
        for (int q = 0; q < gi.np; ++q) {
          const MVPiece p = piece_for(sem, gp[q]);
          raw.push_back({p.flags & 1, p.in_off, p.in_off + p.Kc});
          pcs.push_back(p);
        }
        ivs.assign(raw.begin(), raw.end());
        for (Iv& v : ivs) {
          v.e0 = v.e0 / per16 * per16;
          v.e1 = (v.e1 + per16 - 1) / per16 * per16;
        }
        std::sort(ivs.begin(), ivs.end(), [](const Iv& x, const Iv& y) {
          return x.src != y.src ? x.src < y.src : x.e0 < y.e0;
        });
        {
          merged.clear();
          for (const Iv& v : ivs) {
            if (!merged.empty() && merged.back().src == v.src && v.e0 <= merged.back().e1)
              merged.back().e1 = std::max(merged.back().e1, v.e1);
            else
              merged.push_back(v);
          }
          ivs.swap(merged);
        }
        auto staged = [&]() {
          long long b = 0;
          for (const Iv& v : ivs) b += (long long)(v.e1 - v.e0) * esz;
          return b;
        };
        long long tot = staged();
        while (ivs.size() > 2) {
          int best = -1;
          long long gap = 0;
          for (size_t r = 0; r + 1 < ivs.size(); ++r) {
            if (ivs[r].src != ivs[r + 1].src) continue;
            const long long g2 = (long long)(ivs[r + 1].e0 - ivs[r].e1) * esz;
            if (best < 0 || g2 < gap) {
              best = (int)r;
              gap = g2;
            }
          }
          if (best < 0 || tot + gap > inarea) break;
          ivs[best].e1 = ivs[best + 1].e1;
          ivs.erase(ivs.begin() + best + 1);
          tot += gap;
        }
        piv.clear();  // range index of each piece
        for (const Iv& v : raw) {
          int r = 0;
          while (!(ivs[r].src == v.src && ivs[r].e0 <= v.e0 && v.e1 <= ivs[r].e1)) ++r;
          piv.push_back(r);
        }
        dst.assign(ivs.size(), 0);
        int total = 0;
        for (size_t r = 0; r < ivs.size(); ++r) {
          dst[r] = total;
          total += (ivs[r].e1 - ivs[r].e0) * esz;
        }
        if (total <= inarea) {
          for (size_t r = 0; r < ivs.size(); ++r) {
            const MVRange rg{ivs[r].src, ivs[r].e0, (ivs[r].e1 - ivs[r].e0) * esz, dst[r]};
            rngs.push_back(rg);
            if (r < 2) {
              it.r[4 * r + 0] = rg.src;
              it.r[4 * r + 1] = rg.elem;
              it.r[4 * r + 2] = rg.bytes;
              it.r[4 * r + 3] = rg.dst;
            }
          }
          for (int q = 0; q < gi.np; ++q) {
            MVPiece& p = pcs[it.seg0 + q];
            const Iv& v = ivs[piv[q]];
            p.in_soff = dst[piv[q]] + (p.in_off - v.e0) * esz;
          }
          it.nrng = (int)ivs.size();
          it.inbytes = total;
        } else {
          it.nrng = 0;
          it.inbytes = -1;  // inputs read in place
        }
        items.push_back(it);
      }
    }
  };
  {
    std::vector<std::thread> th;
    std::exception_ptr failure;
    std::mutex fmu;
    std::atomic<size_t> next{0};
    const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (int w = 0; w < nth; ++w)
      th.emplace_back([&] {
        try {
          for (size_t k = next++; k < tasks.size(); k = next++) build_task(tasks[k]);
        } catch (...) {
          std::lock_guard<std::mutex> lk(fmu);
          failure = std::current_exception();
        }
      });
    for (auto& t : th) t.join();
    if (failure) std::rethrow_exception(failure);
    size_t ni[MV_NPASS] = {}, np_[MV_NPASS] = {}, nr[MV_NPASS] = {};
    for (const Task& tk : tasks) {
      ni[tk.pass] += tk.items.size();
      np_[tk.pass] += tk.pcs.size();
      nr[tk.pass] += tk.rngs.size();
    }
    for (int pass = 0; pass < MV_NPASS; ++pass) {
      pass_items[pass].reserve(ni[pass]);
      pass_pcs[pass].reserve(np_[pass]);
      pass_rngs[pass].reserve(nr[pass]);
    }
    for (Task& tk : tasks) {
      const int seg_off = (int)pass_pcs[tk.pass].size(), rng_off = (int)pass_rngs[tk.pass].size();
      for (MVTItem& it : tk.items) {
        it.seg0 += seg_off;
        it.rng0 += rng_off;
      }
      pass_items[tk.pass].insert(pass_items[tk.pass].end(), tk.items.begin(), tk.items.end());
      pass_pcs[tk.pass].insert(pass_pcs[tk.pass].end(), tk.pcs.begin(), tk.pcs.end());
      pass_rngs[tk.pass].insert(pass_rngs[tk.pass].end(), tk.rngs.begin(), tk.rngs.end());
    }
  }
  for (int pass = 0; pass < MV_NPASS; ++pass) {
    if (!(mask & (1u << pass))) continue;
    d_items[pass].upload(pass_items[pass]);
    d_pieces[pass].upload(pass_pcs[pass]);
    d_ranges[pass].upload(pass_rngs[pass]);
    n_items[pass] = (int)pass_items[pass].size();
    const int ip = pass < 4 ? pass : (pass == 4 ? 0 : (pass == 5 ? 1 : (pass == 6 ? 2 : 3)));
    info.mv_ranges[ip] = (int)pass_rngs[pass].size();
    info.mv_items[ip] = n_items[pass];
    npieces += (long long)pass_pcs[pass].size();
  }
  if (npieces > 0 && (mask & 0x30u)) info.mv_segments = (int)npieces;
  else if (npieces > 0 && !keep) info.mv_segments = (int)npieces;
  mv_built |= mask;
  // lists for several right-hand sides (the pass kernel reads the blocks in place there): one
  // piece per span (a dense column chunk, a V2 column chunk, a U2 row chunk, each at most one
  // stage of bytes), so a piece reduces over the whole chunk and each output row receives one
  // atomic per chunk instead of one per column slice; chunks keep the items balanced
  if (multi) {
    mv_multi_built = true;
    std::vector<MVTItem> mi[2];
    std::vector<MVPiece> mp[2];
    auto add = [&](int ph, unsigned long long src, MVPiece pc) {
      pc.ow = std::min(pc.O, 32);
      pc.groups = 32 / pc.ow;
      pc.inv_ow = 1.0f / (float)pc.ow;
      MVTItem it{};
      it.src = src;
      it.seg0 = (int)mp[ph].size();
      it.nseg = 1;
      it.inbytes = -1;
      mp[ph].push_back(pc);
      mi[ph].push_back(it);
    };
    // first piece of a span gives (kind, block, first row/column); the count is the span's total
    auto whole = [&](const Span& sp, const std::vector<GPiece>& pool, int sem) {
      GPiece g = pool[sp.p0];
      for (int q = 1; q < sp.np; ++q) g.cnt += pool[sp.p0 + q].cnt;
      g.soff = 0;
      return piece_raw(sem, g);
    };
    for (const Span& sp : sv) add(0, sp.src, whole(sp, pv, 0));
    for (const Span& sp : sd) add(1, sp.src, whole(sp, pd, 1));
    for (const Span& sp : su) add(1, sp.src, whole(sp, pu, 1));
    // owner-computes lists of y += D x + U2 t: per leaf row cluster, every dense block and
    // low-rank U2 row slice that touches its rows (blocks split along the leaf boundaries)
    {
      std::vector<std::pair<int, int>> lv;  // leaf rows [first, end)
      for (const ClusterH& C : ttest->cl)
        if (C.Child1 < 0) lv.push_back({(int)C.PermuPos, (int)(C.PermuPos + C.Number)});
      std::sort(lv.begin(), lv.end());
      std::vector<std::vector<int4>> per(lv.size());
      auto add_rows = [&](int kind, int blk, int r0, int m) {
        int l = (int)(std::upper_bound(lv.begin(), lv.end(), std::make_pair(r0, INT_MAX)) - lv.begin()) - 1;
        for (l = std::max(l, 0); l < (int)lv.size() && lv[l].first < r0 + m; ++l) {
          const int a0 = std::max(r0, lv[l].first), a1 = std::min(r0 + m, lv[l].second);
          if (a1 > a0) per[l].push_back(make_int4(kind, blk, a0 - r0, a1 - a0));
        }
      };
      for (int k = 0; k < (int)mvdense.size(); ++k) add_rows(0, k, mvdense[k].r0, mvdense[k].m);
      for (int f = 0; f < (int)mvlr.size(); ++f)
        if (mvlr[f].R > 0) add_rows(1, f, mvlr[f].r0, mvlr[f].m);
      std::vector<int4> leaves, ents;
      for (size_t l = 0; l < lv.size(); ++l) {
        const int e0 = (int)ents.size();
        ents.insert(ents.end(), per[l].begin(), per[l].end());
        leaves.push_back(make_int4(lv[l].first, lv[l].second, e0, (int)ents.size()));
      }
      d_ro_leaves.upload(leaves);
      d_ro_ents.upload(ents);
      n_ro_leaves = (int)leaves.size();
    }
    for (int ph = 0; ph < 2; ++ph) {
      d_mr_items[ph].upload(mi[ph]);
      d_mr_pieces[ph].upload(mp[ph]);
      n_mr_items[ph] = (int)mi[ph].size();
    }
  }
  if (d_err.p) return;  // the shared device tables exist already
  d_mvdense.upload(mvdense);
  d_mvlr.upload(mvlr);
  d_err.alloc(sizeof(int));
  BEM_CUDA(cudaMemset(d_err.p, 0, sizeof(int)));
  // [0, 1] claim / finish counters of the pass kernels, [2, 3] claim counters of the two phases
  // of the single-launch matvec, [4, 5] its grid barrier (arrivals, generation)
  d_sched.alloc(8 * sizeof(int));
  BEM_CUDA(cudaMemset(d_sched.p, 0, 8 * sizeof(int)));
  int dev = 0, nsm = 152;
  BEM_CUDA(cudaGetDevice(&dev));
  BEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  mv_grid = nsm;
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
  const int* pin = trans ? (ttest == ttrial ? d_perm_trial.as<int>() : d_perm_test.as<int>()) : d_perm_trial.as<int>();
  const int* pout = trans ? d_perm_trial.as<int>() : (ttest == ttrial ? d_perm_trial.as<int>() : d_perm_test.as<int>());
  std::array<cudaEvent_t, 5> ev{};
  if (profiling) {
    for (auto& e : ev) BEM_CUDA(cudaEventCreate(&e));
    BEM_CUDA(cudaEventRecord(ev[0], s));
  }
  if (tc_eligible(trans, nrhs, s)) {
    mult_tc(alpha, x, beta, y, nrhs, s);
    return;
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
  launch_permute_in(prec, cplx, pin, in_n, nrhs, in_n, x, d_xp.p, s);
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
  launch_permute_out(cplx, pout, out_n, nrhs, out_n, alpha, beta, d_yp.p, y, s);
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
  BEM_CUDA(cudaMemcpy(&e, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  return e;
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
  TrigRule r = make_trig_rule(4);
  const int nq = (int)r.w.size();
  std::vector<std::vector<std::pair<int, double>>> rows(nrows);
  auto shape = [&](const SpaceH& sp, int e, double xi, double eta, double S[3][3], int& dim) {
    const ElemRec64& g = m.rec[e];
    if (sp.kind == BEM_P0) { S[0][0] = sp.dual ? g.invdetJ : 1.0; dim = 1; return; }
    if (sp.kind == BEM_P1) { S[0][0] = xi; S[1][0] = eta; S[2][0] = 1.0 - xi - eta; dim = 1; return; }
    double x[3];
    m.map(e, xi, eta, x);
    for (int a = 0; a < 3; ++a) {
      const int o = (a + 2) % 3;
      double v[3];
      for (int c = 0; c < 3; ++c) v[c] = sp.sign[3 * e + a] * (x[c] - g.p[o][c]) * g.invdetJ;
      // HCurl trace: n x the RT0 shape of the same edge
      for (int c = 0; c < 3; ++c)
        S[a][c] = sp.kind == BEM_HCURL ? g.n[(c + 1) % 3] * v[(c + 2) % 3] - g.n[(c + 2) % 3] * v[(c + 1) % 3] : v[c];
    }
    dim = 3;
  };
  for (int e = 0; e < m.nt; ++e)
    for (int q = 0; q < nq && trial->on(e) && test->on(e); ++q) {
      double Si[3][3], Sj[3][3];
      int di, dj;
      shape(*test, e, r.xi[q], r.eta[q], Si, di);
      shape(*trial, e, r.xi[q], r.eta[q], Sj, dj);
      if (di != dj) throw Error(BEM_ERR_ARG, "mass matrix of scalar and vector spaces");
      const double w = r.w[q] * m.rec[e].detJ;
      for (int a = 0; a < test->nd; ++a)
        for (int b = 0; b < trial->nd; ++b) {
          double s = 0.0;
          for (int c = 0; c < di; ++c) s += Si[a][c] * Sj[b][c];
          rows[test->el_dofs(e)[a]].push_back({trial->el_dofs(e)[b], w * s});
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

}  // namespace bem

namespace bem {

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

namespace bem {

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
