// Assembly of the H-matrix on the GPU and its matvec work lists (reference
// GenericIntegralOperator ctor src/ngbem.cpp:314-330, CalcHMatrix :118-157, HMatrix
// src/hmat.cpp:614-621).  The products are in apply.cpp, the solvers in gmres.cpp.
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
#include <cstdlib>
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

SpaceDev space_dev(const SpaceH& s, int tr, const DevBuf& pinv) {
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
  if (a.curved() || b.curved()) {
    // one geometry order for the union: a flat mesh joined to a curved one takes the curved
    // order with its nodes on the flat triangles
    const int g = std::max(a.gorder, b.gorder), nn = (g + 1) * (g + 2) / 2;
    std::vector<double> G;
    G.reserve((size_t)(a.nt + b.nt) * nn * 3);
    for (const MeshH* m : {&a, &b})
      for (int e = 0; e < m->nt; ++e) {
        int n = 0;
        for (int i = g; i >= 0; --i)
          for (int j = g - i; j >= 0; --j, ++n) {
            double x[3];
            if (m->gorder == g) {
              for (int c = 0; c < 3; ++c) x[c] = m->G[((size_t)e * nn + n) * 3 + c];
            } else {
              m->map(e, (double)i / g, (double)j / g, x);
              // the corner nodes are the vertices themselves
              const int corner = i == g ? 0 : (j == g ? 1 : (g - i - j == g ? 2 : -1));
              if (corner >= 0)
                for (int c = 0; c < 3; ++c) x[c] = m->X[3 * (size_t)m->T[3 * e + corner] + c];
            }
            G.insert(G.end(), x, x + 3);
          }
      }
    own_mesh->set_geometry(g, G.data());
  }
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
  // NGBEM_GB300_ACA_FAIL=k (k > 0): the ACA of every far block whose number in the block list
  // is a multiple of k fails on the host (fault injection; such blocks are assembled densely)
  long long aca_evals = 0;
  int aca_fail_every = 0;
  if (const char* ev = std::getenv("NGBEM_GB300_ACA_FAIL")) aca_fail_every = std::max(0, std::atoi(ev));
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
    a.pgeo = rt.pgeo[prec].p;
    a.nq = nq;
    a.kappa = kappa;
    a.pool = pool->p;
    a.atomic_scatter = (trt == TR_P0 && tet == TR_P0) ? 0 : 1;
    a.sing = np.d_sing.as<SingItem>();
    a.sing_count = np.d_count.as<int>();
    a.sing_cap = np.sing_cap;
    a.err = np.d_err.as<int>();
    a.erec64 = mesh.d_rec64.as<ElemRec64>();
    a.gnodes = mesh.curved() ? mesh.d_gnodes.as<double>() : nullptr;
    a.gorder = mesh.gorder;
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
    aa.pgeo = rt.pgeo[prec].p;
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
    for (int f = 0; f < nf; ++f) {
      const long long pts = (long long)(fd[f].ni + fd[f].nj) * nq;
      for (int c = 0; c < NC; ++c)
        aca_evals += (long long)(status[f] ? fd[f].kcap : ranks[(size_t)f * NC + c] + 1) * pts;
    }
    // host-side fault injection for the tests of the dense fallback: the ACA of the chosen
    // far blocks counts as failed (as if it had reached the rank cap), in every round
    if (aca_fail_every > 0)
      for (int f = 0; f < nf; ++f)
        if (ids[f0 + f] % aca_fail_every == 0) status[f] = 1;
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
    pa.pgeo = rt.pgeo[prec].p;
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
    info.nf_regular_evals += (np.npairs - cnt) * (long long)nq * nq;
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
  info.aca_evals = aca_evals;
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
}  // namespace bem
