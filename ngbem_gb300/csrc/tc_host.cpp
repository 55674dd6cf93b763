// Host side of the tensor-core products for several right-hand sides (kernels in
// tc_matvec.cu): column and row tiles of the blocks, their packed operand panels, a balanced
// static item list per CTA, the per-leaf lists of partial rows, and the application Y = A X for
// 2..32 complex right-hand sides (reference HMatrix::MultAdd, src/hmat.cpp:647-655, applied to
// many vectors at once).
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <map>
#include <mutex>
#include <queue>

#include "host.hpp"

namespace bem {

namespace {

using clk = std::chrono::steady_clock;

// Known-answer check of the instruction and shared-memory descriptor encodings: one
// 128 x 32 x 16 product of small integers and eighths (exact in TF32 and in FP32) against the
// host product.  The tensor-core path is used only on a device where it passed.
int tc_selftest_run() {
  const int N = 32, nkc = 4, K = 16;
  std::vector<float> A(128 * K), Bh(N * K), Bl(N * K);
  for (int r = 0; r < 128; ++r)
    for (int k = 0; k < K; ++k) A[r * K + k] = (float)((r * 7 + k * 3) % 11 - 5);
  for (int n = 0; n < N; ++n)
    for (int k = 0; k < K; ++k) {
      Bh[n * K + k] = (float)((n * 5 + k) % 7 - 3);
      Bl[n * K + k] = (float)((n + 2 * k) % 5 - 2) / 8.0f;
    }
  std::vector<float> pa((size_t)nkc * 128 * 4), pb((size_t)nkc * 2 * N * 4);
  for (int kc = 0; kc < nkc; ++kc)
    for (int r = 0; r < 128; ++r)
      for (int k = 0; k < 4; ++k) pa[((size_t)kc * 128 + r) * 4 + k] = A[r * K + 4 * kc + k];
  for (int kc = 0; kc < nkc; ++kc)
    for (int h = 0; h < 2; ++h)
      for (int n = 0; n < N; ++n)
        for (int k = 0; k < 4; ++k)
          pb[((size_t)(2 * kc + h) * N + n) * 4 + k] = (h ? Bl : Bh)[n * K + 4 * kc + k];
  DevBuf da, db, dd, de;
  da.upload(pa);
  db.upload(pb);
  dd.alloc((size_t)128 * N * sizeof(float));
  de.alloc(sizeof(int));
  BEM_CUDA(cudaMemset(dd.p, 0, dd.bytes));
  BEM_CUDA(cudaMemset(de.p, 0, sizeof(int)));
  BEM_CUDA(launch_tc_selftest(da.p, db.p, N, nkc, dd.as<float>(), de.as<int>(), 0));
  BEM_CUDA(cudaDeviceSynchronize());
  std::vector<float> d((size_t)128 * N);
  int err = 0;
  BEM_CUDA(cudaMemcpy(d.data(), dd.p, dd.bytes, cudaMemcpyDeviceToHost));
  BEM_CUDA(cudaMemcpy(&err, de.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return 0;
  for (int r = 0; r < 128; ++r)
    for (int n = 0; n < N; ++n) {
      double e = 0.0;
      for (int k = 0; k < K; ++k) e += (double)A[r * K + k] * ((double)Bh[n * K + k] + (double)Bl[n * K + k]);
      if ((double)d[(size_t)r * N + n] != e) return 0;
    }
  return 1;
}

// longest-processing-time assignment of items to CTAs; items are reordered so that every
// CTA's list is contiguous
void balance(std::vector<TCItem>& items, const std::vector<double>& cost, int nsm, std::vector<int2>& sched) {
  const int n = (int)items.size();
  const int G = std::max(1, std::min(nsm, n));
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  using E = std::pair<double, int>;
  std::priority_queue<E, std::vector<E>, std::greater<E>> q;
  for (int c = 0; c < G; ++c) q.push({0.0, c});
  std::vector<std::vector<int>> per(G);
  for (int i : order) {
    E e = q.top();
    q.pop();
    per[e.second].push_back(i);
    q.push({e.first + cost[i], e.second});
  }
  std::vector<TCItem> out;
  out.reserve(n);
  sched.assign(G, make_int2(0, 0));
  for (int c = 0; c < G; ++c) {
    sched[c].x = (int)out.size();
    for (int i : per[c]) out.push_back(items[i]);
    sched[c].y = (int)per[c].size();
  }
  items.swap(out);
}

// Stage plans of every CTA: the K ranges of its items' segments in order, packed into
// pipeline stages of `cap` bytes (at most TC_MAXCH ranges, each at least one MMA step of
// K = 8), so that the kernel reads one contiguous run of descriptors per stage.
void plan_stages(const std::vector<TCItem>& items, const std::vector<TCSeg>& segs, const std::vector<int2>& sched,
                 int cap, std::vector<int4>& sched4, std::vector<int2>& stages, std::vector<TCChunk>& chunks) {
  sched4.assign(sched.size(), make_int4(0, 0, 0, 0));
  for (size_t c = 0; c < sched.size(); ++c) {
    const int s0 = (int)stages.size();
    int used = 0, first = (int)chunks.size();
    auto close = [&]() {
      if ((int)chunks.size() > first) {
        chunks.back().flags |= 4;
        stages.push_back(make_int2(first, (int)chunks.size() - first));
      }
      first = (int)chunks.size();
      used = 0;
    };
    for (int ii = sched[c].x; ii < sched[c].x + sched[c].y; ++ii) {
      const TCItem& I = items[ii];
      const int per = 2048 + 32 * I.N;
      bool item_first = true;
      for (int sg = I.seg0; sg < I.seg0 + I.nseg; ++sg) {
        const TCSeg& S = segs[sg];
        for (int kc = 0; kc < S.nkc;) {
          const int fit = ((cap - used) / per) & ~1;
          if (fit < 2 || (int)chunks.size() - first >= TC_MAXCH) {
            close();
            continue;
          }
          const int kcs = std::min(S.nkc - kc, fit);
          TCChunk ch{};
          ch.a = S.a + (unsigned long long)kc * 2048;
          ch.b = S.b + (unsigned long long)kc * 32 * I.N;
          ch.abytes = (unsigned)kcs * 2048;
          ch.bbytes = (unsigned)kcs * 32 * I.N;
          ch.off = (unsigned)used;
          ch.N = (unsigned short)I.N;
          ch.flags = item_first ? 1 : 0;
          item_first = false;
          used += kcs * per;
          kc += kcs;
          if (kc >= S.nkc && sg == I.seg0 + I.nseg - 1) ch.flags |= 2;
          chunks.push_back(ch);
        }
      }
    }
    close();
    sched4[c] = make_int4(sched[c].x, sched[c].y, s0, (int)stages.size() - s0);
  }
}

}  // namespace

int tc_selftest() {
  static std::mutex mu;
  static int state = -2;
  std::lock_guard<std::mutex> lock(mu);
  if (state == -2) state = tc_supported() ? tc_selftest_run() : 0;
  return state;
}

bool HOperator::tc_eligible(int trans, int nrhs, cudaStream_t s) {
  if (!tc_mode || tc_state < 0 || trans || !cplx || prec != 1 || mv_compensated || nrhs < 2 || nrhs > 32 ||
      t_len <= 0)
    return false;
  if (tc_state == 0) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    BEM_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return false;  // built outside a capture only
    build_tc();
  }
  return tc_state == 1;
}

void HOperator::build_tc() {
  const auto t0 = clk::now();
  tc_state = -1;
  if (!cplx || prec != 1 || t_len <= 0 || !tc_selftest()) return;
  for (const LRDesc& L : mvlr)
    if (L.R > 128) return;  // a block's 2 x rank columns must fit one MMA (N <= 256)
  const int nf = (int)mvlr.size();
  std::vector<int> rpad(nf, 0);
  std::vector<long long> taoff(nf, -1);
  long long ta_bytes = 0;
  for (int f = 0; f < nf; ++f)
    if (mvlr[f].R > 0) {
      rpad[f] = (mvlr[f].R + 3) & ~3;
      taoff[f] = ta_bytes;
      ta_bytes += (long long)rpad[f] * 1024;  // 128 rows x 2 rpad FP32
    }
  // pass 0: blocks grouped by column cluster, stacked into column tiles of N <= 256
  std::map<std::pair<int, int>, std::vector<int>> cols, rows;
  for (int f = 0; f < nf; ++f)
    if (rpad[f] > 0) {
      cols[{mvlr[f].c0, mvlr[f].n}].push_back(f);
      rows[{mvlr[f].r0, mvlr[f].m}].push_back(f);
    }
  tc_nkc_x = (width + 3) / 4 + 2;
  std::vector<TCItem> it0;
  std::vector<double> cost0;
  std::vector<TCSeg> sg0;
  std::vector<TCOut> outs;
  std::vector<TCVJob> vjobs;
  std::vector<int4> colmap;
  long long vp_bytes = 0;
  struct OutRef { int f, col; };
  for (auto& kv : cols) {
    const int c0 = kv.first.first, n = kv.first.second;
    const int kc0 = c0 / 4, kc1 = (c0 + n + 3) / 4;
    const int nkc = (kc1 - kc0 + 1) & ~1;
    const std::vector<int>& fs = kv.second;
    for (size_t p = 0; p < fs.size();) {
      std::vector<OutRef> tile;
      int ncol = 0;
      while (p < fs.size() && ncol + 2 * rpad[fs[p]] <= 256) {
        tile.push_back({fs[p], ncol});
        ncol += 2 * rpad[fs[p]];
        ++p;
      }
      const int N = (ncol + 15) & ~15;
      TCVJob J{};
      J.dst = (unsigned long long)vp_bytes;  // offset; rebased after allocation
      J.kc0 = kc0;
      J.nkc = nkc;
      J.N = N;
      J.cm0 = (int)colmap.size();
      for (int c = 0; c < N; ++c) colmap.push_back(make_int4(-1, 0, 0, 0));
      TCItem I{};
      I.seg0 = (int)sg0.size();
      I.nseg = 1;
      I.N = N;
      I.nk2 = nkc / 2;
      I.out0 = (int)outs.size();
      I.nout = (int)tile.size();
      for (const OutRef& o : tile) {
        for (int k = 0; k < mvlr[o.f].R; ++k)
          for (int c = 0; c < 2; ++c) colmap[J.cm0 + o.col + 2 * k + c] = make_int4(o.f, k, c, 0);
        TCOut O{};
        O.ta = (unsigned long long)taoff[o.f];  // offset; rebased
        O.col = o.col;
        O.rpad = rpad[o.f];
        outs.push_back(O);
      }
      TCSeg S{};
      S.a = (unsigned long long)kc0 * 2048;  // offset into the X panel; rebased
      S.b = J.dst;
      S.nkc = nkc;
      sg0.push_back(S);
      vjobs.push_back(J);
      it0.push_back(I);
      cost0.push_back((double)nkc * (2048.0 + 32.0 * N) + 1024.0 * ncol / 2);
      vp_bytes += (long long)nkc * 32 * N;
    }
  }
  // pass 1: low-rank and dense blocks grouped by row cluster; row tiles of <= 256 rows, one
  // segment per block (U2 T for low rank, D X through the second X panel for dense)
  tc_nkc_x2 = (width + 1) / 2 + 2;
  std::map<std::pair<int, int>, std::vector<int>> drows;
  for (int k = 0; k < (int)mvdense.size(); ++k) {
    drows[{mvdense[k].r0, mvdense[k].m}].push_back(k);
    rows[{mvdense[k].r0, mvdense[k].m}];  // make sure the row cluster has an entry
  }
  std::vector<TCItem> it1;
  std::vector<double> cost1;
  std::vector<TCSeg> sg1;
  std::vector<int> sg1_kind;  // 0: U2 segment (A = T panel), 1: dense segment (A = second X panel)
  std::vector<TCUJob> ujobs;
  std::vector<TCDJob> djobs;
  long long up_bytes = 0, dp_bytes = 0, yrows = 0;
  struct RowGroup { int r0, m; long long yoff; };
  std::vector<RowGroup> rgroups;
  const std::vector<int> none;
  for (auto& kv : rows) {
    const int r0 = kv.first.first, m = kv.first.second;
    auto dit = drows.find(kv.first);
    const std::vector<int>& dk = dit == drows.end() ? none : dit->second;
    rgroups.push_back({r0, m, yrows});
    for (int i0 = 0; i0 < m; i0 += 256) {
      const int nr = std::min(256, m - i0);
      const int N = (nr + 15) & ~15;
      TCItem I{};
      I.seg0 = (int)sg1.size();
      I.nseg = (int)(kv.second.size() + dk.size());
      I.N = N;
      I.out0 = (int)(yrows + i0);
      I.nout = nr;
      I.nk2 = 0;
      double c = 256.0 * N;
      for (int f : kv.second) {
        TCUJob J{};
        J.dst = (unsigned long long)up_bytes;
        J.lr = f;
        J.i0 = i0;
        J.rows = nr;
        J.N = N;
        J.nkc = rpad[f] / 2;
        TCSeg S{};
        S.a = (unsigned long long)taoff[f];
        S.b = J.dst;
        S.nkc = J.nkc;
        sg1.push_back(S);
        sg1_kind.push_back(0);
        ujobs.push_back(J);
        I.nk2 += S.nkc / 2;
        c += (double)J.nkc * (2048.0 + 32.0 * N);
        up_bytes += (long long)J.nkc * 32 * N;
      }
      for (int k : dk) {
        const MVDense& D = mvdense[k];
        TCDJob J{};
        J.dst = (unsigned long long)dp_bytes;
        J.blk = k;
        J.i0 = i0;
        J.rows = nr;
        J.N = N;
        J.kc0 = D.c0 / 2;
        J.nkc = ((D.c0 + D.n + 1) / 2 - J.kc0 + 1) & ~1;
        TCSeg S{};
        S.a = (unsigned long long)J.kc0 * 2048;
        S.b = J.dst;
        S.nkc = J.nkc;
        sg1.push_back(S);
        sg1_kind.push_back(1);
        djobs.push_back(J);
        I.nk2 += S.nkc / 2;
        c += (double)J.nkc * (2048.0 + 32.0 * N);
        dp_bytes += (long long)J.nkc * 32 * N;
      }
      it1.push_back(I);
      cost1.push_back(c);
    }
    yrows += m;
  }
  if (yrows > INT_MAX / 2) return;  // partial row offsets are ints
  // device buffers: X panels, T panels, packed V2, U2 and dense panels, partial rows
  d_tc_xa.alloc((size_t)tc_nkc_x * 2048);
  d_tc_xa2.alloc((size_t)tc_nkc_x2 * 2048);
  d_tc_ta.alloc((size_t)std::max(ta_bytes, 16LL));
  d_tc_vp.alloc((size_t)std::max(vp_bytes, 16LL));
  d_tc_up.alloc((size_t)std::max(up_bytes, 16LL));
  d_tc_dp.alloc((size_t)std::max(dp_bytes, 16LL));
  d_tc_y.alloc((size_t)std::max(yrows, 1LL) * 32 * 8);
  const unsigned long long xa = (unsigned long long)d_tc_xa.p, xa2 = (unsigned long long)d_tc_xa2.p;
  const unsigned long long ta = (unsigned long long)d_tc_ta.p, vp = (unsigned long long)d_tc_vp.p;
  const unsigned long long up = (unsigned long long)d_tc_up.p, dp = (unsigned long long)d_tc_dp.p;
  for (TCVJob& J : vjobs) J.dst += vp;
  for (TCSeg& S : sg0) {
    S.a += xa;
    S.b += vp;
  }
  for (TCOut& O : outs) O.ta += ta;
  for (TCUJob& J : ujobs) J.dst += up;
  for (TCDJob& J : djobs) J.dst += dp;
  for (size_t q = 0; q < sg1.size(); ++q) {
    sg1[q].a += sg1_kind[q] ? xa2 : ta;
    sg1[q].b += sg1_kind[q] ? dp : up;
  }
  int dev = 0, nsm = 152;
  BEM_CUDA(cudaGetDevice(&dev));
  BEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  std::vector<int2> sch0, sch1;
  balance(it0, cost0, nsm, sch0);
  balance(it1, cost1, nsm, sch1);
  tc_grid[0] = it0.empty() ? 0 : (int)sch0.size();
  tc_grid[1] = it1.empty() ? 0 : (int)sch1.size();
  d_tc_items[0].upload(it0);
  d_tc_items[1].upload(it1);
  tc_it[0].swap(it0);
  tc_it[1].swap(it1);
  tc_sg[0].swap(sg0);
  tc_sg[1].swap(sg1);
  tc_sch[0].swap(sch0);
  tc_sch[1].swap(sch1);
  plan_tc(tc_nst);
  d_tc_outs.upload(outs);
  // pack the factors (once)
  {
    DevBuf dv, du, dd, dcm;
    dv.upload(vjobs);
    du.upload(ujobs);
    dd.upload(djobs);
    dcm.upload(colmap);
    launch_tc_pack_v(dv.as<TCVJob>(), (int)vjobs.size(), dcm.as<int4>(), d_mvlr.as<LRDesc>(), 0);
    launch_tc_pack_u(du.as<TCUJob>(), (int)ujobs.size(), d_mvlr.as<LRDesc>(), 0);
    launch_tc_pack_d(dd.as<TCDJob>(), (int)djobs.size(), d_mvdense.as<MVDense>(), 0);
    BEM_CUDA(cudaGetLastError());
    BEM_CUDA(cudaDeviceSynchronize());
  }
  // per leaf: the partial-row offsets (row i of the leaf at i + delta) of every row cluster
  // that holds it (row clusters nest, so each either holds the whole leaf or none of it)
  {
    std::vector<std::pair<int, int>> lv;
    for (const ClusterH& C : ttest->cl)
      if (C.Child1 < 0) lv.push_back({(int)C.PermuPos, (int)(C.PermuPos + C.Number)});
    std::sort(lv.begin(), lv.end());
    std::vector<std::vector<int>> per(lv.size());
    for (const RowGroup& g : rgroups) {
      int l = (int)(std::upper_bound(lv.begin(), lv.end(), std::make_pair(g.r0, INT_MAX)) - lv.begin()) - 1;
      for (l = std::max(l, 0); l < (int)lv.size() && lv[l].first < g.r0 + g.m; ++l)
        if (lv[l].first >= g.r0 && lv[l].second <= g.r0 + g.m) per[l].push_back((int)(g.yoff - g.r0));
    }
    std::vector<int4> leaves;
    std::vector<int> deltas;
    for (size_t l = 0; l < lv.size(); ++l) {
      const int e0 = (int)deltas.size();
      deltas.insert(deltas.end(), per[l].begin(), per[l].end());
      leaves.push_back(make_int4(lv[l].first, lv[l].second, e0, (int)deltas.size()));
    }
    d_tc_leaves.upload(leaves);
    d_tc_deltas.upload(deltas);
    n_tc_leaves = (int)leaves.size();
  }
  BEM_CUDA(cudaDeviceSynchronize());
  tc_bytes = (long long)(d_tc_xa.bytes + d_tc_xa2.bytes + d_tc_ta.bytes + d_tc_vp.bytes + d_tc_up.bytes +
                         d_tc_dp.bytes + d_tc_y.bytes);
  tc_items[0] = (int)tc_it[0].size();
  tc_items[1] = (int)tc_it[1].size();
  tc_ms_build = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  tc_state = 1;
}

void HOperator::plan_tc(int nst) {
  if (nst < 2 || nst > TC_NST_MAX) throw Error(BEM_ERR_ARG, "stage count out of range");
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int4> s4;
    std::vector<int2> stg;
    std::vector<TCChunk> chk;
    plan_stages(tc_it[pass], tc_sg[pass], tc_sch[pass], tc_cap(nst), s4, stg, chk);
    d_tc_sched[pass].upload(s4);
    d_tc_stages[pass].upload(stg);
    d_tc_chunks[pass].upload(chk);
  }
  BEM_CUDA(cudaDeviceSynchronize());
  tc_nst = nst;
}

double HOperator::autotune_tc(int reps) {
  if (tc_state == 0 && tc_mode) build_tc();
  if (tc_state != 1) throw Error(BEM_ERR_STATE, "the operator has no tensor-core path");
  reps = std::max(1, reps);
  // zero right-hand sides in both numberings' extents: the kernels do the same work for any values
  const VecMap vm = vec_map(0);
  const int nrhs = 32;
  DevBuf x, y;
  x.alloc((size_t)std::max(vm.ld_in, 1) * nrhs * 16);
  y.alloc((size_t)std::max(vm.ld_out, 1) * nrhs * 16);
  BEM_CUDA(cudaMemset(x.p, 0, x.bytes));
  const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
  cudaEvent_t e0, e1;
  BEM_CUDA(cudaEventCreate(&e0));
  BEM_CUDA(cudaEventCreate(&e1));
  double best = 1e300;
  int best_nst = tc_nst;
  for (int nst = 2; nst <= TC_NST_MAX; ++nst) {
    plan_tc(nst);
    mult_tc(one, x.p, zero, y.p, nrhs, 0);  // warm-up (shared-memory opt-in of the instance)
    BEM_CUDA(cudaEventRecord(e0, 0));
    for (int r = 0; r < reps; ++r) mult_tc(one, x.p, zero, y.p, nrhs, 0);
    BEM_CUDA(cudaEventRecord(e1, 0));
    BEM_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    BEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    tc_tune_ms[nst - 2] = ms / reps;
    if (ms / reps < best) {
      best = ms / reps;
      best_nst = nst;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  plan_tc(best_nst);
  BEM_CUDA(cudaGetLastError());
  if (device_status() != 0) throw Error(BEM_ERR_INTERNAL, "a bounded device wait ran out while tuning");
  return best;
}

void HOperator::release_tc() {
  for (int pass = 0; pass < 2; ++pass) {
    tc_it[pass].clear();
    tc_sg[pass].clear();
    tc_sch[pass].clear();
  }
  for (DevBuf* b : {&d_tc_xa, &d_tc_xa2, &d_tc_ta, &d_tc_vp, &d_tc_up, &d_tc_dp, &d_tc_y, &d_tc_items[0],
                    &d_tc_items[1], &d_tc_stages[0], &d_tc_stages[1], &d_tc_chunks[0], &d_tc_chunks[1],
                    &d_tc_sched[0], &d_tc_sched[1], &d_tc_outs, &d_tc_leaves, &d_tc_deltas})
    b->release();
  tc_state = 0;
  tc_bytes = 0;
}

void HOperator::mult_tc(const double* alpha, const void* x, const double* beta, void* y, int nrhs, cudaStream_t s) {
  const VecMap vm = vec_map(0);
  const int* perm = vm.pin;
  const int* pout = vm.pout;
  std::array<cudaEvent_t, 5> ev{};
  if (profiling) {
    for (auto& e : ev) BEM_CUDA(cudaEventCreate(&e));
    BEM_CUDA(cudaEventRecord(ev[0], s));
  }
  launch_tc_xprep(perm, width, nrhs, vm.ld_in, x, d_tc_xa.p, tc_nkc_x, d_tc_xa2.p, tc_nkc_x2, s);
  if (profiling) BEM_CUDA(cudaEventRecord(ev[1], s));
  for (int pass = 0; pass < 2; ++pass) {
    TCGemmArgs g{};
    g.items = d_tc_items[pass].as<TCItem>();
    g.outs = d_tc_outs.as<TCOut>();
    g.sched = d_tc_sched[pass].as<int4>();
    g.stages = d_tc_stages[pass].as<int2>();
    g.chunks = d_tc_chunks[pass].as<TCChunk>();
    g.ypart = d_tc_y.p;
    g.err = d_err.as<int>();
    BEM_CUDA(launch_tc_gemm(pass, tc_nst, g, tc_grid[pass], s));
    if (profiling && pass == 0) BEM_CUDA(cudaEventRecord(ev[2], s));
  }
  if (profiling) BEM_CUDA(cudaEventRecord(ev[3], s));
  launch_tc_ysum_out(d_tc_leaves.as<int4>(), n_tc_leaves, d_tc_deltas.as<int>(), d_tc_y.p, pout, nrhs, vm.ld_out, alpha,
                     beta, y, s);
  if (profiling) {
    BEM_CUDA(cudaEventRecord(ev[4], s));
    pending.push_back(ev);
    pending_fused.push_back(false);
  }
  BEM_CUDA(cudaGetLastError());
}

}  // namespace bem
