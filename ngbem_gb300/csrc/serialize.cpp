// Saving and loading an assembled H-matrix (no counterpart in the reference, which reassembles
// an operator for every session; listed as the next step after the operator path).
//
// The file holds what the products read: the block partition with ranks and dense-fallback
// flags, every dense block (column-major) and every low-rank block's U2 and V2 factors in
// their chunked device layouts, the operator description and its assembly summary.  Loading
// rebuilds the cluster trees from the spaces (deterministic), checks them against the saved
// permutations and the dofs' elements / vertices / edges, uploads the blocks into fresh device
// pools and builds the work lists, so the loaded operator applies exactly like the saved one.
// The mesh's geometry order and a hash of its curved nodes are recorded too, so that an operator
// is not loaded onto the same triangles with another geometry.  Little-endian binary, version 2.
#include <climits>
#include <cstdio>
#include <cstring>
#include <memory>

#include "host.hpp"

namespace bem {

namespace {

const char kMagic[8] = {'N', 'G', 'B', 'E', 'M', 'H', 'M', '2'};

// FNV-1a over the bytes of the curved nodes (0 for flat meshes)
unsigned long long geometry_hash(const MeshH& m) {
  if (!m.curved()) return 0ull;
  unsigned long long h = 1469598103934665603ull;
  const unsigned char* p = reinterpret_cast<const unsigned char*>(m.G.data());
  for (size_t k = 0; k < m.G.size() * sizeof(double); ++k) {
    h ^= p[k];
    h *= 1099511628211ull;
  }
  return h;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

void put(FILE* f, const void* p, size_t n) {
  if (n && fwrite(p, 1, n, f) != n) throw Error(BEM_ERR_ARG, "write failed");
}
void get(FILE* f, void* p, size_t n) {
  if (n && fread(p, 1, n, f) != n) throw Error(BEM_ERR_ARG, "file truncated or unreadable");
}
template <class T> void put_v(FILE* f, const T& v) { put(f, &v, sizeof(T)); }
template <class T> T get_v(FILE* f) {
  T v;
  get(f, &v, sizeof(T));
  return v;
}
template <class T> void put_vec(FILE* f, const std::vector<T>& v) {
  put_v<long long>(f, (long long)v.size());
  put(f, v.data(), v.size() * sizeof(T));
}
template <class T> std::vector<T> get_vec(FILE* f, long long maxn) {
  const long long n = get_v<long long>(f);
  if (n < 0 || n > maxn) throw Error(BEM_ERR_ARG, "corrupt operator file");
  std::vector<T> v((size_t)n);
  get(f, v.data(), v.size() * sizeof(T));
  return v;
}
// device bytes -> file, through a bounded host buffer
void put_dev(FILE* f, const void* dptr, size_t bytes, std::vector<unsigned char>& buf) {
  const size_t cap = 64u << 20;
  for (size_t o = 0; o < bytes; o += cap) {
    const size_t n = std::min(cap, bytes - o);
    buf.resize(n);
    BEM_CUDA(cudaMemcpy(buf.data(), (const unsigned char*)dptr + o, n, cudaMemcpyDeviceToHost));
    put(f, buf.data(), n);
  }
}
void get_dev(FILE* f, void* dptr, size_t bytes, std::vector<unsigned char>& buf) {
  const size_t cap = 64u << 20;
  for (size_t o = 0; o < bytes; o += cap) {
    const size_t n = std::min(cap, bytes - o);
    buf.resize(n);
    get(f, buf.data(), n);
    BEM_CUDA(cudaMemcpy((unsigned char*)dptr + o, buf.data(), n, cudaMemcpyHostToDevice));
  }
}
size_t u_elems(const LRDesc& L) { return (size_t)((L.m + L.cu - 1) / L.cu) * L.cu * L.R; }
size_t v_elems(const LRDesc& L) { return (size_t)((L.n + L.cv - 1) / L.cv) * L.cv * L.R; }

// Every value read from a file that the kernels or the host index with is checked before
// anything is uploaded: a truncated or corrupt file is refused with BEM_ERR_ARG instead of
// giving blocks that read or write outside the vectors on the device.
void validate_loaded(const HOperator& op) {
  auto bad = [](const char* what) { throw Error(BEM_ERR_ARG, std::string("corrupt operator file: ") + what); };
  if (op.prec != 0 && op.prec != 1) bad("precision");
  if (op.trt < 0 || op.tet < 0) bad("trace evaluators");
  const bem_params_t& p = op.prm;
  if (p.method != BEM_METHOD_ACA && p.method != BEM_METHOD_DENSE) bad("method");
  if (p.method == BEM_METHOD_ACA && p.leafsize < 1) bad("leaf size");
  if (p.intorder < 0 || p.intorder > 40 || p.intorder_singular < 0 || p.intorder_singular > 40 ||
      p.intorder_regular < 0 || p.intorder_regular > 40)
    bad("quadrature orders");
  const size_t nb = op.blocks.size();
  if (op.block_rank.size() != nb || op.block_fallback.size() != nb) bad("block list sizes");
  const long long ncr = (long long)op.ttest->cl.size(), ncc = (long long)op.ttrial->cl.size();
  size_t nlow = 0;
  for (size_t b = 0; b < nb; ++b) {
    const BlockH& B = op.blocks[b];
    if (B.rowcl < 0 || B.rowcl >= ncr || B.colcl < 0 || B.colcl >= ncc) bad("block clusters");
    if (op.block_rank[b] < -1) bad("block rank");
    if (op.block_fallback[b] < 0 || op.block_fallback[b] > 2) bad("fallback flag");
    if (op.block_rank[b] >= 0) ++nlow;
  }
  if (op.mvlr.size() != nlow || op.mvdense.size() != nb - nlow) bad("descriptor counts");
  auto in_range = [](long long o, long long n, long long lim) { return o >= 0 && n >= 0 && o + n <= lim; };
  for (const MVDense& d : op.mvdense)
    if (!in_range(d.r0, d.m, op.height) || !in_range(d.c0, d.n, op.width)) bad("dense block extent");
  // A block's rank is the sum of its kernel terms' ranks (up to six terms), so it may exceed
  // min(m, n); it is bounded here only against overflow, and the payload against the file.
  for (const LRDesc& L : op.mvlr) {
    if (!in_range(L.r0, L.m, op.height) || !in_range(L.c0, L.n, op.width)) bad("low-rank block extent");
    if (L.R < 0 || L.R > (1 << 20)) bad("low-rank block rank");
    if (L.cu < 1 || L.cv < 1 || L.cu > (std::max(L.m, 1) + 3) / 4 * 4 || L.cv > (std::max(L.n, 1) + 3) / 4 * 4)
      bad("factor chunk sizes");
  }
}

// The payload the descriptors announce must be in the file: no allocation is sized by a
// corrupt count.
void check_payload(FILE* f, const HOperator& op) {
  const long pos = ftell(f);
  if (pos < 0 || fseek(f, 0, SEEK_END) != 0) throw Error(BEM_ERR_ARG, "operator file is not seekable");
  const long end = ftell(f);
  if (end < 0 || fseek(f, pos, SEEK_SET) != 0) throw Error(BEM_ERR_ARG, "operator file is not seekable");
  const unsigned long long left = (unsigned long long)(end - pos);
  unsigned long long need = 0;
  auto add = [&](unsigned long long elems) {
    need += elems * (unsigned long long)op.vsize;  // elems < 2^52 and vsize <= 16: no overflow
    if (need > left) throw Error(BEM_ERR_ARG, "corrupt operator file: payload larger than the file");
  };
  for (const MVDense& d : op.mvdense) add((unsigned long long)d.m * (unsigned long long)d.n);
  for (const LRDesc& L : op.mvlr) {
    add(u_elems(L));
    add(v_elems(L));
  }
}

}  // namespace

void save_operator(const HOperator& op, const char* path) {
  File fh;
  fh.f = fopen(path, "wb");
  if (!fh.f) throw Error(BEM_ERR_ARG, std::string("cannot open ") + path + " for writing");
  FILE* f = fh.f;
  BEM_CUDA(cudaDeviceSynchronize());
  put(f, kMagic, sizeof(kMagic));
  put_v<int>(f, op.kid);
  put_v<double>(f, op.kappa);
  put_v<int>(f, op.trial_ev);
  put_v<int>(f, op.test_ev);
  put_v<int>(f, op.prec);
  put_v<bem_params_t>(f, op.prm);
  const int ts[6] = {op.trial->kind, op.trial->ndof, op.trial->dual, op.test->kind, op.test->ndof, op.test->dual};
  put(f, ts, sizeof(ts));
  put_v<int>(f, op.trial->mesh->nv);
  put_v<int>(f, op.trial->mesh->nt);
  put_v<int>(f, op.trial->mesh->gorder);
  put_v<unsigned long long>(f, geometry_hash(*op.trial->mesh));
  put_vec(f, op.ttrial->perm);
  put_vec(f, op.ttest->perm);
  put_vec(f, op.trial->global_dof);  // which elements / vertices / edges the dofs are
  put_vec(f, op.test->global_dof);
  put_vec(f, op.blocks);
  put_vec(f, op.block_rank);
  put_vec(f, op.block_fallback);
  put_v<bem_operator_info_t>(f, op.info);
  std::vector<MVDense> dense = op.mvdense;
  std::vector<LRDesc> lr = op.mvlr;
  for (MVDense& d : dense) d.ptr = 0;
  for (LRDesc& L : lr) L.u = L.v = 0;
  put_vec(f, dense);
  put_vec(f, lr);
  std::vector<unsigned char> buf;
  for (const MVDense& d : op.mvdense) put_dev(f, (const void*)d.ptr, (size_t)d.m * d.n * op.vsize, buf);
  for (const LRDesc& L : op.mvlr) {
    put_dev(f, (const void*)L.u, u_elems(L) * op.vsize, buf);
    put_dev(f, (const void*)L.v, v_elems(L) * op.vsize, buf);
  }
  if (fflush(f) != 0) throw Error(BEM_ERR_ARG, "write failed");
}

std::unique_ptr<HOperator> load_operator(const char* path, SpaceH* trial, SpaceH* test) {
  File fh;
  fh.f = fopen(path, "rb");
  if (!fh.f) throw Error(BEM_ERR_ARG, std::string("cannot open ") + path);
  FILE* f = fh.f;
  char magic[8];
  get(f, magic, sizeof(magic));
  if (std::memcmp(magic, kMagic, sizeof(magic)) != 0) throw Error(BEM_ERR_ARG, "not an operator file");
  auto op = std::make_unique<HOperator>();
  op->kid = get_v<int>(f);
  if (op->kid < 0 || op->kid >= K_NUM) throw Error(BEM_ERR_ARG, "corrupt operator file");
  op->kappa = get_v<double>(f);
  op->trial_ev = get_v<int>(f);
  op->test_ev = get_v<int>(f);
  op->prec = get_v<int>(f);
  op->prm = get_v<bem_params_t>(f);
  int ts[6];
  get(f, ts, sizeof(ts));
  const int nv = get_v<int>(f), nt = get_v<int>(f);
  const int gorder = get_v<int>(f);
  const unsigned long long ghash = get_v<unsigned long long>(f);
  if (ts[0] != trial->kind || ts[1] != trial->ndof || ts[2] != trial->dual || ts[3] != test->kind ||
      ts[4] != test->ndof || ts[5] != test->dual)
    throw Error(BEM_ERR_ARG, "the spaces do not match the saved operator");
  op->trial = trial;
  op->test = test;
  op->merge_meshes();  // spaces on two meshes: the same merged mesh as at assembly
  trial = op->trial;
  test = op->test;
  if (nv != trial->mesh->nv || nt != trial->mesh->nt)
    throw Error(BEM_ERR_ARG, "the spaces do not match the saved operator");
  if (gorder != trial->mesh->gorder || ghash != geometry_hash(*trial->mesh))
    throw Error(BEM_ERR_ARG, "the mesh's geometry (flat or curved) differs from the saved operator's");
  op->trt = trace_kind(trial->kind, op->trial_ev);
  op->tet = trace_kind(test->kind, op->test_ev);
  op->cplx = kernel_complex(op->kid);
  op->vsize = (op->prec == 0 ? 8 : 4) * (op->cplx ? 2 : 1);
  op->height = test->ndof;
  op->width = trial->ndof;
  const long long lim = 1LL << 34;
  const std::vector<int> perm_trial = get_vec<int>(f, lim), perm_test = get_vec<int>(f, lim);
  const std::vector<int> gd_trial = get_vec<int>(f, lim), gd_test = get_vec<int>(f, lim);
  if (gd_trial != trial->global_dof || gd_test != test->global_dof)
    throw Error(BEM_ERR_ARG, "the spaces' dofs differ from the saved operator's (another region?)");
  // the trees are rebuilt from the spaces (the same deterministic construction as assembly)
  const bool dense_method = op->prm.method == BEM_METHOD_DENSE;
  const int leaf = dense_method ? INT_MAX : op->prm.leafsize;
  op->own_trial = trial->tree(leaf);
  op->ttrial = op->own_trial.get();
  if (test == trial) {
    op->ttest = op->ttrial;
  } else {
    op->own_test = test->tree(leaf);
    op->ttest = op->own_test.get();
  }
  if (perm_trial != op->ttrial->perm || perm_test != op->ttest->perm)
    throw Error(BEM_ERR_ARG, "the spaces' cluster trees differ from the saved operator's");
  op->blocks = get_vec<BlockH>(f, lim);
  op->block_rank = get_vec<int>(f, lim);
  op->block_fallback = get_vec<int>(f, lim);
  op->info = get_v<bem_operator_info_t>(f);
  op->mvdense = get_vec<MVDense>(f, lim);
  op->mvlr = get_vec<LRDesc>(f, lim);
  validate_loaded(*op);
  check_payload(f, *op);
  // device pools: every dense block at a 16-byte aligned offset, then the U2 and V2 factors
  const size_t al = 16;
  auto up = [&](size_t b) { return (b + al - 1) / al * al; };
  size_t dbytes = 0, ubytes = 0, vbytes = 0;
  for (const MVDense& d : op->mvdense) dbytes += up((size_t)d.m * d.n * op->vsize);
  for (const LRDesc& L : op->mvlr) {
    ubytes += up(u_elems(L) * op->vsize);
    vbytes += up(v_elems(L) * op->vsize);
  }
  auto dp = std::make_unique<DevBuf>(), upool = std::make_unique<DevBuf>(), vpool = std::make_unique<DevBuf>();
  dp->alloc(std::max<size_t>(dbytes, 16));
  upool->alloc(std::max<size_t>(ubytes, 16));
  vpool->alloc(std::max<size_t>(vbytes, 16));
  std::vector<unsigned char> buf;
  size_t o = 0;
  for (MVDense& d : op->mvdense) {
    const size_t b = (size_t)d.m * d.n * op->vsize;
    d.ptr = (unsigned long long)((unsigned char*)dp->p + o);
    get_dev(f, (void*)d.ptr, b, buf);
    o += up(b);
  }
  size_t ou = 0, ov = 0;
  op->t_len = 0;
  for (LRDesc& L : op->mvlr) {
    const size_t bu = u_elems(L) * op->vsize, bv = v_elems(L) * op->vsize;
    L.u = (unsigned long long)((unsigned char*)upool->p + ou);
    L.v = (unsigned long long)((unsigned char*)vpool->p + ov);
    get_dev(f, (void*)L.u, bu, buf);
    get_dev(f, (void*)L.v, bv, buf);
    ou += up(bu);
    ov += up(bv);
    L.toff = op->t_len;
    op->t_len += L.R;
  }
  op->pools.push_back(std::move(dp));
  op->pools.push_back(std::move(upool));
  op->pools.push_back(std::move(vpool));
  op->d_perm_trial.upload(op->ttrial->perm);
  op->d_pinv_trial.upload(op->ttrial->pinv);
  if (op->ttest != op->ttrial) {
    op->d_perm_test.upload(op->ttest->perm);
    op->d_pinv_test.upload(op->ttest->pinv);
  }
  op->mv_fused = mv_fused_supported();
  op->build_mv_items(op->mv_fused ? 0x30u : 0x03u, false, false);
  BEM_CUDA(cudaDeviceSynchronize());
  return op;
}

}  // namespace bem
