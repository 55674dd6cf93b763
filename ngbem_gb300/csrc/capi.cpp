// extern "C" entry points of libngbem_gb300 (declared in include/ngbem_gb300.h).
// Every call catches C++ exceptions and converts them to an int status plus a
// thread-local message (bem_last_error).
#include <algorithm>
#include <cstring>

#include "host.hpp"

using namespace bem;

static thread_local std::string g_last_error;

template <class F>
static int guarded(F&& f) {
  try {
    f();
    return BEM_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return BEM_ERR_ALLOC;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return BEM_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown error";
    return BEM_ERR_INTERNAL;
  }
}

#define REQUIRE(cond, msg) \
  if (!(cond)) throw Error(BEM_ERR_ARG, msg)

extern "C" {

const char* bem_last_error(void) { return g_last_error.c_str(); }

int bem_params_default(bem_params_t* p) {
  return guarded([&] {
    REQUIRE(p, "null params");
    std::memset(p, 0, sizeof(*p));
    p->intorder = 3;
    p->leafsize = 40;
    p->eta = 2.0;
    p->eps = 1e-6;
    p->method = BEM_METHOD_ACA;
    p->precision = BEM_FP64;
  });
}

int bem_mesh_create(int nv, const double* xyz, int nt, const int* tri, bem_mesh_t* out) {
  return guarded([&] {
    REQUIRE(out && xyz && tri, "null argument");
    auto m = std::make_unique<bem_mesh_s>();
    m->m->build(nv, xyz, nt, tri);
    *out = m.release();
  });
}

int bem_mesh_set_geometry(bem_mesh_t mesh, int order, const double* nodes) {
  return guarded([&] {
    REQUIRE(mesh, "null argument");
    mesh->m->set_geometry(order, nodes);
  });
}

int bem_mesh_num_edges(bem_mesh_t mesh, int* ne) {
  return guarded([&] {
    REQUIRE(mesh && ne, "null argument");
    *ne = mesh->m->ne;
  });
}

int bem_mesh_destroy(bem_mesh_t mesh) {
  return guarded([&] { delete mesh; });
}

int bem_space_create(bem_mesh_t mesh, int kind, int dual_mapping, bem_space_t* out) {
  return guarded([&] {
    REQUIRE(mesh && out, "null argument");
    REQUIRE(kind >= BEM_P0 && kind <= BEM_HCURL4, "unknown space kind");
    REQUIRE(!dual_mapping || kind == BEM_P0, "dual mapping is defined for P0 only");
    auto s = std::make_unique<bem_space_s>();
    s->mesh = mesh->m;
    s->s->build(mesh->m.get(), kind, dual_mapping);
    *out = s.release();
  });
}

int bem_space_create_on(bem_mesh_t mesh, int kind, int dual_mapping, const unsigned char* element_mask,
                        bem_space_t* out) {
  return guarded([&] {
    REQUIRE(mesh && out, "null argument");
    REQUIRE(kind >= BEM_P0 && kind <= BEM_HCURL4, "unknown space kind");
    REQUIRE(!dual_mapping || kind == BEM_P0, "dual mapping is defined for P0 only");
    auto s = std::make_unique<bem_space_s>();
    s->mesh = mesh->m;
    s->s->build(mesh->m.get(), kind, dual_mapping, element_mask);
    *out = s.release();
  });
}

int bem_space_global_dofs(bem_space_t space, int* out) {
  return guarded([&] {
    REQUIRE(space && out, "null argument");
    std::copy(space->s->global_dof.begin(), space->s->global_dof.end(), out);
  });
}

int bem_space_element_dofs(bem_space_t space, int* dofs, int* signs) {
  return guarded([&] {
    REQUIRE(space && dofs, "null argument");
    const SpaceH& s = *space->s;
    const int nt = s.mesh->nt;
    for (int e = 0; e < nt; ++e)
      for (int k = 0; k < 3; ++k) {
        const bool l2p = s.kind >= BEM_L2P1 && s.kind <= BEM_L2P3;
        dofs[3 * e + k] = ((s.nd == 1 || l2p) && k > 0) ? -1 : s.dofs[3 * e + k];
        if (signs) signs[3 * e + k] = s.sign[3 * e + k];
      }
  });
}

int bem_space_dof_table(bem_space_t space, int* nd, int* dofs) {
  return guarded([&] {
    REQUIRE(space && nd, "null argument");
    const SpaceH& s = *space->s;
    *nd = s.nd;
    if (!dofs) return;
    const int nt = s.mesh->nt;
    for (int e = 0; e < nt; ++e)
      for (int a = 0; a < s.nd; ++a) dofs[(size_t)s.nd * e + a] = s.on(e) ? s.dof(e, a) : -1;
  });
}

int bem_space_ndof(bem_space_t space, int* ndof) {
  return guarded([&] {
    REQUIRE(space && ndof, "null argument");
    *ndof = space->s->ndof;
  });
}

int bem_space_destroy(bem_space_t space) {
  return guarded([&] { delete space; });
}

int bem_cluster_tree(bem_space_t space, int leafsize, int* perm, int max_clusters, int* nclusters, long* ci,
                     double* cd) {
  return guarded([&] {
    REQUIRE(space && perm && nclusters, "null argument");
    REQUIRE(leafsize >= 1, "leafsize must be positive");
    ClusterTreeH t;
    t.build(*space->s, leafsize);
    const int nc = (int)t.cl.size();
    *nclusters = nc;
    std::memcpy(perm, t.perm.data(), t.perm.size() * sizeof(int));
    if (nc > max_clusters) throw Error(BEM_ERR_ARG, "max_clusters too small");
    for (int c = 0; c < nc; ++c) {
      const ClusterH& C = t.cl[c];
      if (ci) {
        long* I = ci + 7 * (size_t)c;
        I[0] = C.Level; I[1] = C.Parent; I[2] = C.Child1; I[3] = C.Child2;
        I[4] = C.Number; I[5] = C.PermuPos; I[6] = C.BasisElement;
      }
      if (cd) {
        double* D = cd + 23 * (size_t)c;
        D[0] = C.Radius;
        for (int k = 0; k < 9; ++k) D[1 + k] = C.EVec[k];
        for (int k = 0; k < 3; ++k) {
          D[10 + k] = C.EVal[k];
          D[13 + k] = C.XMin[k];
          D[16 + k] = C.XMax[k];
          D[19 + k] = C.Centre[k];
        }
        D[22] = C.DiagLength;
      }
    }
  });
}

int bem_partition(bem_space_t trial, bem_space_t test, int leafsize, double eta, int max_blocks, int* nblocks,
                  int* rowcl, int* colcl, int* near) {
  return guarded([&] {
    REQUIRE(trial && test && nblocks, "null argument");
    ClusterTreeH tt, ts;
    tt.build(*trial->s, leafsize);
    const ClusterTreeH* row = &tt;
    if (test != trial) {
      ts.build(*test->s, leafsize);
      row = &ts;
    }
    std::vector<BlockH> bl;
    partition_blocks(*row, tt, eta, bl);
    *nblocks = (int)bl.size();
    if ((int)bl.size() > max_blocks) throw Error(BEM_ERR_ARG, "max_blocks too small");
    for (size_t k = 0; k < bl.size(); ++k) {
      if (rowcl) rowcl[k] = bl[k].rowcl;
      if (colcl) colcl[k] = bl[k].colcl;
      if (near) near[k] = bl[k].near ? 1 : 0;
    }
  });
}

int bem_operator_create(int kernel, double kappa, bem_space_t trial, bem_space_t test, int trial_eval, int test_eval,
                        const bem_params_t* params, bem_operator_t* out) {
  return guarded([&] {
    REQUIRE(trial && out && params, "null argument");
    REQUIRE(kernel >= 0 && kernel < K_NUM, "unknown kernel id");
    if (!test) test = trial;
    if (kernel == BEM_MAXWELL_SL) REQUIRE(kappa != 0.0, "Maxwell single layer needs kappa != 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(BEM_ERR_CUDA, "no CUDA device");
    auto op = std::make_unique<HOperator>();
    op->kid = kernel;
    op->kappa = kappa;
    op->trial = trial->s.get();
    op->test = test->s.get();
    op->trial_ev = trial_eval;
    op->test_ev = test_eval;
    op->prm = *params;
    op->assemble();
    auto h = std::make_unique<bem_operator_s>();
    h->keep(trial, test);
    h->op = std::move(op);
    *out = h.release();
  });
}

int bem_mass_create(bem_space_t trial, bem_space_t test, int complex_vectors, bem_operator_t* out) {
  return guarded([&] {
    REQUIRE(trial && test && out, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(BEM_ERR_CUDA, "no CUDA device");
    auto op = std::make_unique<MassOperator>();
    op->build(trial->s.get(), test->s.get(), complex_vectors != 0);
    auto h = std::make_unique<bem_operator_s>();
    h->keep(trial, test);
    h->op = std::move(op);
    *out = h.release();
  });
}

int bem_operator_info(bem_operator_t op, bem_operator_info_t* info) {
  return guarded([&] {
    REQUIRE(op && info, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (h) {
      *info = h->info;
    } else {
      std::memset(info, 0, sizeof(*info));
      info->is_complex = op->op->cplx;
      info->height = op->op->height;
      info->width = op->op->width;
      auto* m = dynamic_cast<MassOperator*>(op->op.get());
      if (m) info->nze = (long long)m->h_val.size();
    }
  });
}

int bem_operator_blocks(bem_operator_t op, int* rowcl, int* colcl, int* near, int* rank, int* fallback) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    for (size_t k = 0; k < h->blocks.size(); ++k) {
      if (rowcl) rowcl[k] = h->blocks[k].rowcl;
      if (colcl) colcl[k] = h->blocks[k].colcl;
      if (near) near[k] = h->blocks[k].near ? 1 : 0;
      if (rank) rank[k] = h->block_rank[k];
      if (fallback) fallback[k] = h->block_fallback[k];
    }
  });
}

namespace {
// The C-ABI products act on vectors in the operator's global numbering when one is set
// (bem_operator_set_global_dofs); the library's own callers (GMRES, the dense copy, the
// autotuner) use the compact numbering.
struct GlobalNumbering {
  HOperator* h;
  explicit GlobalNumbering(OperatorBase* o) : h(dynamic_cast<HOperator*>(o)) {
    if (h) h->apply_gmap = true;
  }
  ~GlobalNumbering() {
    if (h) h->apply_gmap = false;
  }
};
}  // namespace

int bem_operator_mult(bem_operator_t op, int trans, const double* alpha, const void* x, const double* beta, void* y,
                      int nrhs, void* stream) {
  return guarded([&] {
    REQUIRE(op && alpha && beta && x && y, "null argument");
    REQUIRE(nrhs >= 1, "nrhs must be >= 1");
    GlobalNumbering g(op->op.get());
    op->op->mult(trans, alpha, x, beta, y, nrhs, (cudaStream_t)stream);
  });
}

int bem_operator_set_global_dofs(bem_operator_t op, int trial_nglobal, const int* trial_map, int test_nglobal,
                                 const int* test_map) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->set_global_dofs(trial_nglobal, trial_map, test_nglobal, test_map);
  });
}

int bem_operator_mult_noalloc(bem_operator_t op, int trans, const double* alpha, const void* x, const double* beta,
                              void* y, int nrhs, void* stream) {
  return guarded([&] {
    REQUIRE(op && alpha && beta && x && y, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    GlobalNumbering g(h);
    mult_noalloc(*h, trans, alpha, x, beta, y, nrhs, (cudaStream_t)stream);
  });
}

int bem_operator_mult_host(bem_operator_t op, int trans, const double* alpha, const void* x, const double* beta,
                           void* y, int nrhs) {
  return guarded([&] {
    REQUIRE(op && alpha && beta && x && y, "null argument");
    OperatorBase* o = op->op.get();
    GlobalNumbering g(o);
    const size_t esz = o->cplx ? 16 : 8;
    size_t nin = (size_t)(trans ? o->height : o->width) * nrhs;
    size_t nout = (size_t)(trans ? o->width : o->height) * nrhs;
    if (g.h) {
      const HOperator::VecMap vm = g.h->vec_map(trans);
      nin = (size_t)vm.ld_in * nrhs;
      nout = (size_t)vm.ld_out * nrhs;
    }
    // Page-locked host buffers are mapped into the device's address space.  For small products
    // the kernels read x and write y across the host link themselves (no copy launches); their
    // accesses go through the cluster permutations, so each is a scattered access across the
    // link, which for large products costs more than one bulk copy each way.  Larger products,
    // and other host memory, go through device staging.
    const bool small = (nin + nout) * esz <= BEM_HOST_MAPPED_MAX_BYTES;
    auto mapped = [](const void* p) -> void* {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
    };
    void* xm = small ? mapped(x) : nullptr;
    void* ym = xm ? mapped(y) : nullptr;
    // a synchronous call reports a product whose bounded device waits ran out (and clears the
    // operator's device state so that the next product starts clean); the flags are copied on
    // the product's stream before the one synchronisation
    auto* hop = dynamic_cast<HOperator*>(o);
    auto check_status = [&]() {
      auto* h = hop;
      if (!h) return;
      const int st = h->queued_status();
      if (st != 0) {
        h->reset_device_state();
        throw Error(BEM_ERR_INTERNAL, "a bounded device wait of the product ran out (flags " + std::to_string(st) +
                                          "): the result is not valid");
      }
    };
    if (xm && ym) {
      o->mult(trans, alpha, xm, beta, ym, nrhs, 0);
      if (hop) hop->queue_status(0);
      BEM_CUDA(cudaStreamSynchronize(0));
      check_status();
      return;
    }
    if (o->stage_x.bytes < nin * esz) o->stage_x.alloc(nin * esz);
    if (o->stage_y.bytes < nout * esz) o->stage_y.alloc(nout * esz);
    BEM_CUDA(cudaMemcpyAsync(o->stage_x.p, x, nin * esz, cudaMemcpyHostToDevice, 0));
    if (beta[0] != 0.0 || beta[1] != 0.0)
      BEM_CUDA(cudaMemcpyAsync(o->stage_y.p, y, nout * esz, cudaMemcpyHostToDevice, 0));
    o->mult(trans, alpha, o->stage_x.p, beta, o->stage_y.p, nrhs, 0);
    BEM_CUDA(cudaMemcpyAsync(y, o->stage_y.p, nout * esz, cudaMemcpyDeviceToHost, 0));
    if (hop) hop->queue_status(0);
    BEM_CUDA(cudaStreamSynchronize(0));
    check_status();
  });
}

int bem_operator_status(bem_operator_t op, int* flags, int reset) {
  return guarded([&] {
    REQUIRE(op && flags, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) {
      *flags = 0;  // a mass operator has no bounded waits
      return;
    }
    *flags = h->device_status();
    if (reset) h->reset_device_state();
  });
}

int bem_operator_test_waits(bem_operator_t op, long long limit, int extra_arrivals) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    REQUIRE(limit >= 0 && extra_arrivals >= 0 && extra_arrivals <= 1, "limit >= 0, extra_arrivals 0 or 1");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->wait_limit = limit;
    h->bar_extra = (unsigned long long)extra_arrivals;
  });
}

int bem_operator_to_dense(bem_operator_t op, void* out) {
  return guarded([&] {
    REQUIRE(op && out, "null argument");
    if (auto* m = dynamic_cast<MassOperator*>(op->op.get())) {
      // the sparse mass matrix (real entries) as a dense row-major array of its vector type
      const size_t n = (size_t)m->nrows * m->ncols;
      double* o = (double*)out;
      const int w = m->cplx ? 2 : 1;
      std::fill(o, o + n * w, 0.0);
      for (int i = 0; i < m->nrows; ++i)
        for (int k = m->h_rowptr[i]; k < m->h_rowptr[i + 1]; ++k)
          o[((size_t)i * m->ncols + m->h_col[k]) * w] += m->h_val[k];
      return;
    }
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->to_dense(out);
  });
}

int bem_operator_set_accuracy(bem_operator_t op, int compensated) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->mv_compensated = compensated != 0;
  });
}

int bem_operator_save(bem_operator_t op, const char* path) {
  return guarded([&] {
    REQUIRE(op && path, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    save_operator(*h, path);
  });
}

int bem_operator_load(const char* path, bem_space_t trial, bem_space_t test, bem_operator_t* out) {
  return guarded([&] {
    REQUIRE(path && trial && out, "null argument");
    if (!test) test = trial;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(BEM_ERR_CUDA, "no CUDA device");
    auto h = std::make_unique<bem_operator_s>();
    h->keep(trial, test);
    h->op = load_operator(path, trial->s.get(), test->s.get());
    *out = h.release();
  });
}

int bem_operator_set_definedon(bem_operator_t op, const unsigned char* trial_mask, const unsigned char* test_mask) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    REQUIRE(h, "not an integral operator");
    // masks over the caller's meshes, stored over the operator's (merged) mesh
    const int nt = h->trial->mesh->nt;
    h->def_trial.clear();
    h->def_test.clear();
    if (trial_mask) {
      h->def_trial.assign(nt, 0);
      std::copy(trial_mask, trial_mask + h->trial_nt0, h->def_trial.begin() + h->trial_e0);
    }
    if (test_mask) {
      h->def_test.assign(nt, 0);
      std::copy(test_mask, test_mask + h->test_nt0, h->def_test.begin());
    }
  });
}

int bem_operator_potential_dim(bem_operator_t op, int* dim) {
  return guarded([&] {
    REQUIRE(op && dim, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    *dim = potential_dim(h->kid, h->trt);
  });
}

int bem_operator_potential(bem_operator_t op, const void* density, int npts, const double* points,
                           const double* normals, void* out, void* stream) {
  return guarded([&] {
    REQUIRE(op && density && (npts == 0 || (points && out)), "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->potential(density, npts, points, normals, out, (cudaStream_t)stream);
  });
}

int bem_operator_set_tensor_cores(bem_operator_t op, int enable) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    if (!enable) {
      h->release_tc();
      h->tc_mode = 0;
      return;
    }
    h->tc_mode = 1;
    if (h->tc_state == 0) h->build_tc();
  });
}

int bem_operator_tensor_cores(bem_operator_t op, int* state, long long* bytes, int* items0, int* items1,
                              double* ms_build) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    if (state) *state = h->tc_mode ? h->tc_state : 0;
    if (bytes) *bytes = h->tc_bytes;
    if (items0) *items0 = h->tc_items[0];
    if (items1) *items1 = h->tc_items[1];
    if (ms_build) *ms_build = h->tc_ms_build;
  });
}

int bem_operator_autotune_tc(bem_operator_t op, int reps, int* nstages, double* ms) {
  return guarded([&] {
    REQUIRE(op && reps > 0, "null operator or reps < 1");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->autotune_tc(reps);
    if (nstages) *nstages = h->tc_nst;
    if (ms)
      for (int k = 0; k < 3; ++k) ms[k] = h->tc_tune_ms[k];
  });
}

int bem_tc_selftest(int* passed) {
  return guarded([&] {
    REQUIRE(passed, "null argument");
    *passed = tc_selftest();
  });
}

int bem_operator_autotune(bem_operator_t op, int reps, int* piece, int* fused, double* ms) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    const double t = h->autotune(reps, piece, fused);
    if (ms) *ms = t;
  });
}

int bem_operator_set_profiling(bem_operator_t op, int enable) {
  return guarded([&] {
    REQUIRE(op, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->collect_profile();
    h->profiling = enable != 0;
    for (int k = 0; k < 4; ++k) { h->kms[k] = 0.0; h->kcount[k] = 0; }
  });
}

int bem_operator_kernel_times(bem_operator_t op, double* ms, long long* launches) {
  return guarded([&] {
    REQUIRE(op && ms, "null argument");
    auto* h = dynamic_cast<HOperator*>(op->op.get());
    if (!h) throw Error(BEM_ERR_STATE, "not an H-matrix operator");
    h->collect_profile();
    for (int k = 0; k < 4; ++k) {
      ms[k] = h->kms[k];
      if (launches) launches[k] = h->kcount[k];
    }
  });
}

int bem_operator_destroy(bem_operator_t op) {
  return guarded([&] { delete op; });
}

int bem_sl_batch_create(int nprob, const int* nverts, const int* ntris, const int* tris, int intorder_regular,
                        int intorder_singular, int precision, int dual_mapping, bem_slbatch_t* out) {
  return guarded([&] {
    REQUIRE(nverts && ntris && tris && out, "null argument");
    REQUIRE(precision == BEM_FP64 || precision == BEM_MIXED, "unknown precision");
    auto b = std::make_unique<bem_slbatch_s>();
    b->b.build(nprob, nverts, ntris, tris, intorder_regular, intorder_singular, precision == BEM_FP64 ? 0 : 1,
               dual_mapping ? 1 : 0);
    *out = b.release();
  });
}

int bem_sl_batch_eval(bem_slbatch_t batch, const double* X, const double* u, const double* weights, double* energy,
                      double* vu, double* grad, void* stream) {
  return guarded([&] {
    REQUIRE(batch && X && u, "null argument");
    batch->b.eval(X, u, weights, energy, vu, grad, (cudaStream_t)stream);
  });
}

int bem_sl_batch_info(bem_slbatch_t batch, int* nunits, int* nsing, long long* npairs_regular) {
  return guarded([&] {
    REQUIRE(batch, "null argument");
    if (nunits) *nunits = batch->b.nunits;
    if (nsing) *nsing = batch->b.nsing;
    if (npairs_regular) *npairs_regular = batch->b.npairs_regular;
  });
}

int bem_sl_batch_destroy(bem_slbatch_t batch) {
  return guarded([&] { delete batch; });
}

int bem_gmres(int nterms, const bem_operator_t* ops, const double* coef, const void* b, void* x, int maxiter,
              int restart, double tol, int* iters, double* resid, void* stream) {
  return guarded([&] {
    REQUIRE(ops && coef && b && x && nterms >= 1, "null argument");
    std::vector<OperatorBase*> v;
    for (int k = 0; k < nterms; ++k) {
      REQUIRE(ops[k], "null operator");
      v.push_back(ops[k]->op.get());
    }
    gmres_solve(nterms, v.data(), coef, b, x, maxiter, restart, tol, iters, resid, (cudaStream_t)stream);
  });
}

int bem_gmres_batched(int nterms, const bem_operator_t* ops, const double* coef, int nrhs, const void* b, void* x,
                      int maxiter, int restart, double tol, int* iters, double* resid, void* stream) {
  return guarded([&] {
    REQUIRE(ops && coef && b && x && nterms >= 1, "null argument");
    REQUIRE(nrhs >= 1, "nrhs must be >= 1");
    std::vector<OperatorBase*> v;
    for (int k = 0; k < nterms; ++k) {
      REQUIRE(ops[k], "null operator");
      v.push_back(ops[k]->op.get());
    }
    gmres_batched_solve(nterms, v.data(), coef, nrhs, b, x, maxiter, restart, tol, iters, resid,
                        (cudaStream_t)stream);
  });
}

}  // extern "C"
