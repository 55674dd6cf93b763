// H-matrix application whose scratch is a fixed, file-scope device array
// (bem_operator_mult_noalloc in include/ngbem_gb300.h).
//
// bem_operator_mult keeps its scratch -- the permuted input, the FP64 output accumulator, the
// pool t of the R^T x products and t's input form -- in buffers that the operator owns and
// grows on first use or when nrhs grows.  Growing means cudaFree + cudaMalloc, and cudaFree
// waits for the whole device.  A caller that cannot let a matvec allocate -- a solver loop
// beside other streams that must not be stalled by that device-wide wait, or a process whose
// memory is already reserved by its own allocator so that a late cudaMalloc can fail halfway
// through a solve -- calls this variant instead.  It runs the same kernels on the same
// operator data; only the scratch comes from g_scratch below.
//
// Limits and rules:
// - the scratch holds at most BEM_NOALLOC_SCRATCH_BYTES; a call that would need more
//   (large operators, many right-hand sides) is rejected before anything is launched;
// - the first call on a device looks the array up (cudaGetSymbolAddress, which can load this
//   file's device code): make that first call before any stream capture on that device;
// - the work lists come from the operator and are never built here (building them
//   allocates).  Assembly and loading build those of the non-transposed single-vector
//   product; those of another form (transposed, several right-hand sides) are built by the
//   operator's first bem_operator_mult of that form.  A call whose lists are missing returns
//   BEM_ERR_STATE and launches nothing;
// - there is one array per device and per process, so calls that overlap on a device (two
//   streams, two host threads, two operators) race on it: order them on one stream or with
//   events;
// - the array keeps whatever the last call left in it; every region that a product expects
//   at zero (the claim counters and the grid barrier, the output accumulator, t and its input
//   form) is cleared by every call;
// - a bounded device wait that runs out sets the operator's error flags, which
//   bem_operator_status reads (and clears): check it after a sequence of calls.
#include <mutex>

#include "host.hpp"
#include "kernels.h"

namespace bem {

namespace {

__device__ __align__(256) unsigned char g_scratch[BEM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_ptr[kMaxDevices] = {};

// device address of g_scratch on the current device (looked up once per device)
void* scratch_on_current_device() {
  int dev = 0;
  BEM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error(BEM_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p)
      throw Error(BEM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_ptr[dev] = p;
  }
  return g_ptr[dev];
}

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

void mult_noalloc(HOperator& op, int trans, const double* alpha, const void* x, const double* beta, void* y,
                  int nrhs, cudaStream_t s) {
  if (nrhs < 1) throw Error(BEM_ERR_ARG, "nrhs must be >= 1");
  const int in_n = trans ? op.height : op.width;
  const int out_n = trans ? op.width : op.height;
  const size_t dsz = op.cplx ? 16 : 8;                          // FP64 accumulators
  const size_t xsz = (size_t)mv_x_bytes(op.prec, op.cplx);        // permuted input values
  const size_t tn = (size_t)std::max(op.t_len, 0) * nrhs;
  // layout: [counters | y accumulator | t | t input form] (cleared each call), then [permuted x]
  const size_t off_yp = 256;
  const size_t off_t = off_yp + round256((size_t)out_n * nrhs * dsz);
  const size_t off_tx = off_t + round256(tn * dsz);
  const size_t off_xp = off_tx + (op.prec == 0 ? 0 : round256(tn * xsz));
  const size_t need = off_xp + round256((size_t)in_n * nrhs * xsz);
  if (need > (size_t)BEM_NOALLOC_SCRATCH_BYTES)
    throw Error(BEM_ERR_ARG, "bem_operator_mult_noalloc: this operator with nrhs=" + std::to_string(nrhs) +
                                 " needs " + std::to_string(need) + " bytes of scratch, the fixed area holds " +
                                 std::to_string((size_t)BEM_NOALLOC_SCRATCH_BYTES));
  // the schedule bem_operator_mult would run for this form, on lists the operator already has
  const unsigned fused_mask = trans ? 0xC0u : 0x30u, pass_mask = trans ? 0x0Cu : 0x03u;
  const bool use_fused = nrhs == 1 && op.mv_fused && (op.mv_built & fused_mask) == fused_mask;
  const bool use_multi = !use_fused && nrhs > 1 && !trans && op.mv_multi_built;
  const bool use_pass = !use_fused && !use_multi && (op.mv_built & pass_mask) == pass_mask;
  if (!use_fused && !use_multi && !use_pass)
    throw Error(BEM_ERR_STATE, "bem_operator_mult_noalloc: the work lists of this product (trans=" +
                                   std::to_string(trans) + ", " + (nrhs == 1 ? "one right-hand side" :
                                   "several right-hand sides") + ") are not built; one bem_operator_mult "
                                   "call of the same form builds them (with the tensor cores off for several "
                                   "complex right-hand sides: bem_operator_set_tensor_cores(op, 0))");
  unsigned char* base = (unsigned char*)scratch_on_current_device();
  const HOperator::VecMap vm = op.vec_map(trans);
  const int* pin = vm.pin;
  const int* pout = vm.pout;
  if (vm.n_free_out > 0) launch_scale_rows(op.cplx, vm.free_out, vm.n_free_out, nrhs, vm.ld_out, beta, y, s);
  BEM_CUDA(cudaMemsetAsync(base, 0, off_xp, s));
  void* tx = op.prec == 0 ? (void*)(base + off_t) : (void*)(base + off_tx);
  if (use_fused) {
    // the single cooperative launch on the scratch: claim counters at bytes 0 and 4, the grid
    // barrier's arrival counter at byte 8 (zero: a multiple of the grid, as the kernel needs)
    MVFusedArgs f{};
    f.a.xp = base + off_xp;
    f.a.t = base + off_t;
    f.a.tx = tx;
    f.a.yp = base + off_yp;
    f.a.nrhs = 1;
    f.a.compensated = op.mv_compensated;
    f.a.in_esz = op.cplx ? 16 : 8;
    f.a.err = op.d_err.as<int>();
    f.a.t_f32 = (op.prec == 1 && !op.mv_compensated) ? 1 : 0;
    const int p0 = trans ? 6 : 4;
    for (int ph = 0; ph < 2; ++ph) {
      f.items[ph] = op.d_items[p0 + ph].as<MVTItem>();
      f.pieces[ph] = op.d_pieces[p0 + ph].as<MVPiece>();
      f.ranges[ph] = op.d_ranges[p0 + ph].as<MVRange>();
      f.nitems[ph] = op.n_items[p0 + ph];
      f.ctr[ph] = (int*)base + ph;
    }
    f.bar = (unsigned long long*)(base + 8);
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
    f.t_len = op.t_len;
    f.wait_limit = op.wait_limit;
    f.bar_extra = op.bar_extra;
    BEM_CUDA(launch_mv_fused(op.prec, op.cplx, f, s));
    return;
  }
  launch_permute_in(op.prec, op.cplx, pin, in_n, nrhs, vm.ld_in, x, base + off_xp, s);
  MVArgs2 a{};
  a.xp = base + off_xp;
  a.t = base + off_t;
  a.tx = tx;
  a.yp = base + off_yp;
  a.nrhs = nrhs;
  a.compensated = op.mv_compensated;
  a.in_esz = op.cplx ? 16 : 8;
  a.err = op.d_err.as<int>();
  a.sched = (int*)base;
  if (op.t_len > 0) {
    a.pass = trans ? 2 : 0;
    a.items = op.d_items[a.pass].as<MVTItem>();
    a.pieces = op.d_pieces[a.pass].as<MVPiece>();
    a.ranges = op.d_ranges[a.pass].as<MVRange>();
    a.nitems = op.n_items[a.pass];
    if (use_multi) {
      a.items = op.d_mr_items[0].as<MVTItem>();
      a.pieces = op.d_mr_pieces[0].as<MVPiece>();
      a.nitems = op.n_mr_items[0];
      a.chunked = 1;
    }
    launch_mv_pass(op.prec, op.cplx, a, op.mv_grid, s);
    launch_t_to_x(op.prec, op.cplx, base + off_t, tx, (long long)tn, s);
  }
  a.pass = trans ? 3 : 1;
  a.items = op.d_items[a.pass].as<MVTItem>();
  a.pieces = op.d_pieces[a.pass].as<MVPiece>();
  a.ranges = op.d_ranges[a.pass].as<MVRange>();
  a.nitems = op.n_items[a.pass];
  a.chunked = 0;
  if (use_multi && op.prec == 0) {
    a.items = op.d_mr_items[1].as<MVTItem>();
    a.pieces = op.d_mr_pieces[1].as<MVPiece>();
    a.nitems = op.n_mr_items[1];
    a.chunked = 1;
    launch_mv_pass(op.prec, op.cplx, a, op.mv_grid, s);
  } else if (use_multi) {
    MVRowArgs ra{};
    ra.leaves = op.d_ro_leaves.as<int4>();
    ra.nleaves = op.n_ro_leaves;
    ra.ents = op.d_ro_ents.as<int4>();
    ra.dense = op.d_mvdense.as<MVDense>();
    ra.lr = op.d_mvlr.as<LRDesc>();
    ra.xp = base + off_xp;
    ra.tx = tx;
    ra.yp = base + off_yp;
    ra.nrhs = nrhs;
    ra.compensated = op.mv_compensated;
    launch_mv_rowowner(op.prec, op.cplx, ra, s);
  } else {
    launch_mv_pass(op.prec, op.cplx, a, op.mv_grid, s);
  }
  launch_permute_out(op.cplx, pout, out_n, nrhs, vm.ld_out, alpha, beta, base + off_yp, y, s);
  BEM_CUDA(cudaGetLastError());
}

}  // namespace bem
