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
// - there is one array per device and per process, so calls that overlap on a device (two
//   streams, two host threads, two operators) race on it: order them on one stream or with
//   events;
// - the array keeps whatever the last call left in it; the regions that the kernels accumulate
//   into (the item counters, the output accumulator and t) are cleared by every call.
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
  op.ensure_mv(trans ? 0x0Cu : 0x03u, false, s);  // the four-pass lists (built on first use)
  const int in_n = trans ? op.height : op.width;
  const int out_n = trans ? op.width : op.height;
  const size_t dsz = op.cplx ? 16 : 8;                          // FP64 accumulators
  const size_t xsz = (size_t)mv_x_bytes(op.prec, op.cplx);        // permuted input values
  const size_t tn = (size_t)std::max(op.t_len, 0) * nrhs;
  // layout: [counters | y accumulator | t] (cleared each call) then [permuted x | t input form]
  const size_t off_yp = 256;
  const size_t off_t = off_yp + round256((size_t)out_n * nrhs * dsz);
  const size_t off_xp = off_t + round256(tn * dsz);
  const size_t off_tx = off_xp + round256((size_t)in_n * nrhs * xsz);
  const size_t need = off_tx + (op.prec == 0 ? 0 : round256(tn * xsz));
  if (need > (size_t)BEM_NOALLOC_SCRATCH_BYTES)
    throw Error(BEM_ERR_ARG, "bem_operator_mult_noalloc: this operator with nrhs=" + std::to_string(nrhs) +
                                 " needs " + std::to_string(need) + " bytes of scratch, the fixed area holds " +
                                 std::to_string((size_t)BEM_NOALLOC_SCRATCH_BYTES));
  unsigned char* base = (unsigned char*)scratch_on_current_device();
  const int* pin = trans ? (op.ttest == op.ttrial ? op.d_perm_trial.as<int>() : op.d_perm_test.as<int>())
                         : op.d_perm_trial.as<int>();
  const int* pout = trans ? op.d_perm_trial.as<int>()
                          : (op.ttest == op.ttrial ? op.d_perm_trial.as<int>() : op.d_perm_test.as<int>());
  BEM_CUDA(cudaMemsetAsync(base, 0, off_xp, s));
  launch_permute_in(op.prec, op.cplx, pin, in_n, nrhs, in_n, x, base + off_xp, s);
  MVArgs2 a{};
  a.xp = base + off_xp;
  a.t = base + off_t;
  a.tx = op.prec == 0 ? (const void*)(base + off_t) : (const void*)(base + off_tx);
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
    launch_mv_pass(op.prec, op.cplx, a, op.mv_grid, s);
    launch_t_to_x(op.prec, op.cplx, base + off_t, base + off_tx, (long long)tn, s);
  }
  a.pass = trans ? 3 : 1;
  a.items = op.d_items[a.pass].as<MVTItem>();
  a.pieces = op.d_pieces[a.pass].as<MVPiece>();
  a.ranges = op.d_ranges[a.pass].as<MVRange>();
  a.nitems = op.n_items[a.pass];
  launch_mv_pass(op.prec, op.cplx, a, op.mv_grid, s);
  launch_permute_out(op.cplx, pout, out_n, nrhs, out_n, alpha, beta, base + off_yp, y, s);
  BEM_CUDA(cudaGetLastError());
}

}  // namespace bem
