// Several-right-hand-side products of the low-rank blocks on the tcgen05 tensor cores
// (complex FP32 storage).  The reference applies each low-rank block as y += U2 (V2 x) one
// vector at a time (LowRankMatrix::Mult / BEMBlock::MultAdd, src/hmat.cpp:473-565, summed by
// HMatrix::MultAdd, :647-666); with 32 right-hand sides those products are GEMMs:
//
//   pass 0: T_b = V2_b X[cols b] for every low-rank block b.  The blocks of one column cluster
//           are stacked along N (one X panel feeds all of them); every block's T is written
//           once, as the A panel of pass 1.
//   pass 1: Y_tau = sum_b U2_b T_b + sum_d D_d X[cols d] over the low-rank blocks b and the
//           dense blocks d of one row cluster tau; the tensor memory accumulates over all of
//           them and the tile is stored once into a per-row-cluster partial buffer.  A last
//           kernel sums, for each row, the partials of every row cluster that holds it and
//           writes y through the output permutation with alpha and beta.
//
// Complex products run as real products.  Rows of the A side are (right-hand side r, real or
// imaginary part a, TF32 high or low part h) at 4 r + 2 a + h, so M = 128 for 32 right-hand
// sides; the B side holds the TF32 high and low parts of the stored factor and both are issued
// into one accumulator.  Summing the two h rows gives (a_hi + a_lo)(b_hi + b_lo): a split-TF32
// product about 2^-21 from the exact one, accumulated in FP32 (TMEM).
//
// Kernel roles (320 threads, one CTA per SM, persistent over a host-balanced item list):
//   warp 0      bulk copies (cp.async.bulk + mbarrier complete_tx) of A and B K-ranges into a
//               ring of 2 to 4 stages (NST, the operator's stage plan);
//   warp 1      owns the tensor memory (512 columns: two 256-column buffers) and one thread
//               issues tcgen05.mma, releasing stages and buffers by tcgen05.commit;
//   warps 2-9   epilogue: tcgen05.ld of their TMEM lane quarter (two warps per quarter, one
//               per half of the item's columns), FP32 sums of the accumulators, combination of
//               the real and imaginary and high and low rows with warp shuffles, global stores.
// Accuracy: tcgen05.mma accumulates with rounding toward zero, so the error of one accumulator
// grows linearly with the MMAs it takes.  A buffer holds A = 256 / round_up(N, 32) accumulators
// of the item; its K steps go to them round-robin, at most TC_CHAIN each, and the buffer then
// goes to the epilogue, whose sums round to nearest (kernels.h).
// Every wait is bounded: a wait that runs out sets an error bit, the CTA drains what it
// issued and frees its tensor memory.
#include <algorithm>
#include <cstdint>

#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

#define TC_THREADS 320  // warp 0 copies, warp 1 MMAs, warps 2-9 epilogue
#define TC_ACC_COLS 256
#define TC_HDR 4096  // barriers, then the range descriptors of each stage (TC_MAXCH x 32 bytes)
static_assert(1024 + TC_NST_MAX * TC_MAXCH * 32 <= TC_HDR, "range descriptors fit the header");
#define TC_DESC 1024
#define TC_ERR_WAIT 0x100

namespace {

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
// One potentially blocking test of the phase of `parity`: the warp is suspended in hardware
// until the phase completes or about a microsecond has passed (no issue slots spent polling).
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity), "r"(1000u)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of `parity` to complete (at most 2^21 suspended tests: about two
// seconds at most).  Returns false when the CTA is aborting or when the limit ran out (then the
// error bit is set and the CTA aborts).
__device__ bool bar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, int* err) {
  for (int i = 0; i < (1 << 21); ++i) {
    if (bar_try(b, parity)) return true;
    if ((i & 255) == 255 && *abort_flag) return false;
  }
  atomicOr(err, TC_ERR_WAIT);
  *abort_flag = 1;
  return false;
}
__device__ __forceinline__ void expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   su32(dst)),
               "l"(src), "r"(bytes), "r"(su32(b))
               : "memory");
}

// ---- tcgen05 --------------------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major without swizzle: start address, leading-dimension
// byte offset (between core matrices adjacent in K), stride byte offset (between 8-row groups
// adjacent in M or N), descriptor version 1 (bits 46-47), no base offset, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// the mbarrier gets one arrival when every MMA this thread issued so far has completed
__device__ __forceinline__ void mma_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b))
               : "memory");
}
// 8 consecutive accumulator columns of this thread's TMEM lane; the values are defined after
// tmem_wait (which takes them as operands so that no use moves above it)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}
// 8 columns into v[8 J .. 8 J + 7] of a 16-value batch (tmem_wait16 completes the batch)
template <int J>
__device__ __forceinline__ void tmem_ld8_at(uint32_t taddr, float (&v)[16]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[8 * J + k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_wait16(float (&v)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                 "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]),
                 "+f"(v[15])
               :
               : "memory");
}
__device__ __forceinline__ void tmem_wait(float (&v)[8]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7])
               :
               : "memory");
}

// round to TF32 (10 stored mantissa bits, nearest, ties away from zero), low 13 bits cleared:
// adding half a TF32 unit (bit 12) to the bit pattern rounds the magnitude, a carry moving into
// the exponent as it should (finite values far below FLT_MAX).  Two integer operations on the
// full-rate pipes instead of a conversion: the epilogue rounds every T entry twice.
__device__ __forceinline__ float tf32_rn(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// high (h = 0) or low (h = 1) TF32 part of v; v - hi is exact in FP32
__device__ __forceinline__ float tf32_part(float v, int h) {
  const float hi = tf32_rn(v);
  return h ? tf32_rn(v - hi) : hi;
}

struct TCSmem {
  uint64_t full[TC_NST_MAX], empty[TC_NST_MAX], accf[2], acce[2], fin;
  uint32_t tmem;
  int abort_flag;
};

}  // namespace

// ---- the grouped GEMM -----------------------------------------------------------------------
template <int PASS, int NST>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_gemm_kernel(TCGemmArgs g) {
  constexpr int TC_NST = NST;
  constexpr int TC_CAP = tc_cap(NST);
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
  TCSmem& S = *(TCSmem*)base;
  unsigned char* stages = base + TC_HDR;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_NST; ++s) {
      bar_init(&S.full[s], 1);
      bar_init(&S.empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      bar_init(&S.accf[a], 1);
      bar_init(&S.acce[a], TC_THREADS / 32 - 2);  // one arrival per epilogue warp
    }
    bar_init(&S.fin, 1);
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(&S.tmem, 2 * TC_ACC_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  volatile int* abort_flag = &S.abort_flag;
  const int4 my = g.sched[blockIdx.x];

  const int iend = my.x + my.y;
  TCChunk* desc = (TCChunk*)(base + TC_DESC);  // [TC_NST][TC_MAXCH]
  if (warp == 0) {
    // producer warp: lane c loads range c of the next stage while the current stage's slot is
    // awaited, then every lane issues its own range's two bulk copies, and lane 0 copies the
    // range descriptors next to the payload for the MMA thread
    const int s_end = my.z + my.w;
    int it = 0;
    int2 st = my.w > 0 ? g.stages[my.z] : make_int2(0, 0);
    TCChunk cd{};
    if (my.w > 0 && lane < st.y) cd = g.chunks[st.x + lane];
    for (int si = my.z; si < s_end; ++si, ++it) {
      // prefetch the next stage's descriptors
      int2 st_n = make_int2(0, 0);
      TCChunk cd_n{};
      if (si + 1 < s_end) {
        st_n = g.stages[si + 1];
        if (lane < st_n.y) cd_n = g.chunks[st_n.x + lane];
      }
      uint32_t bytes = lane < st.y ? cd.abytes + cd.bbytes : 0u;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
      const int slot = it % TC_NST;
      int ok = 1;
      if (lane == 0) {
        ok = bar_wait(&S.empty[slot], ((it / TC_NST) & 1) ^ 1, abort_flag, g.err) ? 1 : 0;
        if (ok) expect_tx(&S.full[slot], bytes + (uint32_t)st.y * (uint32_t)sizeof(TCChunk));
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      unsigned char* sp = stages + (size_t)slot * TC_CAP;
      if (lane < st.y) {
        bulk_g2s(sp + cd.off, (const void*)cd.a, cd.abytes, &S.full[slot]);
        bulk_g2s(sp + cd.off + cd.abytes, (const void*)cd.b, cd.bbytes, &S.full[slot]);
      }
      if (lane == 0)
        bulk_g2s(desc + slot * TC_MAXCH, g.chunks + st.x, (uint32_t)st.y * (uint32_t)sizeof(TCChunk), &S.full[slot]);
      st = st_n;
      cd = cd_n;
    }
    // drain: wait until the MMA thread released every stage still filled, so that no copy
    // or commit arrival is in flight when the CTA ends
    if (lane == 0)
      for (int j = it > TC_NST ? it - TC_NST : 0; j < it; ++j)
        bar_wait(&S.empty[j % TC_NST], (j / TC_NST) & 1, abort_flag, g.err);
  } else if (warp == 1) {
    if (lane == 0) {
      int acc_it = 0, buf = 0, A = 1, stride = TC_ACC_COLS, rlen = TC_CHAIN, r = 0, ai = 0;
      uint32_t base = 0, idesc = 0;
      bool ok = true, issued = false, fresh = true;
      // the next buffer, once the epilogue has released it
      auto take_buffer = [&]() -> bool {
        buf = acc_it & 1;
        if (!bar_wait(&S.acce[buf], ((acc_it >> 1) & 1) ^ 1, abort_flag, g.err)) return false;
        tc_fence_after();
        base = tmem + (uint32_t)(buf * TC_ACC_COLS);
        return true;
      };
      for (int it = 0; ok && it < my.w; ++it) {
        const int slot = it % TC_NST;
        if (!bar_wait(&S.full[slot], (it / TC_NST) & 1, abort_flag, g.err)) break;
        tc_fence_after();
        const uint32_t sp = su32(stages + (size_t)slot * TC_CAP);
        const TCChunk* cds = desc + slot * TC_MAXCH;
        for (int c = 0; c < TC_MAXCH; ++c) {
          const TCChunk cd = cds[c];
          if (cd.flags & 1) {
            // first range of an item: its accumulators, round-robin over a fresh buffer
            stride = ((int)cd.N + 31) & ~31;
            A = TC_ACC_COLS / stride;
            rlen = A * TC_CHAIN;
            r = 0;
            ai = 0;
            fresh = true;
            idesc = idesc_tf32(128, cd.N);
            if (!take_buffer()) {
              ok = false;
              break;
            }
          }
          const uint32_t N = cd.N, bstride = 32u * N, kcs = cd.abytes / 2048u;
          const uint32_t sa = sp + cd.off, sb = sa + cd.abytes;
          for (uint32_t k2 = 0; k2 < kcs; k2 += 2) {
            if (r == 0 && !fresh) {
              // every accumulator of the buffer took TC_CHAIN K steps: the epilogue adds them
              // into its sums while the other buffer takes the next ones
              mma_commit(&S.accf[buf]);
              ++acc_it;
              if (!take_buffer()) {
                ok = false;
                break;
              }
            }
            fresh = false;
            const uint32_t d = base + (uint32_t)(ai * stride);
            const uint64_t ad = sdesc(sa + k2 * 2048u, 2048u, 128u);
            const uint64_t bh = sdesc(sb + k2 * bstride, bstride, 128u);
            const uint64_t bl = sdesc(sb + k2 * bstride + 16u * N, bstride, 128u);
            mma_tf32(d, ad, bh, idesc, r >= A ? 1u : 0u);  // the first K step of an accumulator overwrites it
            mma_tf32(d, ad, bl, idesc, 1u);
            if (++ai == A) ai = 0;
            if (++r == rlen) r = 0;
          }
          if (!ok) break;
          issued = true;
          if (cd.flags & 2) {
            // last range of the item: hand its last buffer to the epilogue
            mma_commit(&S.accf[buf]);
            ++acc_it;
          }
          if (cd.flags & 4) break;
        }
        if (!ok) break;
        mma_commit(&S.empty[slot]);
      }
      if (issued) {
        mma_commit(&S.fin);
        bar_wait(&S.fin, 0, abort_flag, g.err);
      }
    }
  } else {
    // epilogue: warps 2..9.  Warp w reads TMEM lanes [32 (w % 4), +32) (accumulator row
    // 32 (w % 4) + lane) and half of the item's columns (hc = (w - 2) / 4 picks the half).
    // Every buffer of an item is added into the warp's FP32 sums (round to nearest); after the
    // last one the sums are combined and stored.
    const int q4 = warp & 3, hc = (warp - 2) >> 2;
    const int row = 32 * q4 + lane;
    const int rhs = row >> 2, a = (row >> 1) & 1, h = row & 1;
    const unsigned FULL = 0xffffffffu;
    int acc_it = 0;
    TCItem In{};
    if (my.y > 0) In = g.items[my.x];
    bool ok = true;
    for (int ii = my.x; ok && ii < iend; ++ii) {
      const TCItem I = In;
      if (ii + 1 < iend) In = g.items[ii + 1];  // next item's descriptor, loaded early
      // pass 0: lane o holds the output descriptor of block o of the tile (at most 32 blocks:
      // N <= 256 and a block takes at least 8 columns), loaded before the accumulator wait
      TCOut oc{};
      if (PASS == 0 && lane < I.nout) oc = g.outs[I.out0 + lane];
      // the two warps of a lane quarter split the item's columns (N is a multiple of 16)
      const int half = I.N >> 1;
      const int c0 = hc * half;   // first column of this warp
      const int ng8 = half >> 3;  // its 8-column groups (<= 16)
      const int stride = (I.N + 31) & ~31, A = TC_ACC_COLS / stride, rlen = A * TC_CHAIN;
      const int nround = (I.nk2 + rlen - 1) / rlen;
      float sum[4][32];
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int k = 0; k < 32; ++k) sum[b][k] = 0.f;
      for (int rd = 0; rd < nround; ++rd) {
        const int used = min(A, I.nk2 - rd * rlen);  // accumulators written in this round
        const int buf = acc_it & 1;
        int w = 1;
        if (lane == 0) w = bar_wait(&S.accf[buf], (acc_it >> 1) & 1, abort_flag, g.err) ? 1 : 0;
        if (!__shfl_sync(FULL, w, 0)) {
          ok = false;
          break;
        }
        tc_fence_after();
        for (int ac = 0; ac < used; ++ac) {
          const uint32_t tb = tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(buf * TC_ACC_COLS + ac * stride + c0);
#pragma unroll
          for (int b = 0; b < 4; ++b) {
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
              // 16 columns at a time (register pressure: the sums hold 128)
              const int g0 = 4 * b + 2 * hf;
              if (g0 < ng8) {
                float v[16];
                const uint32_t t0 = tb + (uint32_t)(8 * g0);
                tmem_ld8_at<0>(t0, v);
                if (g0 + 1 < ng8) tmem_ld8_at<1>(t0 + 8, v);
                tmem_wait16(v);
#pragma unroll
                for (int J = 0; J < 2; ++J)
                  if (g0 + J < ng8)  // only the groups that were loaded
#pragma unroll
                    for (int k = 0; k < 8; ++k) sum[b][16 * hf + 8 * J + k] += v[8 * J + k];
              }
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) bar_arrive(&S.acce[buf]);
        ++acc_it;
      }
      if (!ok) break;
      const int nb = (ng8 + 3) >> 2;
      if (PASS == 0) {
        // columns (rank k, real/imaginary c) of each block: T = V2 x combined from the four
        // real products, written as the block's pass-1 A panel: row (r, a', h') holds, for
        // K = (k, c), the h' part of  a' = 0: (Re T_k, -Im T_k);  a' = 1: (Im T_k, Re T_k)
        // the block holding the current column group: its T panel and columns [col, cend);
        // blocks are stacked in column order, so it is looked up again only past cend
        float4* ta = nullptr;
        int col = 0, cend = -1;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          if (b >= nb) break;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (4 * b + j >= ng8) break;           // past this warp's columns
            const int gcol = c0 + 32 * b + 8 * j;  // warp-uniform
            if (gcol >= cend) {
              const unsigned m = __ballot_sync(FULL, lane < I.nout && oc.col <= gcol);
              const int o = __popc(m) - 1;
              ta = (float4*)__shfl_sync(FULL, oc.ta, o < 0 ? 0 : o);
              col = __shfl_sync(FULL, oc.col, o < 0 ? 0 : o);
              cend = o < 0 ? -1 : col + 2 * __shfl_sync(FULL, oc.rpad, o < 0 ? 0 : o);
              if (gcol >= cend) continue;  // padding columns after the last block
            }
            float sm[8], pm[8], out[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) sm[k] = sum[b][8 * j + k] + __shfl_xor_sync(FULL, sum[b][8 * j + k], 1);
#pragma unroll
            for (int k = 0; k < 8; ++k) pm[k] = __shfl_xor_sync(FULL, sm[k], 2);  // the other part a
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const float rr = a ? pm[2 * k] : sm[2 * k];          // sum_j Re x Re V
              const float ri = a ? pm[2 * k + 1] : sm[2 * k + 1];  // sum_j Re x Im V
              const float ir = a ? sm[2 * k] : pm[2 * k];          // sum_j Im x Re V
              const float ii2 = a ? sm[2 * k + 1] : pm[2 * k + 1]; // sum_j Im x Im V
              const float tr = rr - ii2, ti = ri + ir;
              out[2 * k] = tf32_part(a ? ti : tr, h);
              out[2 * k + 1] = tf32_part(a ? tr : -ti, h);
            }
            const int kc = (gcol - col) >> 2;
            ta[(size_t)kc * 128 + row] = make_float4(out[0], out[1], out[2], out[3]);
            ta[(size_t)(kc + 1) * 128 + row] = make_float4(out[4], out[5], out[6], out[7]);
          }
        }
      } else {
        // columns = rows i of the row tile; row (r, a, h) holds the h part of Re/Im (U2 T)_i
        float2* yp = (float2*)g.ypart;
        const int u = lane & 3;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          if (b >= nb) break;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (4 * b + j >= ng8) break;  // past this warp's columns
            const int i0 = c0 + 32 * b + 8 * j;
            if (i0 >= I.nout) break;
            float sm[8], pm[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) sm[k] = sum[b][8 * j + k] + __shfl_xor_sync(FULL, sum[b][8 * j + k], 1);
#pragma unroll
            for (int k = 0; k < 8; ++k) pm[k] = __shfl_xor_sync(FULL, sm[k], 2);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int i = i0 + k;
              if ((k >> 1) == u && i < I.nout)
                yp[(size_t)(I.out0 + i) * 32 + rhs] = make_float2(a ? pm[k] : sm[k], a ? sm[k] : pm[k]);
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * TC_ACC_COLS);
  }
}

int tc_smem_bytes() { return TC_HDR + TC_STAGE_BYTES + 1024; }

int tc_supported() {
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return 0;
  return major == 10 ? 1 : 0;
}

template <int PASS, int NST>
static cudaError_t tc_gemm_t(const TCGemmArgs& g, int grid, cudaStream_t s) {
  cudaError_t e = smem_optin<tc_gemm_kernel<PASS, NST>>(tc_smem_bytes());
  if (e != cudaSuccess) return e;
  tc_gemm_kernel<PASS, NST><<<grid, TC_THREADS, tc_smem_bytes(), s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_tc_gemm(int pass, int nst, const TCGemmArgs& g, int grid, cudaStream_t s) {
  if (grid <= 0) return cudaSuccess;
  if (nst == 3) return pass == 0 ? tc_gemm_t<0, 3>(g, grid, s) : tc_gemm_t<1, 3>(g, grid, s);
  if (nst == 4) return pass == 0 ? tc_gemm_t<0, 4>(g, grid, s) : tc_gemm_t<1, 4>(g, grid, s);
  return pass == 0 ? tc_gemm_t<0, 2>(g, grid, s) : tc_gemm_t<1, 2>(g, grid, s);
}

// ---- operand preparation ----------------------------------------------------------------------
// A panels of x: xa with K = dof (core kc: dofs 4 kc .. 4 kc + 3), xa2 with K = (dof, c) (core
// kc: dofs 2 kc, 2 kc + 1), row 4 r + 2 a + h
// one CTA (128 threads) per K core of xa (4 dofs), which also fills cores 2 kc and 2 kc + 1 of
// xa2: the 4 x 32 complex values are read once (through the permutation) and rounded to FP32
// in shared memory (one FP64 conversion per value: the FP64 pipe is narrow on this part), then
// thread = panel row splits them in FP32 and writes one 16-byte entry of each core
__global__ void __launch_bounds__(128) tc_xprep_kernel(const int* perm, int n, int nrhs, int ld, const double2* x,
                                                       float4* xa, int nkc, float4* xa2, int nkc2) {
  __shared__ float2 z[32][4];
  const int t = threadIdx.x;
  const int r = t >> 2, a = (t >> 1) & 1, h = t & 1;
  for (int kc = blockIdx.x; kc < nkc; kc += gridDim.x) {
    {
      const int j = 4 * kc + (t & 3);
      float2 v = make_float2(0.f, 0.f);
      if (j < n && (t >> 2) < nrhs) {
        const double2 w = x[(size_t)(t >> 2) * ld + perm[j]];
        v = make_float2((float)w.x, (float)w.y);
      }
      z[t >> 2][t & 3] = v;
    }
    __syncthreads();
    float o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = tf32_part(a ? z[r][k].y : z[r][k].x, h);
    xa[(size_t)kc * 128 + t] = make_float4(o[0], o[1], o[2], o[3]);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (2 * kc + q >= nkc2) break;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const float2 v = z[r][2 * q + k];
        o[2 * k] = tf32_part(a ? v.y : v.x, h);
        o[2 * k + 1] = tf32_part(a ? v.x : -v.y, h);
      }
      xa2[(size_t)(2 * kc + q) * 128 + t] = make_float4(o[0], o[1], o[2], o[3]);
    }
    __syncthreads();
  }
}

void launch_tc_xprep(const int* perm, int n, int nrhs, int ld, const void* x, void* xa, int nkc, void* xa2, int nkc2,
                     cudaStream_t s) {
  const int grid = std::max(1, std::min(nkc, 152 * 16));
  tc_xprep_kernel<<<grid, 128, 0, s>>>(perm, n, nrhs, ld, (const double2*)x, (float4*)xa, nkc, (float4*)xa2, nkc2);
}

// V2 panel of a column tile: column n = (block, rank k, part c) from the column map (x < 0:
// zero column), K = dof; entries outside the block's columns are zero
__global__ void tc_pack_v_kernel(const TCVJob* jobs, const int4* colmap, const LRDesc* lr) {
  const TCVJob J = jobs[blockIdx.x];
  float4* dst = (float4*)J.dst;
  const long long total = (long long)J.nkc * 2 * J.N;
  for (long long e = threadIdx.x; e < total; e += blockDim.x) {
    const int n = (int)(e % J.N);
    const int hk = (int)(e / J.N);
    const int hl = hk & 1, kc = hk >> 1;
    const int4 cm = colmap[J.cm0 + n];
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    if (cm.x >= 0) {
      const LRDesc L = lr[cm.x];
      const float2* V = (const float2*)L.v;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int j = 4 * (J.kc0 + kc) + k - L.c0;
        if (j >= 0 && j < L.n) {
          const float2 z = V[lr_v_index(L, cm.y, j)];
          o[k] = tf32_part(cm.z ? z.y : z.x, hl);
        }
      }
    }
    dst[e] = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// U2 panel of (row tile, block): row n = block row i0 + n, K = (rank k, part c) at 2 k + c
__global__ void tc_pack_u_kernel(const TCUJob* jobs, const LRDesc* lr) {
  const TCUJob J = jobs[blockIdx.x];
  const LRDesc L = lr[J.lr];
  const float2* U = (const float2*)L.u;
  float4* dst = (float4*)J.dst;
  const long long total = (long long)J.nkc * 2 * J.N;
  for (long long e = threadIdx.x; e < total; e += blockDim.x) {
    const int n = (int)(e % J.N);
    const int hk = (int)(e / J.N);
    const int hl = hk & 1, kc = hk >> 1;
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    if (n < J.rows) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int K = 4 * kc + k, rk = K >> 1;
        if (rk < L.R) {
          const float2 z = U[lr_u_index(L, J.i0 + n, rk)];
          o[k] = tf32_part((K & 1) ? z.y : z.x, hl);
        }
      }
    }
    dst[e] = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// panel of (row tile, dense block): row n = block row i0 + n, K = (column j, part c) with the
// columns of core kc at 2 kc, 2 kc + 1 (absolute, cluster order); the block is column-major
__global__ void tc_pack_d_kernel(const TCDJob* jobs, const MVDense* dense) {
  const TCDJob J = jobs[blockIdx.x];
  const MVDense D = dense[J.blk];
  const float2* A = (const float2*)D.ptr;
  float4* dst = (float4*)J.dst;
  const long long total = (long long)J.nkc * 2 * J.N;
  for (long long e = threadIdx.x; e < total; e += blockDim.x) {
    const int n = (int)(e % J.N);
    const int hk = (int)(e / J.N);
    const int hl = hk & 1, kc = hk >> 1;
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    if (n < J.rows) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int j = 2 * (J.kc0 + kc) + (k >> 1) - D.c0;
        if (j >= 0 && j < D.n) {
          const float2 z = A[(size_t)(J.i0 + n) + (size_t)j * D.m];
          o[k] = tf32_part((k & 1) ? z.y : z.x, hl);
        }
      }
    }
    dst[e] = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// y = alpha * (sum of the partial rows of every row cluster holding the row) + beta * y, written
// through the output permutation; one CTA per leaf, thread per (row, right-hand side)
#define TC_YS_MAXE 64
// error-free sum of a float pair accumulator (s, c) and v (Knuth TwoSum, FP32)
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float v) {
  const float t = s + v;
  const float bp = t - s;
  c += (s - (t - bp)) + (v - bp);
  s = t;
}
// Partials are summed in FP32 with TwoSum compensation (the FP64 pipe is narrow on this part);
// the FP64 result is hi + lo, formed once per component.
__global__ void __launch_bounds__(256) tc_ysum_out_kernel(const int4* leaves, const int* deltas, const float2* ypart,
                                                          const int* perm, int nrhs, int ld, double ar, double ai,
                                                          double br, double bi, int use_alpha, int use_beta,
                                                          double2* y) {
  __shared__ int dl[TC_YS_MAXE];
  const int4 L = leaves[blockIdx.x];
  const int ne = L.w - L.z, ns = min(ne, TC_YS_MAXE);
  for (int e = threadIdx.x; e < ns; e += blockDim.x) dl[e] = deltas[L.z + e];
  __syncthreads();
  const int total = (L.y - L.x) * 32;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int i = L.x + (t >> 5), r = t & 31;
    if (r >= nrhs) continue;
    float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
#pragma unroll 4
    for (int e = 0; e < ns; ++e) {
      const float2 v = ypart[(size_t)(i + dl[e]) * 32 + r];
      two_sum_acc(sr, cr, v.x);
      two_sum_acc(si, ci, v.y);
    }
    for (int e = ns; e < ne; ++e) {
      const float2 v = ypart[(size_t)(i + deltas[L.z + e]) * 32 + r];
      two_sum_acc(sr, cr, v.x);
      two_sum_acc(si, ci, v.y);
    }
    double2 o = make_double2((double)sr + (double)cr, (double)si + (double)ci);
    if (use_alpha) o = make_double2(ar * o.x - ai * o.y, ar * o.y + ai * o.x);
    double2* yo = y + (size_t)r * ld + perm[i];
    if (use_beta) {
      const double2 w = *yo;
      o.x += br * w.x - bi * w.y;
      o.y += br * w.y + bi * w.x;
    }
    *yo = o;
  }
}

void launch_tc_pack_d(const TCDJob* jobs, int njobs, const MVDense* dense, cudaStream_t s) {
  if (njobs > 0) tc_pack_d_kernel<<<njobs, 256, 0, s>>>(jobs, dense);
}

void launch_tc_ysum_out(const int4* leaves, int nleaves, const int* deltas, const void* ypart, const int* perm,
                        int nrhs, int ld, const double* alpha, const double* beta, void* y, cudaStream_t s) {
  const int use_beta = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
  const int use_alpha = (alpha[0] != 1.0 || alpha[1] != 0.0) ? 1 : 0;
  if (nleaves > 0)
    tc_ysum_out_kernel<<<nleaves, 256, 0, s>>>(leaves, deltas, (const float2*)ypart, perm, nrhs, ld, alpha[0], alpha[1],
                                               beta[0], beta[1], use_alpha, use_beta, (double2*)y);
}

void launch_tc_pack_v(const TCVJob* jobs, int njobs, const int4* colmap, const LRDesc* lr, cudaStream_t s) {
  if (njobs > 0) tc_pack_v_kernel<<<njobs, 256, 0, s>>>(jobs, colmap, lr);
}
void launch_tc_pack_u(const TCUJob* jobs, int njobs, const LRDesc* lr, cudaStream_t s) {
  if (njobs > 0) tc_pack_u_kernel<<<njobs, 256, 0, s>>>(jobs, lr);
}

// ---- self-test: one CTA, one 128 x N x (4 nkc) product ----------------------------------------
// Shared memory leaves room beyond both panels, so that the descriptor reads stay inside the
// allocation whatever the panel sizes of the test (N <= 64, nkc <= 4).
#define TC_ST_A 40960
#define TC_ST_B 16384
__global__ void __launch_bounds__(128, 1) tc_selftest_kernel(const float4* a, const float4* b, int N, int nkc, float* d,
                                                            int* err) {
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
  TCSmem& S = *(TCSmem*)base;
  unsigned char* sa = base + TC_HDR;
  unsigned char* sb = sa + TC_ST_A;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < (TC_ST_A + TC_ST_B) / 16; i += blockDim.x)
    ((float4*)sa)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (threadIdx.x == 0) {
    bar_init(&S.full[0], 1);
    bar_init(&S.fin, 1);
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) tmem_alloc(&S.tmem, 64);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  volatile int* abort_flag = &S.abort_flag;
  if (threadIdx.x == 0) {
    const uint32_t ab = (uint32_t)nkc * 2048u, bb = (uint32_t)nkc * 32u * (uint32_t)N;
    expect_tx(&S.full[0], ab + bb);
    bulk_g2s(sa, a, ab, &S.full[0]);
    bulk_g2s(sb, b, bb, &S.full[0]);
    if (bar_wait(&S.full[0], 0, abort_flag, err)) {
      tc_fence_after();
      const uint32_t idesc = idesc_tf32(128, N), bstride = 32u * (uint32_t)N;
      for (int k2 = 0; k2 < nkc; k2 += 2) {
        const uint64_t ad = sdesc(su32(sa) + (uint32_t)k2 * 2048u, 2048u, 128u);
        const uint64_t bh = sdesc(su32(sb) + (uint32_t)k2 * bstride, bstride, 128u);
        const uint64_t bl = sdesc(su32(sb) + (uint32_t)k2 * bstride + 16u * (uint32_t)N, bstride, 128u);
        mma_tf32(tmem, ad, bh, idesc, k2 > 0 ? 1u : 0u);
        mma_tf32(tmem, ad, bl, idesc, 1u);
      }
      mma_commit(&S.fin);
      bar_wait(&S.fin, 0, abort_flag, err);
    }
  }
  __syncthreads();
  tc_fence_after();
  if (!*abort_flag) {
    const int row = 32 * warp + lane;
    for (int c = 0; c < N; c += 8) {
      float v[8];
      tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
      tmem_wait(v);
#pragma unroll
      for (int k = 0; k < 8; ++k) d[(size_t)row * N + c + k] = v[k];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 64);
  }
}

cudaError_t launch_tc_selftest(const void* a, const void* b, int N, int nkc, float* d, int* err, cudaStream_t s) {
  if (N < 16 || N > 64 || N % 16 != 0 || nkc < 2 || nkc > 4 || nkc % 2 != 0) return cudaErrorInvalidValue;
  const int smem = TC_HDR + TC_ST_A + TC_ST_B + 1024;
  cudaError_t e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  tc_selftest_kernel<<<1, 128, smem, s>>>((const float4*)a, (const float4*)b, N, nkc, d, err);
  return cudaGetLastError();
}

}  // namespace bem
