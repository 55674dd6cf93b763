// H-matrix application (reference BEMBlock::MultAdd / LowRankMatrix::Mult / HMatrix::MultAdd,
// src/hmat.cpp:473-515, 527-565, 647-666).
//
// Vectors are permuted once into cluster order, where every block is a contiguous row range
// [r0, r0+m) x column range [c0, c0+n): the gather/scatter of the reference becomes a slice.
// Stage 1 computes t = V2 x for every low-rank block (column chunks, atomics into t);
// the apply pass computes y += D x (dense) and y += U2 t (low rank) over row chunks,
// accumulating into an FP64 (complex128) permuted vector with atomics; a final kernel
// un-permutes and applies alpha/beta.  Storage precision S is fp64 or fp32; products are
// formed in S and block partial sums are added in FP64.
#include <algorithm>
#include <type_traits>

#include "bem_device.cuh"
#include "kernels.h"

namespace bem {

template <class A> struct acc_of;
template <> struct acc_of<float> { using type = double; };
template <> struct acc_of<double> { using type = double; };
template <> struct acc_of<cpx<float>> { using type = cpx<double>; };
template <> struct acc_of<cpx<double>> { using type = cpx<double>; };

__device__ __forceinline__ double to_acc(float v) { return (double)v; }
__device__ __forceinline__ double to_acc(double v) { return v; }
__device__ __forceinline__ cpx<double> to_acc(cpx<float> v) { return {(double)v.x, (double)v.y}; }
__device__ __forceinline__ cpx<double> to_acc(cpx<double> v) { return v; }

// ---------------------------------------------------------------------------------------


template <class VD>
__global__ void permute_out_kernel(const int* perm, int n, int nrhs, int ld, VD alpha, VD beta, int use_beta,
                                   const VD* yp, VD* y) {
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / nrhs), r = (int)(t - (long long)k * nrhs);
    VD* dst = y + (size_t)r * ld + perm[k];
    VD v = alpha * yp[t];
    if (use_beta) v += beta * (*dst);
    *dst = v;
  }
}

__device__ __forceinline__ double scal_mul(double a, double b) { return a * b; }

template <class D> __device__ __forceinline__ D mk_d(double re, double im);
template <> __device__ __forceinline__ double mk_d<double>(double re, double) { return re; }
template <> __device__ __forceinline__ cpx<double> mk_d<cpx<double>>(double re, double im) { return mkc(re, im); }

// ---------------------------------------------------------------------------------------
// Item-based passes.  The H-matrix payload (dense blocks column-major, U2 row chunks, V2
// column chunks) is grouped into work items of at most MV_STAGE bytes; a pass streams its
// items through shared memory with cp.async.bulk (TMA bulk copies completing on mbarriers,
// MV_NSTAGE-deep pipeline, persistent grid) and each warp applies the segments of an item.
// Pass 0: t = V2 x; 1: y += D x + U2 t; 2: t = U2^T x; 3: y += D^T x + V2^T t.
//
// FP32 storage uses error-free transformations: x is split into hi + lo FP32 parts and every
// product a*x_hi is formed exactly (a*x_hi = p + e with an FMA) and summed with TwoSum, so the
// only rounding of the mixed matvec is the FP32 rounding of the stored entries: the operator
// it applies is linear and consistent to ~1e-13, which GMRES needs to reach 1e-8.
// ---------------------------------------------------------------------------------------
template <class VS> struct MT;
template <> struct MT<float> { using X = float2; using D = double; };
template <> struct MT<double> { using X = double; using D = double; };
template <> struct MT<cpx<float>> { using X = float4; using D = cpx<double>; };
template <> struct MT<cpx<double>> { using X = cpx<double>; using D = cpx<double>; };

__device__ __forceinline__ float2 split_x(double v) {
  float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ float4 split_x(cpx<double> v) {
  float2 a = split_x(v.x), b = split_x(v.y);
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ double split_x_d(double v) { return v; }

// FP64 additions into shared memory (several warps add to one row)
__device__ __forceinline__ void shared_add(double* p, double v) { atomicAdd(p, v); }
__device__ __forceinline__ void shared_add(cpx<double>* p, cpx<double> v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

template <class VS> __device__ __forceinline__ typename MT<VS>::X to_x(typename MT<VS>::D v);
template <> __device__ __forceinline__ float2 to_x<float>(double v) { return split_x(v); }
template <> __device__ __forceinline__ double to_x<double>(double v) { return v; }
template <> __device__ __forceinline__ float4 to_x<cpx<float>>(cpx<double> v) { return split_x(v); }
template <> __device__ __forceinline__ cpx<double> to_x<cpx<double>>(cpx<double> v) { return v; }

// compensated FP32 accumulator
struct CAcc { float h, l; };
__device__ __forceinline__ void cadd(CAcc& s, float a, float xh, float xl) {
  const float p = __fmul_rn(a, xh);
  const float e = fmaf(a, xh, -p);
  const float t = __fadd_rn(s.h, p);
  const float bb = __fsub_rn(t, s.h);
  const float err = __fadd_rn(__fsub_rn(s.h, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  s.h = t;
  s.l = __fadd_rn(s.l, __fadd_rn(err, fmaf(a, xl, e)));
}
__device__ __forceinline__ void cmerge(CAcc& s, float oh, float ol) {
  const float t = __fadd_rn(s.h, oh);
  const float bb = __fsub_rn(t, s.h);
  const float err = __fadd_rn(__fsub_rn(s.h, __fsub_rn(t, bb)), __fsub_rn(oh, bb));
  s.h = t;
  s.l = __fadd_rn(s.l, __fadd_rn(ol, err));
}

template <class VS> struct Acc;
template <> struct Acc<float> {
  CAcc a{0.f, 0.f};
  __device__ __forceinline__ void add(float m, float2 x) { cadd(a, m, x.x, x.y); }
  __device__ __forceinline__ Acc from_lane(int src) const {
    Acc r;
    r.a.h = __shfl_sync(0xffffffffu, a.h, src);
    r.a.l = __shfl_sync(0xffffffffu, a.l, src);
    return r;
  }
  __device__ __forceinline__ void merge(const Acc& o) { cmerge(a, o.a.h, o.a.l); }
  __device__ __forceinline__ void merge_xor(int mask) {
    float oh = __shfl_xor_sync(0xffffffffu, a.h, mask), ol = __shfl_xor_sync(0xffffffffu, a.l, mask);
    cmerge(a, oh, ol);
  }
  __device__ __forceinline__ double val() const { return (double)a.h + (double)a.l; }
};
template <> struct Acc<cpx<float>> {
  CAcc re{0.f, 0.f}, im{0.f, 0.f};
  __device__ __forceinline__ Acc from_lane(int src) const {
    Acc r;
    r.re.h = __shfl_sync(0xffffffffu, re.h, src);
    r.re.l = __shfl_sync(0xffffffffu, re.l, src);
    r.im.h = __shfl_sync(0xffffffffu, im.h, src);
    r.im.l = __shfl_sync(0xffffffffu, im.l, src);
    return r;
  }
  __device__ __forceinline__ void merge(const Acc& o) { cmerge(re, o.re.h, o.re.l); cmerge(im, o.im.h, o.im.l); }
  __device__ __forceinline__ void add(cpx<float> m, float4 x) {
    cadd(re, m.x, x.x, x.y);
    cadd(re, -m.y, x.z, x.w);
    cadd(im, m.x, x.z, x.w);
    cadd(im, m.y, x.x, x.y);
  }
  __device__ __forceinline__ void merge_xor(int mask) {
    float a = __shfl_xor_sync(0xffffffffu, re.h, mask), b = __shfl_xor_sync(0xffffffffu, re.l, mask);
    float c = __shfl_xor_sync(0xffffffffu, im.h, mask), d = __shfl_xor_sync(0xffffffffu, im.l, mask);
    cmerge(re, a, b);
    cmerge(im, c, d);
  }
  __device__ __forceinline__ cpx<double> val() const { return {(double)re.h + (double)re.l, (double)im.h + (double)im.l}; }
};
// plain FP32 accumulation (x_hi only): one FMA per product
struct AccF {
  float a = 0.f;
  __device__ __forceinline__ void add(float m, float2 x) { a = fmaf(m, x.x, a); }
  __device__ __forceinline__ AccF from_lane(int src) const { AccF r; r.a = __shfl_sync(0xffffffffu, a, src); return r; }
  __device__ __forceinline__ void merge(const AccF& o) { a += o.a; }
  __device__ __forceinline__ double val() const { return (double)a; }
};
struct AccCF {
  float re = 0.f, im = 0.f;
  __device__ __forceinline__ void add(cpx<float> m, float4 x) {
    re = fmaf(m.x, x.x, re);
    re = fmaf(-m.y, x.z, re);
    im = fmaf(m.x, x.z, im);
    im = fmaf(m.y, x.x, im);
  }
  __device__ __forceinline__ AccCF from_lane(int src) const {
    AccCF r;
    r.re = __shfl_sync(0xffffffffu, re, src);
    r.im = __shfl_sync(0xffffffffu, im, src);
    return r;
  }
  __device__ __forceinline__ void merge(const AccCF& o) { re += o.re; im += o.im; }
  __device__ __forceinline__ cpx<double> val() const { return {(double)re, (double)im}; }
};
// t in FP32: add a plain accumulator to the high part(s) of entry i of the input form (float2
// hi/lo per real value, float4 re hi/lo, im hi/lo per complex value)
__device__ __forceinline__ void add_hi(float* tx, long long i, const AccF& s) { atomicAdd(tx + 2 * i, s.a); }
__device__ __forceinline__ void add_hi(float* tx, long long i, const AccCF& s) {
  atomicAdd(tx + 4 * i, s.re);
  atomicAdd(tx + 4 * i + 2, s.im);
}
template <class VS, bool COMP> struct AccSel { using type = Acc<VS>; };
template <> struct AccSel<float, false> { using type = AccF; };
template <> struct AccSel<cpx<float>, false> { using type = AccCF; };

template <> struct Acc<double> {
  double a = 0.0;
  __device__ __forceinline__ Acc from_lane(int src) const { Acc r; r.a = __shfl_sync(0xffffffffu, a, src); return r; }
  __device__ __forceinline__ void merge(const Acc& o) { a += o.a; }
  __device__ __forceinline__ void add(double m, double x) { a = fma(m, x, a); }
  __device__ __forceinline__ void merge_xor(int mask) { a += __shfl_xor_sync(0xffffffffu, a, mask); }
  __device__ __forceinline__ double val() const { return a; }
};
template <> struct Acc<cpx<double>> {
  cpx<double> a{0.0, 0.0};
  __device__ __forceinline__ Acc from_lane(int src) const {
    Acc r;
    r.a.x = __shfl_sync(0xffffffffu, a.x, src);
    r.a.y = __shfl_sync(0xffffffffu, a.y, src);
    return r;
  }
  __device__ __forceinline__ void merge(const Acc& o) { a += o.a; }
  __device__ __forceinline__ void add(cpx<double> m, cpx<double> x) { a += m * x; }
  __device__ __forceinline__ void merge_xor(int mask) { a += shfl_xor(a, mask); }
  __device__ __forceinline__ cpx<double> val() const { return a; }
};

// pipeline shape: MV_NSTAGE stages, each with MV_STAGE payload bytes, MV_MAXPC piece
// descriptors and MV_INAREA bytes of staged inputs (all within one SM's shared memory).
// Measured on the single-vector matvec (V at L5): 5 x 32 KB 66.5 us, 4 x 48 KB 58.7 us,
// 3 x 64 KB 59.1 us, 2 x 96 KB 66.9 us -- larger items with three or four in flight.
#ifndef MV_STAGE
#define MV_STAGE 49152
#endif
#ifndef MV_PIECE
#define MV_PIECE 512  // target stored elements per piece (one consumer warp's task)
#endif
#ifndef MV_NSTAGE
#define MV_NSTAGE 4
#endif
#define MV_THREADS 1024
#define MV_CONSUMERS (MV_THREADS / 32 - 1)
#define MV_INBUF 128
#ifndef MV_MAXPC
#define MV_MAXPC 32
#endif
#ifndef MV_INAREA
#define MV_INAREA 6144
#endif
#define MV_CHMAX 8   // items per claimed chunk, at most
#define MV_HDR (128 + MV_NSTAGE * 32 + 2 * MV_CHMAX * 80)

// what the producer tells the consumers about the item in a stage (nseg < 0: no more items)
struct MVStageHdr {
  int nseg, bytes, inbytes, pad;
  unsigned long long src;
  unsigned long long pad2;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, int bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false after ~1<<22 polls (the phase never completed)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// bounded wait with a short sleep between polls, for the many consumer warps (leaves the
// issue slots to the producer warp and to warps with work)
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 20); ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    __nanosleep(64);
  }
  return false;
}

// out[o] += sum_k A[o*so + k*sk] * in[k] for o < O, one warp.  When O < 32 the lanes form
// G = 32/O groups (lane = o + g*O) that split k and are combined by shuffles, so G*O lanes
// work; with so = 1 and sk = O consecutive lanes read consecutive shared-memory words.
template <class VS, bool COMP, class InF, class OutF>
__device__ __forceinline__ void warp_gemv(const VS* A, int so, int sk, int O, int Kc, InF in, OutF out,
                                          typename MT<VS>::X* buf, int lane, bool first_staged = false) {
  using AccT = typename AccSel<VS, COMP>::type;
  using X = typename MT<VS>::X;
  const int Ow = O < 32 ? O : 32;
  const int G = 32 / Ow;
  const int g = lane / Ow, ol = lane - g * Ow;
  const bool active = g < G;
  for (int kc0 = 0; kc0 < Kc; kc0 += MV_INBUF) {
    const int kn = min(MV_INBUF, Kc - kc0);
    if (!(first_staged && kc0 == 0)) {
      __syncwarp();
      for (int k = lane; k < kn; k += 32) buf[k] = in(kc0 + k);
    }
    __syncwarp();
    for (int o0 = 0; o0 < O; o0 += Ow) {
      const int o = o0 + ol;
      AccT acc;
      if (active && o < O) {
        const VS* Ap = A + o * so + (kc0 + g) * sk;
        const X* bp = buf + g;
        const int astep = G * sk;
        int k = g;
#pragma unroll 4
        for (; k < kn; k += G) {
          acc.add(*Ap, *bp);
          Ap += astep;
          bp += G;
        }
      }
      // combine the G groups into group 0 (source lanes o + j*Ow)
      for (int j = 1; j < G; ++j) {
        AccT other = acc.from_lane(ol + j * Ow);
        if (g == 0) acc.merge(other);
      }
      if (g == 0 && o < O) out(o, acc.val());
    }
  }
}

// out[o] += sum_k A[o*so + k*sk] * in[k] for o < O, one warp, inputs already in shared
// memory.  When O < 32 the lanes form G = 32/O groups (lane = o + g*O) that split k and are
// combined by shuffles; with so = 1 and sk = O consecutive lanes read consecutive words.
template <class VS, bool COMP, class InF, class OutF>
__device__ __forceinline__ void warp_gemv_s(const VS* A, int so, int sk, int O, int Kc, int Ow, int G, float inv_ow,
                                            InF in, OutF out, int lane) {
  using AccT = typename AccSel<VS, COMP>::type;
  const int g = __float2int_rz(((float)lane + 0.5f) * inv_ow);
  const int ol = lane - g * Ow;
  const bool active = g < G;
  for (int o0 = 0; o0 < O; o0 += Ow) {
    const int o = o0 + ol;
    AccT acc;
    if (active && o < O) {
      const VS* Ap = A + o * so + g * sk;
      const int astep = G * sk;
#pragma unroll 4
      for (int k = g; k < Kc; k += G) {
        acc.add(*Ap, in(k));
        Ap += astep;
      }
    }
    for (int j = 1; j < G; ++j) {
      AccT other = acc.from_lane(ol + j * Ow);
      if (g == 0) acc.merge(other);
    }
    if (g == 0 && o < O) out(o, acc);
  }
}

template <class VS, bool COMP>
__device__ __forceinline__ void run_piece_s(const MVArgs2& a, const MVPiece& pc, const VS* A, const typename MT<VS>::X* xin,
                                            int lane) {
  using D = typename MT<VS>::D;
  if constexpr (!COMP && (std::is_same<VS, float>::value || std::is_same<VS, cpx<float>>::value)) {
    if ((pc.flags & 2) && a.t_f32) {
      float* tx = (float*)a.tx;
      warp_gemv_s<VS, COMP>(A, pc.so, pc.sk, pc.O, pc.Kc, pc.ow, pc.groups, pc.inv_ow, [&](int k) { return xin[k]; },
                            [&](int o, const auto& s) { add_hi(tx, (long long)pc.out_off + o, s); }, lane);
      return;
    }
  }
  D* out = ((pc.flags & 2) ? (D*)a.t : (D*)a.yp) + pc.out_off;
  warp_gemv_s<VS, COMP>(A, pc.so, pc.sk, pc.O, pc.Kc, pc.ow, pc.groups, pc.inv_ow, [&](int k) { return xin[k]; },
                        [&](int o, const auto& s) { atomic_add(&out[o], s.val()); }, lane);
}

// Persistent single right-hand-side pass, warp specialised.  Warp 0 (the producer) streams
// items into MV_NSTAGE shared-memory stages with bulk copies: the payload, the item's piece
// descriptors and the input ranges its pieces read (slices of the permuted x or of t), all
// counted on the stage's full barrier.  The consumer warps take the pieces of each item
// round-robin -- reading only shared memory -- and release the stage on its empty barrier.
//
// Items are handed out in chunks of consecutive items.  A CTA's first chunk is fixed
// (blockIdx.x * w0 ...); later chunks are claimed from a counter, with sizes that shrink as
// the items run out (guided scheduling), so SMs whose copies land later do fewer items
// instead of setting the kernel time.  The descriptors of a chunk are bulk-copied into one of
// two shared-memory buffers while the previous chunk is issued, and each claim is made one
// chunk ahead, so the issue loop never waits on a global load.  After its last item the
// producer pushes a stop marker (nseg < 0) through the next stage; the consumers release it
// like an item, so a second pass can run through the same pipeline.
// an item issued before its inputs were ready: its stage and input ranges
struct MVPend {
  int stage, rng0, nrng, pad;
  int r[8];
};

struct MVSmem {
  uint64_t* full;        // MV_NSTAGE barriers: stage filled
  uint64_t* empty;       // MV_NSTAGE barriers: stage released by all consumer warps
  uint64_t* dbar;        // 2 barriers: descriptor buffers filled
  MVStageHdr* hdr;       // per stage: what the item holds
  MVTItem* dring;        // 2 x MV_CHMAX item descriptors
  unsigned char* stage;  // per stage: MV_STAGE payload bytes
  MVPiece* dstage;       // per stage: MV_MAXPC piece descriptors
  unsigned char* istage; // per stage: MV_INAREA staged input bytes
  MVPend* pend;          // MV_NSTAGE items whose input ranges wait for the gate (producer only)
  volatile int* gate;    // phase gate of the single-launch matvec (inputs of phase p ready: >= p + 1)
};

__device__ __forceinline__ MVSmem mv_smem(unsigned char* smem) {
  MVSmem m;
  m.full = (uint64_t*)smem;
  m.empty = m.full + MV_NSTAGE;
  m.dbar = m.empty + MV_NSTAGE;
  m.hdr = (MVStageHdr*)(smem + 128);
  m.dring = (MVTItem*)(smem + 128 + MV_NSTAGE * sizeof(MVStageHdr));
  m.stage = smem + MV_HDR;
  m.dstage = (MVPiece*)(m.stage + MV_NSTAGE * MV_STAGE);
  m.istage = (unsigned char*)(m.dstage + MV_NSTAGE * MV_MAXPC);
  m.pend = (MVPend*)(m.istage + MV_NSTAGE * MV_INAREA);
  m.gate = (volatile int*)(m.pend + MV_NSTAGE);
  return m;
}

__device__ __forceinline__ void mv_init_barriers(const MVSmem& m) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < MV_NSTAGE; ++s) {
      mbar_init(&m.full[s], 1);
      mbar_init(&m.empty[s], MV_CONSUMERS);
    }
    mbar_init(&m.dbar[0], 1);
    mbar_init(&m.dbar[1], 1);
    *m.gate = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
}

// pipeline position of the producer warp / of one consumer warp (carried across passes)
struct MVProd { uint32_t ephase = 0, dphase = 0; int it = 0; };
struct MVCons { uint32_t fphase = 0; int it = 0; int pbase = 0; };

// Producer warp: streams items [0, nit) (first chunk fixed, the rest claimed from *ctr), then
// the stop marker.  Returns false if a wait timed out (error flag set; copies drained).
// need > 0: the inputs (x or t) of this pass are written by other CTAs; they are ready once the
// gate reaches need.  Until then every item's payload and descriptors are issued at once and
// its input-range copies are parked (the item's full barrier already expects their bytes, so no
// consumer starts on it); the stage waits keep watching the gate, so the parked copies go out
// as soon as it opens even while all stages are taken.
__device__ bool mv_produce(const MVArgs2& a, const MVTItem* items, int nit, int* ctr, const MVSmem& m, MVProd& p,
                           int lane, int need = 0) {
  const int G = gridDim.x;
  int ok = 1;
  const int it0 = p.it;
  bool open = need <= 0 || *m.gate >= need;
  int npend = 0;
  auto issue_ranges = [&](int s, int rng0, int nrng, const int* rin) {
    unsigned char* ia = m.istage + s * MV_INAREA;
    for (int r = lane; r < nrng; r += 32) {
      MVRange rg;
      if (r < 2) rg = MVRange{rin[4 * r], rin[4 * r + 1], rin[4 * r + 2], rin[4 * r + 3]};
      else rg = a.ranges[rng0 + r];
      const unsigned char* gsrc = (const unsigned char*)(rg.src ? a.tx : a.xp) + (size_t)rg.elem * a.in_esz;
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   ::"r"(smem_u32(ia + rg.dst)), "l"((const void*)gsrc), "r"(rg.bytes),
                   "r"(smem_u32(&m.full[s])) : "memory");
    }
  };
  auto open_gate = [&]() {  // whole warp: the inputs are ready, issue the parked copies
    __threadfence();
    asm volatile("fence.proxy.async.global;" ::: "memory");
    open = true;
    for (int k = 0; k < npend; ++k) issue_ranges(m.pend[k].stage, m.pend[k].rng0, m.pend[k].nrng, m.pend[k].r);
    __syncwarp();
    npend = 0;
  };
  // wait for a free stage; meanwhile open the gate if it has become ready
  auto wait_empty = [&](int s, uint32_t parity) -> int {
    for (int i = 0; i < (1 << 22); ++i) {
      int st = 0;
      if (lane == 0) {
        st = mbar_try_wait(&m.empty[s], parity) ? 1 : 0;
        if (!open && *m.gate >= need) st |= 2;
      }
      st = __shfl_sync(0xffffffffu, st, 0);
      if (st & 2) open_gate();
      if (st & 1) return 1;
    }
    return 0;
  };
  // global data written before this pass by ordinary stores (x, t) is read by bulk copies
  asm volatile("fence.proxy.async.global;" ::: "memory");
  auto chunk_size = [&](int remaining) {
    const int w = remaining / (4 * G);
    return w < 2 ? 2 : (w > MV_CHMAX ? MV_CHMAX : w);
  };
  auto fetch_descs = [&](int buf, int c0, int cn) {  // lane 0
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bulk_load(m.dring + buf * MV_CHMAX, items + c0, cn * (int)sizeof(MVTItem), &m.dbar[buf]);
  };
  // fixed first chunk, then claims at w0 * G + counter
  const int w0 = chunk_size(nit);
  const int base = w0 * G;
  int c0 = blockIdx.x * w0;
  int cn = c0 < nit ? min(w0, nit - c0) : 0;
  int sc = 0;
  int dpend = -1;  // descriptor buffer with a copy in flight that nobody has waited for
  if (cn > 0) {
    if (lane == 0) fetch_descs(0, c0, cn);
    dpend = 0;
  }
  int want = chunk_size(nit - base), tok = 0;
  bool pend = base < nit;
  if (pend && lane == 0) tok = atomicAdd(ctr, want);
  while (cn > 0) {
    ok = mbar_wait(&m.dbar[sc], (p.dphase >> sc) & 1u) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) break;
    p.dphase ^= 1u << sc;
    dpend = -1;
    int n0 = 0, nn = 0, wnext = 0;
    for (int j = 0; j < cn; ++j) {
      const MVTItem* d = m.dring + sc * MV_CHMAX + j;
      const unsigned long long src = d->src;
      const int bytes = d->bytes, seg0 = d->seg0, nseg = d->nseg, rng0 = d->rng0, nrng = d->nrng;
      const int inbytes = d->inbytes;
      const int s = p.it % MV_NSTAGE;
      if (!open && inbytes < 0) {
        // inputs read in place: nothing may be issued for this item before they are ready
        int st = 0;
        for (int i = 0; i < (1 << 24) && !st; ++i) {
          if (lane == 0) st = *m.gate >= need ? 1 : 0;
          st = __shfl_sync(0xffffffffu, st, 0);
          if (!st) __nanosleep(64);
        }
        if (!st) {
          ok = 0;
          break;
        }
        open_gate();
      }
      // the first use of a stage passes at once (parity of the phase before the first)
      ok = wait_empty(s, ((p.ephase >> s) & 1u) ^ 1u);
      if (!ok) break;
      p.ephase ^= 1u << s;
      const int dbytes = nseg * (int)sizeof(MVPiece);
      if (lane == 0) {
        m.hdr[s].nseg = nseg;
        m.hdr[s].bytes = bytes;
        m.hdr[s].inbytes = inbytes;
        m.hdr[s].src = src;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        // one arrival carries the transaction bytes of all copies of the item
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&m.full[s])),
                     "r"(bytes + dbytes + (inbytes > 0 ? inbytes : 0)) : "memory");
        if (bytes > 0)
          asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                       ::"r"(smem_u32(m.stage + s * MV_STAGE)), "l"((const void*)src), "r"(bytes),
                       "r"(smem_u32(&m.full[s])) : "memory");
        if (dbytes > 0)
          asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                       ::"r"(smem_u32(m.dstage + s * MV_MAXPC)), "l"((const void*)(a.pieces + seg0)),
                       "r"(dbytes), "r"(smem_u32(&m.full[s])) : "memory");
      }
      if (open) {
        issue_ranges(s, rng0, nrng, d->r);
      } else if (nrng > 0) {
        if (lane == 0) {
          MVPend& e = m.pend[npend];
          e.stage = s;
          e.rng0 = rng0;
          e.nrng = nrng;
#pragma unroll
          for (int k = 0; k < 8; ++k) e.r[k] = d->r[k];
        }
        ++npend;  // at most MV_NSTAGE: a parked item holds its stage until its inputs land
      }
      __syncwarp();
      ++p.it;
      if (pend) {
        // the claim made a chunk ago: start copying the descriptors of the next chunk
        pend = false;
        const int k = base + __shfl_sync(0xffffffffu, tok, 0);
        n0 = k;
        nn = k < nit ? min(want, nit - k) : 0;
        wnext = nit - (k + want);
        if (nn > 0) {
          if (lane == 0) fetch_descs(sc ^ 1, n0, nn);
          dpend = sc ^ 1;
        }
      }
    }
    if (!ok) break;
    __syncwarp();
    sc ^= 1;
    c0 = n0;
    cn = nn;
    if (cn > 0 && wnext > 0) {
      want = chunk_size(wnext);
      pend = true;
      if (lane == 0) tok = atomicAdd(ctr, want);
    }
  }
  if (ok && !open) {
    // all items issued before the inputs were ready: wait for the gate (bounded)
    int st = 0;
    for (int i = 0; i < (1 << 24) && !st; ++i) {
      if (lane == 0) st = *m.gate >= need ? 1 : 0;
      st = __shfl_sync(0xffffffffu, st, 0);
      if (!st) __nanosleep(64);
    }
    if (st) open_gate();
    else ok = 0;
  }
  if (lane == 0) {
    if (!ok) {
      atomicOr(a.err, 2);
      // every issued copy must land before shared memory is reused or the CTA exits
      for (int j = max(it0, p.it - MV_NSTAGE); j < p.it; ++j) {
        const int s = j % MV_NSTAGE;
        const uint32_t par = (uint32_t)((j / MV_NSTAGE) & 1);
        mbar_wait(&m.full[s], par);
      }
      if (dpend >= 0) mbar_wait(&m.dbar[dpend], (p.dphase >> dpend) & 1u);
    }
    // stop marker (a wait that times out leaves the consumers to time out on their own)
    const int s = p.it % MV_NSTAGE;
    if (mbar_wait(&m.empty[s], ((p.ephase >> s) & 1u) ^ 1u)) {
      m.hdr[s].nseg = -1;
      mbar_arrive(&m.full[s]);
    } else {
      ok = 0;
      atomicOr(a.err, 2);
    }
  }
  ++p.it;
  p.ephase ^= 1u << ((p.it - 1) % MV_NSTAGE);
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// One consumer warp (cw = 0 .. MV_CONSUMERS-1): applies its pieces of every item until the
// stop marker.
template <class VS, bool COMP>
__device__ void mv_consume(const MVArgs2& a, const MVSmem& m, MVCons& c, int cw, int lane) {
  for (;; ++c.it) {
    const int s = c.it % MV_NSTAGE;
    if (!mbar_wait_sleep(&m.full[s], (c.fphase >> s) & 1u)) {
      if (lane == 0) atomicOr(a.err, 2);
      ++c.it;
      return;
    }
    c.fphase ^= 1u << s;
    const int nseg = m.hdr[s].nseg;
    if (nseg < 0) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&m.empty[s]);
      ++c.it;
      return;
    }
    const bool sa = m.hdr[s].bytes > 0, si = m.hdr[s].inbytes >= 0;
    int q0 = cw - c.pbase % MV_CONSUMERS;  // warp cw takes pieces with (pbase + q) % C == cw
    if (q0 < 0) q0 += MV_CONSUMERS;
    c.pbase += nseg;
    const MVPiece* pcs = m.dstage + s * MV_MAXPC;
    // separate paths so that staged operands are read with shared-memory loads
    using X = typename MT<VS>::X;
    const unsigned char* sbase = m.stage + s * MV_STAGE;
    const unsigned char* ia = m.istage + s * MV_INAREA;
    if (sa && si) {
      for (int q = q0; q < nseg; q += MV_CONSUMERS) {
        const MVPiece pc = pcs[q];
        run_piece_s<VS, COMP>(a, pc, (const VS*)(sbase + pc.soff), (const X*)(ia + pc.in_soff), lane);
      }
    } else {
      const unsigned char* gbase = (const unsigned char*)m.hdr[s].src;
      for (int q = q0; q < nseg; q += MV_CONSUMERS) {
        const MVPiece pc = pcs[q];
        const X* gin = (const X*)((const unsigned char*)((pc.flags & 1) ? a.tx : a.xp) + (size_t)pc.in_off * a.in_esz);
        if (sa) run_piece_s<VS, COMP>(a, pc, (const VS*)(sbase + pc.soff), gin, lane);
        else if (si) run_piece_s<VS, COMP>(a, pc, (const VS*)(gbase + pc.soff), (const X*)(ia + pc.in_soff), lane);
        else run_piece_s<VS, COMP>(a, pc, (const VS*)(gbase + pc.soff), gin, lane);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&m.empty[s]);
  }
}

// One pass as its own launch.  The chunk-claim counter a.sched[0] is reset by the last CTA to
// finish (counter a.sched[1]), which leaves both zero for the next launch on the stream.
template <class VS, bool COMP>
__global__ void __launch_bounds__(MV_THREADS, 1) mv_tma_kernel(MVArgs2 a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const MVSmem m = mv_smem(smem);
  mv_init_barriers(m);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    MVProd p;
    mv_produce(a, a.items, a.nitems, a.sched, m, p, lane);
    if (lane == 0) {
      __threadfence();
      if (atomicAdd(a.sched + 1, 1) == (int)gridDim.x - 1) {
        atomicExch(a.sched, 0);
        atomicExch(a.sched + 1, 0);
      }
    }
    return;
  }
  MVCons c;
  mv_consume<VS, COMP>(a, m, c, warp - 1, lane);
}

// Grid-wide barrier of the consumer warps of a cooperative launch (all CTAs resident; the
// producer warp of each CTA keeps streaming meanwhile): named barrier 1 over the consumer
// threads, then thread 32 adds its arrival to the 64-bit counter *bar and waits until the
// counter reaches this barrier's target.  The counter only grows: every launch passes the
// same number of barriers with all CTAs, so it is a multiple of the grid size when a launch
// starts, and barrier j of the launch completes at base + j * grid size.  One atomic and one
// observation per CTA; nobody resets anything.  A wait that runs past its limit sets the
// error flag and returns false instead of hanging.
struct MVGridBar {
  unsigned long long* ctr;
  unsigned long long base;
  int n;  // barriers passed in this launch
  long long limit;            // polls before the wait gives up
  unsigned long long extra;   // added to every target (a test makes the waits run out with 1)
};
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ bool mv_grid_sync_cons(MVGridBar& g, int* err, int* flag) {
  asm volatile("bar.sync 1, %0;" ::"r"(MV_THREADS - 32) : "memory");
  if (threadIdx.x == 32) {
    int ok = 1;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(g.ctr) : "memory");
    g.n += 1;
    const unsigned long long target = g.base + (unsigned long long)g.n * gridDim.x + g.extra;
    long long i = 0;
    while (ld_acquire_u64(g.ctr) < target) {
      if (++i > g.limit) {
        ok = 0;
        atomicOr(err, 4);
        break;
      }
      __nanosleep(20);
    }
    __threadfence();
    *flag = ok;
  }
  asm volatile("bar.sync 1, %0;" ::"r"(MV_THREADS - 32) : "memory");
  return *flag != 0;
}

// One whole matvec per launch.  Warp 0 of each CTA streams phase A from the start and phase B
// right after it, issuing payloads and descriptors ahead of the grid barriers and parking the
// input-range copies until the gate says the inputs are ready (gate 1: permuted x, after the
// prologue barrier; gate 2: t in input form, after the phase-A barrier and the conversion).
// The consumer warps do the prologue, the conversion and the epilogue with grid-stride loops
// and hold the grid barriers.  The claim counters of the two phases are zero on entry (set at
// operator build, reset again by the epilogue once every CTA has finished claiming).
template <class VS, bool COMP>
__global__ void __launch_bounds__(MV_THREADS, 1) mv_fused_kernel(MVFusedArgs f) {
  using D = typename MT<VS>::D;
  using X = typename MT<VS>::X;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int bflag;
  const MVSmem m = mv_smem(smem);
  mv_init_barriers(m);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  MVArgs2 a = f.a;
  auto set_phase = [&](int ph) {
    a.items = f.items[ph];
    a.pieces = f.pieces[ph];
    a.ranges = f.ranges[ph];
    a.nitems = f.nitems[ph];
  };
  if (warp == 0) {
    MVProd p;
    for (int ph = 0; ph < 2; ++ph) {
      set_phase(ph);
      if (a.nitems > 0) mv_produce(a, a.items, a.nitems, f.ctr[ph], m, p, lane, ph + 1);
    }
    return;
  }
  const long long ct = (long long)blockIdx.x * (MV_THREADS - 32) + (tid - 32);
  const long long cs = (long long)gridDim.x * (MV_THREADS - 32);
  MVGridBar gb{f.bar, 0ull, 0, f.wait_limit > 0 ? f.wait_limit : MV_WAIT_LIMIT, f.bar_extra};
  if (tid == 32) {
    // no CTA of this launch can have passed its first barrier yet: round down to the launch's base
    const unsigned long long c0 = ld_acquire_u64(f.bar);
    gb.base = c0 - c0 % gridDim.x;
  }
  // prologue: permuted input.  The accumulators yp, t and tx are zero on entry: every matvec
  // of the operator leaves them zero (this kernel's epilogue, a memset after the multi-pass
  // schedule); only after an error (a launch that may have stopped early) are they zeroed here.
  constexpr bool FP32S = !std::is_same<VS, double>::value && !std::is_same<VS, cpx<double>>::value;
  const bool t32 = a.t_f32 != 0;
  {
    const D* x = (const D*)f.x;
    X* xp = (X*)a.xp;
    for (long long k = ct; k < f.n_in; k += cs) xp[k] = to_x<VS>(x[f.perm_in[k]]);
    if (*(volatile int*)a.err != 0) {
      D* yp = (D*)a.yp;
      for (long long k = ct; k < f.n_out; k += cs) yp[k] = D{};
      D* t = (D*)a.t;
      for (long long k = ct; k < f.t_len; k += cs) t[k] = D{};
      if (FP32S) {
        X* tx = (X*)a.tx;
        for (long long k = ct; k < f.t_len; k += cs) tx[k] = X{};
      }
    }
  }
  mv_grid_sync_cons(gb, a.err, &bflag);
  if (tid == 32) *m.gate = 1;
  MVCons c;
  set_phase(0);
  if (a.nitems > 0) mv_consume<VS, COMP>(a, m, c, warp - 1, lane);
  mv_grid_sync_cons(gb, a.err, &bflag);
  // t is complete: its input form for phase B (already in place when t accumulates in FP32)
  if constexpr (FP32S) {
    if (!t32) {
      const D* t = (const D*)a.t;
      X* tx = (X*)a.tx;
      for (long long k = ct; k < f.t_len; k += cs) tx[k] = to_x<VS>(t[k]);
      mv_grid_sync_cons(gb, a.err, &bflag);
    }
  }
  if (tid == 32) *m.gate = 2;
  set_phase(1);
  if (a.nitems > 0) mv_consume<VS, COMP>(a, m, c, warp - 1, lane);
  mv_grid_sync_cons(gb, a.err, &bflag);
  // every CTA has finished claiming: zero the claim counters for the next launch
  if (blockIdx.x == 0 && tid == 32) {
    *f.ctr[0] = 0;
    *f.ctr[1] = 0;
  }
  // epilogue: y = alpha yp + beta y in the caller's numbering; yp and t (tx) are zeroed for
  // the next launch (every entry by the thread that read it; t is no longer read after the
  // last barrier)
  {
    D* yp = (D*)a.yp;
    D* y = (D*)f.y;
    const D al = mk_d<D>(f.alpha[0], f.alpha[1]), be = mk_d<D>(f.beta[0], f.beta[1]);
    for (long long k = ct; k < f.n_out; k += cs) {
      D* dst = y + f.perm_out[k];
      D v = al * yp[k];
      if (f.use_beta) v += be * (*dst);
      *dst = v;
      yp[k] = D{};
    }
    if (!t32) {
      D* t = (D*)a.t;
      for (long long k = ct; k < f.t_len; k += cs) t[k] = D{};
    }
    if (FP32S) {
      X* tx = (X*)a.tx;
      for (long long k = ct; k < f.t_len; k += cs) tx[k] = X{};
    }
  }
}

// generic pass for several right-hand sides (payload read in place): lane = rhs
template <class VS, bool COMP>
__global__ void __launch_bounds__(256) mv_multi_kernel(MVArgs2 a) {
  using AccT = typename AccSel<VS, COMP>::type;
  using X = typename MT<VS>::X;
  using D = typename MT<VS>::D;
  const MVTItem item = a.items[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const X* xp = (const X*)a.xp;
  D* t = (D*)a.t;
  D* yp = (D*)a.yp;
  const int nr = a.nrhs;
  for (int q = warp; q < item.nseg; q += nwarp) {
    const MVPiece pc = a.pieces[item.seg0 + q];
    const VS* A = (const VS*)((const unsigned char*)item.src + pc.soff);
    const bool in_t = pc.flags & 1, out_t = pc.flags & 2;
    for (int o = 0; o < pc.O; ++o)
      for (int g = 0; g < nr; g += 32) {
        const int rh = g + lane;
        if (rh >= nr) continue;
        AccT acc;
        for (int k = 0; k < pc.Kc; ++k) {
          const size_t idx = (size_t)(pc.in_off + k) * nr + rh;
          const X xv = in_t ? ((const X*)a.tx)[idx] : xp[idx];
          acc.add(A[(long long)o * pc.so + (long long)k * pc.sk], xv);
        }
        D* dst = (out_t ? t : yp) + (size_t)(pc.out_off + o) * nr + rh;
        atomic_add(dst, acc.val());
      }
  }
}

// Several right-hand sides over chunk items (one piece per chunk, lane = right-hand side).
// Long reductions (Kc >= MV_MC_SPLIT: dense and V2 column chunks): the 8 warps split the
// columns, each keeps partial sums for MV_MR rows in registers (one input load feeds MV_MR
// products), and the partials are added across warps in shared memory before a single atomic
// per output row and right-hand side.  Short reductions (U2 chunks, Kc = rank): the warps
// split the rows and each row is reduced by one warp.
#define MV_MR 8
#define MV_MC_SPLIT 64
template <class VS, bool COMP>
__global__ void __launch_bounds__(256) mv_multi_chunk_kernel(MVArgs2 a) {
  using AccT = typename AccSel<VS, COMP>::type;
  using X = typename MT<VS>::X;
  using D = typename MT<VS>::D;
  __shared__ D part[8][MV_MR][32];
  const MVTItem item = a.items[blockIdx.x];
  const MVPiece pc = a.pieces[item.seg0];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const VS* A = (const VS*)((const unsigned char*)item.src + pc.soff);
  const X* xin = (const X*)((pc.flags & 1) ? a.tx : a.xp);
  D* out = ((pc.flags & 2) ? (D*)a.t : (D*)a.yp) + (size_t)pc.out_off * a.nrhs;
  const int nr = a.nrhs;
  if (pc.Kc < MV_MC_SPLIT) {
    for (int o = warp; o < pc.O; o += 8)
      for (int g = 0; g < nr; g += 32) {
        const int rh = g + lane;
        if (rh >= nr) continue;
        AccT acc;
        const X* xk = xin + (size_t)pc.in_off * nr + rh;
        for (int k = 0; k < pc.Kc; ++k) acc.add(A[(long long)o * pc.so + (long long)k * pc.sk], xk[(size_t)k * nr]);
        atomic_add(out + (size_t)o * nr + rh, acc.val());
      }
    return;
  }
  const int k0 = (int)(((long long)pc.Kc * warp) / 8), k1 = (int)(((long long)pc.Kc * (warp + 1)) / 8);
  for (int o0 = 0; o0 < pc.O; o0 += MV_MR) {
    const int no = min(MV_MR, pc.O - o0);
    for (int g = 0; g < nr; g += 32) {
      const int rh = g + lane;
      AccT acc[MV_MR];
      if (rh < nr) {
        const X* xk = xin + (size_t)(pc.in_off + k0) * nr + rh;
        const VS* Ak = A + (long long)o0 * pc.so + (long long)k0 * pc.sk;
        for (int k = k0; k < k1; ++k) {
          const X xv = *xk;
#pragma unroll
          for (int r = 0; r < MV_MR; ++r)
            if (r < no) acc[r].add(Ak[(long long)r * pc.so], xv);
          xk += nr;
          Ak += pc.sk;
        }
      }
#pragma unroll
      for (int r = 0; r < MV_MR; ++r) part[warp][r][lane] = acc[r].val();
      __syncthreads();
      {
        const int r = tid >> 5, l = tid & 31;  // 256 threads = MV_MR rows x 32 lanes
        if (r < no && g + l < nr) {
          D sum = part[0][r][l];
#pragma unroll
          for (int w = 1; w < 8; ++w) sum += part[w][r][l];
          atomic_add(out + (size_t)(o0 + r) * nr + g + l, sum);
        }
      }
      __syncthreads();
    }
  }
}

#define MV_RO_ROWS 64
template <class VS, bool COMP>
__global__ void __launch_bounds__(256) mv_rowowner_kernel(MVRowArgs a) {
  using AccT = typename AccSel<VS, COMP>::type;
  using X = typename MT<VS>::X;
  using D = typename MT<VS>::D;
  __shared__ D ysm[MV_RO_ROWS][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int4 L = a.leaves[blockIdx.x];  // rows [L.x, L.y), entries [L.z, L.w)
  const int nr = a.nrhs;
  const X* xp = (const X*)a.xp;
  const X* tx = (const X*)a.tx;
  D* yp = (D*)a.yp;
  for (int t0 = L.x; t0 < L.y; t0 += MV_RO_ROWS) {
    const int t1 = min(L.y, t0 + MV_RO_ROWS);
    for (int g = 0; g < nr; g += 32) {
      for (int q = tid; q < MV_RO_ROWS * 32; q += 256) ysm[q >> 5][q & 31] = D{};
      __syncthreads();
      const int rh = g + lane;
      for (int e = L.z + warp; e < L.w; e += 8) {
        const int4 E = a.ents[e];
        // rows of this entry (global, permuted) inside the tile
        int i0, i1, gr0;
        if (E.x == 0) gr0 = a.dense[E.y].r0;
        else gr0 = a.lr[E.y].r0;
        i0 = max(t0, gr0 + E.z);
        i1 = min(t1, gr0 + E.z + E.w);
        if (rh >= nr) continue;
        for (int ib = i0; ib < i1; ib += MV_MR) {
          const int no = min(MV_MR, i1 - ib);
          AccT acc[MV_MR];
          if (E.x == 0) {
            const MVDense Dd = a.dense[E.y];
            const VS* A = (const VS*)Dd.ptr + (ib - Dd.r0);
            const X* xk = xp + (size_t)Dd.c0 * nr + rh;
            for (int k = 0; k < Dd.n; ++k) {
              const X xv = xk[(size_t)k * nr];
              const VS* Ak = A + (long long)k * Dd.m;
#pragma unroll
              for (int r = 0; r < MV_MR; ++r)
                if (r < no) acc[r].add(Ak[r], xv);
            }
          } else {
            const LRDesc Lr = a.lr[E.y];
            const VS* U = (const VS*)Lr.u;
            long long base[MV_MR];
#pragma unroll
            for (int r = 0; r < MV_MR; ++r) {
              const int i = ib - Lr.r0 + (r < no ? r : 0);
              base[r] = lr_u_index(Lr, i, 0);
            }
            const X* xk = tx + (size_t)Lr.toff * nr + rh;
            for (int k = 0; k < Lr.R; ++k) {
              const X xv = xk[(size_t)k * nr];
#pragma unroll
              for (int r = 0; r < MV_MR; ++r)
                if (r < no) acc[r].add(U[base[r] + (long long)k * Lr.cu], xv);
            }
          }
#pragma unroll
          for (int r = 0; r < MV_MR; ++r)
            if (r < no) shared_add(&ysm[ib + r - t0][lane], acc[r].val());
        }
      }
      __syncthreads();
      for (int q = tid; q < (t1 - t0) * 32; q += 256) {
        const int i = q >> 5, l = q & 31;
        if (g + l < nr) yp[(size_t)(t0 + i) * nr + g + l] = ysm[i][l];
      }
      __syncthreads();
    }
  }
}

template <class VS, bool COMP>
static void rowowner_t(const MVRowArgs& a, cudaStream_t s) {
  if (a.nleaves > 0) mv_rowowner_kernel<VS, COMP><<<a.nleaves, 256, 0, s>>>(a);
}

void launch_mv_rowowner(int prec, bool cplx, const MVRowArgs& a, cudaStream_t s) {
  if (prec == 0) {
    if (cplx) rowowner_t<cpx<double>, true>(a, s);
    else rowowner_t<double, true>(a, s);
  } else if (a.compensated) {
    if (cplx) rowowner_t<cpx<float>, true>(a, s);
    else rowowner_t<float, true>(a, s);
  } else {
    if (cplx) rowowner_t<cpx<float>, false>(a, s);
    else rowowner_t<float, false>(a, s);
  }
}

int mv_smem_bytes() {
  static_assert(16 * MV_NSTAGE + 16 <= 128 && sizeof(MVStageHdr) == 32 && sizeof(MVTItem) == 80,
                "matvec header area");
  return MV_HDR + MV_NSTAGE * (MV_STAGE + MV_MAXPC * (int)sizeof(MVPiece) + MV_INAREA) +
         MV_NSTAGE * (int)sizeof(MVPend) + 16;
}
int mv_in_bytes() { return MV_INAREA; }
int mv_max_pieces() { return MV_MAXPC; }

template <class VS, bool COMP>
static void pass_t(const MVArgs2& a, int grid, cudaStream_t s) {
  if (a.nitems <= 0) return;
  if (a.nrhs == 1) {
    const int smem = mv_smem_bytes();
    if (smem_optin<mv_tma_kernel<VS, COMP>>(smem) != cudaSuccess) return;  // left for cudaGetLastError
    mv_tma_kernel<VS, COMP><<<std::min(grid, a.nitems), MV_THREADS, smem, s>>>(a);
  } else if (a.chunked) {
    mv_multi_chunk_kernel<VS, COMP><<<a.nitems, 256, 0, s>>>(a);
  } else {
    mv_multi_kernel<VS, COMP><<<a.nitems, 256, 0, s>>>(a);
  }
}

void launch_mv_pass(int prec, bool cplx, const MVArgs2& a, int grid, cudaStream_t s) {
  if (prec == 0) {
    if (cplx) pass_t<cpx<double>, true>(a, grid, s);
    else pass_t<double, true>(a, grid, s);
  } else if (a.compensated) {
    if (cplx) pass_t<cpx<float>, true>(a, grid, s);
    else pass_t<float, true>(a, grid, s);
  } else {
    if (cplx) pass_t<cpx<float>, false>(a, grid, s);
    else pass_t<float, false>(a, grid, s);
  }
}

int mv_stage_bytes() { return MV_STAGE; }
int mv_piece_elems() { return MV_PIECE; }

template <class VS, bool COMP>
static cudaError_t fused_t(const MVFusedArgs& f, cudaStream_t s) {
  const int smem = mv_smem_bytes();
  cudaError_t e = smem_optin<mv_fused_kernel<VS, COMP>>(smem);
  if (e != cudaSuccess) return e;
  // SM count and residency, queried once per device (host time on every matvec otherwise)
  static std::atomic<int> cache_nsm[64], cache_nb[64];
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int nsm = dev >= 0 && dev < 64 ? cache_nsm[dev].load() : 0;
  int nb = dev >= 0 && dev < 64 ? cache_nb[dev].load() : 0;
  if (nsm <= 0 || nb <= 0) {
    e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mv_fused_kernel<VS, COMP>, MV_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) {
      cache_nsm[dev].store(nsm);
      cache_nb[dev].store(nb);
    }
  }
  if (nb < 1) return cudaErrorCooperativeLaunchTooLarge;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nsm);  // one CTA per SM, all resident: the grid barriers rely on it
  cfg.blockDim = dim3(MV_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, mv_fused_kernel<VS, COMP>, f);
}

bool mv_fused_supported() {
  int dev = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return false;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return optin >= mv_smem_bytes();
}

cudaError_t launch_mv_fused(int prec, bool cplx, const MVFusedArgs& f, cudaStream_t s) {
  if (prec == 0) return cplx ? fused_t<cpx<double>, true>(f, s) : fused_t<double, true>(f, s);
  if (f.a.compensated) return cplx ? fused_t<cpx<float>, true>(f, s) : fused_t<float, true>(f, s);
  return cplx ? fused_t<cpx<float>, false>(f, s) : fused_t<float, false>(f, s);
}

template <class VS>
__global__ void permute_in_kernel(const int* perm, int n, int nrhs, int ld, const void* xv, void* xpv) {
  using D = typename MT<VS>::D;
  using X = typename MT<VS>::X;
  const D* x = (const D*)xv;
  X* xp = (X*)xpv;
  const long long total = (long long)n * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / nrhs), r = (int)(t - (long long)k * nrhs);
    xp[t] = to_x<VS>(x[(size_t)r * ld + perm[k]]);
  }
}

template <class VS>
__global__ void t_to_x_kernel(const void* tv, void* txv, long long n) {
  using D = typename MT<VS>::D;
  using X = typename MT<VS>::X;
  const D* t = (const D*)tv;
  X* tx = (X*)txv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    tx[i] = to_x<VS>(t[i]);
}

static int grid_for(long long total) {
  long long g = (total + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

void launch_permute_in(int prec, bool cplx, const int* perm, int n, int nrhs, int ld, const void* x, void* xp,
                       cudaStream_t s) {
  int g = grid_for((long long)n * nrhs);
  if (prec == 0) {
    if (cplx) permute_in_kernel<cpx<double>><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, xp);
    else permute_in_kernel<double><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, xp);
  } else {
    if (cplx) permute_in_kernel<cpx<float>><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, xp);
    else permute_in_kernel<float><<<g, 256, 0, s>>>(perm, n, nrhs, ld, x, xp);
  }
}

void launch_permute_out(bool cplx, const int* perm, int n, int nrhs, int ld, const double* alpha, const double* beta,
                        const void* yp, void* y, cudaStream_t s) {
  int g = grid_for((long long)n * nrhs);
  int use_beta = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
  if (cplx)
    permute_out_kernel<cpx<double>><<<g, 256, 0, s>>>(perm, n, nrhs, ld, mkc(alpha[0], alpha[1]), mkc(beta[0], beta[1]),
                                                      use_beta, (const cpx<double>*)yp, (cpx<double>*)y);
  else
    permute_out_kernel<double><<<g, 256, 0, s>>>(perm, n, nrhs, ld, alpha[0], beta[0], use_beta, (const double*)yp,
                                                 (double*)y);
}

template <class D>
__global__ void scale_rows_kernel(const int* rows, int nrows, int nrhs, int ld, D beta, int zero, D* y) {
  const long long total = (long long)nrows * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nrows), r = (int)(t / nrows);
    D* dst = y + (size_t)r * ld + rows[i];
    *dst = zero ? vzero<D>() : beta * (*dst);
  }
}

void launch_scale_rows(bool cplx, const int* rows, int nrows, int nrhs, int ld, const double* beta, void* y,
                       cudaStream_t s) {
  if (nrows <= 0) return;
  const int g = grid_for((long long)nrows * nrhs);
  const int zero = (beta[0] == 0.0 && beta[1] == 0.0) ? 1 : 0;
  if (cplx)
    scale_rows_kernel<cpx<double>><<<g, 256, 0, s>>>(rows, nrows, nrhs, ld, mkc(beta[0], beta[1]), zero,
                                                     (cpx<double>*)y);
  else
    scale_rows_kernel<double><<<g, 256, 0, s>>>(rows, nrows, nrhs, ld, beta[0], zero, (double*)y);
}

// ---------------------------------------------------------------------------------------
// CSR SpMV (mass matrices).  trans: y = alpha A^T x + beta y via atomics into y after scaling.
template <class VD>
__global__ void spmv_kernel(int nrows, const int* rowptr, const int* col, const double* val, VD alpha, VD beta,
                            int use_beta, const VD* x, VD* y, int nrhs, int ldx, int ldy) {
  const long long total = (long long)nrows * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nrows), r = (int)(t / nrows);
    VD s = vzero<VD>();
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += x[(size_t)r * ldx + col[k]] * val[k];
    VD* dst = y + (size_t)r * ldy + i;
    VD v = alpha * s;
    if (use_beta) v += beta * (*dst);
    *dst = v;
  }
}
template <class VD>
__global__ void scale_kernel(VD* y, long long n, VD beta, int zero) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    y[t] = zero ? vzero<VD>() : beta * y[t];
}
template <class VD>
__global__ void spmv_t_kernel(int nrows, const int* rowptr, const int* col, const double* val, VD alpha, const VD* x,
                              VD* y, int nrhs, int ldx, int ldy) {
  const long long total = (long long)nrows * nrhs;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nrows), r = (int)(t / nrows);
    const VD xi = alpha * x[(size_t)r * ldx + i];
    for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) atomic_add(&y[(size_t)r * ldy + col[k]], xi * val[k]);
  }
}

void launch_spmv(bool cplx, bool trans, int nrows, int ncols, const int* rowptr, const int* col, const double* val,
                 const double* alpha, const double* beta, const void* x, void* y, int nrhs, cudaStream_t s) {
  int use_beta = (beta[0] != 0.0 || beta[1] != 0.0) ? 1 : 0;
  if (!trans) {
    int g = grid_for((long long)nrows * nrhs);
    if (cplx)
      spmv_kernel<cpx<double>><<<g, 256, 0, s>>>(nrows, rowptr, col, val, mkc(alpha[0], alpha[1]), mkc(beta[0], beta[1]),
                                                 use_beta, (const cpx<double>*)x, (cpx<double>*)y, nrhs, ncols, nrows);
    else
      spmv_kernel<double><<<g, 256, 0, s>>>(nrows, rowptr, col, val, alpha[0], beta[0], use_beta, (const double*)x,
                                            (double*)y, nrhs, ncols, nrows);
  } else {
    long long ny = (long long)ncols * nrhs;
    int g1 = grid_for(ny), g2 = grid_for((long long)nrows * nrhs);
    if (cplx) {
      scale_kernel<cpx<double>><<<g1, 256, 0, s>>>((cpx<double>*)y, ny, mkc(beta[0], beta[1]), use_beta ? 0 : 1);
      spmv_t_kernel<cpx<double>><<<g2, 256, 0, s>>>(nrows, rowptr, col, val, mkc(alpha[0], alpha[1]),
                                                    (const cpx<double>*)x, (cpx<double>*)y, nrhs, nrows, ncols);
    } else {
      scale_kernel<double><<<g1, 256, 0, s>>>((double*)y, ny, beta[0], use_beta ? 0 : 1);
      spmv_t_kernel<double><<<g2, 256, 0, s>>>(nrows, rowptr, col, val, alpha[0], (const double*)x, (double*)y, nrhs,
                                               nrows, ncols);
    }
  }
}

// ---------------------------------------------------------------------------------------
// GMRES helpers (fp64 / complex128): h = Q^H w, w -= Q h, ||w||, q = w / ||w||, x += Q y
template <class VD>
__global__ void __launch_bounds__(256) gemv_ct_kernel(int n, const VD* Q, const VD* w, VD* h) {
  __shared__ VD sb[8];
  const int c = blockIdx.x;
  const VD* q = Q + (size_t)c * n;
  VD s = vzero<VD>();
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += conjv(q[i]) * w[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    VD t = sb[0];
    for (int k = 1; k < 8; ++k) t += sb[k];
    h[c] = t;
  }
}
template <class VD>
__global__ void gemv_sub_kernel(int n, int k, const VD* Q, const VD* h, VD* w, int sign) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    VD s = vzero<VD>();
    for (int c = 0; c < k; ++c) s += Q[(size_t)c * n + i] * h[c];
    if (sign < 0) w[i] -= s;
    else w[i] += s;
  }
}
template <class VD>
__global__ void __launch_bounds__(256) nrm2_kernel(int n, const VD* w, double* out) {
  __shared__ double sb[8];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += norm2v(w[i]);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < 8; ++k) t += sb[k];
    *out = sqrt(t);
  }
}
template <class VD>
__global__ void scale_copy_kernel(int n, const VD* w, double inv, VD* q) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) q[i] = w[i] * inv;
}
template <class VD>
__global__ void residual_kernel(int n, const VD* b, VD* r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r[i] = b[i] - r[i];
}

void launch_gemv_ct(bool cplx, int n, int k, const void* Q, const void* w, void* h, cudaStream_t s) {
  if (k <= 0) return;
  if (cplx) gemv_ct_kernel<cpx<double>><<<k, 256, 0, s>>>(n, (const cpx<double>*)Q, (const cpx<double>*)w, (cpx<double>*)h);
  else gemv_ct_kernel<double><<<k, 256, 0, s>>>(n, (const double*)Q, (const double*)w, (double*)h);
}
void launch_gemv_sub(bool cplx, int n, int k, const void* Q, const void* h, void* w, cudaStream_t s) {
  if (k <= 0) return;
  int g = grid_for(n);
  if (cplx) gemv_sub_kernel<cpx<double>><<<g, 256, 0, s>>>(n, k, (const cpx<double>*)Q, (const cpx<double>*)h, (cpx<double>*)w, -1);
  else gemv_sub_kernel<double><<<g, 256, 0, s>>>(n, k, (const double*)Q, (const double*)h, (double*)w, -1);
}
void launch_axpy_basis(bool cplx, int n, int k, const void* Q, const void* y, void* x, cudaStream_t s) {
  if (k <= 0) return;
  int g = grid_for(n);
  if (cplx) gemv_sub_kernel<cpx<double>><<<g, 256, 0, s>>>(n, k, (const cpx<double>*)Q, (const cpx<double>*)y, (cpx<double>*)x, 1);
  else gemv_sub_kernel<double><<<g, 256, 0, s>>>(n, k, (const double*)Q, (const double*)y, (double*)x, 1);
}
void launch_nrm2(bool cplx, int n, const void* w, double* out, cudaStream_t s) {
  if (cplx) nrm2_kernel<cpx<double>><<<1, 256, 0, s>>>(n, (const cpx<double>*)w, out);
  else nrm2_kernel<double><<<1, 256, 0, s>>>(n, (const double*)w, out);
}
void launch_scale_copy(bool cplx, int n, const void* w, double inv, void* q, cudaStream_t s) {
  int g = grid_for(n);
  if (cplx) scale_copy_kernel<cpx<double>><<<g, 256, 0, s>>>(n, (const cpx<double>*)w, inv, (cpx<double>*)q);
  else scale_copy_kernel<double><<<g, 256, 0, s>>>(n, (const double*)w, inv, (double*)q);
}
void launch_residual(bool cplx, int n, const void* b, void* r, cudaStream_t s) {
  int g = grid_for(n);
  if (cplx) residual_kernel<cpx<double>><<<g, 256, 0, s>>>(n, (const cpx<double>*)b, (cpx<double>*)r);
  else residual_kernel<double><<<g, 256, 0, s>>>(n, (const double*)b, (double*)r);
}

void launch_t_to_x(int prec, bool cplx, const void* t, void* tx, long long n, cudaStream_t s) {
  if (n <= 0 || prec == 0) return;  // fp64 storage: t is already the input form
  const int g = grid_for(n);
  if (cplx) t_to_x_kernel<cpx<float>><<<g, 256, 0, s>>>(t, tx, n);
  else t_to_x_kernel<float><<<g, 256, 0, s>>>(t, tx, n);
}

}  // namespace bem
