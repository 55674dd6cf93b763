// Device-side building blocks: complex arithmetic, Green's functions with their term
// tables, trace evaluators and warp/block reductions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "bem_shared.h"

namespace bem {

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per kernel and device.  The opt-in is
// a per-device property of the function, so a process that launches FN on several devices
// sets it on each (devices 0..63 are remembered; others set it on every call).
template <auto FN>
cudaError_t smem_optin(int smem) {
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const bool track = dev >= 0 && dev < 64;
  if (track && ((done.load(std::memory_order_acquire) >> dev) & 1ull)) return cudaSuccess;
  e = cudaFuncSetAttribute(FN, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess && track) done.fetch_or(1ull << dev, std::memory_order_acq_rel);
  return e;
}

// ----------------------------------------------------------------------------------------
// complex numbers
// ----------------------------------------------------------------------------------------
template <class R>
struct cpx {
  R x, y;
};
template <class R> __host__ __device__ __forceinline__ cpx<R> mkc(R a, R b) { return cpx<R>{a, b}; }
template <class R> __host__ __device__ __forceinline__ cpx<R> operator+(cpx<R> a, cpx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <class R> __host__ __device__ __forceinline__ cpx<R> operator-(cpx<R> a, cpx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <class R> __host__ __device__ __forceinline__ cpx<R> operator*(cpx<R> a, cpx<R> b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
template <class R> __host__ __device__ __forceinline__ cpx<R> operator*(R s, cpx<R> a) { return {s * a.x, s * a.y}; }
template <class R> __host__ __device__ __forceinline__ cpx<R> operator*(cpx<R> a, R s) { return {s * a.x, s * a.y}; }
template <class R> __host__ __device__ __forceinline__ cpx<R>& operator+=(cpx<R>& a, cpx<R> b) { a.x += b.x; a.y += b.y; return a; }
template <class R> __host__ __device__ __forceinline__ cpx<R>& operator-=(cpx<R>& a, cpx<R> b) { a.x -= b.x; a.y -= b.y; return a; }
template <class R> __host__ __device__ __forceinline__ cpx<R>& operator*=(cpx<R>& a, cpx<R> b) { a = a * b; return a; }
template <class R> __host__ __device__ __forceinline__ cpx<R>& operator*=(cpx<R>& a, R s) { a.x *= s; a.y *= s; return a; }

template <class V> struct scal;
template <> struct scal<float> { using R = float; static constexpr bool cplx = false; };
template <> struct scal<double> { using R = double; static constexpr bool cplx = false; };
template <> struct scal<cpx<float>> { using R = float; static constexpr bool cplx = true; };
template <> struct scal<cpx<double>> { using R = double; static constexpr bool cplx = true; };

template <bool C, class R> struct VT_ { using type = R; };
template <class R> struct VT_<true, R> { using type = cpx<R>; };
template <bool C, class R> using VT = typename VT_<C, R>::type;

__device__ __forceinline__ float zero_of(float) { return 0.f; }
__device__ __forceinline__ double zero_of(double) { return 0.0; }
template <class R> __device__ __forceinline__ cpx<R> zero_of(cpx<R>) { return {R(0), R(0)}; }
template <class V> __device__ __forceinline__ V vzero() { return zero_of(V()); }

__device__ __forceinline__ float conjv(float a) { return a; }
__device__ __forceinline__ double conjv(double a) { return a; }
template <class R> __device__ __forceinline__ cpx<R> conjv(cpx<R> a) { return {a.x, -a.y}; }
__device__ __forceinline__ float absv(float a) { return fabsf(a); }
__device__ __forceinline__ double absv(double a) { return fabs(a); }
__device__ __forceinline__ float absv(cpx<float> a) { return sqrtf(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ double absv(cpx<double> a) { return sqrt(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ float norm2v(float a) { return a * a; }
__device__ __forceinline__ double norm2v(double a) { return a * a; }
template <class R> __device__ __forceinline__ R norm2v(cpx<R> a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ float realv(float a) { return a; }
__device__ __forceinline__ double realv(double a) { return a; }
template <class R> __device__ __forceinline__ R realv(cpx<R> a) { return a.x; }
// 1/a for real or complex a
__device__ __forceinline__ float invv(float a) { return 1.f / a; }
__device__ __forceinline__ double invv(double a) { return 1.0 / a; }
template <class R> __device__ __forceinline__ cpx<R> invv(cpx<R> a) { R d = a.x * a.x + a.y * a.y; return {a.x / d, -a.y / d}; }

// conversions between storage and accumulation types
__device__ __forceinline__ void cvt(float& d, double s) { d = (float)s; }
__device__ __forceinline__ void cvt(double& d, double s) { d = s; }
__device__ __forceinline__ void cvt(double& d, float s) { d = (double)s; }
__device__ __forceinline__ void cvt(float& d, float s) { d = s; }
template <class A, class B> __device__ __forceinline__ void cvt(cpx<A>& d, cpx<B> s) { cvt(d.x, s.x); cvt(d.y, s.y); }
template <class A> __device__ __forceinline__ void cvt(cpx<A>& d, double s) { cvt(d.x, s); d.y = A(0); }
template <class A> __device__ __forceinline__ void cvt(cpx<A>& d, float s) { cvt(d.x, s); d.y = A(0); }

__device__ __forceinline__ void atomic_add(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add(double* p, double v) { atomicAdd(p, v); }
template <class R> __device__ __forceinline__ void atomic_add(cpx<R>* p, cpx<R> v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

__device__ __forceinline__ float rsqrt_(float a) { return rsqrtf(a); }
__device__ __forceinline__ double rsqrt_(double a) { return 1.0 / sqrt(a); }
__device__ __forceinline__ void sincos_(float a, float* s, float* c) { sincosf(a, s, c); }
__device__ __forceinline__ void sincos_(double a, double* s, double* c) { sincos(a, s, c); }
__device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
__device__ __forceinline__ double sqrt_(double a) { return sqrt(a); }

// ----------------------------------------------------------------------------------------
// Green's functions (reference src/ngbem.hpp:226-468).  eval() takes d = x - y, the normals
// and kappa and returns the NC kernel components.  Term tables (fac, kernel comp, trial comp,
// test comp): fac kind 0 = 1, 1 = kappa, 2 = -1/kappa.
// ----------------------------------------------------------------------------------------
#define BEM_INV4PI 0.079577471545947667884441881686257181

template <int KID> struct Green;

template <> struct Green<K_LAPLACE_SL> {
  static constexpr bool CPLX = false; static constexpr int NC = 1; static constexpr int NT = 1;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = false;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int) { return 0; }
  __host__ __device__ static constexpr int tec(int) { return 0; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R*, R, R* out) {
    R ir = rsqrt_(dx * dx + dy * dy + dz * dz);
    out[0] = ir * R(BEM_INV4PI);
  }
};

template <> struct Green<K_LAPLACE_DL> {
  static constexpr bool CPLX = false; static constexpr int NC = 1; static constexpr int NT = 1;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = true;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int) { return 0; }
  __host__ __device__ static constexpr int tec(int) { return 0; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R* ny, R, R* out) {
    R ir = rsqrt_(dx * dx + dy * dy + dz * dz);
    R nxy = ny[0] * dx + ny[1] * dy + ny[2] * dz;
    out[0] = nxy * (ir * ir * ir) * R(BEM_INV4PI);
  }
};

template <> struct Green<K_LAPLACE_HS> {
  static constexpr bool CPLX = false; static constexpr int NC = 1; static constexpr int NT = 3;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = false;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int t) { return t; }
  __host__ __device__ static constexpr int tec(int t) { return t; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R*, R, R* out) {
    R ir = rsqrt_(dx * dx + dy * dy + dz * dz);
    out[0] = ir * R(BEM_INV4PI);
  }
};

template <> struct Green<K_HELMHOLTZ_SL> {
  static constexpr bool CPLX = true; static constexpr int NC = 1; static constexpr int NT = 1;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = false;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int) { return 0; }
  __host__ __device__ static constexpr int tec(int) { return 0; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R*, R kappa, cpx<R>* out) {
    R r2 = dx * dx + dy * dy + dz * dz;
    R ir = rsqrt_(r2);
    R s, c;
    sincos_(kappa * (r2 * ir), &s, &c);
    R f = ir * R(BEM_INV4PI);
    out[0] = mkc(c * f, s * f);
  }
};

// d/dkappa of the Helmholtz single-layer kernel: d/dk e^{ikr}/(4 pi r) = i e^{ikr}/(4 pi), a
// bounded kernel (the derivative of the bilinear form with respect to the wavenumber)
template <> struct Green<K_HELMHOLTZ_SL_DKAPPA> {
  static constexpr bool CPLX = true; static constexpr int NC = 1; static constexpr int NT = 1;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = false;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int) { return 0; }
  __host__ __device__ static constexpr int tec(int) { return 0; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R*, R kappa, cpx<R>* out) {
    R r2 = dx * dx + dy * dy + dz * dz;
    R s, c;
    sincos_(kappa * sqrt_(r2), &s, &c);
    out[0] = mkc(-s * R(BEM_INV4PI), c * R(BEM_INV4PI));
  }
};

template <> struct Green<K_MAXWELL_SL> {
  static constexpr bool CPLX = true; static constexpr int NC = 1; static constexpr int NT = 4;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = false;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int t) { return t; }
  __host__ __device__ static constexpr int tec(int t) { return t; }
  __host__ __device__ static constexpr int fk(int t) { return t < 3 ? 1 : 2; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R* nx, const R* ny, R kappa, cpx<R>* out) {
    Green<K_HELMHOLTZ_SL>::eval(dx, dy, dz, nx, ny, kappa, out);
  }
};

template <> struct Green<K_HELMHOLTZ_DL> {
  static constexpr bool CPLX = true; static constexpr int NC = 1; static constexpr int NT = 1;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = true;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int) { return 0; }
  __host__ __device__ static constexpr int tec(int) { return 0; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R* ny, R kappa, cpx<R>* out) {
    R r2 = dx * dx + dy * dy + dz * dz;
    R ir = rsqrt_(r2);
    R r = r2 * ir;
    R s, c;
    sincos_(kappa * r, &s, &c);
    R nxy = ny[0] * dx + ny[1] * dy + ny[2] * dz;
    R f = nxy * (ir * ir * ir) * R(BEM_INV4PI);
    // e^{ikr} * f * (1 - i kappa r)
    cpx<R> e = mkc(c * f, s * f);
    out[0] = e * mkc(R(1), -kappa * r);
  }
};

template <> struct Green<K_HELMHOLTZ_CF> {
  static constexpr bool CPLX = true; static constexpr int NC = 1; static constexpr int NT = 1;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = true;
  __host__ __device__ static constexpr int kc(int) { return 0; }
  __host__ __device__ static constexpr int trc(int) { return 0; }
  __host__ __device__ static constexpr int tec(int) { return 0; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R* ny, R kappa, cpx<R>* out) {
    R r2 = dx * dx + dy * dy + dz * dz;
    R ir = rsqrt_(r2);
    R r = r2 * ir;
    R s, c;
    sincos_(kappa * r, &s, &c);
    R nxy = ny[0] * dx + ny[1] * dy + ny[2] * dz;
    R f = (ir * ir * ir) * R(BEM_INV4PI);
    // e^{ikr}/(4 pi r^3) * (nxy (1 - i kappa r) - i kappa r^2)
    cpx<R> e = mkc(c * f, s * f);
    out[0] = e * mkc(nxy, -kappa * r * nxy - kappa * r2);
  }
};

template <> struct Green<K_HELMHOLTZ_HS> {
  static constexpr bool CPLX = true; static constexpr int NC = 2; static constexpr int NT = 4;
  static constexpr bool NEEDS_NX = true, NEEDS_NY = true;
  __host__ __device__ static constexpr int kc(int t) { return t < 3 ? 0 : 1; }
  __host__ __device__ static constexpr int trc(int t) { return t; }
  __host__ __device__ static constexpr int tec(int t) { return t; }
  __host__ __device__ static constexpr int fk(int) { return 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R* nx, const R* ny, R kappa, cpx<R>* out) {
    R r2 = dx * dx + dy * dy + dz * dz;
    R ir = rsqrt_(r2);
    R s, c;
    sincos_(kappa * (r2 * ir), &s, &c);
    R f = ir * R(BEM_INV4PI);
    cpx<R> kern = mkc(c * f, s * f);
    R nxny = nx[0] * ny[0] + nx[1] * ny[1] + nx[2] * ny[2];
    out[0] = kern;
    out[1] = kern * (-kappa * kappa * nxny);
  }
};

// Maxwell double layer (reference MaxwellDLKernel<3>, src/ngbem.hpp:475-510): the gradient
// e^{ikr}/(4 pi r^3) (i k r - 1)(x - y) in three components, applied as the cross product
// test . (grad x trial) through six terms of factor +-1
template <> struct Green<K_MAXWELL_DL> {
  static constexpr bool CPLX = true; static constexpr int NC = 3; static constexpr int NT = 6;
  static constexpr bool NEEDS_NX = false, NEEDS_NY = false;
  __host__ __device__ static constexpr int kc(int t) { return t >> 1; }
  __host__ __device__ static constexpr int trc(int t) { return t == 0 ? 1 : (t == 1 ? 2 : (t == 2 ? 2 : (t == 3 ? 0 : (t == 4 ? 0 : 1)))); }
  __host__ __device__ static constexpr int tec(int t) { return t == 0 ? 2 : (t == 1 ? 1 : (t == 2 ? 0 : (t == 3 ? 2 : (t == 4 ? 1 : 0)))); }
  __host__ __device__ static constexpr int fk(int t) { return (t & 1) ? 3 : 0; }
  template <class R>
  __device__ static __forceinline__ void eval(R dx, R dy, R dz, const R*, const R*, R kappa, cpx<R>* out) {
    R r2 = dx * dx + dy * dy + dz * dz;
    R ir = rsqrt_(r2);
    R r = r2 * ir;
    R s, c;
    sincos_(kappa * r, &s, &c);
    R f = (ir * ir * ir) * R(BEM_INV4PI);
    const cpx<R> g = mkc(c * f, s * f) * mkc(R(-1), kappa * r);
    out[0] = g * dx;
    out[1] = g * dy;
    out[2] = g * dz;
  }
};

template <class G, class R>
__device__ __forceinline__ R term_fac(int t, R kappa) {
  int k = G::fk(t);
  return k == 0 ? R(1) : (k == 1 ? kappa : (k == 3 ? R(-1) : R(-1) / kappa));
}

// ----------------------------------------------------------------------------------------
// Trace evaluators.  ND local dofs, DIM components.  Values at a point with reference
// coordinates (xi, eta) and physical offsets xp[k][c] = x - p_k (vertex k):
//   P0   : 1 (or 1/|J| with dual mapping)
//   P1   : lambda_a = (xi, eta, 1 - xi - eta)
//   ROT  : n x grad lambda_a                       (DiffOpBoundaryRot)
//   HELM : [n x grad lambda_a ; lambda_a]          (DiffOpHelmholtz)
//   MAX  : [sigma_a (x - p_opp(a)) / |J| ; 2 sigma_a / |J|]  (DiffOpMaxwellNew, RT0)
//   RT0ID: sigma_a (x - p_opp(a)) / |J|           (HDivSurface identity trace)
// Local RT0 edge a joins vertices (a, a+1 mod 3); its opposite vertex is (a+2) mod 3.
// ----------------------------------------------------------------------------------------
// the primary template serves HDivSurface / HCurl of order 1..4 (hdiv_trace)
template <int TR> struct TraceInfo {
  static_assert(hdiv_trace(TR), "trace kind without a TraceInfo");
  static constexpr int ND = (hdiv_order(TR) + 1) * (hdiv_order(TR) + 2);
  static constexpr int DIM = (bdm_variant(TR) == 1 || bdm_variant(TR) == 4) ? 4 : 3;
};
template <> struct TraceInfo<TR_P0> { static constexpr int ND = 1, DIM = 1; };
template <> struct TraceInfo<TR_P1> { static constexpr int ND = 3, DIM = 1; };
template <> struct TraceInfo<TR_ROT> { static constexpr int ND = 3, DIM = 3; };
template <> struct TraceInfo<TR_HELM> { static constexpr int ND = 3, DIM = 4; };
template <> struct TraceInfo<TR_MAX> { static constexpr int ND = 3, DIM = 4; };
template <> struct TraceInfo<TR_RT0ID> { static constexpr int ND = 3, DIM = 3; };
template <> struct TraceInfo<TR_NED> { static constexpr int ND = 3, DIM = 3; };
template <> struct TraceInfo<TR_NEDROT> { static constexpr int ND = 3, DIM = 3; };
template <> struct TraceInfo<TR_NEDMAX> { static constexpr int ND = 3, DIM = 4; };
template <> struct TraceInfo<TR_L2P1> { static constexpr int ND = 3, DIM = 1; };
template <> struct TraceInfo<TR_L2P2> { static constexpr int ND = 6, DIM = 1; };
template <> struct TraceInfo<TR_L2P3> { static constexpr int ND = 10, DIM = 1; };
template <> struct TraceInfo<TR_H1P2> { static constexpr int ND = 6, DIM = 1; };
template <> struct TraceInfo<TR_H1P3> { static constexpr int ND = 10, DIM = 1; };
template <> struct TraceInfo<TR_H1P2ROT> { static constexpr int ND = 6, DIM = 3; };
template <> struct TraceInfo<TR_H1P3ROT> { static constexpr int ND = 10, DIM = 3; };
template <> struct TraceInfo<TR_H1P2HELM> { static constexpr int ND = 6, DIM = 4; };
template <> struct TraceInfo<TR_H1P3HELM> { static constexpr int ND = 10, DIM = 4; };
// traces that read the element's n x grad(lambda_a) table
// the geometry of a curved element's rule point (PGeo): normal, rotated gradients, 1 / |J| and
// the Piola offsets
template <class P>
__device__ __forceinline__ void point_geo(const PGeo<P>& g, P n[3], P rot[3][3], P& inv, P xp[3][3]) {
  inv = g.invdetJ;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    n[c] = g.n[c];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      rot[a][c] = g.rot[a][c];
      xp[a][c] = g.xp[a][c];
    }
  }
}

// traces that read 1 / |J| (the dual P0 and the Piola-mapped edge shapes) and, for the edge
// shapes, the offsets x - p_o
__host__ __device__ constexpr bool piola_trace(int tr) { return tr == TR_P0 || edge_trace(tr); }

// the parts of a rule point's geometry that a kernel side reads: the normal (N), the rotated
// gradients (ROT), 1 / |J| and the Piola offsets (PIOLA)
template <class P, bool N, bool ROT, bool PIOLA>
__device__ __forceinline__ void pgeo_load(const PGeo<P>& g, P n[3], P rot[3][3], P& inv, P xp[3][3]) {
  if constexpr (N) {
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c] = g.n[c];
  }
  if constexpr (ROT) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) rot[a][c] = g.rot[a][c];
  }
  if constexpr (PIOLA) {
    inv = g.invdetJ;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) xp[a][c] = g.xp[a][c];
  }
}

__host__ __device__ constexpr bool needs_rot(int tr) { return tr == TR_ROT || tr == TR_HELM || h1p_rot(tr); }  // incl. HELM
// sign slots a kernel keeps per element (at least the three edge signs)
template <int TR> struct SignSlots { static constexpr int N = TraceInfo<TR>::ND > 3 ? TraceInfo<TR>::ND : 3; };

// the element's second dof record, read only by traces that need it (H1 of order >= 2)
template <int TR>
__device__ __forceinline__ int4 dof_aux(const int4* sign, int e) {
  if constexpr (h1p_trace(TR) || hdiv_trace(TR)) return sign[e];
  else return make_int4(0, 0, 0, 0);
}
// global dof of local dof a of an element (dn: the element's dof record; aux: dof_aux).  H1 of
// order p >= 2: dn = (the three vertex dofs, first face dof), aux = per local edge its
// orientation sign times (first edge dof + 1)
// HDivSurface of order K: dn = (the three lowest-order edge dofs, first interior dof), aux = per
// local edge its orientation sign times (first higher-order dof of the edge + 1)
template <int TR>
__device__ __forceinline__ int elem_dof(const int4& dn, const int4& aux, int a) {
  if (l2p_trace(TR)) return dn.x + a;
  if constexpr (hdiv_trace(TR)) {
    constexpr int K = hdiv_order(TR);
    if (a >= 3 * (K + 1)) return dn.w + (a - 3 * (K + 1));
    const int k = a / (K + 1), m = a % (K + 1);
    if (m == 0) return k == 0 ? dn.x : (k == 1 ? dn.y : dn.z);
    const int g = k == 0 ? aux.x : (k == 1 ? aux.y : aux.z);
    return (g < 0 ? -g : g) - 1 + (m - 1);
  }
  if constexpr (h1p_trace(TR)) {
    constexpr int P = h1p_order(TR);
    if (a >= 3 && a < 3 + 3 * (P - 1)) {
      const int k = (a - 3) / (P - 1), m = (a - 3) % (P - 1);
      const int g = k == 0 ? aux.x : (k == 1 ? aux.y : aux.z);
      return (g < 0 ? -g : g) - 1 + m;
    }
    if (a >= 3) return dn.w + (a - 3 - 3 * (P - 1));
  }
  return a == 0 ? dn.x : (a == 1 ? dn.y : dn.z);
}
// per-local-dof sign argument of trace_val: edge orientations, or the vertex order code of an
// L2 element of order >= 1 (the same for all its dofs), else 1
template <int TR, int N>
__device__ __forceinline__ void elem_signs(const int4* sign, int e, int (&sg)[N]) {
#pragma unroll
  for (int k = 0; k < N; ++k) sg[k] = 1;
  if constexpr (hdiv_trace(TR)) {
    // every dof of local edge k: the edge's orientation; interior dofs: 1
    constexpr int K = hdiv_order(TR);
    const int4 g = sign[e];
#pragma unroll
    for (int a = 0; a < 3 * (K + 1) && a < N; ++a) {
      const int k = a / (K + 1);
      sg[a] = (k == 0 ? g.x : (k == 1 ? g.y : g.z)) < 0 ? -1 : 1;
    }
    return;
  }
  if (edge_trace(TR)) {
    const int4 g = sign[e];
    sg[0] = g.x;
    sg[1] = g.y;
    sg[2] = g.z;
  }
  if (l2p_trace(TR)) {
    const int4 g = sign[e];
    const int code = g.x + 3 * g.y;
#pragma unroll
    for (int k = 0; k < N; ++k) sg[k] = code;
  }
  if constexpr (h1p_trace(TR)) {
    // edge dof of degree m + 2: the edge's orientation sign to the power m
    constexpr int P = h1p_order(TR);
    const int4 g = sign[e];
#pragma unroll
    for (int a = 3; a < 3 + 3 * (P - 1) && a < N; ++a) {
      const int k = (a - 3) / (P - 1), m = (a - 3) % (P - 1);
      const int o = (k == 0 ? g.x : (k == 1 ? g.y : g.z)) < 0 ? -1 : 1;
      sg[a] = (m & 1) ? o : 1;
    }
  }
}

// value of trace component c of local dof a (nrm: the element's unit normal, read by TR_NED)
template <int TR, class R>
__device__ __forceinline__ R trace_val(int a, int c, R xi, R eta, const R (*xp)[3], R invdetJ,
                                       const R (*rot)[3], int sgn, bool dual, const R* nrm) {
  if (TR == TR_P0) return dual ? invdetJ : R(1);
  if (TR == TR_P1) return a == 0 ? xi : (a == 1 ? eta : R(1) - xi - eta);
  if (l2p_trace(TR)) return dubiner<R>(l2p_order(TR), a, xi, eta, sgn);
  if constexpr (h1p_trace(TR)) {
    const R l[3] = {xi, eta, R(1) - xi - eta};
    R d[3];
    const R v = h1p_shape<R>(h1p_order(TR), a, l, d);
    if (!h1p_rot(TR) || c == 3) return R(sgn) * v;
    return R(sgn) * (d[0] * rot[0][c] + d[1] * rot[1][c] + d[2] * rot[2][c]);
  }
  if (TR == TR_ROT) return rot[a][c];
  if (TR == TR_HELM) {
    if (c < 3) return rot[a][c];
    return a == 0 ? xi : (a == 1 ? eta : R(1) - xi - eta);
  }
  if constexpr (hdiv_trace(TR)) {
    // HDivSurface of order K: the Piola map of the reference field, J = (xp_2 - xp_0, xp_2 - xp_1);
    // HCurl of order K: n x it (ID), its negative (ROT, MAX), the divergence as the curl (MAX)
    R vx, vy;
    const R dv = hdiv_shape<R>(hdiv_order(TR), a, xi, eta, sgn, vx, vy);
    if (c == 3) return dv * invdetJ;
    if constexpr (normal_trace(TR)) {
      const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
      const R p1 = ((xp[2][c2] - xp[0][c2]) * vx + (xp[2][c2] - xp[1][c2]) * vy) * invdetJ;
      const R p2 = ((xp[2][c1] - xp[0][c1]) * vx + (xp[2][c1] - xp[1][c1]) * vy) * invdetJ;
      return nrm[c1] * p1 - nrm[c2] * p2;
    }
    const R v = ((xp[2][c] - xp[0][c]) * vx + (xp[2][c] - xp[1][c]) * vy) * invdetJ;
    return hcurl_hi_trace(TR) ? -v : v;
  }
  // edge dofs: the RT0 shape sgn (x - p_o) / |J| (o the vertex opposite the edge)
  const int o = (a + 2) % 3;
  if (TR == TR_NED) {  // n x RT0 shape
    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    return R(sgn) * (nrm[c1] * xp[o][c2] - nrm[c2] * xp[o][c1]) * invdetJ;
  }
  if (c < 3) {
    const R v = R(sgn) * xp[o][c] * invdetJ;
    return (TR == TR_NEDROT || TR == TR_NEDMAX) ? -v : v;
  }
  return R(2 * sgn) * invdetJ;  // surface divergence (RT0) = surface curl (Nedelec)
}

// ----------------------------------------------------------------------------------------
// reductions
// ----------------------------------------------------------------------------------------
__device__ __forceinline__ float shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
template <class R> __device__ __forceinline__ cpx<R> shfl_xor(cpx<R> v, int m) { return {shfl_xor(v.x, m), shfl_xor(v.y, m)}; }

template <class V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v += shfl_xor(v, m);
  return v;
}

// argmax with lowest-index tie-break; idx < 0 means "none".
template <class R>
__device__ __forceinline__ void argmax_combine(R& v, int& i, R v2, int i2) {
  if (i2 >= 0 && (i < 0 || v2 > v || (v2 == v && i2 < i))) { v = v2; i = i2; }
}
template <class R>
__device__ __forceinline__ void warp_argmax(R& v, int& i) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    R v2 = shfl_xor(v, m);
    int i2 = __shfl_xor_sync(0xffffffffu, i, m);
    argmax_combine(v, i, v2, i2);
  }
}

}  // namespace bem
