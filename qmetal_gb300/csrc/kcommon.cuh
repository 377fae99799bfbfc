// kcommon.cuh -- shared device helpers for the statevector kernels.
//
// Layout: the state is 2^n complex64 amplitudes, interleaved, LSB-first.
// Most kernels address it as float4 "vectors": vector v holds amplitudes 2v
// (lanes x,y) and 2v+1 (lanes z,w), so amplitude bit 0 is the lane and
// amplitude bit b >= 1 is vector bit b-1. Every global access is then a
// 16-byte load or store, and a warp touches 512 contiguous bytes whenever
// the vector bits below 5 are free.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace qmk {

constexpr int kThreads = 256;

struct M2 {
  float2 a, b, c, d;  // [[a b] [c d]]
};

__host__ inline M2 m2_from(const float m[8]) {
  M2 r;
  r.a = make_float2(m[0], m[1]);
  r.b = make_float2(m[2], m[3]);
  r.c = make_float2(m[4], m[5]);
  r.d = make_float2(m[6], m[7]);
  return r;
}

__device__ __forceinline__ float2 cmul(float2 x, float2 y) {
  return make_float2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// m0 * u + m1 * v
__device__ __forceinline__ float2 cmac2(float2 m0, float2 u, float2 m1, float2 v) {
  return make_float2(m0.x * u.x - m0.y * u.y + m1.x * v.x - m1.y * v.y,
                     m0.x * u.y + m0.y * u.x + m1.x * v.y + m1.y * v.x);
}

__device__ __forceinline__ void apply2(const M2 &m, float2 &u, float2 &v) {
  const float2 nu = cmac2(m.a, u, m.b, v);
  const float2 nv = cmac2(m.c, u, m.d, v);
  u = nu;
  v = nv;
}

// Structure of a 2x2, found on the host: the specialised forms below drop
// products with exact zeros of the general form (RY-like real matrices,
// RX-like real diagonal with imaginary off-diagonal, diagonal matrices), so
// they halve the multiply-adds and round the same way.
enum : int8_t { kMatGeneral = 0, kMatReal = 1, kMatRx = 2, kMatDiag = 3 };

__host__ inline int8_t m2_class(const M2 &m) {
  if (m.b.x == 0.0f && m.b.y == 0.0f && m.c.x == 0.0f && m.c.y == 0.0f) return kMatDiag;
  if (m.a.y == 0.0f && m.b.y == 0.0f && m.c.y == 0.0f && m.d.y == 0.0f) return kMatReal;
  if (m.a.y == 0.0f && m.d.y == 0.0f && m.b.x == 0.0f && m.c.x == 0.0f) return kMatRx;
  return kMatGeneral;
}

// s * own + t * other, where s is the row's own coefficient and t the other
// one, for a matrix of class cls (t is imaginary for kMatRx, zero for kMatDiag).
__device__ __forceinline__ float2 cmac2c(int cls, float2 s, float2 own, float2 t, float2 other) {
  switch (cls) {
    case kMatReal:
      return make_float2(s.x * own.x + t.x * other.x, s.x * own.y + t.x * other.y);
    case kMatRx:
      return make_float2(s.x * own.x - t.y * other.y, s.x * own.y + t.y * other.x);
    case kMatDiag:
      return make_float2(s.x * own.x - s.y * own.y, s.x * own.y + s.y * own.x);
    default:
      return cmac2(s, own, t, other);
  }
}

__device__ __forceinline__ void apply2c(int cls, const M2 &m, float2 &u, float2 &v) {
  const float2 nu = cmac2c(cls, m.a, u, m.b, v);
  const float2 nv = cmac2c(cls, m.d, v, m.c, u);
  u = nu;
  v = nv;
}

__device__ __forceinline__ float2 lo2(const float4 &x) { return make_float2(x.x, x.y); }
__device__ __forceinline__ float2 hi2(const float4 &x) { return make_float2(x.z, x.w); }
__device__ __forceinline__ float4 pack4(float2 a, float2 b) {
  return make_float4(a.x, a.y, b.x, b.y);
}

// The two amplitudes of one vector held as (re0, re1) and (im0, im1): an op
// on any wire but 0 updates both amplitudes with the same coefficients, so
// each real multiply-add runs as one packed FP32x2 instruction (sm_100 and
// later) instead of two.
struct Cx2 {
  float2 re, im;
};
__device__ __forceinline__ Cx2 split2(const float4 &v) {
  return {make_float2(v.x, v.z), make_float2(v.y, v.w)};
}
__device__ __forceinline__ float4 join2(const Cx2 &c) {
  return make_float4(c.re.x, c.im.x, c.re.y, c.im.y);
}
__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }

// s * own + t * other for both amplitudes, s and t of a class-cls matrix
// (the packed counterpart of cmac2c), from their parts as broadcast pairs:
// sr = (s.x, s.x), si = (s.y, s.y), nsi = -si, and the same for t.
template <int CLS>
__device__ __forceinline__ Cx2 cmacx6(float2 sr, float2 si, float2 nsi, float2 tr, float2 ti,
                                      float2 nti, const Cx2 &own, const Cx2 &oth) {
  Cx2 r;
  if (CLS == kMatReal) {
    r.re = __ffma2_rn(tr, oth.re, __fmul2_rn(sr, own.re));
    r.im = __ffma2_rn(tr, oth.im, __fmul2_rn(sr, own.im));
  } else if (CLS == kMatRx) {
    r.re = __ffma2_rn(nti, oth.im, __fmul2_rn(sr, own.re));
    r.im = __ffma2_rn(ti, oth.re, __fmul2_rn(sr, own.im));
  } else if (CLS == kMatDiag) {
    r.re = __ffma2_rn(nsi, own.im, __fmul2_rn(sr, own.re));
    r.im = __ffma2_rn(si, own.re, __fmul2_rn(sr, own.im));
  } else {
    r.re = __ffma2_rn(nti, oth.im,
                      __ffma2_rn(tr, oth.re, __ffma2_rn(nsi, own.im, __fmul2_rn(sr, own.re))));
    r.im = __ffma2_rn(ti, oth.re,
                      __ffma2_rn(tr, oth.im, __ffma2_rn(si, own.re, __fmul2_rn(sr, own.im))));
  }
  return r;
}

template <int CLS>
__device__ __forceinline__ Cx2 cmacx(float2 s, const Cx2 &own, float2 t, const Cx2 &oth) {
  return cmacx6<CLS>(bc2(s.x), bc2(s.y), bc2(-s.y), bc2(t.x), bc2(t.y), bc2(-t.y), own, oth);
}

// A 2x2 with its parts pre-broadcast to pairs (imaginary parts also
// negated): the operands of the packed updates, built once on the host.
struct MX {
  float2 ar, ai, nai, br, bi, nbi, cr, ci, nci, dr, di, ndi;
};
__host__ inline MX mx_from(const M2 &m) {
  auto b = [](float x) { return make_float2(x, x); };
  return {b(m.a.x), b(m.a.y), b(-m.a.y), b(m.b.x), b(m.b.y), b(-m.b.y),
          b(m.c.x), b(m.c.y), b(-m.c.y), b(m.d.x), b(m.d.y), b(-m.d.y)};
}

// (u, v) <- m (u, v) for a pair of vectors across one wire >= 1.
template <int CLS>
__device__ __forceinline__ void applyx(const MX &m, Cx2 &u, Cx2 &v) {
  const Cx2 nu = cmacx6<CLS>(m.ar, m.ai, m.nai, m.br, m.bi, m.nbi, u, v);
  const Cx2 nv = cmacx6<CLS>(m.dr, m.di, m.ndi, m.cr, m.ci, m.nci, v, u);
  u = nu;
  v = nv;
}

// m on wire 0: the two amplitudes of one vector are the pair.
template <int CLS>
__device__ __forceinline__ void apply_w0x(const M2 &m, Cx2 &x) {
  float2 u = make_float2(x.re.x, x.im.x), v = make_float2(x.re.y, x.im.y);
  apply2c(CLS, m, u, v);
  x.re = make_float2(u.x, v.x);
  x.im = make_float2(u.y, v.y);
}

// Insert a zero bit at position p (bits >= p move up one).
__device__ __forceinline__ uint64_t ins0(uint64_t x, uint32_t p) {
  const uint64_t low = x & ((1ull << p) - 1ull);
  return ((x >> p) << (p + 1)) | low;
}

__device__ __forceinline__ int parity64(uint64_t x) { return __popcll(x) & 1; }

// The partner lane's vector (lane ^ mask), for ops on wires 1..5.
__device__ __forceinline__ float4 shfl4(const float4 &v, int mask) {
  return make_float4(__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask),
                     __shfl_xor_sync(0xffffffffu, v.z, mask), __shfl_xor_sync(0xffffffffu, v.w, mask));
}

// e^{i phi} for an angle summed in FP64: reduced to [-pi, pi] in FP64, then
// evaluated with the single-precision sincosf (about 1 ulp there).
__device__ __forceinline__ float2 expi_reduced(double phi) {
  const double two_pi = 6.283185307179586476925286766559;
  const double k = rint(phi * (1.0 / two_pi));
  const double r = fma(-k, two_pi, phi);
  float s, c;
  sincosf(static_cast<float>(r), &s, &c);
  return make_float2(c, s);
}

// FP64 warp sum.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block of kThreads threads; returns the block sum in thread 0 (other threads
// get unspecified values). `sm` needs kThreads/32 doubles.
__device__ __forceinline__ double block_sum(double v, double *sm) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sm[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < kThreads / 32) ? sm[l] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

}  // namespace qmk

// Device / grid helpers shared by the launchers (host side).
namespace qmk_host {
int num_sms();
inline unsigned grid_for(uint64_t items, uint64_t per_block) {
  uint64_t g = (items + per_block - 1) / per_block;
  if (g == 0) g = 1;
  return static_cast<unsigned>(g);
}
inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : static_cast<int>(e);
}
}  // namespace qmk_host
