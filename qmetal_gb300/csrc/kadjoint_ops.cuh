// kadjoint_ops.cuh -- the per-op pieces of the window-tile adjoint kernels
// (k_adjoint_tiles.cu, k_adjoint_uniform.cu): a tile holds both states in
// registers, NV vectors of each per thread, and every op takes the overlap
// of its generator before applying its inverse 2x2 to both states.
#pragma once

#include "kadjoint.cuh"

namespace qmk_adj {

using namespace qmk;

// ---------------------------------------------------------------------------
// Wider window tiles for both states: a warp owns 32 consecutive vectors
// (lane = vector bits 0..4, i.e. wires 1..5) for every combination of up to
// KH wires >= 6 held in registers, so all accesses are full 512-byte warp
// accesses. Wire 0 pairs the lanes of a vector; a wire in 1..5 exchanges
// with the partner lane by shuffle, and each lane then takes its own half of
// the overlap (the two halves of a pair sum to the pair's term).



// Im(conj(l) w) and Re(conj(l) w) summed over both amplitudes of a vector.
__device__ __forceinline__ float im_dot4(const float4 &l, const float4 &w) {
  return (l.x * w.y - l.y * w.x) + (l.z * w.w - l.w * w.z);
}
__device__ __forceinline__ float re_dot4(const float4 &l, const float4 &w) {
  return (l.x * w.x + l.y * w.y) + (l.z * w.z + l.w * w.w);
}

// One op on a lane wire for every register vector. Each lane owns one
// element of each pair: own' = s own + t other with (s, t) = (a, b) on the
// wire's 0 side and (d, c) on its 1 side, and it takes its own half of the
// pair's overlap: X: Im(conj(l) other); Y: -/+ Re(conj(l) other); Z: +/-
// Im(conj(l) own). A diagonal op needs no partner unless its generator is X
// or Y (a rotation by zero). GEN is a template parameter so the unrolled
// body has no branch and the vectors' chains interleave.
template <int NV, int CLS, int GEN>
__device__ __forceinline__ float lane_op_g(float4 (&P)[NV], float4 (&L)[NV], int mask, bool one,
                                           const M2 &m) {
  const float2 s = one ? m.d : m.a, t = one ? m.c : m.b;
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int l = 0; l < NV; l++) {
    if (CLS == kMatDiag && GEN != 1 && GEN != 2) {
      if (GEN == 3) acc[l & 3] += im_dot4(L[l], P[l]);
      P[l] = pack4(cmac2c(CLS, s, lo2(P[l]), t, lo2(P[l])), cmac2c(CLS, s, hi2(P[l]), t, hi2(P[l])));
      L[l] = pack4(cmac2c(CLS, s, lo2(L[l]), t, lo2(L[l])), cmac2c(CLS, s, hi2(L[l]), t, hi2(L[l])));
    } else {
      const float4 Po = shfl4(P[l], mask), Lo = shfl4(L[l], mask);
      if (GEN == 1) acc[l & 3] += im_dot4(L[l], Po);
      if (GEN == 2) acc[l & 3] += re_dot4(L[l], Po);
      if (GEN == 3) acc[l & 3] += im_dot4(L[l], P[l]);
      P[l] = pack4(cmac2c(CLS, s, lo2(P[l]), t, lo2(Po)), cmac2c(CLS, s, hi2(P[l]), t, hi2(Po)));
      L[l] = pack4(cmac2c(CLS, s, lo2(L[l]), t, lo2(Lo)), cmac2c(CLS, s, hi2(L[l]), t, hi2(Lo)));
    }
  }
  const float ov = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  if (GEN == 2) return one ? ov : -ov;
  if (GEN == 3) return one ? -ov : ov;
  return ov;
}

template <int NV, int CLS>
__device__ __forceinline__ float lane_op(float4 (&P)[NV], float4 (&L)[NV], int mask, bool one,
                                         int gen, const M2 &m) {
  switch (gen) {
    case 1: return lane_op_g<NV, CLS, 1>(P, L, mask, one, m);
    case 2: return lane_op_g<NV, CLS, 2>(P, L, mask, one, m);
    case 3: return lane_op_g<NV, CLS, 3>(P, L, mask, one, m);
    default: return lane_op_g<NV, CLS, 0>(P, L, mask, one, m);
  }
}

// Overlap of the pairs (p0, p1) = (P[l], P[h]) or the two halves of one
// vector, before the op is applied: a separate loop per generator, so the
// apply loop that follows is branch free.
template <int GEN>
__device__ __forceinline__ float pair_ov(const float4 &pa, const float4 &pb, const float4 &la,
                                         const float4 &lb) {
  return overlap(GEN, lo2(pa), lo2(pb), lo2(la), lo2(lb)) +
         overlap(GEN, hi2(pa), hi2(pb), hi2(la), hi2(lb));
}

template <int NV, int GEN>
__device__ __forceinline__ float wire0_ov(const float4 (&P)[NV], const float4 (&L)[NV]) {
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int l = 0; l < NV; l++)
    acc[l & 3] += overlap(GEN, lo2(P[l]), hi2(P[l]), lo2(L[l]), hi2(L[l]));
  return (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

template <int NV, int J, int GEN>
__device__ __forceinline__ float reg_ov(const float4 (&P)[NV], const float4 (&L)[NV]) {
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  int k = 0;
#pragma unroll
  for (int l = 0; l < NV; l++) {
    if ((l >> J) & 1) continue;
    const int h = l | (1 << J);
    acc[k & 3] += pair_ov<GEN>(P[l], P[h], L[l], L[h]);
    k++;
  }
  return (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// One op on wire 0 (the two amplitudes of each vector).
template <int NV, int CLS>
__device__ __forceinline__ float wire0_op(float4 (&P)[NV], float4 (&L)[NV], int gen, const M2 &m) {
  float ov = 0.0f;
  if (gen == 1) ov = wire0_ov<NV, 1>(P, L);
  else if (gen == 2) ov = wire0_ov<NV, 2>(P, L);
  else if (gen == 3) ov = wire0_ov<NV, 3>(P, L);
#pragma unroll
  for (int l = 0; l < NV; l++) {
    float2 p0 = lo2(P[l]), p1 = hi2(P[l]), l0 = lo2(L[l]), l1 = hi2(L[l]);
    apply2c(CLS, m, p0, p1);
    apply2c(CLS, m, l0, l1);
    P[l] = pack4(p0, p1);
    L[l] = pack4(l0, l1);
  }
  return ov;
}

// One op on register bit J.
template <int NV, int J, int CLS>
__device__ __forceinline__ float reg_op(float4 (&P)[NV], float4 (&L)[NV], int gen, const M2 &m) {
  float ov = 0.0f;
  if (gen == 1) ov = reg_ov<NV, J, 1>(P, L);
  else if (gen == 2) ov = reg_ov<NV, J, 2>(P, L);
  else if (gen == 3) ov = reg_ov<NV, J, 3>(P, L);
#pragma unroll
  for (int l = 0; l < NV; l++) {
    if ((l >> J) & 1) continue;
    const int h = l | (1 << J);
    float2 pa = lo2(P[l]), pb = lo2(P[h]), qa = hi2(P[l]), qb = hi2(P[h]);
    float2 la = lo2(L[l]), lb = lo2(L[h]), ma = hi2(L[l]), mb = hi2(L[h]);
    apply2c(CLS, m, pa, pb);
    apply2c(CLS, m, qa, qb);
    apply2c(CLS, m, la, lb);
    apply2c(CLS, m, ma, mb);
    P[l] = pack4(pa, qa);
    P[h] = pack4(pb, qb);
    L[l] = pack4(la, ma);
    L[h] = pack4(lb, mb);
  }
  return ov;
}

template <int NV, int CLS>
__device__ __forceinline__ float reg_op_any(float4 (&P)[NV], float4 (&L)[NV], int j, int gen,
                                            const M2 &m) {
  constexpr int KH = NV == 1 ? 0 : (NV == 2 ? 1 : (NV == 4 ? 2 : (NV == 8 ? 3 : 4)));
  float ov = 0.0f;
  if (KH > 0 && j == 0) ov = reg_op<NV, 0, CLS>(P, L, gen, m);
  if (KH > 1 && j == 1) ov = reg_op<NV, (KH > 1 ? 1 : 0), CLS>(P, L, gen, m);
  if (KH > 2 && j == 2) ov = reg_op<NV, (KH > 2 ? 2 : 0), CLS>(P, L, gen, m);
  if (KH > 3 && j == 3) ov = reg_op<NV, (KH > 3 ? 3 : 0), CLS>(P, L, gen, m);
  return ov;
}

template <int NV, int CLS>
__device__ __forceinline__ float warp_op(float4 (&P)[NV], float4 (&L)[NV], int kind, int arg,
                                         int gen, const M2 &m, uint32_t lane) {
  if (kind == 0) return wire0_op<NV, CLS>(P, L, gen, m);
  if (kind == 1) return lane_op<NV, CLS>(P, L, 1 << arg, (lane >> arg) & 1, gen, m);
  return reg_op_any<NV, CLS>(P, L, arg, gen, m);
}

// Tiles of up to three register wires keep two blocks resident per SM.

// ---------------------------------------------------------------------------
// Window tiles with four wires >= 6, two warps per tile: each thread holds the
// eight vectors of both states for three of the four register wires, and the
// two warps of a pair hold the two values of the fourth. An op on that fourth
// wire trades the pair's vectors through shared memory (each thread then
// takes its own half, as a lane op does); every other op is the one-warp
// tile's. Half the registers per thread of the one-warp tile, so twice the
// resident warps to hide the loads and the dependent arithmetic.

constexpr int kPairNV = 8;

// Barrier of the two warps of pair p only (named barrier p + 1; barrier 0 is
// the block's), so the block's pairs run out of step with each other and
// one pair's loads overlap another's arithmetic.
__device__ __forceinline__ void pair_sync(uint32_t p) {
  asm volatile("bar.sync %0, 64;" ::"r"(p + 1) : "memory");
}
static_assert(kThreads / 64 + 1 <= 16, "one named barrier per warp pair");

// The op on the fourth wire for every register vector: own' = s own + t
// other, own half of the overlap; the partner's vectors come from shared
// memory (written before the barrier that precedes this call).
template <int CLS, int GEN>
__device__ __forceinline__ float split_op_g(float4 (&P)[kPairNV], float4 (&L)[kPairNV],
                                            const float4 *__restrict__ oth_p,
                                            const float4 *__restrict__ oth_l, bool one,
                                            const M2 &m) {
  const float2 s = one ? m.d : m.a, t = one ? m.c : m.b;
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int l = 0; l < kPairNV; l++) {
    const float4 Po = oth_p[l * 32], Lo = oth_l[l * 32];
    if (GEN == 1) acc[l & 3] += im_dot4(L[l], Po);
    if (GEN == 2) acc[l & 3] += re_dot4(L[l], Po);
    if (GEN == 3) acc[l & 3] += im_dot4(L[l], P[l]);
    P[l] = pack4(cmac2c(CLS, s, lo2(P[l]), t, lo2(Po)), cmac2c(CLS, s, hi2(P[l]), t, hi2(Po)));
    L[l] = pack4(cmac2c(CLS, s, lo2(L[l]), t, lo2(Lo)), cmac2c(CLS, s, hi2(L[l]), t, hi2(Lo)));
  }
  const float ov = (acc[0] + acc[1]) + (acc[2] + acc[3]);
  if (GEN == 2) return one ? ov : -ov;
  if (GEN == 3) return one ? -ov : ov;
  return ov;
}

template <int CLS>
__device__ __forceinline__ float split_op(float4 (&P)[kPairNV], float4 (&L)[kPairNV],
                                          const float4 *oth_p, const float4 *oth_l, bool one,
                                          int gen, const M2 &m) {
  switch (gen) {
    case 1: return split_op_g<CLS, 1>(P, L, oth_p, oth_l, one, m);
    case 2: return split_op_g<CLS, 2>(P, L, oth_p, oth_l, one, m);
    case 3: return split_op_g<CLS, 3>(P, L, oth_p, oth_l, one, m);
    default: return split_op_g<CLS, 0>(P, L, oth_p, oth_l, one, m);
  }
}

}  // namespace qmk_adj
