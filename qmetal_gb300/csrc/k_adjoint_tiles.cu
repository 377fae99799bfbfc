// k_adjoint_tiles.cu -- backward passes over windows of one-qubit gates:
// both states held in registers as warp tiles, each window's gates undone in
// reverse with the overlap of every rotation taken first. Split from
// k_adjoint.cu so the two compile in parallel.
#include <algorithm>

#include "kadjoint.cuh"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

namespace qmk_adj {
namespace {

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
template <int KH, int NG>
__global__ void __launch_bounds__(kThreads, KH >= 4 ? 1 : 2)
k_adj_warp(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nwsites, WarpAdjArgs g,
           Area a, OutSlots<(NG > 0 ? NG : 1)> out) {
  constexpr int NV = 1 << KH;
  constexpr int NA = NG > 0 ? NG : 1;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gw = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (kThreads / 32);
  // FP32 per thread over its sites (a few dozen at most), FP64 from the warp
  // up. The per-thread partials live in shared memory, one column per
  // thread, so an op adds to its slot with one indexed access instead of a
  // compare-and-add over every register slot.
  __shared__ float sacc[NA][kThreads];
#pragma unroll
  for (int t = 0; t < NA; t++) sacc[t][threadIdx.x] = 0.0f;
  for (uint64_t ws = gw; ws < nwsites; ws += nwarps) {
    uint64_t b = ws;
#pragma unroll
    for (int j = 0; j < KH; j++) b = ins0(b, g.hpos[j]);
    const uint64_t base = (b << 5) | lane;
    float4 P[NV], L[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < KH; j++)
        if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
      P[l] = psi[v];
      L[l] = lam[v];
    }
    for (uint32_t o = 0; o < g.nops; o++) {
      const int kind = g.kind[o], arg = g.arg[o], gen = g.gen[o];
      const M2 m = g.m[o];
      float ov;
      switch (g.cls[o]) {
        case kMatReal: ov = warp_op<NV, kMatReal>(P, L, kind, arg, gen, m, lane); break;
        case kMatRx: ov = warp_op<NV, kMatRx>(P, L, kind, arg, gen, m, lane); break;
        case kMatDiag: ov = warp_op<NV, kMatDiag>(P, L, kind, arg, gen, m, lane); break;
        default: ov = warp_op<NV, kMatGeneral>(P, L, kind, arg, gen, m, lane); break;
      }
      if (NG > 0) sacc[g.slotidx[o]][threadIdx.x] += gen ? ov : 0.0f;
    }
#pragma unroll
    for (int l = 0; l < NV; l++) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < KH; j++)
        if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
      psi[v] = P[l];
      lam[v] = L[l];
    }
  }
  if constexpr (NG > 0) {
    double acc[NA];
#pragma unroll
    for (int t = 0; t < NA; t++) acc[t] = sacc[t][threadIdx.x];
    finish<NG>(acc, static_cast<int>(g.ngrad), a, out);
  }
}

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

template <int NG>
__global__ void __launch_bounds__(kThreads, 2)
k_adj_pair(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nwsites, WarpAdjArgs g,
           Area a, OutSlots<(NG > 0 ? NG : 1)> out) {
  constexpr int NV = kPairNV;
  constexpr int NA = NG > 0 ? NG : 1;
  extern __shared__ __align__(16) float4 xs[];   // [warp][state][NV][32 lanes]
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t half = warp & 1;                // value of the fourth wire
  const uint64_t per_round = static_cast<uint64_t>(gridDim.x) * (kThreads / 64);
  const uint64_t rounds = (nwsites + per_round - 1) / per_round;
  float4 *mine_p = xs + (warp * 2 + 0) * NV * 32 + lane;
  float4 *mine_l = xs + (warp * 2 + 1) * NV * 32 + lane;
  const float4 *oth_p = xs + ((warp ^ 1) * 2 + 0) * NV * 32 + lane;
  const float4 *oth_l = xs + ((warp ^ 1) * 2 + 1) * NV * 32 + lane;
  __shared__ float sacc[NA][kThreads];   // per-thread FP32 gradient partials
#pragma unroll
  for (int t = 0; t < NA; t++) sacc[t][tid] = 0.0f;
  // Both warps of a pair run the same rounds (the barriers of their
  // exchanges must match); a pair past the last tile works on zeros and
  // stores nothing.
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t ws = r * per_round + static_cast<uint64_t>(blockIdx.x) * (kThreads / 64) +
                        (warp >> 1);
    const bool active = ws < nwsites;
    uint64_t base = 0;
    if (active) {
      uint64_t b = ws;
#pragma unroll
      for (int j = 0; j < 4; j++) b = ins0(b, g.hpos[j]);
      base = (b << 5) | lane | (static_cast<uint64_t>(half) << (g.hpos[3] + 5));
    }
    auto vec_of = [&](int l) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < 3; j++)
        if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
      return v;
    };
    float4 P[NV], L[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      if (active) {
        const uint64_t v = vec_of(l);
        P[l] = psi[v];
        L[l] = lam[v];
      } else {
        P[l] = L[l] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    for (uint32_t o = 0; o < g.nops; o++) {
      const int kind = g.kind[o], arg = g.arg[o], gen = g.gen[o], cls = g.cls[o];
      const M2 m = g.m[o];
      float ov;
      if (kind == 3) {
        const bool need = cls != kMatDiag || gen == 1 || gen == 2;
        if (need) {
#pragma unroll
          for (int l = 0; l < NV; l++) {
            mine_p[l * 32] = P[l];
            mine_l[l * 32] = L[l];
          }
          pair_sync(warp >> 1);
        }
        const bool one = half != 0;
        switch (cls) {
          case kMatReal: ov = split_op<kMatReal>(P, L, oth_p, oth_l, one, gen, m); break;
          case kMatRx: ov = split_op<kMatRx>(P, L, oth_p, oth_l, one, gen, m); break;
          case kMatDiag: ov = split_op<kMatDiag>(P, L, oth_p, oth_l, one, gen, m); break;
          default: ov = split_op<kMatGeneral>(P, L, oth_p, oth_l, one, gen, m); break;
        }
        if (need) pair_sync(warp >> 1);
      } else {
        switch (cls) {
          case kMatReal: ov = warp_op<NV, kMatReal>(P, L, kind, arg, gen, m, lane); break;
          case kMatRx: ov = warp_op<NV, kMatRx>(P, L, kind, arg, gen, m, lane); break;
          case kMatDiag: ov = warp_op<NV, kMatDiag>(P, L, kind, arg, gen, m, lane); break;
          default: ov = warp_op<NV, kMatGeneral>(P, L, kind, arg, gen, m, lane); break;
        }
      }
      if (NG > 0) sacc[g.slotidx[o]][tid] += gen ? ov : 0.0f;
    }
    if (active) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        const uint64_t v = vec_of(l);
        psi[v] = P[l];
        lam[v] = L[l];
      }
    }
  }
  if constexpr (NG > 0) {
    double acc[NA];
#pragma unroll
    for (int t = 0; t < NA; t++) acc[t] = sacc[t][tid];
    finish<NG>(acc, static_cast<int>(g.ngrad), a, out);
  }
}

// ---------------------------------------------------------------------------
// Uniform warp-pair tiles: one rotation per wire, every op of the same kind
// (all RX, all RY or all RZ), on wire 0 and all five lane wires or on the
// four register wires alone -- the mixer and rotation layers of QAOA, TFIM
// and hardware-efficient circuits. The op list is then known at compile
// time: no per-op dispatch, gradient partials in registers at fixed
// indices, and the compiler free to interleave one op's shuffles with
// another's arithmetic. Same per-op arithmetic and order as k_adj_pair.

struct UniArgs {
  uint32_t hpos[4];   // wires >= 6: vector bit - 5, ascending; hpos[3] is split
  uint32_t lbit[5];   // lane wires' vector bits
  M2 m0, ml[5], mh[4];
};

template <bool W0, int NL, int CLS, int GEN>
__global__ void __launch_bounds__(kThreads, 2)
k_adj_pair_uni(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nwsites, UniArgs g,
               Area a, OutSlots<(W0 ? 1 : 0) + NL + 4> out) {
  constexpr int NV = kPairNV;
  constexpr int NOPS = (W0 ? 1 : 0) + NL + 4;
  constexpr int LANE0 = W0 ? 1 : 0, REG0 = LANE0 + NL;
  extern __shared__ __align__(16) float4 xs[];   // [warp][state][NV][32 lanes]
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t half = warp & 1;
  const uint64_t per_round = static_cast<uint64_t>(gridDim.x) * (kThreads / 64);
  const uint64_t rounds = (nwsites + per_round - 1) / per_round;
  float4 *mine_p = xs + (warp * 2 + 0) * NV * 32 + lane;
  float4 *mine_l = xs + (warp * 2 + 1) * NV * 32 + lane;
  const float4 *oth_p = xs + ((warp ^ 1) * 2 + 0) * NV * 32 + lane;
  const float4 *oth_l = xs + ((warp ^ 1) * 2 + 1) * NV * 32 + lane;
  float accf[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) accf[t] = 0.0f;
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t ws = r * per_round + static_cast<uint64_t>(blockIdx.x) * (kThreads / 64) +
                        (warp >> 1);
    const bool active = ws < nwsites;
    uint64_t base = 0;
    if (active) {
      uint64_t b = ws;
#pragma unroll
      for (int j = 0; j < 4; j++) b = ins0(b, g.hpos[j]);
      base = (b << 5) | lane | (static_cast<uint64_t>(half) << (g.hpos[3] + 5));
    }
    auto vec_of = [&](int l) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < 3; j++)
        if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
      return v;
    };
    float4 P[NV], L[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      if (active) {
        const uint64_t v = vec_of(l);
        P[l] = psi[v];
        L[l] = lam[v];
      } else {
        P[l] = L[l] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (W0) accf[0] += wire0_op<NV, CLS>(P, L, GEN, g.m0);
#pragma unroll
    for (int k = 0; k < NL; k++)
      accf[LANE0 + k] += lane_op_g<NV, CLS, GEN>(P, L, 1 << g.lbit[k], (lane >> g.lbit[k]) & 1,
                                                 g.ml[k]);
    accf[REG0 + 0] += reg_op<NV, 0, CLS>(P, L, GEN, g.mh[0]);
    accf[REG0 + 1] += reg_op<NV, 1, CLS>(P, L, GEN, g.mh[1]);
    accf[REG0 + 2] += reg_op<NV, 2, CLS>(P, L, GEN, g.mh[2]);
    constexpr bool kNeed = CLS != kMatDiag || GEN == 1 || GEN == 2;
    if (kNeed) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        mine_p[l * 32] = P[l];
        mine_l[l * 32] = L[l];
      }
      pair_sync(warp >> 1);
    }
    accf[REG0 + 3] += split_op_g<CLS, GEN>(P, L, oth_p, oth_l, half != 0, g.mh[3]);
    if (kNeed) pair_sync(warp >> 1);
    if (active) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        const uint64_t v = vec_of(l);
        psi[v] = P[l];
        lam[v] = L[l];
      }
    }
  }
  double acc[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) acc[t] = accf[t];
  finish<NOPS>(acc, NOPS, a, out);
}

template <bool W0, int NL, int CLS, int GEN>
int launch_adj_pair_uni(float4 *psi, float4 *lam, uint64_t nwsites, const UniArgs &g,
                        double *grad, const uint32_t *slots, Area a, cudaStream_t s) {
  constexpr int NOPS = (W0 ? 1 : 0) + NL + 4;
  OutSlots<NOPS> out{};
  out.p = grad;
  for (int t = 0; t < NOPS; t++) out.slot[t] = slots[t];
  unsigned grid = grid_for(nwsites, kThreads / 64);
  grid = std::min<unsigned>(grid, reduce_grid());
  const size_t smem = static_cast<size_t>(kThreads / 32) * 2 * kPairNV * 32 * sizeof(float4);
  static bool opted[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(k_adj_pair_uni<W0, NL, CLS, GEN>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  k_adj_pair_uni<W0, NL, CLS, GEN><<<grid, kThreads, smem, s>>>(psi, lam, nwsites, g, a, out);
  return launch_status();
}

// A four-register-wire tile with one rotation per wire, all RX (class RX,
// generator X), all RY (real, Y) or all RZ (diagonal, Z), on the four
// register wires alone or with wire 0 and all five lane wires, goes to the
// uniform kernel. Returns 1 (nothing launched) for any other tile.
int launch_uniform(float4 *psi, float4 *lam, uint64_t nw, const WarpAdjArgs &g,
                   const OutSlots<kMaxGen> &out, Area a, cudaStream_t s) {
  if (g.nops != 4 && g.nops != 10) return 1;
  const int cls = g.cls[0], gen = g.gen[0];
  if (!((cls == kMatRx && gen == 1) || (cls == kMatReal && gen == 2) ||
        (cls == kMatDiag && gen == 3)))
    return 1;
  UniArgs u{};
  for (int j = 0; j < 4; j++) u.hpos[j] = g.hpos[j];
  int w0 = 0, nl = 0;
  bool seen_h[4] = {false, false, false, false};
  uint32_t lanes_seen = 0, slot_w0 = 0, slot_l[5] = {}, slot_h[4] = {};
  for (uint32_t o = 0; o < g.nops; o++) {
    if (g.cls[o] != cls || g.gen[o] != gen) return 1;
    const uint32_t slot = out.slot[g.slotidx[o]];
    if (g.kind[o] == 0) {
      if (w0) return 1;
      w0 = 1;
      u.m0 = g.m[o];
      slot_w0 = slot;
    } else if (g.kind[o] == 1) {
      const int b = g.arg[o];
      if (b < 0 || b > 4 || ((lanes_seen >> b) & 1u)) return 1;
      lanes_seen |= 1u << b;
      u.lbit[nl] = static_cast<uint32_t>(b);
      u.ml[nl] = g.m[o];
      slot_l[nl] = slot;
      nl++;
    } else if (g.kind[o] == 2) {
      const int j = g.arg[o];
      if (j < 0 || j > 3 || seen_h[j]) return 1;
      seen_h[j] = true;
      u.mh[j] = g.m[o];
      slot_h[j] = slot;
    } else {
      return 1;
    }
  }
  for (int j = 0; j < 4; j++)
    if (!seen_h[j]) return 1;
  const bool wide = w0 == 1 && nl == 5;
  if (!wide && !(w0 == 0 && nl == 0)) return 1;
  uint32_t slots[10];
  int t = 0;
  if (w0) slots[t++] = slot_w0;
  for (int k = 0; k < nl; k++) slots[t++] = slot_l[k];
  for (int j = 0; j < 4; j++) slots[t++] = slot_h[j];
  double *p = out.p;
  if (wide) {
    if (gen == 1) return launch_adj_pair_uni<true, 5, kMatRx, 1>(psi, lam, nw, u, p, slots, a, s);
    if (gen == 2) return launch_adj_pair_uni<true, 5, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
    return launch_adj_pair_uni<true, 5, kMatDiag, 3>(psi, lam, nw, u, p, slots, a, s);
  }
  if (gen == 1) return launch_adj_pair_uni<false, 0, kMatRx, 1>(psi, lam, nw, u, p, slots, a, s);
  if (gen == 2) return launch_adj_pair_uni<false, 0, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
  return launch_adj_pair_uni<false, 0, kMatDiag, 3>(psi, lam, nw, u, p, slots, a, s);
}

template <int NG>
int launch_adj_pair(float4 *psi, float4 *lam, uint64_t nwsites, const WarpAdjArgs &g,
                    const OutSlots<kMaxGen> &slots, Area a, cudaStream_t s) {
  OutSlots<(NG > 0 ? NG : 1)> out{};
  out.p = slots.p;
  for (int t = 0; t < (NG > 0 ? NG : 1); t++) out.slot[t] = slots.slot[t];
  unsigned grid = grid_for(nwsites, kThreads / 64);
  grid = std::min<unsigned>(grid, reduce_grid());
  const size_t smem = static_cast<size_t>(kThreads / 32) * 2 * kPairNV * 32 * sizeof(float4);
  // The opt-in above 48 KiB is per device; set it once on each.
  static bool opted[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_adj_pair<NG>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  k_adj_pair<NG><<<grid, kThreads, smem, s>>>(psi, lam, nwsites, g, a, out);
  return launch_status();
}

template <int KH, int NG>
void launch_adj_warp(float4 *psi, float4 *lam, uint64_t nwsites, const WarpAdjArgs &g,
                     const OutSlots<kMaxGen> &slots, Area a, cudaStream_t s) {
  OutSlots<(NG > 0 ? NG : 1)> out{};
  out.p = slots.p;
  for (int t = 0; t < (NG > 0 ? NG : 1); t++) out.slot[t] = slots.slot[t];
  const uint64_t per_block = kThreads / 32;
  unsigned grid = grid_for(nwsites, per_block);
  if (NG > 0) grid = std::min<unsigned>(grid, reduce_grid());
  k_adj_warp<KH, NG><<<grid, kThreads, 0, s>>>(psi, lam, nwsites, g, a, out);
}


}  // namespace

int launch_tiles(int kh, int ng, float4 *psi, float4 *lam, uint64_t nw, WarpAdjArgs &g,
                 const OutSlots<kMaxGen> &out, Area a, cudaStream_t s) {
  if (kh == 4) {
    const int rc = launch_uniform(psi, lam, nw, g, out, a, s);
    if (rc != 1) return rc;
    // two warps per tile: the fourth register wire is split across the pair
    for (uint32_t o = 0; o < g.nops; o++)
      if (g.kind[o] == 2 && g.arg[o] == 3) g.kind[o] = 3;
    if (ng == 0) return launch_adj_pair<0>(psi, lam, nw, g, out, a, s);
    if (ng == 4) return launch_adj_pair<4>(psi, lam, nw, g, out, a, s);
    if (ng == 8) return launch_adj_pair<8>(psi, lam, nw, g, out, a, s);
    return launch_adj_pair<16>(psi, lam, nw, g, out, a, s);
  }
#define QMK_ADJ_WARP_CASE(KH)                                                   \
  if (kh == KH) {                                                               \
    if (ng == 0) launch_adj_warp<KH, 0>(psi, lam, nw, g, out, a, s);            \
    else if (ng == 4) launch_adj_warp<KH, 4>(psi, lam, nw, g, out, a, s);       \
    else if (ng == 8) launch_adj_warp<KH, 8>(psi, lam, nw, g, out, a, s);       \
    else launch_adj_warp<KH, 16>(psi, lam, nw, g, out, a, s);                   \
    return launch_status();                                                     \
  }
  QMK_ADJ_WARP_CASE(0)
  QMK_ADJ_WARP_CASE(1)
  QMK_ADJ_WARP_CASE(2)
  QMK_ADJ_WARP_CASE(3)
#undef QMK_ADJ_WARP_CASE
  return -1;
}

}  // namespace qmk_adj
