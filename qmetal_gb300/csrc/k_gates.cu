// k_gates.cu -- in-place gate kernels: basis init, dense / controlled 2x2,
// masked phase, register groups, shared-memory blocks, swap.
//
// Work is enumerated by "sites": the free vector-index bits left after the
// op's own wires are taken out. A site expands to the one or more float4
// vectors the op touches, so every thread moves whole 16-byte vectors and
// consecutive threads move consecutive vectors. Each thread handles U sites
// spaced kThreads apart (loads for all U first, then math, then stores) so
// enough bytes are in flight to cover HBM latency.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

#include "kcommon.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;

namespace {

constexpr int U = 2;  // sites per thread

__device__ __forceinline__ uint64_t site_of(int k) {
  return (static_cast<uint64_t>(blockIdx.x) * U + k) * kThreads + threadIdx.x;
}

// Up to three ascending vector-bit positions to open, then forced-one bits.
struct Fix {
  uint32_t nfix;
  uint32_t pos[3];
  uint64_t set;
};

__device__ __forceinline__ uint64_t expand(uint64_t s, const Fix &f) {
#pragma unroll
  for (uint32_t j = 0; j < 3; j++)
    if (j < f.nfix) s = ins0(s, f.pos[j]);
  return s | f.set;
}

__global__ void k_init_basis(float4 *__restrict__ st, uint64_t nvec) {
#pragma unroll
  for (int k = 0; k < U; k++) {
    const uint64_t v = site_of(k);
    if (v < nvec) st[v] = make_float4(v == 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
  }
}

// MODE 0: the target is amplitude bit 0, so the pair is the two lanes of one
//         vector; controls (all >= 1) are forced-one vector bits.
// MODE 1: target >= 1: the pair is vectors v and v|tbit, both lanes.
// MODE 2: target >= 1 and amplitude bit 0 is a control: only the odd lane.
template <int MODE>
__global__ void __launch_bounds__(kThreads)
k_pair(float4 *__restrict__ st, uint64_t nsites, Fix f, uint64_t tbit, M2 m) {
  uint64_t v[U];
  float4 A[U], B[U];
#pragma unroll
  for (int k = 0; k < U; k++) {
    const uint64_t s = site_of(k);
    v[k] = (s < nsites) ? expand(s, f) : ~0ull;
    if (v[k] != ~0ull) {
      A[k] = st[v[k]];
      if (MODE != 0) B[k] = st[v[k] | tbit];
    }
  }
#pragma unroll
  for (int k = 0; k < U; k++) {
    if (v[k] == ~0ull) continue;
    if (MODE == 0) {
      float2 x = lo2(A[k]), y = hi2(A[k]);
      apply2(m, x, y);
      st[v[k]] = pack4(x, y);
    } else if (MODE == 1) {
      float2 a0 = lo2(A[k]), b0 = lo2(B[k]), a1 = hi2(A[k]), b1 = hi2(B[k]);
      apply2(m, a0, b0);
      apply2(m, a1, b1);
      st[v[k]] = pack4(a0, a1);
      st[v[k] | tbit] = pack4(b0, b1);
    } else {
      float2 a1 = hi2(A[k]), b1 = hi2(B[k]);
      apply2(m, a1, b1);
      float2 *s2 = reinterpret_cast<float2 *>(st);
      s2[2 * v[k] + 1] = a1;
      s2[2 * (v[k] | tbit) + 1] = b1;
    }
  }
}

// Multiply amplitudes with every mask bit set by `ph`. ODD: amplitude bit 0
// is in the mask, so only the odd lane of each vector changes.
template <bool ODD>
__global__ void __launch_bounds__(kThreads)
k_phase(float4 *__restrict__ st, uint64_t nsites, Fix f, float2 ph) {
  if (ODD) {
    float2 *s2 = reinterpret_cast<float2 *>(st);
#pragma unroll
    for (int k = 0; k < U; k++) {
      const uint64_t s = site_of(k);
      if (s < nsites) {
        const uint64_t i = 2 * expand(s, f) + 1;
        s2[i] = cmul(ph, s2[i]);
      }
    }
  } else {
    uint64_t v[U];
    float4 A[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
      const uint64_t s = site_of(k);
      v[k] = (s < nsites) ? expand(s, f) : ~0ull;
      if (v[k] != ~0ull) A[k] = st[v[k]];
    }
#pragma unroll
    for (int k = 0; k < U; k++)
      if (v[k] != ~0ull) st[v[k]] = pack4(cmul(ph, lo2(A[k])), cmul(ph, hi2(A[k])));
  }
}

struct GroupArgs {
  uint32_t pos[5];  // vector-bit positions of the wires >= 1, ascending
  M2 m[5];          // their matrices
  M2 m0;            // matrix of wire 0 when W0
};

// KP wires >= 1 (plus wire 0 when W0): a site owns 2^KP vectors in registers.
// CLS: the structure every matrix of the launch shares (kMat*), so RX-, RY-
// and phase-like layers take half the multiply-adds of general ones.
template <int KP, bool W0, int CLS>
__global__ void __launch_bounds__(kThreads)
k_group(float4 *__restrict__ st, uint64_t nsites, GroupArgs g) {
  constexpr int NV = 1 << KP;
  const uint64_t s = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x;
  if (s >= nsites) return;
  uint64_t base = s;
#pragma unroll
  for (int j = 0; j < KP; j++) base = ins0(base, g.pos[j]);
  // Scalar arithmetic: at up to 32 vectors a thread this kernel is bound by
  // its one block per SM, and the packed form's extra registers cost more
  // than its saved instructions.
  float4 r[NV];
#pragma unroll
  for (int l = 0; l < NV; l++) {
    uint64_t v = base;
#pragma unroll
    for (int j = 0; j < KP; j++)
      if ((l >> j) & 1) v |= 1ull << g.pos[j];
    r[l] = st[v];
  }
  if (W0) {
#pragma unroll
    for (int l = 0; l < NV; l++) {
      float2 x = lo2(r[l]), y = hi2(r[l]);
      apply2c(CLS, g.m0, x, y);
      r[l] = pack4(x, y);
    }
  }
#pragma unroll
  for (int j = 0; j < KP; j++) {
#pragma unroll
    for (int l = 0; l < NV; l++) {
      if ((l >> j) & 1) continue;
      const int h = l | (1 << j);
      float2 a0 = lo2(r[l]), b0 = lo2(r[h]), a1 = hi2(r[l]), b1 = hi2(r[h]);
      apply2c(CLS, g.m[j], a0, b0);
      apply2c(CLS, g.m[j], a1, b1);
      r[l] = pack4(a0, a1);
      r[h] = pack4(b0, b1);
    }
  }
#pragma unroll
  for (int l = 0; l < NV; l++) {
    uint64_t v = base;
#pragma unroll
    for (int j = 0; j < KP; j++)
      if ((l >> j) & 1) v |= 1ull << g.pos[j];
    st[v] = r[l];
  }
}

// Five wires >= 1 on a warp pair: a site's 32 vectors are split by the bit
// of the fifth wire between the two warps of a pair, each thread holding 16
// in registers (half the registers of k_group<5>, so two blocks fit per SM
// and twice the warps hide the loads). Ops on the first four wires pair
// registers; the fifth trades vectors through shared memory and each thread
// updates its own half. A pair covers 32 consecutive sites (lane = site).
constexpr int kPairVecs = 16;

__device__ __forceinline__ void group_pair_sync(uint32_t p) {
  asm volatile("bar.sync %0, 64;" ::"r"(p + 1) : "memory");
}

template <bool W0, int CLS>
__global__ void __launch_bounds__(kThreads, 2)
k_group5_pair(float4 *__restrict__ st, uint64_t nsites, GroupArgs g) {
  constexpr int NV = kPairVecs;
  extern __shared__ __align__(16) float4 xg[];   // [warp][NV][32 lanes]
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t half = warp & 1, pair = warp >> 1;
  const uint64_t s = (static_cast<uint64_t>(blockIdx.x) * (kThreads / 64) + pair) * 32 + lane;
  // Both warps of a pair reach the exchange barrier: the pair's 32 sites
  // are all valid or all invalid (nsites is a multiple of 32 here).
  const bool active = s < nsites;
  uint64_t base = s;
#pragma unroll
  for (int j = 0; j < 5; j++) base = ins0(base, g.pos[j]);
  base |= static_cast<uint64_t>(half) << g.pos[4];
  auto vec_of = [&](int l) {
    uint64_t v = base;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if ((l >> j) & 1) v |= 1ull << g.pos[j];
    return v;
  };
  float4 r[NV];
#pragma unroll
  for (int l = 0; l < NV; l++) r[l] = active ? st[vec_of(l)] : make_float4(0.f, 0.f, 0.f, 0.f);
  if (W0) {
#pragma unroll
    for (int l = 0; l < NV; l++) {
      float2 x = lo2(r[l]), y = hi2(r[l]);
      apply2c(CLS, g.m0, x, y);
      r[l] = pack4(x, y);
    }
  }
#pragma unroll
  for (int j = 0; j < 4; j++) {
#pragma unroll
    for (int l = 0; l < NV; l++) {
      if ((l >> j) & 1) continue;
      const int h = l | (1 << j);
      float2 a0 = lo2(r[l]), b0 = lo2(r[h]), a1 = hi2(r[l]), b1 = hi2(r[h]);
      apply2c(CLS, g.m[j], a0, b0);
      apply2c(CLS, g.m[j], a1, b1);
      r[l] = pack4(a0, a1);
      r[h] = pack4(b0, b1);
    }
  }
  // The fifth wire: own' = s own + t other, (a, b) on its 0 side, (d, c) on
  // its 1 side.
  float4 *mine = xg + warp * NV * 32 + lane;
  const float4 *other = xg + (warp ^ 1) * NV * 32 + lane;
  if (CLS != kMatDiag) {
#pragma unroll
    for (int l = 0; l < NV; l++) mine[l * 32] = r[l];
    group_pair_sync(pair);
  }
  const M2 &m = g.m[4];
  const float2 cs = half ? m.d : m.a, ct = half ? m.c : m.b;
#pragma unroll
  for (int l = 0; l < NV; l++) {
    const float4 o = CLS != kMatDiag ? other[l * 32] : r[l];
    r[l] = pack4(cmac2c(CLS, cs, lo2(r[l]), ct, lo2(o)), cmac2c(CLS, cs, hi2(r[l]), ct, hi2(o)));
  }
  if (active) {
#pragma unroll
    for (int l = 0; l < NV; l++) st[vec_of(l)] = r[l];
  }
}

// Six or seven wires >= 6 in one pass (optionally with wire 0) on a block
// of warps: a site is 2^(4 + WB) rows of 32 vectors, held by 2^WB warps with
// sixteen vectors per thread. A thread's four register bits are the site's
// first four wires and its warp's index the others, so those four wires'
// 2x2s run in registers; the site then trades places through shared memory
// (WB register bits become warp bits and the warp bits register bits) and
// the last WB wires run in registers too. One shared-memory round trip per
// site instead of a pair exchange per wire; every load and store is a
// 512-byte warp row.
struct BlkGroupArgs {
  uint32_t pos[7];   // the wires' vector bits (wire - 1), ascending, all >= 5
  M2 m[7];
  M2 m0;             // wire 0 when W0
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(smem))),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Blocks loop over sites. Each thread copies its next site's sixteen vectors
// into its own first-layout slots (16-byte cp.async, waited for by the
// thread that issued them) once every warp of the site has read the current
// second layout, so the copies overlap the second half of the arithmetic and
// the stores.
template <int WB, bool W0, int CLS>
__global__ void __launch_bounds__(kThreads, 2)
k_group_blk(float4 *__restrict__ st, uint64_t nsites, BlkGroupArgs g) {
  constexpr int NV = 16;
  constexpr int KB = 4 + WB;                  // wires >= 6 in the group
  constexpr int NW = 1 << WB;                 // warps per site
  constexpr int SPB = (kThreads / 32) / NW;   // sites per block
  constexpr int ROWS = NV * NW;
  static_assert(SPB >= 1 && SPB * NW == kThreads / 32, "whole sites per block");
  extern __shared__ __align__(16) float4 xq[];   // [site][row][32 lanes]
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t sib = warp / NW, wsl = warp % NW;
  float4 *site = xq + static_cast<size_t>(sib) * ROWS * 32;
  const uint64_t per_round = static_cast<uint64_t>(gridDim.x) * SPB;
  const uint64_t rounds = (nsites + per_round - 1) / per_round;
  // Rows in the first layout (register bits = wires 0..3 of the group, warp
  // bits = wires 4..) and the second (register bits = wires 4.., then wires
  // WB..3; warp bits = wires 0..WB-1); each warp's offsets worked out once.
  auto row_a = [&](int l) { return static_cast<uint32_t>(l) | (wsl << 4); };
  auto row_b = [&](int l) {
    const uint32_t lo = static_cast<uint32_t>(l) & (NW - 1u), hi = static_cast<uint32_t>(l) >> WB;
    return wsl | (hi << WB) | (lo << 4);
  };
  __shared__ uint64_t row_off[kThreads / 32][2][NV];
  {
    const int l = lane & (NV - 1);
    const uint32_t row = lane < NV ? row_a(l) : row_b(l);
    uint64_t v = 0;
#pragma unroll
    for (int j = 0; j < KB; j++)
      if ((row >> j) & 1u) v |= 1ull << g.pos[j];
    row_off[warp][lane / NV][l] = v;
  }
  __syncwarp();
  auto site_of = [&](uint64_t r) {
    return r * per_round + static_cast<uint64_t>(blockIdx.x) * SPB + sib;
  };
  auto base_of = [&](uint64_t sidx) {
    uint64_t b = sidx * 32 + lane;
#pragma unroll
    for (int j = 0; j < KB; j++) b = ins0(b, g.pos[j]);
    return b;
  };
  auto site_sync = [&]() {
    if constexpr (SPB == 1) {
      __syncthreads();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(sib + 1), "r"(NW * 32) : "memory");
    }
  };
  auto prefetch = [&](uint64_t r) {
    const uint64_t sidx = site_of(r);
    if (r < rounds && sidx < nsites) {
      const uint64_t base = base_of(sidx);
#pragma unroll
      for (int l = 0; l < NV; l++)
        cp_async16(site + row_a(l) * 32 + lane, st + (base | row_off[warp][0][l]));
    }
    cp_async_commit();
  };
  auto reg_wire = [&](float4 (&r)[NV], int j, const M2 &m) {
#pragma unroll
    for (int l = 0; l < NV; l++) {
      if ((l >> j) & 1) continue;
      const int h = l | (1 << j);
      float2 a0 = lo2(r[l]), b0 = lo2(r[h]), a1 = hi2(r[l]), b1 = hi2(r[h]);
      apply2c(CLS, m, a0, b0);
      apply2c(CLS, m, a1, b1);
      r[l] = pack4(a0, a1);
      r[h] = pack4(b0, b1);
    }
  };
  prefetch(0);
  for (uint64_t rd = 0; rd < rounds; rd++) {
    const uint64_t sidx = site_of(rd);
    const bool active = sidx < nsites;   // uniform over the site's warps
    float4 r[NV];
    cp_async_wait_all();                 // this thread's copies of this round
    if (active) {
#pragma unroll
      for (int l = 0; l < NV; l++) r[l] = site[row_a(l) * 32 + lane];
      if (W0) {
#pragma unroll
        for (int l = 0; l < NV; l++) {
          float2 x = lo2(r[l]), y = hi2(r[l]);
          apply2c(CLS, g.m0, x, y);
          r[l] = pack4(x, y);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++) reg_wire(r, j, g.m[j]);
#pragma unroll
      for (int l = 0; l < NV; l++) site[row_a(l) * 32 + lane] = r[l];
    }
    site_sync();   // the first layout is written back
    if (active) {
#pragma unroll
      for (int l = 0; l < NV; l++) r[l] = site[row_b(l) * 32 + lane];
    }
    site_sync();   // every warp has read its second layout: the slots are free
    prefetch(rd + 1);
    if (active) {
#pragma unroll
      for (int j = 0; j < WB; j++) reg_wire(r, j, g.m[4 + j]);
      const uint64_t base = base_of(sidx);
#pragma unroll
      for (int l = 0; l < NV; l++) st[base | row_off[warp][1][l]] = r[l];
    }
  }
  cp_async_wait_all();
}

struct WarpGroupArgs {
  uint32_t nlow;     // wires 1..5: lane bits
  uint32_t lbit[5];  // their vector bits (0..4)
  M2 lm[5];
  uint32_t hpos[4];  // wires >= 6: vector bits - 5 (warp-site bits), ascending
  MX hm[4];
  M2 m0;             // wire 0 (lanes) when W0
};

// Groups with wires inside one warp's 512 bytes. A warp owns 32 consecutive
// vectors (lane = vector bits 0..4) for each combination of the KH high
// wires, so every load and store is a full 512-byte warp access. Wire 0 is a
// lane-pair update, wires 1..5 exchange with the partner lane by shuffle,
// wires >= 6 pair registers. Each thread takes UW warp-sites.
template <int KH, bool W0, int CLS>
__global__ void __launch_bounds__(kThreads, 2)
k_group_warp(float4 *__restrict__ st, uint64_t nwsites, WarpGroupArgs g) {
  constexpr int NV = 1 << KH;
  constexpr int UW = KH <= 1 ? 4 : (KH == 2 ? 2 : 1);
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t warp = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  uint64_t base[UW];
  Cx2 r[UW][NV];
#pragma unroll
  for (int u = 0; u < UW; u++) {
    const uint64_t ws = warp * UW + u;
    base[u] = ~0ull;
    if (ws >= nwsites) continue;
    uint64_t b = ws;
#pragma unroll
    for (int j = 0; j < KH; j++) b = ins0(b, g.hpos[j]);
    base[u] = (b << 5) | lane;
#pragma unroll
    for (int l = 0; l < NV; l++) {
      uint64_t v = base[u];
#pragma unroll
      for (int j = 0; j < KH; j++)
        if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
      r[u][l] = split2(st[v]);
    }
  }
#pragma unroll
  for (int u = 0; u < UW; u++) {
    // Warp-uniform: the sites of one warp are all valid or all invalid.
    if (base[u] == ~0ull) continue;
    if (W0) {
#pragma unroll
      for (int l = 0; l < NV; l++) apply_w0x<CLS>(g.m0, r[u][l]);
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
      if (k >= static_cast<int>(g.nlow)) continue;   // (a break here spills)
      const uint32_t b = g.lbit[k];
      const bool one = (lane >> b) & 1;
      const M2 m = g.lm[k];
      // own' = s own + t other: (a, b) on the wire's 0 side, (d, c) on its 1 side
      const float2 cs = one ? m.d : m.a, ct = one ? m.c : m.b;
#pragma unroll
      for (int l = 0; l < NV; l++) {
        if (CLS == kMatDiag) {
          r[u][l] = cmacx<CLS>(cs, r[u][l], ct, r[u][l]);
        } else {
          const Cx2 mine = r[u][l];
          Cx2 other;
          other.re.x = __shfl_xor_sync(0xffffffffu, mine.re.x, 1 << b);
          other.re.y = __shfl_xor_sync(0xffffffffu, mine.re.y, 1 << b);
          other.im.x = __shfl_xor_sync(0xffffffffu, mine.im.x, 1 << b);
          other.im.y = __shfl_xor_sync(0xffffffffu, mine.im.y, 1 << b);
          r[u][l] = cmacx<CLS>(cs, mine, ct, other);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < KH; j++) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        if ((l >> j) & 1) continue;
        applyx<CLS>(g.hm[j], r[u][l], r[u][l | (1 << j)]);
      }
    }
#pragma unroll
    for (int l = 0; l < NV; l++) {
      uint64_t v = base[u];
#pragma unroll
      for (int j = 0; j < KH; j++)
        if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
      st[v] = join2(r[u][l]);
    }
  }
}

constexpr int kMaxBlockedGates = 96;
struct BlockedArgs {
  uint32_t count;
  uint8_t q[kMaxBlockedGates];
  M2 m[kMaxBlockedGates];
};

// One CTA per 2^b block: stage it in shared memory, apply every gate in
// order with a barrier between gates, write it back once.
__global__ void __launch_bounds__(kThreads)
k_blocked(float2 *__restrict__ st, uint32_t b, uint64_t nblocks, BlockedArgs g) {
  extern __shared__ float4 smem4[];
  float2 *tile = reinterpret_cast<float2 *>(smem4);
  const uint32_t block = 1u << b;
  const uint32_t pairs = block >> 1;
  for (uint64_t blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
    const uint64_t base = blk << b;
    const float4 *src = reinterpret_cast<const float4 *>(st + base);
    for (uint32_t i = threadIdx.x; i < block / 2; i += kThreads) smem4[i] = src[i];
    __syncthreads();
    for (uint32_t k = 0; k < g.count; k++) {
      const uint32_t q = g.q[k], stride = 1u << q;
      const M2 m = g.m[k];
      for (uint32_t t = threadIdx.x; t < pairs; t += kThreads) {
        const uint32_t i = ((t >> q) << (q + 1)) | (t & (stride - 1));
        float2 x = tile[i], y = tile[i + stride];
        apply2(m, x, y);
        tile[i] = x;
        tile[i + stride] = y;
      }
      __syncthreads();
    }
    float4 *dst = reinterpret_cast<float4 *>(st + base);
    for (uint32_t i = threadIdx.x; i < block / 2; i += kThreads) dst[i] = smem4[i];
    __syncthreads();
  }
}

// A block of b <= 10 low wires as a warp tile: lane = vector bits 0..4
// (wires 1..5), registers = wires 6..b-1, wire 0 inside each vector. The
// block's gates run in order on registers and shuffles, with no barrier and
// no shared-memory round trip per gate; every global access is a whole
// 512-byte warp access.
constexpr int kSeqOps = 64;
struct SeqArgs {
  uint32_t count;
  int8_t kind[kSeqOps];   // 0: wire 0, 1: lane bit, 2: register bit
  int8_t arg[kSeqOps];
  int8_t cls[kSeqOps];    // kMat* structure of m
  M2 m[kSeqOps];
};

template <int NV, int J, int CLS>
__device__ __forceinline__ void seq_reg(float4 (&P)[NV], const M2 &m) {
#pragma unroll
  for (int l = 0; l < NV; l++) {
    if ((l >> J) & 1) continue;
    const int h = l | (1 << J);
    float2 pa = lo2(P[l]), pb = lo2(P[h]), qa = hi2(P[l]), qb = hi2(P[h]);
    apply2c(CLS, m, pa, pb);
    apply2c(CLS, m, qa, qb);
    P[l] = pack4(pa, qa);
    P[h] = pack4(pb, qb);
  }
}

template <int KH, int CLS>
__device__ __forceinline__ void seq_op(float4 (&P)[1 << KH], int kind, int arg, const M2 &m,
                                       uint32_t lane) {
  constexpr int NV = 1 << KH;
  if (kind == 0) {
#pragma unroll
    for (int l = 0; l < NV; l++) {
      float2 p0 = lo2(P[l]), p1 = hi2(P[l]);
      apply2c(CLS, m, p0, p1);
      P[l] = pack4(p0, p1);
    }
  } else if (kind == 1) {
    const bool one = (lane >> arg) & 1;
    const float2 s = one ? m.d : m.a, t = one ? m.c : m.b;
#pragma unroll
    for (int l = 0; l < NV; l++) {
      const float4 o = (CLS == kMatDiag) ? P[l] : shfl4(P[l], 1 << arg);
      P[l] = pack4(cmac2c(CLS, s, lo2(P[l]), t, lo2(o)), cmac2c(CLS, s, hi2(P[l]), t, hi2(o)));
    }
  } else {
    if (KH > 0 && arg == 0) seq_reg<NV, 0, CLS>(P, m);
    if (KH > 1 && arg == 1) seq_reg<NV, (KH > 1 ? 1 : 0), CLS>(P, m);
    if (KH > 2 && arg == 2) seq_reg<NV, (KH > 2 ? 2 : 0), CLS>(P, m);
    if (KH > 3 && arg == 3) seq_reg<NV, (KH > 3 ? 3 : 0), CLS>(P, m);
  }
}

template <int KH>
__global__ void __launch_bounds__(kThreads)
k_seq_warp(float4 *__restrict__ st, uint64_t nwsites, SeqArgs g) {
  constexpr int NV = 1 << KH;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gw = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (kThreads / 32);
  for (uint64_t ws = gw; ws < nwsites; ws += nwarps) {
    // registers take vector bits 5 .. 4 + KH (wires 6 .. 5 + KH); the site
    // index fills the bits above them
    const uint64_t base = (ws << (5 + KH)) | lane;
    float4 P[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) P[l] = st[base | (static_cast<uint64_t>(l) << 5)];
    for (uint32_t o = 0; o < g.count; o++) {
      const int kind = g.kind[o], arg = g.arg[o];
      const M2 m = g.m[o];
      switch (g.cls[o]) {
        case kMatReal: seq_op<KH, kMatReal>(P, kind, arg, m, lane); break;
        case kMatRx: seq_op<KH, kMatRx>(P, kind, arg, m, lane); break;
        case kMatDiag: seq_op<KH, kMatDiag>(P, kind, arg, m, lane); break;
        default: seq_op<KH, kMatGeneral>(P, kind, arg, m, lane); break;
      }
    }
#pragma unroll
    for (int l = 0; l < NV; l++) st[base | (static_cast<uint64_t>(l) << 5)] = P[l];
  }
}

// Swap for wires a < b. A0: a == 0, so lane z,w of vector v (a=1,b=0) trades
// with lanes x,y of v|tb (a=0,b=1). Otherwise whole vectors trade.
template <bool A0>
__global__ void __launch_bounds__(kThreads)
k_swap(float4 *__restrict__ st, uint64_t nsites, Fix f, uint64_t ta, uint64_t tb) {
#pragma unroll
  for (int k = 0; k < U; k++) {
    const uint64_t s = site_of(k);
    if (s >= nsites) continue;
    const uint64_t v = expand(s, f);
    if (A0) {
      float4 A = st[v], B = st[v | tb];
      st[v] = make_float4(A.x, A.y, B.x, B.y);
      st[v | tb] = make_float4(A.z, A.w, B.z, B.w);
    } else {
      const float4 A = st[v | ta], B = st[v | tb];
      st[v | ta] = B;
      st[v | tb] = A;
    }
  }
}

Fix make_fix(std::vector<uint32_t> pos, uint64_t set) {
  std::sort(pos.begin(), pos.end());
  Fix f{};
  f.nfix = static_cast<uint32_t>(pos.size());
  for (size_t j = 0; j < pos.size(); j++) f.pos[j] = pos[j];
  f.set = set;
  return f;
}

bool valid_state(const float *p, uint32_t n) {
  return p && n >= 1 && n <= 40 && (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

}  // namespace

namespace qmk_host {
int num_sms() {
  // Read by every launcher, from as many host threads as there are batch
  // lanes; a race to fill an entry only stores the same count twice.
  static std::atomic<int> cache[64];   // zero-initialised: not yet read
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (!v) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      return 152;   // not cached: the next call asks again
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}
}  // namespace qmk_host

using qmk_host::grid_for;
using qmk_host::launch_status;

extern "C" int qmk_init_basis(float *state, uint32_t n, void *stream) {
  if (!valid_state(state, n)) return -1;
  const uint64_t nvec = 1ull << (n - 1);
  k_init_basis<<<grid_for(nvec, kThreads * U), kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<float4 *>(state), nvec);
  return launch_status();
}

// Shared launcher for the controlled family (no controls == dense 2x2).
static int launch_controlled(float *state, uint32_t n, const uint32_t *ctrl,
                             uint32_t nctrl, uint32_t t, const float m8[8],
                             cudaStream_t stream) {
  if (!valid_state(state, n) || t >= n || nctrl > 2) return -1;
  bool ctrl0 = false;
  std::vector<uint32_t> pos;
  uint64_t set = 0;
  for (uint32_t j = 0; j < nctrl; j++) {
    if (ctrl[j] >= n || ctrl[j] == t) return -1;
    for (uint32_t k = 0; k < j; k++)
      if (ctrl[k] == ctrl[j]) return -1;
    if (ctrl[j] == 0) {
      ctrl0 = true;
    } else {
      pos.push_back(ctrl[j] - 1);
      set |= 1ull << (ctrl[j] - 1);
    }
  }
  const M2 m = m2_from(m8);
  float4 *st = reinterpret_cast<float4 *>(state);
  if (t == 0) {
    const Fix f = make_fix(pos, set);
    const uint64_t nsites = 1ull << (n - 1 - f.nfix);
    k_pair<0><<<grid_for(nsites, kThreads * U), kThreads, 0, stream>>>(st, nsites, f, 0, m);
    return launch_status();
  }
  pos.push_back(t - 1);
  const Fix f = make_fix(pos, set);
  if (n - 1 < f.nfix) return -1;
  const uint64_t nsites = 1ull << (n - 1 - f.nfix);
  const uint64_t tbit = 1ull << (t - 1);
  if (ctrl0)
    k_pair<2><<<grid_for(nsites, kThreads * U), kThreads, 0, stream>>>(st, nsites, f, tbit, m);
  else
    k_pair<1><<<grid_for(nsites, kThreads * U), kThreads, 0, stream>>>(st, nsites, f, tbit, m);
  return launch_status();
}

extern "C" int qmk_apply_1q(float *state, uint32_t n, uint32_t q,
                            const float m[8], void *stream) {
  return launch_controlled(state, n, nullptr, 0, q, m, (cudaStream_t)stream);
}

extern "C" int qmk_apply_controlled(float *state, uint32_t n,
                                    uint32_t num_controls,
                                    const uint32_t *controls, uint32_t target,
                                    const float m[8], void *stream) {
  if (num_controls < 1 || num_controls > 2 || !controls) return -1;
  return launch_controlled(state, n, controls, num_controls, target, m,
                           (cudaStream_t)stream);
}

extern "C" int qmk_apply_phase(float *state, uint32_t n, uint64_t mask,
                               float re, float im, void *stream) {
  if (!valid_state(state, n) || mask == 0 || (n < 64 && (mask >> n)) ||
      __builtin_popcountll(mask) > 3)
    return -1;
  std::vector<uint32_t> pos;
  uint64_t set = 0;
  for (uint32_t b = 1; b < n; b++)
    if (mask >> b & 1) {
      pos.push_back(b - 1);
      set |= 1ull << (b - 1);
    }
  const Fix f = make_fix(pos, set);
  const uint64_t nsites = 1ull << (n - 1 - f.nfix);
  const float2 ph = make_float2(re, im);
  float4 *st = reinterpret_cast<float4 *>(state);
  if (mask & 1)
    k_phase<true><<<grid_for(nsites, kThreads * U), kThreads, 0, (cudaStream_t)stream>>>(st, nsites, f, ph);
  else
    k_phase<false><<<grid_for(nsites, kThreads * U), kThreads, 0, (cudaStream_t)stream>>>(st, nsites, f, ph);
  return launch_status();
}

// The narrowest kMat* structure all k matrices share (kMatGeneral if none).
static int8_t common_class(const M2 *ms, int k) {
  bool diag = true, rx = true, real = true;
  for (int j = 0; j < k; j++) {
    const M2 &m = ms[j];
    diag &= m.b.x == 0.0f && m.b.y == 0.0f && m.c.x == 0.0f && m.c.y == 0.0f;
    rx &= m.a.y == 0.0f && m.d.y == 0.0f && m.b.x == 0.0f && m.c.x == 0.0f;
    real &= m.a.y == 0.0f && m.b.y == 0.0f && m.c.y == 0.0f && m.d.y == 0.0f;
  }
  return diag ? kMatDiag : (rx ? kMatRx : (real ? kMatReal : kMatGeneral));
}

template <int KP, bool W0>
static void launch_group(float4 *st, uint64_t nsites, const GroupArgs &g, int cls,
                         cudaStream_t stream) {
  const unsigned grid = grid_for(nsites, kThreads);
  switch (cls) {
    case kMatDiag: k_group<KP, W0, kMatDiag><<<grid, kThreads, 0, stream>>>(st, nsites, g); break;
    case kMatRx: k_group<KP, W0, kMatRx><<<grid, kThreads, 0, stream>>>(st, nsites, g); break;
    case kMatReal: k_group<KP, W0, kMatReal><<<grid, kThreads, 0, stream>>>(st, nsites, g); break;
    default: k_group<KP, W0, kMatGeneral><<<grid, kThreads, 0, stream>>>(st, nsites, g); break;
  }
}

template <bool W0, int CLS>
static int launch_group5_pair_cls(float4 *st, uint64_t nsites, const GroupArgs &g,
                                  cudaStream_t s) {
  const size_t smem = static_cast<size_t>(kThreads / 32) * kPairVecs * 32 * sizeof(float4);
  // The opt-in above 48 KiB is per device; set it once on each.
  static std::atomic<bool> opted[64];   // zero-initialised: false
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_group5_pair<W0, CLS>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  k_group5_pair<W0, CLS><<<grid_for(nsites, kThreads / 2), kThreads, smem, s>>>(st, nsites, g);
  return launch_status();
}

template <int WB, bool W0, int CLS>
static int launch_group_blk_cls(float4 *st, uint64_t nsites, const BlkGroupArgs &g,
                                cudaStream_t s) {
  constexpr int SPB = (kThreads / 32) >> WB;
  const size_t smem = static_cast<size_t>(SPB) * (16 << WB) * 32 * sizeof(float4);
  // The opt-in above 48 KiB is per device; set it once on each.
  static std::atomic<bool> opted[64];   // zero-initialised: false
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_group_blk<WB, W0, CLS>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  // Resident blocks only: each loops over its sites.
  const unsigned grid = std::min<unsigned>(grid_for(nsites, SPB),
                                           static_cast<unsigned>(qmk_host::num_sms()) * 2);
  k_group_blk<WB, W0, CLS><<<grid, kThreads, smem, s>>>(st, nsites, g);
  return launch_status();
}

template <int WB, bool W0>
static int launch_group_blk(float4 *st, uint64_t nsites, const BlkGroupArgs &g, int cls,
                            cudaStream_t s) {
  switch (cls) {
    case kMatDiag: return launch_group_blk_cls<WB, W0, kMatDiag>(st, nsites, g, s);
    case kMatRx: return launch_group_blk_cls<WB, W0, kMatRx>(st, nsites, g, s);
    case kMatReal: return launch_group_blk_cls<WB, W0, kMatReal>(st, nsites, g, s);
    default: return launch_group_blk_cls<WB, W0, kMatGeneral>(st, nsites, g, s);
  }
}

template <bool W0>
static int launch_group5_pair(float4 *st, uint64_t nsites, const GroupArgs &g, int cls,
                              cudaStream_t s) {
  switch (cls) {
    case kMatDiag: return launch_group5_pair_cls<W0, kMatDiag>(st, nsites, g, s);
    case kMatRx: return launch_group5_pair_cls<W0, kMatRx>(st, nsites, g, s);
    case kMatReal: return launch_group5_pair_cls<W0, kMatReal>(st, nsites, g, s);
    default: return launch_group5_pair_cls<W0, kMatGeneral>(st, nsites, g, s);
  }
}

template <int KH, bool W0>
static void launch_group_warp(float4 *st, uint64_t nw, const WarpGroupArgs &g, int cls,
                              unsigned grid, cudaStream_t s) {
  switch (cls) {
    case kMatDiag: k_group_warp<KH, W0, kMatDiag><<<grid, kThreads, 0, s>>>(st, nw, g); break;
    case kMatRx: k_group_warp<KH, W0, kMatRx><<<grid, kThreads, 0, s>>>(st, nw, g); break;
    case kMatReal: k_group_warp<KH, W0, kMatReal><<<grid, kThreads, 0, s>>>(st, nw, g); break;
    default: k_group_warp<KH, W0, kMatGeneral><<<grid, kThreads, 0, s>>>(st, nw, g); break;
  }
}

extern "C" int qmk_apply_group(float *state, uint32_t n, uint32_t k,
                               const uint32_t *qubits, const float *mats,
                               void *stream) {
  if (!valid_state(state, n) || k < 1 || k > 10 || !qubits || !mats) return -1;
  for (uint32_t j = 0; j < k; j++) {
    if (qubits[j] >= n) return -1;
    if (j && qubits[j] <= qubits[j - 1]) return -1;  // ascending, distinct
  }
  const bool w0 = qubits[0] == 0;
  cudaStream_t s = (cudaStream_t)stream;
  float4 *st = reinterpret_cast<float4 *>(state);
  {
    // Wires 1..5 sit inside one warp's 512 bytes: the warp-tile kernel keeps
    // every access a whole 512-byte warp access.
    WarpGroupArgs wg{};
    int kh = 0;
    for (uint32_t j = 0; j < k; j++) {
      const uint32_t q = qubits[j];
      if (q == 0) {
        wg.m0 = m2_from(mats + 8 * j);
      } else if (q <= 5) {
        wg.lbit[wg.nlow] = q - 1;
        wg.lm[wg.nlow] = m2_from(mats + 8 * j);
        wg.nlow++;
      } else {
        if (kh == 4) { kh = -1; break; }
        wg.hpos[kh] = q - 6;
        wg.hm[kh] = mx_from(m2_from(mats + 8 * j));
        kh++;
      }
    }
    if (wg.nlow > 0 && kh >= 0 && n >= 6u + static_cast<uint32_t>(kh)) {
      const uint64_t nw = 1ull << (n - 6 - kh);
      const int uw = kh <= 1 ? 4 : (kh == 2 ? 2 : 1);
      const unsigned grid = grid_for(nw, (kThreads / 32) * uw);
      std::vector<M2> all;
      for (uint32_t j = 0; j < k; j++) all.push_back(m2_from(mats + 8 * j));
      const int cls = common_class(all.data(), static_cast<int>(k));
      switch (kh * 2 + (w0 ? 1 : 0)) {
        case 0: launch_group_warp<0, false>(st, nw, wg, cls, grid, s); break;
        case 1: launch_group_warp<0, true>(st, nw, wg, cls, grid, s); break;
        case 2: launch_group_warp<1, false>(st, nw, wg, cls, grid, s); break;
        case 3: launch_group_warp<1, true>(st, nw, wg, cls, grid, s); break;
        case 4: launch_group_warp<2, false>(st, nw, wg, cls, grid, s); break;
        case 5: launch_group_warp<2, true>(st, nw, wg, cls, grid, s); break;
        case 6: launch_group_warp<3, false>(st, nw, wg, cls, grid, s); break;
        case 7: launch_group_warp<3, true>(st, nw, wg, cls, grid, s); break;
        case 8: launch_group_warp<4, false>(st, nw, wg, cls, grid, s); break;
        case 9: launch_group_warp<4, true>(st, nw, wg, cls, grid, s); break;
        default: return -1;
      }
      return launch_status();
    }
  }
  {
    // Six or seven wires >= 6 (and perhaps wire 0): the block route.
    const uint32_t kh = k - (w0 ? 1u : 0u);
    bool high_only = true;
    for (uint32_t j = 0; j < k; j++) high_only &= qubits[j] == 0 || qubits[j] >= 6;
    if (high_only && (kh == 6 || kh == 7) && n - 1 >= 5 + kh) {
      BlkGroupArgs bg{};
      uint32_t kb = 0;
      std::vector<M2> all;
      for (uint32_t j = 0; j < k; j++) {
        const M2 m = m2_from(mats + 8 * j);
        all.push_back(m);
        if (qubits[j] == 0) {
          bg.m0 = m;
        } else {
          bg.pos[kb] = qubits[j] - 1;
          bg.m[kb] = m;
          kb++;
        }
      }
      const int cls = common_class(all.data(), static_cast<int>(k));
      const uint64_t nsites = 1ull << (n - 1 - 5 - kh);
      if (kh == 6) return w0 ? launch_group_blk<2, true>(st, nsites, bg, cls, s)
                             : launch_group_blk<2, false>(st, nsites, bg, cls, s);
      return w0 ? launch_group_blk<3, true>(st, nsites, bg, cls, s)
                : launch_group_blk<3, false>(st, nsites, bg, cls, s);
    }
  }
  if (k - (w0 ? 1u : 0u) > 5) return -1;  // register path: at most five wires >= 1
  GroupArgs g{};
  int kp = 0;
  for (uint32_t j = 0; j < k; j++) {
    if (qubits[j] == 0) {
      g.m0 = m2_from(mats + 8 * j);
    } else {
      g.pos[kp] = qubits[j] - 1;
      g.m[kp] = m2_from(mats + 8 * j);
      kp++;
    }
  }
  if (static_cast<uint32_t>(kp) > n - 1) return -1;
  const uint64_t nsites = 1ull << (n - 1 - kp);
  std::vector<M2> all;
  for (uint32_t j = 0; j < k; j++) all.push_back(m2_from(mats + 8 * j));
  const int cls = common_class(all.data(), static_cast<int>(k));
  switch (kp * 2 + (w0 ? 1 : 0)) {
    case 1: launch_group<0, true>(st, nsites, g, cls, s); break;
    case 2: launch_group<1, false>(st, nsites, g, cls, s); break;
    case 3: launch_group<1, true>(st, nsites, g, cls, s); break;
    case 4: launch_group<2, false>(st, nsites, g, cls, s); break;
    case 5: launch_group<2, true>(st, nsites, g, cls, s); break;
    case 6: launch_group<3, false>(st, nsites, g, cls, s); break;
    case 7: launch_group<3, true>(st, nsites, g, cls, s); break;
    case 8: launch_group<4, false>(st, nsites, g, cls, s); break;
    case 9: launch_group<4, true>(st, nsites, g, cls, s); break;
    // Five register wires: on warp pairs once a pair's 32 sites exist.
    case 10:
      if (nsites >= 32) return launch_group5_pair<false>(st, nsites, g, cls, s);
      launch_group<5, false>(st, nsites, g, cls, s);
      break;
    case 11:
      if (nsites >= 32) return launch_group5_pair<true>(st, nsites, g, cls, s);
      launch_group<5, true>(st, nsites, g, cls, s);
      break;
    default: return -1;
  }
  return launch_status();
}

extern "C" int qmk_apply_blocked(float *state, uint32_t n, uint32_t b,
                                 uint32_t count, const uint32_t *qubits,
                                 const float *mats, void *stream) {
  if (!valid_state(state, n) || b < 2 || b > 14 || b > n) return -1;
  if (count && (!qubits || !mats)) return -1;
  for (uint32_t k = 0; k < count; k++)
    if (qubits[k] >= b) return -1;
  const uint32_t tile = b < 6 ? 6u : b;           // wires the warp tile spans
  if (b <= 10 && n >= tile) {
    const int kh = static_cast<int>(tile) - 6;
    const uint64_t nw = 1ull << (n - 1 - 5 - kh);
    const unsigned grid = grid_for(nw, kThreads / 32);
    float4 *st = reinterpret_cast<float4 *>(state);
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t done = 0;
    do {
      SeqArgs g{};
      g.count = std::min<uint32_t>(count - done, kSeqOps);
      for (uint32_t k = 0; k < g.count; k++) {
        const uint32_t q = qubits[done + k];
        g.kind[k] = q == 0 ? 0 : (q <= 5 ? 1 : 2);
        g.arg[k] = static_cast<int8_t>(q == 0 ? 0 : (q <= 5 ? q - 1 : q - 6));
        g.m[k] = m2_from(mats + 8 * (done + k));
        g.cls[k] = m2_class(g.m[k]);
      }
      switch (kh) {
        case 0: k_seq_warp<0><<<grid, kThreads, 0, s>>>(st, nw, g); break;
        case 1: k_seq_warp<1><<<grid, kThreads, 0, s>>>(st, nw, g); break;
        case 2: k_seq_warp<2><<<grid, kThreads, 0, s>>>(st, nw, g); break;
        case 3: k_seq_warp<3><<<grid, kThreads, 0, s>>>(st, nw, g); break;
        default: k_seq_warp<4><<<grid, kThreads, 0, s>>>(st, nw, g); break;
      }
      done += g.count;
    } while (done < count);
    return launch_status();
  }
  const size_t smem = sizeof(float2) << b;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_blocked, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
  }
  const uint64_t nblocks = 1ull << (n - b);
  // Runs longer than one argument block go in consecutive passes; each pass
  // applies its gates in order, so the composition is unchanged.
  uint32_t done = 0;
  do {
    BlockedArgs g{};
    g.count = std::min<uint32_t>(count - done, kMaxBlockedGates);
    for (uint32_t k = 0; k < g.count; k++) {
      g.q[k] = static_cast<uint8_t>(qubits[done + k]);
      g.m[k] = m2_from(mats + 8 * (done + k));
    }
    const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(nblocks, 1u << 20));
    k_blocked<<<grid, kThreads, smem, (cudaStream_t)stream>>>(
        reinterpret_cast<float2 *>(state), b, nblocks, g);
    int rc = launch_status();
    if (rc) return rc;
    done += g.count;
  } while (done < count);
  return 0;
}

extern "C" int qmk_apply_swap(float *state, uint32_t n, uint32_t a, uint32_t b,
                              void *stream) {
  if (!valid_state(state, n) || a >= n || b >= n) return -1;
  if (a == b) return 0;
  if (a > b) std::swap(a, b);
  float4 *st = reinterpret_cast<float4 *>(state);
  cudaStream_t s = (cudaStream_t)stream;
  if (a == 0) {
    const Fix f = make_fix({b - 1}, 0);
    const uint64_t nsites = 1ull << (n - 2);
    k_swap<true><<<grid_for(nsites, kThreads * U), kThreads, 0, s>>>(st, nsites, f, 0, 1ull << (b - 1));
  } else {
    const Fix f = make_fix({a - 1, b - 1}, 0);
    const uint64_t nsites = 1ull << (n - 3);
    k_swap<false><<<grid_for(nsites, kThreads * U), kThreads, 0, s>>>(
        st, nsites, f, 1ull << (a - 1), 1ull << (b - 1));
  }
  return launch_status();
}
