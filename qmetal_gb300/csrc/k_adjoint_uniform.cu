// k_adjoint_uniform.cu -- window tiles whose op list is fixed at compile
// time: every wire of the tile carries the same short sequence of rotations
// (one RX, RY or RZ per wire -- the mixer and rotation layers of QAOA and
// TFIM circuits -- or RZ then RY, the backward order of a hardware-efficient
// layer). With the sequence known there is no per-op dispatch, the gradient
// partials sit in registers at fixed indices, and the compiler may interleave
// one op's shuffles with another's arithmetic. The per-op arithmetic is that
// of the general tiles (k_adjoint_tiles.cu, through kadjoint_ops.cuh); the
// pipelined warp-pair tiles run the split wire's ops first.
#include <algorithm>
#include <atomic>

#include "kadjoint_ops.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

namespace qmk_adj {
namespace {

// Matrices of a uniform tile: op k of wire 0, of lane wire i, of register
// wire j.
struct UniArgs {
  uint32_t hpos[6];   // wires >= 6: vector bit - 5, ascending
  uint32_t lbit[5];   // lane wires' vector bits, in op order
  M2 m0[2], ml[5][2], mh[6][2];
  // Tiles of RZ and RY on every wire: the RZ undos of the register wires
  // of one layout as one phase per register vector (index l: the product of
  // a or d of each wire's RZ by bit j of l), for the wires of mh[0..2]
  // (first layout) and of mh[3..] (second layout of a block tile). In the
  // tile of wire 0 and wires 1..5, ph[0][2 l + b] also takes wire 0's entry
  // by amplitude bit b, and lph[lane] is the lane wires' product by the
  // lane's bits.
  float2 ph[2][8];
  float2 lph[32];
};

// The M ops of one wire: op k has class Ck and generator Gk.
template <int M, int NV, int C0, int G0, int C1, int G1>
__device__ __forceinline__ void w0_ops(float4 (&P)[NV], float4 (&L)[NV], const M2 (&m)[2],
                                       float *acc) {
  acc[0] += wire0_op<NV, C0>(P, L, G0, m[0]);
  if constexpr (M > 1) acc[1] += wire0_op<NV, C1>(P, L, G1, m[1]);
}
template <int M, int NV, int C0, int G0, int C1, int G1>
__device__ __forceinline__ void lane_ops(float4 (&P)[NV], float4 (&L)[NV], uint32_t bit,
                                         uint32_t lane, const M2 (&m)[2], float *acc) {
  const int mask = 1 << bit;
  const bool one = (lane >> bit) & 1;
  acc[0] += lane_op_g<NV, C0, G0>(P, L, mask, one, m[0]);
  if constexpr (M > 1) acc[1] += lane_op_g<NV, C1, G1>(P, L, mask, one, m[1]);
}
template <int M, int NV, int J, int C0, int G0, int C1, int G1>
__device__ __forceinline__ void reg_ops(float4 (&P)[NV], float4 (&L)[NV], const M2 (&m)[2],
                                        float *acc) {
  acc[0] += reg_op<NV, J, C0>(P, L, G0, m[0]);
  if constexpr (M > 1) acc[1] += reg_op<NV, J, C1>(P, L, G1, m[1]);
}

// The RZ ops of K register wires (bits 0..K-1 of a vector's register
// index) at once, for tiles with an RZ on every wire. Their gradients need
// only q = Im(conj(l) p) of each amplitude, which the other wires' RZ phases
// leave alone and which commutes with the other wires' ops: wire j's
// overlap is the sum over vectors of +-Q (Q = q of both amplitudes, sign by
// bit j), as pair by pair in reg_op. Then one phase per vector undoes all K
// RZs: ph[l] is the product of the wires' diagonal entries picked by l.
template <int NV, int K>
__device__ __forceinline__ void rz_block(float4 (&P)[NV], float4 (&L)[NV], const float2 (&ph)[8],
                                         float *acc, int stride) {
  float a[K];
#pragma unroll
  for (int j = 0; j < K; j++) a[j] = 0.0f;
#pragma unroll
  for (int l = 0; l < NV; l++) {
    const float q = (L[l].x * P[l].y - L[l].y * P[l].x) + (L[l].z * P[l].w - L[l].w * P[l].z);
#pragma unroll
    for (int j = 0; j < K; j++) a[j] += ((l >> j) & 1) ? -q : q;
    const float2 f = ph[l & 7];
    P[l] = pack4(cmul(f, lo2(P[l])), cmul(f, hi2(P[l])));
    L[l] = pack4(cmul(f, lo2(L[l])), cmul(f, hi2(L[l])));
  }
#pragma unroll
  for (int j = 0; j < K; j++) acc[j * stride] += a[j];
}

// The RZ ops of wire 0, the five lane wires and KH register wires at once
// (the tile of wires 0..5 with an RZ on every wire): wire 0's overlap is
// q0 - q1 of each vector's two amplitudes, a register wire's +-Q as in
// rz_block, and a lane wire's the lane's sign times the sum of Q over the
// thread's vectors (sl; the sign goes on after the last site), as is that of
// a wire split across a warp pair (by the warp's half). One phase per
// amplitude, lp ph[2 l + b], undoes them all (lp: the lane wires' product,
// and the split wire's entry).
template <int NV, int KH>
__device__ __forceinline__ void rz_wide(float4 (&P)[NV], float4 (&L)[NV], const float2 *ph,
                                        float2 lp, float &a0, float &sl, float *ar, int stride) {
  static_assert(NV <= 8, "three register wires at most (a table of 2 NV phases)");
  float r[KH > 0 ? KH : 1];
#pragma unroll
  for (int j = 0; j < KH; j++) r[j] = 0.0f;
#pragma unroll
  for (int l = 0; l < NV; l++) {
    const float q0 = L[l].x * P[l].y - L[l].y * P[l].x;
    const float q1 = L[l].z * P[l].w - L[l].w * P[l].z;
    a0 += q0 - q1;
    const float q = q0 + q1;
    sl += q;
#pragma unroll
    for (int j = 0; j < KH; j++) r[j] += ((l >> j) & 1) ? -q : q;
    const float2 f0 = cmul(lp, ph[2 * l]), f1 = cmul(lp, ph[2 * l + 1]);
    P[l] = pack4(cmul(f0, lo2(P[l])), cmul(f1, hi2(P[l])));
    L[l] = pack4(cmul(f0, lo2(L[l])), cmul(f1, hi2(L[l])));
  }
#pragma unroll
  for (int j = 0; j < KH; j++) ar[j * stride] += r[j];
}

// The ops of K register wires of a tile whose wires carry RZ and RY (in
// either undo order): the RZs of all K wires as one phase, the RYs one wire
// at a time. M2 m[j][k] is op k of wire j; acc[j * 2 + k] its gradient.
template <int NV, int K, int C0>
__device__ __forceinline__ void rzry_ops(float4 (&P)[NV], float4 (&L)[NV], const M2 (*m)[2],
                                         const float2 (&ph)[8], float *acc) {
  constexpr int RZ = C0 == kMatDiag ? 0 : 1;   // the RZ's position in undo order
  if constexpr (RZ == 0) rz_block<NV, K>(P, L, ph, acc, 2);
  acc[1 - RZ] += reg_op<NV, 0, kMatReal>(P, L, 2, m[0][1 - RZ]);
  if constexpr (K > 1) acc[2 + 1 - RZ] += reg_op<NV, (K > 1 ? 1 : 0), kMatReal>(P, L, 2, m[1][1 - RZ]);
  if constexpr (K > 2) acc[4 + 1 - RZ] += reg_op<NV, (K > 2 ? 2 : 0), kMatReal>(P, L, 2, m[2][1 - RZ]);
  if constexpr (RZ == 1) rz_block<NV, K>(P, L, ph, acc + 1, 2);
}

// One op on the wire split across a warp pair: the pair trades vectors
// through shared memory unless the op is diagonal with a Z (or no)
// generator.
template <int C, int G>
__device__ __forceinline__ float split_one(float4 (&P)[kPairNV], float4 (&L)[kPairNV],
                                           float4 *mine_p, float4 *mine_l, const float4 *oth_p,
                                           const float4 *oth_l, bool one, uint32_t pair,
                                           const M2 &m) {
  constexpr bool kNeed = C != kMatDiag || G == 1 || G == 2;
  if (kNeed) {
#pragma unroll
    for (int l = 0; l < kPairNV; l++) {
      mine_p[l * 32] = P[l];
      mine_l[l * 32] = L[l];
    }
    pair_sync(pair);
  }
  const float ov = split_op_g<C, G>(P, L, oth_p, oth_l, one, m);
  if (kNeed) pair_sync(pair);
  return ov;
}

// Bulk copies through the TMA engine: one 512-byte row per instruction,
// completion counted in bytes on a shared-memory mbarrier. Every wait is
// bounded: a wait that gives up is counted in the workspace's wait counter
// (Area::waits, read by the host after the pass), the warp stops streaming
// and drains its copies in flight before it exits, and the kernel goes on,
// so it cannot hang. A test may shorten the bound of the in-loop waits
// through the workspace (Area::polls; qmk_set_wait_poll_limit), down to
// giving up at once; the drain before exit always keeps the full bound, so
// every copy lands before its block ends.
constexpr uint32_t kMaxWaitPolls = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *mb, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mb, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_row(void *dst, const void *src, uint32_t bytes, uint64_t *mb) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mb))
      : "memory");
}
// Order this thread's earlier shared-memory accesses (and, after a barrier,
// its partners') before the async proxy's next writes to the same bytes.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Bounded wait for a phase of the barrier; false if it gave up. Called by a
// whole warp, which reduces the answer to one warp-uniform flag.
__device__ __forceinline__ bool mbar_wait(uint64_t *mb, uint32_t parity,
                                          uint32_t limit = kMaxWaitPolls) {
  for (uint32_t polls = 0; polls < limit; polls++)
    if (mbar_try_wait(mb, parity)) return true;
  return false;
}

// The in-loop wait bound of this workspace: the full bound unless a test set
// one (stored as polls + 1, so that the zeroed workspace means the default).
__device__ __forceinline__ uint32_t wait_limit(const Area &a) {
  const uint32_t v = *a.polls;
  return v == 0 ? kMaxWaitPolls : min(v - 1, kMaxWaitPolls);
}

// Four register wires on a warp pair (the fourth split across the pair),
// optionally with wire 0 and the five lane wires. With the op list this
// short the tile is bound by load latency; where a round has enough work to
// hide a load behind (two ops per wire, or the ten-wire tile), the warp's
// vectors for the next round stream into its shared-memory slots while the
// current round computes, as 16 bulk copies of one 512-byte row each issued
// by one lane: a round reads its slots, runs the split wire's ops first
// (they commute with the other wires' ops; their exchanges go through the
// same slots), then sends out the next round's copies and runs the rest.
// The four-op tile loads directly (measured: the staging costs it more
// than it hides).
template <bool W0, int NL, int M, int C0, int G0, int C1, int G1>
__global__ void __launch_bounds__(kThreads, 2)
k_adj_pair_uni(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nwsites, UniArgs g,
               Area a, OutSlots<M *((W0 ? 1 : 0) + NL + 4)> out) {
  constexpr int NV = kPairNV;
  constexpr int NOPS = M * ((W0 ? 1 : 0) + NL + 4);
  constexpr int LANE0 = M * (W0 ? 1 : 0), REG0 = LANE0 + M * NL;
  constexpr bool kPipe = M > 1 || W0;
  // Wires 0..5 and four wires >= 6 with RZ then RY (undo order) on every
  // wire: the RZs of all ten go as one phase (rz_wide), the split wire's by
  // the warp's half.
  constexpr bool kRzRy = M == 2 && W0 && NL == 5 && C0 == kMatDiag && G0 == 3 &&
                         C1 == kMatReal && G1 == 2;
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
  float sl = 0.0f;   // kRzRy: the lane and split wires' RZ overlap before its sign
  auto site = [&](uint64_t r) {
    return r * per_round + static_cast<uint64_t>(blockIdx.x) * (kThreads / 64) + (warp >> 1);
  };
  auto base_of = [&](uint64_t ws) {
    uint64_t b = ws;
#pragma unroll
    for (int j = 0; j < 4; j++) b = ins0(b, g.hpos[j]);
    return (b << 5) | lane | (static_cast<uint64_t>(half) << (g.hpos[3] + 5));
  };
  auto vec_of = [&](uint64_t base, int l) {
    uint64_t v = base;
#pragma unroll
    for (int j = 0; j < 3; j++)
      if ((l >> j) & 1) v |= 1ull << (g.hpos[j] + 5);
    return v;
  };
  __shared__ uint64_t mbar[kThreads / 32];   // one per warp: its next round's rows
  uint32_t parity = 0;
  // A wait that gives up (counted in the workspace; the pass's results are
  // then refused by the host) leaves one batch of copies in flight: the warp
  // issues no more and waits for none (its slots' contents no longer
  // matter), and before it exits waits once more, bounded, for that batch
  // to land.
  bool stalled = false;
  uint32_t stalled_parity = 0;
  uint32_t limit = kMaxWaitPolls;
  if constexpr (kPipe) {
    limit = wait_limit(a);
    if (lane == 0) mbar_init(&mbar[warp], 1);
    fence_proxy_async();
    __syncwarp();
  }
  // The next round's rows of this warp (8 of each state), if it has one.
  auto prefetch = [&](uint64_t r) {
    const uint64_t ws = site(r);
    if (r < rounds && ws < nwsites && !stalled) {
      const uint64_t row0 = base_of(ws) & ~31ull;
      __syncwarp();
      if (lane == 0) {
        fence_proxy_async();
        mbar_expect_tx(&mbar[warp], 2 * NV * 32 * sizeof(float4));
#pragma unroll
        for (int l = 0; l < NV; l++) {
          const uint64_t v = vec_of(row0, l);
          bulk_row(mine_p - lane + l * 32, psi + v, 32 * sizeof(float4), &mbar[warp]);
          bulk_row(mine_l - lane + l * 32, lam + v, 32 * sizeof(float4), &mbar[warp]);
        }
      }
    }
  };
  if constexpr (kPipe) prefetch(0);
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t ws = site(r);
    const bool active = ws < nwsites;
    const uint64_t base = active ? base_of(ws) : 0;
    if constexpr (kPipe) {
      if (active && !stalled) {
        const bool landed = mbar_wait(&mbar[warp], parity, limit);
        if (!__all_sync(0xffffffffu, landed)) {
          if (lane == 0) atomicAdd(a.waits, 1u);
          stalled = true;
          stalled_parity = parity;
        }
        parity ^= 1u;
      }
    }
    float4 P[NV], L[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      if (!active) {
        P[l] = L[l] = make_float4(0.f, 0.f, 0.f, 0.f);
      } else if (kPipe) {
        P[l] = mine_p[l * 32];
        L[l] = mine_l[l * 32];
      } else {
        const uint64_t v = vec_of(base, l);
        P[l] = psi[v];
        L[l] = lam[v];
      }
    }
    auto split_ops = [&]() {
      accf[REG0 + 3 * M] += split_one<C0, G0>(P, L, mine_p, mine_l, oth_p, oth_l, half != 0,
                                              warp >> 1, g.mh[3][0]);
      if constexpr (M > 1)
        accf[REG0 + 3 * M + 1] += split_one<C1, G1>(P, L, mine_p, mine_l, oth_p, oth_l,
                                                    half != 0, warp >> 1, g.mh[3][1]);
    };
    // Pipelined: the split wire's ops first. They rewrite all of P and L, so
    // by their end this thread's slot reads are done; the partner's reads of
    // its slots end at the barrier that closes an exchange.
    if constexpr (kRzRy) {
      // every wire's RZ as one phase, then the split wire's RY (an exchange),
      // the next round's copies, and the other wires' RYs
      {
        // the lane wires' phase and the split wire's, formed each round (kept
        // across the loop it pushed the tile into spills)
        const float2 lp = cmul(g.lph[lane], half ? g.mh[3][0].d : g.mh[3][0].a);
        rz_wide<NV, 3>(P, L, &g.ph[0][0], lp, accf[0], sl, accf + REG0, M);
      }
      accf[REG0 + 3 * M + 1] += split_one<kMatReal, 2>(P, L, mine_p, mine_l, oth_p, oth_l,
                                                        half != 0, warp >> 1, g.mh[3][1]);
      prefetch(r + 1);
      accf[1] += wire0_op<NV, kMatReal>(P, L, 2, g.m0[1]);
#pragma unroll
      for (int k = 0; k < NL; k++)
        accf[LANE0 + M * k + 1] += lane_op_g<NV, kMatReal, 2>(
            P, L, 1 << g.lbit[k], (lane >> g.lbit[k]) & 1, g.ml[k][1]);
      accf[REG0 + 1] += reg_op<NV, 0, kMatReal>(P, L, 2, g.mh[0][1]);
      accf[REG0 + M + 1] += reg_op<NV, 1, kMatReal>(P, L, 2, g.mh[1][1]);
      accf[REG0 + 2 * M + 1] += reg_op<NV, 2, kMatReal>(P, L, 2, g.mh[2][1]);
    } else {
      if constexpr (kPipe) {
        split_ops();
        prefetch(r + 1);
      }
      if constexpr (W0) w0_ops<M, NV, C0, G0, C1, G1>(P, L, g.m0, accf);
#pragma unroll
      for (int k = 0; k < NL; k++)
        lane_ops<M, NV, C0, G0, C1, G1>(P, L, g.lbit[k], lane, g.ml[k], accf + LANE0 + M * k);
      reg_ops<M, NV, 0, C0, G0, C1, G1>(P, L, g.mh[0], accf + REG0);
      reg_ops<M, NV, 1, C0, G0, C1, G1>(P, L, g.mh[1], accf + REG0 + M);
      reg_ops<M, NV, 2, C0, G0, C1, G1>(P, L, g.mh[2], accf + REG0 + 2 * M);
      if constexpr (!kPipe) split_ops();
    }
    // A warp that gave up a wait computed on slots that may not have held
    // this round's rows: it leaves the states alone (the host refuses the
    // pass and resets the simulator's state).
    if (active && !stalled) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        const uint64_t v = vec_of(base, l);
        psi[v] = P[l];
        lam[v] = L[l];
      }
    }
  }
  if constexpr (kPipe) {
    if (stalled && !__all_sync(0xffffffffu, mbar_wait(&mbar[warp], stalled_parity)) && lane == 0)
      atomicAdd(a.waits, 1u);
  }
  if constexpr (kRzRy) {
#pragma unroll
    for (int k = 0; k < NL; k++)
      accf[LANE0 + M * k] += ((lane >> g.lbit[k]) & 1) ? -sl : sl;
    accf[REG0 + 3 * M] += half ? -sl : sl;
  }
  double acc[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) acc[t] = accf[t];
  finish<NOPS>(acc, NOPS, a, out);
}

// KH <= 3 register wires on one warp, optionally with wire 0 and the five
// lane wires.
template <int KH, bool W0, int NL, int M, int C0, int G0, int C1, int G1>
__global__ void __launch_bounds__(kThreads, 2)
k_adj_warp_uni(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nwsites, UniArgs g,
               Area a, OutSlots<M *((W0 ? 1 : 0) + NL + KH)> out) {
  constexpr int NV = 1 << KH;
  constexpr int NOPS = M * ((W0 ? 1 : 0) + NL + KH);
  constexpr int LANE0 = M * (W0 ? 1 : 0), REG0 = LANE0 + M * NL;
  // Wires 0..5 and up to two register wires, RZ and RY on every wire (either
  // undo order): the RZs of all of them go as one phase (rz_wide).
  constexpr bool kRzRy = M == 2 && W0 && NL == 5 && KH <= 2 &&
                         ((C0 == kMatDiag && G0 == 3 && C1 == kMatReal && G1 == 2) ||
                          (C0 == kMatReal && G0 == 2 && C1 == kMatDiag && G1 == 3));
  constexpr int RZ = C0 == kMatDiag ? 0 : 1;   // the RZ's position in undo order
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gw = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (kThreads / 32);
  float accf[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) accf[t] = 0.0f;
  float sl = 0.0f;   // kRzRy: the lane wires' RZ overlap before its sign
  const float2 lp = kRzRy ? g.lph[lane] : make_float2(1.0f, 0.0f);
  // The RY ops of wire 0, the lane wires and the register wires (kRzRy).
  auto ry_all = [&](float4(&P)[NV], float4(&L)[NV]) {
    accf[1 - RZ] += wire0_op<NV, kMatReal>(P, L, 2, g.m0[1 - RZ]);
#pragma unroll
    for (int k = 0; k < NL; k++)
      accf[LANE0 + M * k + 1 - RZ] += lane_op_g<NV, kMatReal, 2>(
          P, L, 1 << g.lbit[k], (lane >> g.lbit[k]) & 1, g.ml[k][1 - RZ]);
    if constexpr (KH > 0)
      accf[REG0 + 1 - RZ] += reg_op<NV, 0, kMatReal>(P, L, 2, g.mh[0][1 - RZ]);
    if constexpr (KH > 1)
      accf[REG0 + M + 1 - RZ] += reg_op<NV, (KH > 1 ? 1 : 0), kMatReal>(P, L, 2, g.mh[1][1 - RZ]);
  };
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
    if constexpr (kRzRy) {
      if constexpr (RZ == 1) ry_all(P, L);
      rz_wide<NV, KH>(P, L, &g.ph[0][0], lp, accf[RZ], sl, accf + REG0 + RZ, M);
      if constexpr (RZ == 0) ry_all(P, L);
    } else {
      if constexpr (W0) w0_ops<M, NV, C0, G0, C1, G1>(P, L, g.m0, accf);
#pragma unroll
      for (int k = 0; k < NL; k++)
        lane_ops<M, NV, C0, G0, C1, G1>(P, L, g.lbit[k], lane, g.ml[k], accf + LANE0 + M * k);
      if constexpr (KH > 0) reg_ops<M, NV, 0, C0, G0, C1, G1>(P, L, g.mh[0], accf + REG0);
      if constexpr (KH > 1) reg_ops<M, NV, (KH > 1 ? 1 : 0), C0, G0, C1, G1>(P, L, g.mh[1], accf + REG0 + M);
      if constexpr (KH > 2) reg_ops<M, NV, (KH > 2 ? 2 : 0), C0, G0, C1, G1>(P, L, g.mh[2], accf + REG0 + 2 * M);
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
  if constexpr (kRzRy) {
#pragma unroll
    for (int k = 0; k < NL; k++)
      accf[LANE0 + M * k + RZ] += ((lane >> g.lbit[k]) & 1) ? -sl : sl;
  }
  double acc[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) acc[t] = accf[t];
  finish<NOPS>(acc, NOPS, a, out);
}

// Five or six wires >= 6 per pass on a block tile: a site is 2^(3 + WB)
// rows of 32 vectors of each state, held by 2^WB warps with eight vectors of
// each state per thread. Register bits 0..2 of a thread are the site's first
// three wires and its warp's index in the site the others, so the first three
// wires' ops run in registers; the site then trades places through shared
// memory -- WB of the register bits become warp bits and the warp bits
// register bits -- and the remaining wires' ops run in registers too. One
// shared-memory round trip per round replaces an exchange per op on a wire
// split across warps. The rows stream in by bulk copies (one batch per warp:
// the rows of its first layout), and the next round's copies go out once
// every warp of the site has read its second layout, so they overlap the
// second half of the arithmetic and the stores. Waits are bounded as in
// k_adj_pair_uni. Stores go from the second layout: every warp store is
// still one 512-byte row.
template <int WB, int M, int C0, int G0, int C1, int G1>
__global__ void __launch_bounds__(kThreads, 2)
k_adj_blk_uni(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nsites, UniArgs g,
              Area a, OutSlots<M *(3 + WB)> out) {
  constexpr int NV = 8;
  constexpr int KH = 3 + WB;                  // wires >= 6 in the tile
  constexpr int NW = 1 << WB;                 // warps per site
  constexpr int SPB = (kThreads / 32) / NW;   // sites per block
  constexpr int ROWS = NV * NW;               // rows of one state in a site
  constexpr int NOPS = M * KH;
  // RZ and RY on every wire (either undo order): the RZs of a layout's
  // register wires go as one phase per vector (rzry_ops).
  constexpr bool kRzRy = M == 2 && ((C0 == kMatDiag && G0 == 3 && C1 == kMatReal && G1 == 2) ||
                                    (C0 == kMatReal && G0 == 2 && C1 == kMatDiag && G1 == 3));
  static_assert(SPB >= 1 && SPB * NW == kThreads / 32, "whole sites per block");
  extern __shared__ __align__(16) float4 xb[];   // [site][state][row][32 lanes]
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t sib = warp / NW, wsl = warp % NW;
  float4 *site_p = xb + static_cast<size_t>(sib) * 2 * ROWS * 32;
  float4 *site_l = site_p + ROWS * 32;
  const uint64_t per_round = static_cast<uint64_t>(gridDim.x) * SPB;
  const uint64_t rounds = (nsites + per_round - 1) / per_round;
  // Row of register vector l in the first layout (register bits = the
  // site's wires 0..2, warp bits = wires 3..) and in the second (register
  // bits = wires 3.., then the rest of wires 0..2; warp bits = wires 0..WB-1).
  auto row_a = [&](int l) { return static_cast<uint32_t>(l) | (wsl << 3); };
  auto row_b = [&](int l) {
    const uint32_t lo = static_cast<uint32_t>(l) & ((1u << WB) - 1u);   // -> wires 3..
    const uint32_t hi = static_cast<uint32_t>(l) >> WB;                 // -> wires WB..2
    return wsl | (hi << WB) | (lo << 3);
  };
  auto site_of = [&](uint64_t r) {
    return r * per_round + static_cast<uint64_t>(blockIdx.x) * SPB + sib;
  };
  auto row0_of = [&](uint64_t st) {
    uint64_t b = st;
#pragma unroll
    for (int j = 0; j < KH; j++) b = ins0(b, g.hpos[j]);
    return b << 5;
  };
  auto vec_of = [&](uint64_t row0, uint32_t row) {
    uint64_t v = row0;
#pragma unroll
    for (int j = 0; j < KH; j++)
      if ((row >> j) & 1u) v |= 1ull << (g.hpos[j] + 5);
    return v;
  };
  auto site_sync = [&]() {
    if constexpr (SPB == 1) {
      __syncthreads();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(sib + 1), "r"(NW * 32) : "memory");
    }
  };
  // Each warp's eight row offsets (the row's wire bits, as a vector index)
  // in both layouts, worked out once: a round then adds them to its site's
  // first row instead of testing six wire bits per vector.
  __shared__ uint64_t row_off[kThreads / 32][2][NV];
  if (lane < 2 * NV) {
    const int l = lane & (NV - 1);
    row_off[warp][lane / NV][l] = vec_of(0, lane < NV ? row_a(l) : row_b(l));
  }
  float accf[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) accf[t] = 0.0f;
  __shared__ uint64_t mbar[kThreads / 32];   // one per warp: its rows of the next round
  uint32_t parity = 0;
  bool stalled = false;
  uint32_t stalled_parity = 0;
  const uint32_t limit = wait_limit(a);
  if (lane == 0) mbar_init(&mbar[warp], 1);
  fence_proxy_async();
  __syncthreads();
  auto prefetch = [&](uint64_t r) {
    const uint64_t st = site_of(r);
    if (r < rounds && st < nsites && !stalled && lane == 0) {
      const uint64_t row0 = row0_of(st);
      fence_proxy_async();
      mbar_expect_tx(&mbar[warp], 2 * NV * 32 * sizeof(float4));
#pragma unroll
      for (int l = 0; l < NV; l++) {
        const uint32_t row = row_a(l);
        const uint64_t v = row0 | row_off[warp][0][l];
        bulk_row(site_p + row * 32, psi + v, 32 * sizeof(float4), &mbar[warp]);
        bulk_row(site_l + row * 32, lam + v, 32 * sizeof(float4), &mbar[warp]);
      }
    }
  };
  prefetch(0);
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t st = site_of(r);
    const bool active = st < nsites;   // uniform over the site's warps
    float4 P[NV], L[NV];
    if (active) {
      if (!stalled) {
        const bool landed = mbar_wait(&mbar[warp], parity, limit);
        if (!__all_sync(0xffffffffu, landed)) {
          if (lane == 0) atomicAdd(a.waits, 1u);
          stalled = true;
          stalled_parity = parity;
        }
        parity ^= 1u;
      }
#pragma unroll
      for (int l = 0; l < NV; l++) {
        P[l] = site_p[row_a(l) * 32 + lane];
        L[l] = site_l[row_a(l) * 32 + lane];
      }
      if constexpr (kRzRy) {
        rzry_ops<NV, 3, C0>(P, L, g.mh, g.ph[0], accf);
      } else {
        reg_ops<M, NV, 0, C0, G0, C1, G1>(P, L, g.mh[0], accf);
        reg_ops<M, NV, 1, C0, G0, C1, G1>(P, L, g.mh[1], accf + M);
        reg_ops<M, NV, 2, C0, G0, C1, G1>(P, L, g.mh[2], accf + 2 * M);
      }
#pragma unroll
      for (int l = 0; l < NV; l++) {
        site_p[row_a(l) * 32 + lane] = P[l];
        site_l[row_a(l) * 32 + lane] = L[l];
      }
    }
    site_sync();   // the first layout is written back
    if (active) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        P[l] = site_p[row_b(l) * 32 + lane];
        L[l] = site_l[row_b(l) * 32 + lane];
      }
    }
    site_sync();   // every warp has read its second layout: the slots are free
    if (active) {
      prefetch(r + 1);
      if constexpr (kRzRy) {
        rzry_ops<NV, WB, C0>(P, L, g.mh + 3, g.ph[1], accf + 3 * M);
      } else {
        reg_ops<M, NV, 0, C0, G0, C1, G1>(P, L, g.mh[3], accf + 3 * M);
        if constexpr (WB > 1) reg_ops<M, NV, 1, C0, G0, C1, G1>(P, L, g.mh[4], accf + 4 * M);
        if constexpr (WB > 2) reg_ops<M, NV, 2, C0, G0, C1, G1>(P, L, g.mh[5], accf + 5 * M);
      }
      // A warp that gave up a wait leaves the states alone (the host refuses
      // the pass and resets the simulator's state).
      if (!stalled) {
        const uint64_t row0 = row0_of(st) | lane;
#pragma unroll
        for (int l = 0; l < NV; l++) {
          const uint64_t v = row0 | row_off[warp][1][l];
          psi[v] = P[l];
          lam[v] = L[l];
        }
      }
    }
  }
  if (stalled && !__all_sync(0xffffffffu, mbar_wait(&mbar[warp], stalled_parity)) && lane == 0)
    atomicAdd(a.waits, 1u);
  double acc[NOPS];
#pragma unroll
  for (int t = 0; t < NOPS; t++) acc[t] = accf[t];
  finish<NOPS>(acc, NOPS, a, out);
}

template <int WB, int M, int C0, int G0, int C1, int G1>
int launch_blk(float4 *psi, float4 *lam, uint64_t nsites, const UniArgs &g, double *grad,
               const uint32_t *slots, Area a, cudaStream_t s) {
  constexpr int NOPS = M * (3 + WB);
  constexpr int SPB = (kThreads / 32) >> WB;
  OutSlots<NOPS> out{};
  out.p = grad;
  for (int t = 0; t < NOPS; t++) out.slot[t] = slots[t];
  unsigned grid = grid_for(nsites, SPB);
  grid = std::min<unsigned>(grid, reduce_grid());
  const size_t smem = static_cast<size_t>(SPB) * 2 * (8 << WB) * 32 * sizeof(float4);
  // The opt-in above 48 KiB is per device; set it once on each.
  static std::atomic<bool> opted[64];   // zero-initialised: false
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_adj_blk_uni<WB, M, C0, G0, C1, G1>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  k_adj_blk_uni<WB, M, C0, G0, C1, G1><<<grid, kThreads, smem, s>>>(psi, lam, nsites, g, a, out);
  return launch_status();
}

template <bool W0, int NL, int M, int C0, int G0, int C1, int G1>
int launch_pair(float4 *psi, float4 *lam, uint64_t nw, const UniArgs &g, double *grad,
                const uint32_t *slots, Area a, cudaStream_t s) {
  constexpr int NOPS = M * ((W0 ? 1 : 0) + NL + 4);
  OutSlots<NOPS> out{};
  out.p = grad;
  for (int t = 0; t < NOPS; t++) out.slot[t] = slots[t];
  unsigned grid = grid_for(nw, kThreads / 64);
  grid = std::min<unsigned>(grid, reduce_grid());
  const size_t smem = static_cast<size_t>(kThreads / 32) * 2 * kPairNV * 32 * sizeof(float4);
  // The opt-in above 48 KiB is per device; set it once on each.
  static std::atomic<bool> opted[64];   // zero-initialised: false
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_adj_pair_uni<W0, NL, M, C0, G0, C1, G1>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  k_adj_pair_uni<W0, NL, M, C0, G0, C1, G1><<<grid, kThreads, smem, s>>>(psi, lam, nw, g, a, out);
  return launch_status();
}

template <int KH, bool W0, int NL, int M, int C0, int G0, int C1, int G1>
int launch_warp(float4 *psi, float4 *lam, uint64_t nw, const UniArgs &g, double *grad,
                const uint32_t *slots, Area a, cudaStream_t s) {
  constexpr int NOPS = M * ((W0 ? 1 : 0) + NL + KH);
  OutSlots<NOPS> out{};
  out.p = grad;
  for (int t = 0; t < NOPS; t++) out.slot[t] = slots[t];
  unsigned grid = grid_for(nw, kThreads / 32);
  grid = std::min<unsigned>(grid, reduce_grid());
  k_adj_warp_uni<KH, W0, NL, M, C0, G0, C1, G1><<<grid, kThreads, 0, s>>>(psi, lam, nw, g, a, out);
  return launch_status();
}

// The rotation kinds a uniform tile takes: (class, generator) of RX, RY, RZ.
constexpr int kRx = 0, kRy = 1, kRz = 2;
int kind_of(int cls, int gen) {
  if (cls == kMatRx && gen == 1) return kRx;
  if (cls == kMatReal && gen == 2) return kRy;
  if (cls == kMatDiag && gen == 3) return kRz;
  return -1;
}

}  // namespace

int launch_uniform(int kh, float4 *psi, float4 *lam, uint64_t nw, const WarpAdjArgs &g,
                   const OutSlots<kMaxGen> &out, Area a, cudaStream_t s) {
  if (kh < 1 || kh > 6 || g.nops < 1 || g.nops > 20) return 1;
  // Wires in op order (a wire's ops are consecutive), each with its ops.
  struct Wire {
    int kind, arg, n;
    int op[2];
  };
  Wire w[16];
  int nwires = 0;
  for (uint32_t o = 0; o < g.nops; o++) {
    const int kind = g.kind[o], arg = g.arg[o];
    if (nwires > 0 && w[nwires - 1].kind == kind && w[nwires - 1].arg == arg) {
      Wire &c = w[nwires - 1];
      if (c.n == 2) return 1;
      c.op[c.n++] = static_cast<int>(o);
      continue;
    }
    for (int i = 0; i < nwires; i++)
      if (w[i].kind == kind && w[i].arg == arg) return 1;   // a wire's ops not together
    if (nwires == 16 || kind < 0 || kind > 2) return 1;
    w[nwires++] = {kind, arg, 1, {static_cast<int>(o), -1}};
  }
  const int M = w[0].n;
  int seq[2];
  for (int k = 0; k < M; k++) {
    seq[k] = kind_of(g.cls[w[0].op[k]], g.gen[w[0].op[k]]);
    if (seq[k] < 0) return 1;
  }
  UniArgs u{};
  for (int j = 0; j < 6; j++) u.hpos[j] = g.hpos[j];
  int w0 = 0, nl = 0, nh = 0;
  uint32_t slots[20];
  int order[16], no = 0;   // wires in kernel order: wire 0, lanes, registers by index
  for (int i = 0; i < nwires; i++) {
    if (w[i].n != M) return 1;
    for (int k = 0; k < M; k++)
      if (kind_of(g.cls[w[i].op[k]], g.gen[w[i].op[k]]) != seq[k]) return 1;
    if (w[i].kind == 0) w0++;
    else if (w[i].kind == 1) nl++;
    else nh++;
  }
  if (w0 > 1 || nh != kh) return 1;
  for (int i = 0; i < nwires; i++)
    if (w[i].kind == 0) order[no++] = i;
  for (int i = 0; i < nwires; i++)
    if (w[i].kind == 1) order[no++] = i;
  for (int j = 0; j < kh; j++) {
    int found = -1;
    for (int i = 0; i < nwires; i++)
      if (w[i].kind == 2 && w[i].arg == j) found = i;
    if (found < 0) return 1;
    order[no++] = found;
  }
  int t = 0, li = 0;
  for (int q = 0; q < no; q++) {
    const Wire &c = w[order[q]];
    for (int k = 0; k < M; k++) {
      const int o = c.op[k];
      slots[t++] = out.slot[g.slotidx[o]];
      if (c.kind == 0) u.m0[k] = g.m[o];
      else if (c.kind == 1) u.ml[li][k] = g.m[o];
      else u.mh[c.arg][k] = g.m[o];
    }
    if (c.kind == 1) u.lbit[li++] = static_cast<uint32_t>(c.arg);
  }
  const bool wide = w0 == 1 && nl == 5, narrow = w0 == 0 && nl == 0;
  if (!wide && !narrow) return 1;
  // RZ and RY on every wire: each layout's RZ undos of the register wires as
  // one phase per register vector, multiplied out in double from the
  // narrowed matrices (one rounding instead of one per wire).
  if (M == 2 && (seq[0] == kRz) != (seq[1] == kRz)) {
    const int rz = seq[0] == kRz ? 0 : 1;
    auto phase = [&](int j0, int cnt, float2(&out)[8]) {
      for (int l = 0; l < 8; l++) {
        double re = 1.0, im = 0.0;
        for (int j = 0; j < cnt; j++) {
          const float2 e = ((l >> j) & 1) ? u.mh[j0 + j][rz].d : u.mh[j0 + j][rz].a;
          const double nr = re * e.x - im * e.y, ni = re * e.y + im * e.x;
          re = nr;
          im = ni;
        }
        out[l] = make_float2(static_cast<float>(re), static_cast<float>(im));
      }
    };
    if (wide) {
      // ph[2 l + b] (both rows as one table): the register wires' entries by
      // l (up to three wires; a fourth is split across a warp pair) times
      // wire 0's by b
      float2 reg[8];
      const int kr = std::min(kh, 3);
      phase(0, kr, reg);
      float2 *flat = &u.ph[0][0];
      for (int l = 0; l < (1 << kr); l++)
        for (int b = 0; b < 2; b++) {
          const float2 r = reg[l], e = b ? u.m0[rz].d : u.m0[rz].a;
          const double re = static_cast<double>(r.x) * e.x - static_cast<double>(r.y) * e.y;
          const double im = static_cast<double>(r.x) * e.y + static_cast<double>(r.y) * e.x;
          flat[2 * l + b] = make_float2(static_cast<float>(re), static_cast<float>(im));
        }
      for (int ln = 0; ln < 32; ln++) {
        double re = 1.0, im = 0.0;
        for (int k = 0; k < 5; k++) {
          const float2 e = ((ln >> u.lbit[k]) & 1) ? u.ml[k][rz].d : u.ml[k][rz].a;
          const double nr = re * e.x - im * e.y, ni = re * e.y + im * e.x;
          re = nr;
          im = ni;
        }
        u.lph[ln] = make_float2(static_cast<float>(re), static_cast<float>(im));
      }
    } else {
      phase(0, std::min(kh, 3), u.ph[0]);
      if (kh > 3) phase(3, kh - 3, u.ph[1]);
    }
  }
  double *p = out.p;
  if (kh >= 5) {
    if (!narrow) return 1;
#define QMK_UNI_BLK(WB)                                                                        \
  if (kh == 3 + WB) {                                                                          \
    if (M == 1 && seq[0] == kRx) return launch_blk<WB, 1, kMatRx, 1, 0, 0>(psi, lam, nw, u, p, slots, a, s);   \
    if (M == 1 && seq[0] == kRy) return launch_blk<WB, 1, kMatReal, 2, 0, 0>(psi, lam, nw, u, p, slots, a, s); \
    if (M == 1) return launch_blk<WB, 1, kMatDiag, 3, 0, 0>(psi, lam, nw, u, p, slots, a, s);                  \
    if (seq[0] == kRz && seq[1] == kRy)                                                        \
      return launch_blk<WB, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);    \
    if (seq[0] == kRy && seq[1] == kRz)                                                        \
      return launch_blk<WB, 2, kMatReal, 2, kMatDiag, 3>(psi, lam, nw, u, p, slots, a, s);    \
    return 1;                                                                                  \
  }
    QMK_UNI_BLK(2)
    QMK_UNI_BLK(3)
#undef QMK_UNI_BLK
    return 1;
  }
  if (M == 1 && kh == 4) {
    if (wide) {
      if (seq[0] == kRx) return launch_pair<true, 5, 1, kMatRx, 1, 0, 0>(psi, lam, nw, u, p, slots, a, s);
      if (seq[0] == kRy) return launch_pair<true, 5, 1, kMatReal, 2, 0, 0>(psi, lam, nw, u, p, slots, a, s);
      return launch_pair<true, 5, 1, kMatDiag, 3, 0, 0>(psi, lam, nw, u, p, slots, a, s);
    }
    if (seq[0] == kRx) return launch_pair<false, 0, 1, kMatRx, 1, 0, 0>(psi, lam, nw, u, p, slots, a, s);
    if (seq[0] == kRy) return launch_pair<false, 0, 1, kMatReal, 2, 0, 0>(psi, lam, nw, u, p, slots, a, s);
    return launch_pair<false, 0, 1, kMatDiag, 3, 0, 0>(psi, lam, nw, u, p, slots, a, s);
  }
  if (M == 2 && kh == 4 && narrow) {
    if (seq[0] == kRz && seq[1] == kRy)
      return launch_pair<false, 0, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
    if (seq[0] == kRy && seq[1] == kRz)
      return launch_pair<false, 0, 2, kMatReal, 2, kMatDiag, 3>(psi, lam, nw, u, p, slots, a, s);
    return 1;
  }
  if (M == 1 && seq[0] == kRx && kh <= 3) {
#define QMK_UNI_RX(KH)                                                                        \
  if (kh == KH) {                                                                             \
    if (wide) return launch_warp<KH, true, 5, 1, kMatRx, 1, 0, 0>(psi, lam, nw, u, p, slots, a, s); \
    return launch_warp<KH, false, 0, 1, kMatRx, 1, 0, 0>(psi, lam, nw, u, p, slots, a, s);   \
  }
    QMK_UNI_RX(1)
    QMK_UNI_RX(2)
    QMK_UNI_RX(3)
#undef QMK_UNI_RX
  }
  if (M == 2 && seq[0] == kRz && seq[1] == kRy && wide && kh == 4)
    return launch_pair<true, 5, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
  if (M == 2 && seq[0] == kRz && seq[1] == kRy && kh <= 3) {
    if (wide && kh == 2)
      return launch_warp<2, true, 5, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
    if (narrow && kh == 1)
      return launch_warp<1, false, 0, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
    if (narrow && kh == 2)
      return launch_warp<2, false, 0, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
    if (narrow && kh == 3)
      return launch_warp<3, false, 0, 2, kMatDiag, 3, kMatReal, 2>(psi, lam, nw, u, p, slots, a, s);
  }
  return 1;
}

}  // namespace qmk_adj
