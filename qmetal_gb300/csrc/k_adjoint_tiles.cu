// k_adjoint_tiles.cu -- backward passes over windows of one-qubit gates:
// both states held in registers as warp tiles, each window's gates undone in
// reverse with the overlap of every rotation taken first. Split from
// k_adjoint.cu so the two compile in parallel.
#include <algorithm>
#include <atomic>

#include "kadjoint_ops.cuh"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

namespace qmk_adj {
namespace {

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
  static std::atomic<bool> opted[64];   // zero-initialised: false
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
  const int rc = launch_uniform(kh, psi, lam, nw, g, out, a, s);
  if (rc != 1) return rc;
  if (kh == 4) {
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
