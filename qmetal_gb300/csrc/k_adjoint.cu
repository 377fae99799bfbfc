// k_adjoint.cu -- the fused adjoint sweep: co-state of Z Hamiltonians and
// block-wise backward passes that take every gradient of a commuting block
// and undo the block on both states in one pass.
//
// The reference sweep (src/metal/simulator.mm:914-959) visits one gate at a
// time: a two-state reduction per parameter, then the inverse gate on psi and
// on lambda, each a full pass. Two facts let whole blocks go at once:
//  * gates that commute with each other and with a gate's generator P leave
//    <lambda|P|psi> unchanged when undone on both states, so every gradient of
//    a block of commuting gates can be read at the block boundary;
//  * a diagonal block's gradients need only F(i) = Im(conj(lambda_i) psi_i)
//    weighted by the generators' signs, and F is itself unchanged by the
//    block's phases.
// A diagonal block (ZZ couplings, RZ, CZ, CP ...) is therefore one pass that
// reads both states, accumulates all its RZ / ZZ gradients, applies the
// conjugate phase and writes both states; a window of one-qubit gates is
// undone a few wires at a time with the wires' gates in reverse order held in
// registers. Gradients land straight in the gate-indexed gradient array.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "kquad.cuh"
#include "kreduce.cuh"
#include "kadjoint.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;
using qmk_adj::kMaxDiagGen;
using qmk_adj::kMaxGen;
using qmk_adj::kMaxWarpOps;
using qmk_adj::overlap;
using qmk_adj::WarpAdjArgs;

namespace {

// ---------------------------------------------------------------------------
// Co-state of a Hamiltonian of Z strings with at most two bits each:
// lambda_i = D(i) psi_i with the real quadratic form
// D(i) = sum_t c_t (-1)^{x_a} or c_t (-1)^{x_a + x_b}; energy = sum D |psi|^2.

__global__ void __launch_bounds__(kThreads)
k_zdiag(float4 *__restrict__ lam, const float4 *__restrict__ psi, const DiagDesc *__restrict__ d,
        const float2 *__restrict__ table2, uint64_t ntiles, Area a, double *out) {
  __shared__ float cr[kWMax];
  __shared__ float hr;
  __shared__ __align__(16) float Y1[64];
  __shared__ float Y2[1 << (kWMax - 6)];
  const uint32_t W = d->W, tid = threadIdx.x, nv = 1u << (W - 1);
  double acc[1] = {0.0};
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    tile_coeffs<false>(d, tile, nullptr, nullptr, cr, &hr, false);
    __syncthreads();
    tile_real_tables(W, cr, hr, Y1, Y2);
    __syncthreads();
    const uint64_t base = tile << (W - 1);
    float part = 0.0f;
    constexpr int UU = 4;
    for (uint32_t e0 = tid; e0 < nv; e0 += kThreads * UU) {
      float4 x[UU];
      float2 t[UU];
#pragma unroll
      for (int k = 0; k < UU; k++) {
        const uint32_t e = e0 + k * kThreads;
        if (e < nv) {
          x[k] = psi[base + e];
          t[k] = table2[e];   // table of floats read two at a time
        }
      }
#pragma unroll
      for (int k = 0; k < UU; k++) {
        const uint32_t e = e0 + k * kThreads;
        if (e >= nv) continue;
        const uint32_t lo = 2 * e;
        const float2 y1 = *reinterpret_cast<const float2 *>(&Y1[lo & 63]);
        const float y2 = Y2[lo >> 6];
        const float d0 = t[k].x + (y1.x + y2), d1 = t[k].y + (y1.y + y2);
        const float4 v = x[k];
        lam[base + e] = make_float4(d0 * v.x, d0 * v.y, d1 * v.z, d1 * v.w);
        part += d0 * (v.x * v.x + v.y * v.y) + d1 * (v.z * v.z + v.w * v.w);
      }
    }
    acc[0] += part;
    __syncthreads();
  }
  finish<1>(acc, 1, a, OutContig{out, false});
}

// ---------------------------------------------------------------------------
// Adjoint of a diagonal block. Thread t of a tile owns amplitude bits 1..8
// (= t) and visits the 32 amplitudes spanned by bit 0 (lane) and bits 9..12
// (loop k): j = lane | k << 1. The gradient of a Z-string generator with mask
// m is sum_j F_j (-1)^{popcount(j & vm)} times the sign of the thread's fixed
// bits, i.e. one coefficient of the 32-point Walsh-Hadamard transform of F.


template <int T>
struct DiagAdjArgs {
  uint32_t ngen;
  uint32_t undo;
  uint64_t fixmask[T > 0 ? T : 1];   // generator bits outside {0, 9..12}
  uint8_t vm[T > 0 ? T : 1];         // generator bits inside, as j bits
};

template <int T>
__device__ __forceinline__ void adj_diag_body(float4 *__restrict__ psi, float4 *__restrict__ lam,
                                              const DiagDesc *__restrict__ d,
                                              const float4 *__restrict__ table4, uint64_t ntiles,
                                              const DiagAdjArgs<T> &g, Area a,
                                              const OutSlots<(T > 0 ? T : 1)> &out) {
  __shared__ float2 f[kWMax];
  __shared__ float2 eH;
  __shared__ __align__(16) float2 Y1[64];
  __shared__ float2 Y2[1 << (kWMax - 6)];
  __shared__ float Fs[T > 0 ? kThreads * 33 : 1];
  const uint32_t W = d->W, tid = threadIdx.x, nv = 1u << (W - 1);
  // FP32 per thread over its tiles (a few dozen at most), FP64 from the warp up.
  float accf[T > 0 ? T : 1];
#pragma unroll
  for (int t = 0; t < (T > 0 ? T : 1); t++) accf[t] = 0.0f;
  // Generator signs outside the 32 transformed amplitudes: bit t is the
  // parity of (fixed bits & fixmask[t]); the thread's own bits give a mask
  // that holds for every tile, the tile's bits one that every thread shares
  // (lane t computes bit t, a ballot hands the word to the warp).
  // (More than 32 generators: a 64-bit sign word and a second ballot.)
  using Sign = std::conditional_t<(T > 32), uint64_t, uint32_t>;
  __shared__ uint64_t fm[T > 0 ? T : 1];
  Sign own_sign = 0;
  if constexpr (T > 0) {
    const uint64_t mine = static_cast<uint64_t>(tid) << 1;
    for (int t = 0; t < T && t < static_cast<int>(g.ngen); t++)
      own_sign |= static_cast<Sign>(parity64(mine & g.fixmask[t])) << t;
    if (tid < static_cast<uint32_t>(T)) fm[tid] = g.fixmask[tid];
  }
  __syncthreads();
  const uint32_t lane = tid & 31;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t base = tile << (W - 1);
    // Four vectors of both states (and their table entries) are loaded
    // before any is used, so each thread keeps 8-12 loads in flight; the
    // first four are issued before the tile's phase tables are built, so the
    // table set-up runs under their latency.
    constexpr int UU = 4;
    float4 P[UU], L[UU], tb[UU];
    auto load_chunk = [&](int c) {
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const uint32_t e = tid + (c + u) * kThreads;
        if (e < nv) {
          P[u] = psi[base + e];
          L[u] = lam[base + e];
          if (g.undo) tb[u] = table4[e];
        }
      }
    };
    load_chunk(0);
    if (g.undo) {
      tile_coeffs<true>(d, tile, f, &eH, nullptr, nullptr, true);
      __syncthreads();
      tile_phase_tables(W, f, eH, Y1, Y2);
      __syncthreads();
    }
    float F[32];
#pragma unroll
    for (int j = 0; j < 32; j++) F[j] = 0.0f;
#pragma unroll
    for (int c = 0; c < 16; c += UU) {
      if (c > 0) load_chunk(c);
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const int k = c + u;
        const uint32_t e = tid + k * kThreads;
        if (e >= nv) continue;
        float4 p = P[u], l = L[u];
        if (T > 0) {
          F[2 * k] = l.x * p.y - l.y * p.x;
          F[2 * k + 1] = l.z * p.w - l.w * p.z;
        }
        if (g.undo) {
          const uint32_t lo = 2 * e;
          const float4 t = tb[u];
          const float4 y1 = *reinterpret_cast<const float4 *>(&Y1[lo & 63]);
          const float2 y2 = Y2[lo >> 6];
          const float2 f0 = cmul(cmul(make_float2(t.x, -t.y), lo2(y1)), y2);
          const float2 f1 = cmul(cmul(make_float2(t.z, -t.w), hi2(y1)), y2);
          p = pack4(cmul(f0, lo2(p)), cmul(f1, hi2(p)));
          l = pack4(cmul(f0, lo2(l)), cmul(f1, hi2(l)));
          psi[base + e] = p;
          lam[base + e] = l;
        }
      }
    }
    if constexpr (T > 0) {
#pragma unroll
      for (int h = 1; h < 32; h <<= 1) {
#pragma unroll
        for (int j = 0; j < 32; j++) {
          if (j & h) continue;
          const float u = F[j], v = F[j | h];
          F[j] = u + v;
          F[j | h] = u - v;
        }
      }
      float *row = &Fs[tid * 33];
#pragma unroll
      for (int j = 0; j < 32; j++) row[j] = F[j];
      const int ng = static_cast<int>(g.ngen);
      const uint64_t tbits = tile << W;
      const bool mine = static_cast<int>(lane) < ng && static_cast<int>(lane) < T;
      Sign tile_sign =
          __ballot_sync(0xffffffffu, mine && parity64(tbits & fm[lane < T ? lane : 0]));
      if constexpr (T > 32) {
        const int t2 = 32 + static_cast<int>(lane);
        const bool mine2 = t2 < ng && t2 < T;
        const uint32_t hi = __ballot_sync(0xffffffffu, mine2 && parity64(tbits & fm[mine2 ? t2 : 0]));
        tile_sign |= static_cast<Sign>(hi) << 32;
      }
      const Sign sign = own_sign ^ tile_sign;
#pragma unroll
      for (int t = 0; t < T; t++) {
        const float v = t < ng ? row[g.vm[t]] : 0.0f;
        accf[t] += ((sign >> t) & 1u) ? -v : v;
      }
    }
    __syncthreads();
  }
  double acc[T > 0 ? T : 1];
#pragma unroll
  for (int t = 0; t < (T > 0 ? T : 1); t++) acc[t] = accf[t];
  if constexpr (T > 0) finish<T>(acc, g.ngen, a, out);
}

template <int T>
__global__ void __launch_bounds__(kThreads)
k_adj_diag(float4 *__restrict__ psi, float4 *__restrict__ lam, const DiagDesc *__restrict__ d,
           const float4 *__restrict__ table4, uint64_t ntiles, DiagAdjArgs<T> g, Area a,
           OutSlots<(T > 0 ? T : 1)> out) {
  adj_diag_body<T>(psi, lam, d, table4, ntiles, g, a, out);
}

// More than 32 generators: left unbounded the kernel takes 172 registers (one
// block a multiprocessor); held to two blocks it spills a few words.
template <int T>
__global__ void __launch_bounds__(kThreads, 2)
k_adj_diag_wide(float4 *__restrict__ psi, float4 *__restrict__ lam, const DiagDesc *__restrict__ d,
                const float4 *__restrict__ table4, uint64_t ntiles, DiagAdjArgs<T> g, Area a,
                OutSlots<(T > 0 ? T : 1)> out) {
  adj_diag_body<T>(psi, lam, d, table4, ntiles, g, a, out);
}

// ---------------------------------------------------------------------------
// Adjoint of a window of one-qubit gates on up to four wires (wire 0 in the
// lanes plus up to three vector bits), both states in registers. Ops run in
// the given order (each wire's gates last-to-first); an op with a generator
// first takes Im<lambda|P|psi> over the tile, then applies the inverse gate.

constexpr int kMaxOps = 16;

struct GroupAdjArgs {
  uint32_t pos[3];        // vector bits of the tile's wires >= 1, ascending
  uint32_t nops;
  uint32_t ngrad;         // ops with a generator (results written)
  int8_t where[kMaxOps];  // -1: wire 0 (lanes); j >= 0: pos[j]
  int8_t gen[kMaxOps];    // 0 none, 1 X, 2 Y, 3 Z
  uint8_t slotidx[kMaxOps];
  M2 m[kMaxOps];
};


template <int KP, int NG>
__global__ void __launch_bounds__(kThreads)
k_adj_group(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nsites, GroupAdjArgs g,
            Area a, OutSlots<(NG > 0 ? NG : 1)> out) {
  constexpr int NV = 1 << KP;
  double acc[NG > 0 ? NG : 1];
#pragma unroll
  for (int t = 0; t < (NG > 0 ? NG : 1); t++) acc[t] = 0.0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kThreads;
  for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x; s < nsites;
       s += stride) {
    uint64_t base = s;
#pragma unroll
    for (int j = 0; j < KP; j++) base = ins0(base, g.pos[j]);
    float4 P[NV], L[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < KP; j++)
        if ((l >> j) & 1) v |= 1ull << g.pos[j];
      P[l] = psi[v];
      L[l] = lam[v];
    }
    float part[NG > 0 ? NG : 1];
#pragma unroll
    for (int t = 0; t < (NG > 0 ? NG : 1); t++) part[t] = 0.0f;
    for (uint32_t o = 0; o < g.nops; o++) {
      const int w = g.where[o], gen = g.gen[o];
      const M2 m = g.m[o];
      float ov = 0.0f;
      if (w < 0) {
#pragma unroll
        for (int l = 0; l < NV; l++) {
          float2 p0 = lo2(P[l]), p1 = hi2(P[l]), l0 = lo2(L[l]), l1 = hi2(L[l]);
          if (gen) ov += overlap(gen, p0, p1, l0, l1);
          apply2(m, p0, p1);
          apply2(m, l0, l1);
          P[l] = pack4(p0, p1);
          L[l] = pack4(l0, l1);
        }
      } else {
#pragma unroll
        for (int j = 0; j < KP; j++) {
          if (j != w) continue;
#pragma unroll
          for (int l = 0; l < NV; l++) {
            if ((l >> j) & 1) continue;
            const int h = l | (1 << j);
            float2 pa = lo2(P[l]), pb = lo2(P[h]), qa = hi2(P[l]), qb = hi2(P[h]);
            float2 la = lo2(L[l]), lb = lo2(L[h]), ma = hi2(L[l]), mb = hi2(L[h]);
            if (gen) ov += overlap(gen, pa, pb, la, lb) + overlap(gen, qa, qb, ma, mb);
            apply2(m, pa, pb);
            apply2(m, qa, qb);
            apply2(m, la, lb);
            apply2(m, ma, mb);
            P[l] = pack4(pa, qa);
            P[h] = pack4(pb, qb);
            L[l] = pack4(la, ma);
            L[h] = pack4(lb, mb);
          }
        }
      }
      if (NG > 0 && gen) {
#pragma unroll
        for (int t = 0; t < (NG > 0 ? NG : 1); t++)
          if (t == g.slotidx[o]) part[t] += ov;
      }
    }
#pragma unroll
    for (int l = 0; l < NV; l++) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < KP; j++)
        if ((l >> j) & 1) v |= 1ull << g.pos[j];
      psi[v] = P[l];
      lam[v] = L[l];
    }
#pragma unroll
    for (int t = 0; t < (NG > 0 ? NG : 1); t++) acc[t] += part[t];
  }
  if constexpr (NG > 0) finish<NG>(acc, static_cast<int>(g.ngrad), a, out);
}

bool ok_ws(void *ws, size_t bytes, uint32_t n) {
  return ws && bytes >= qmk_workspace_bytes(n);
}

template <int T>
int launch_adj_diag(float *psi, float *lam, uint32_t n, const DiagDesc *dd, const float2 *table,
                    uint32_t ngen, const uint64_t *gm, const uint32_t *slots, double *grad,
                    bool undo, void *ws, cudaStream_t s) {
  DiagAdjArgs<T> g{};
  OutSlots<(T > 0 ? T : 1)> out{};
  out.p = grad;
  g.ngen = ngen;
  g.undo = undo ? 1u : 0u;
  const uint64_t inner = 1ull | (0xFull << 9);   // amplitude bits 0 and 9..12
  for (uint32_t t = 0; t < ngen && T > 0; t++) {
    const uint64_t m = gm[t];
    g.fixmask[t] = m & ~inner;
    g.vm[t] = static_cast<uint8_t>((m & 1ull) | (((m >> 9) & 0xFull) << 1));
    out.slot[t] = slots[t];
  }
  const uint32_t W = std::min<uint32_t>(n, kWMax);
  const uint64_t ntiles = 1ull << (n - W);
  float4 *p4 = reinterpret_cast<float4 *>(psi), *l4 = reinterpret_cast<float4 *>(lam);
  const float4 *t4 = reinterpret_cast<const float4 *>(table);
  if constexpr (T > 32) {
    // 64 partials a block: at most kMaxBlocks / 2 blocks; one wave of two
    // blocks a multiprocessor.
    const unsigned cap = std::min<unsigned>(kMaxBlocks / 2, 2u * qmk_host::num_sms());
    const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(ntiles, cap));
    k_adj_diag_wide<T><<<grid, kThreads, 0, s>>>(p4, l4, dd, t4, ntiles, g, area_of(ws), out);
  } else {
    const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(ntiles, reduce_grid()));
    k_adj_diag<T><<<grid, kThreads, 0, s>>>(p4, l4, dd, t4, ntiles, g, area_of(ws), out);
  }
  return launch_status();
}

template <int KP, int NG>
void launch_adj_group(float4 *psi, float4 *lam, uint64_t nsites, const GroupAdjArgs &g,
                      const OutSlots<kMaxOps> &slots, Area a, cudaStream_t s) {
  OutSlots<(NG > 0 ? NG : 1)> out{};
  out.p = slots.p;
  for (int t = 0; t < (NG > 0 ? NG : 1); t++) out.slot[t] = slots.slot[t];
  const unsigned grid = NG > 0 ? std::min<unsigned>(reduce_grid(), grid_for(nsites, kThreads))
                               : grid_for(nsites, kThreads);
  k_adj_group<KP, NG><<<grid, kThreads, 0, s>>>(psi, lam, nsites, g, a, out);
}

}  // namespace

extern "C" int qmk_zdiag_costate(float *lam, const float *psi, uint32_t n, uint32_t nt,
                                 const uint64_t *zmasks, const double *coeffs, double *d_energy,
                                 void *ws, size_t ws_bytes, void *stream) {
  if (!lam || !psi || !d_energy || n < 1 || n > 40 || (nt && (!zmasks || !coeffs)) ||
      !ok_ws(ws, ws_bytes, n))
    return -1;
  // Expand each Z string into quadratic-form terms: (-1)^{x_a} = 1 - 2 x_a,
  // (-1)^{x_a + x_b} = 1 - 2 x_a - 2 x_b + 4 x_a x_b.
  std::vector<uint64_t> m;
  std::vector<double> c;
  double c0 = 0.0;
  for (uint32_t t = 0; t < nt; t++) {
    const uint64_t z = zmasks[t];
    const int pc = __builtin_popcountll(z);
    if (pc > 2) return -1;
    c0 += coeffs[t];
    if (pc >= 1) {
      for (uint64_t r = z; r; r &= r - 1) {
        m.push_back(r & (~r + 1));
        c.push_back(-2.0 * coeffs[t]);
      }
    }
    if (pc == 2) {
      m.push_back(z);
      c.push_back(4.0 * coeffs[t]);
    }
  }
  DiagDesc d;
  if (build_quad_desc(n, static_cast<uint32_t>(m.size()), m.data(), c.data(), c0, d, nullptr,
                      nullptr) != 0)
    return -1;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t *base = static_cast<uint8_t *>(ws);
  DiagDesc *dd = reinterpret_cast<DiagDesc *>(base);
  float *table = reinterpret_cast<float *>(base + kDescBytes);
  k_quad_prep<false><<<grid_for(1u << d.W, kThreads), kThreads, 0, s>>>(d, dd, table);
  int rc = launch_status();
  if (rc) return rc;
  const uint64_t ntiles = 1ull << (n - d.W);
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(ntiles, reduce_grid()));
  k_zdiag<<<grid, kThreads, 0, s>>>(reinterpret_cast<float4 *>(lam),
                                    reinterpret_cast<const float4 *>(psi), dd,
                                    reinterpret_cast<const float2 *>(table), ntiles, area_of(ws),
                                    d_energy);
  return launch_status();
}

extern "C" int qmk_adjoint_diagonal(float *psi, float *lam, uint32_t n, uint32_t nt,
                                    const uint64_t *masks, const double *angles,
                                    double global_phase, uint32_t ngen, const uint64_t *gen_masks,
                                    const uint32_t *slots, double *d_grad, int undo, void *ws,
                                    size_t ws_bytes, void *stream) {
  if (!psi || !lam || n < 1 || n > 40 || (nt && (!masks || !angles)) || !ok_ws(ws, ws_bytes, n))
    return -1;
  if (ngen > kMaxDiagGen || (ngen && (!gen_masks || !slots || !d_grad))) return -1;
  for (uint32_t t = 0; t < ngen; t++)
    if (n < 64 && (gen_masks[t] >> n)) return -1;
  if (!undo && ngen == 0) return 0;
  DiagDesc d;
  if (build_quad_desc(n, nt, masks, angles, global_phase, d, nullptr, nullptr) != 0) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t *base = static_cast<uint8_t *>(ws);
  DiagDesc *dd = reinterpret_cast<DiagDesc *>(base);
  float2 *table = reinterpret_cast<float2 *>(base + kDescBytes);
  if (undo) {
    k_quad_prep<true><<<grid_for(1u << d.W, kThreads), kThreads, 0, s>>>(d, dd, table);
    int rc = launch_status();
    if (rc) return rc;
  } else {
    // Gradient only: the kernel still reads W from the descriptor.
    k_quad_prep<true><<<1, kThreads, 0, s>>>(d, dd, table);
    int rc = launch_status();
    if (rc) return rc;
  }
  if (ngen == 0)
    return launch_adj_diag<0>(psi, lam, n, dd, table, 0, nullptr, nullptr, nullptr, undo != 0, ws, s);
  // Up to 16 generators take the 16-slot kernel (an 8-slot one measured
  // 15-25% slower on the same blocks), up to 32 the 32-slot one, more the
  // 48-slot one (MaxCut layers on 3-regular graphs of 22-32 vertices).
  if (ngen <= 16)
    return launch_adj_diag<16>(psi, lam, n, dd, table, ngen, gen_masks, slots, d_grad, undo != 0, ws, s);
  if (ngen <= 32)
    return launch_adj_diag<32>(psi, lam, n, dd, table, ngen, gen_masks, slots, d_grad, undo != 0, ws, s);
  return launch_adj_diag<48>(psi, lam, n, dd, table, ngen, gen_masks, slots, d_grad, undo != 0, ws, s);
}

extern "C" int qmk_adjoint_group(float *psi, float *lam, uint32_t n, uint32_t nops,
                                 const uint32_t *wires, const float *minv, const int *gens,
                                 const uint32_t *slots, double *d_grad, void *ws, size_t ws_bytes,
                                 void *stream) {
  if (!psi || !lam || n < 1 || n > 40 || nops < 1 || nops > kMaxWarpOps || !wires || !minv ||
      !gens || !ok_ws(ws, ws_bytes, n))
    return -1;
  // Distinct wires of the tile.
  uint32_t distinct[kMaxWarpOps], high[kMaxWarpOps];
  uint32_t nd = 0, nh = 0;
  int ngrad = 0;
  bool low = false;   // any wire below 6
  for (uint32_t o = 0; o < nops; o++) {
    if (wires[o] >= n || gens[o] < 0 || gens[o] > 3) return -1;
    if (gens[o] && (!slots || !d_grad)) return -1;
    if (gens[o]) ngrad++;
    low |= wires[o] < 6;
    if (wires[o] == 0) continue;   // wire 0 pairs the lanes of every vector: no tile bit
    bool seen = false;
    for (uint32_t k = 0; k < nd; k++) seen |= distinct[k] == wires[o];
    if (!seen) {
      distinct[nd++] = wires[o];
      if (wires[o] >= 6) high[nh++] = wires[o];
    }
  }
  // Sixteen gradients a pass, or twenty in the compile-time tile of wire 0,
  // wires 1..5 and four wires >= 6 with RZ then RY on every wire.
  if (ngrad > 20) return -1;
  if ((nh == 5 || nh == 6) && !low && n >= 6 + nh) {
    // Block tile: only the compile-time (uniform) kernels take five or six
    // wires >= 6 in one pass; any other tile of that shape is refused.
    std::sort(high, high + nh);
    WarpAdjArgs g{};
    OutSlots<kMaxGen> out{};
    out.p = d_grad;
    g.nops = nops;
    g.ngrad = static_cast<uint32_t>(ngrad);
    for (uint32_t k = 0; k < nh; k++) g.hpos[k] = high[k] - 6;
    int gi = 0;
    for (uint32_t o = 0; o < nops; o++) {
      g.kind[o] = 2;
      g.arg[o] = static_cast<int8_t>(std::find(high, high + nh, wires[o]) - high);
      g.gen[o] = static_cast<int8_t>(gens[o]);
      g.m[o] = m2_from(minv + 8 * o);
      g.cls[o] = m2_class(g.m[o]);
      g.slotidx[o] = 0;
      if (gens[o]) {
        g.slotidx[o] = static_cast<int8_t>(gi);
        out.slot[gi] = slots[o];
        gi++;
      }
    }
    const uint64_t nsites = 1ull << (n - 6 - nh);
    const int rc = qmk_adj::launch_uniform(static_cast<int>(nh), reinterpret_cast<float4 *>(psi),
                                           reinterpret_cast<float4 *>(lam), nsites, g, out,
                                           area_of(ws), (cudaStream_t)stream);
    return rc == 1 ? -1 : rc;
  }
  if (nh <= 4 && n >= 6 + nh) {
    // Warp tile: lanes carry wires 1..5, registers the wires >= 6.
    std::sort(high, high + nh);
    WarpAdjArgs g{};
    OutSlots<kMaxGen> out{};
    out.p = d_grad;
    g.nops = nops;
    g.ngrad = static_cast<uint32_t>(ngrad);
    for (uint32_t k = 0; k < nh; k++) g.hpos[k] = high[k] - 6;
    int gi = 0;
    for (uint32_t o = 0; o < nops; o++) {
      const uint32_t q = wires[o];
      if (q == 0) {
        g.kind[o] = 0;
        g.arg[o] = 0;
      } else if (q <= 5) {
        g.kind[o] = 1;
        g.arg[o] = static_cast<int8_t>(q - 1);
      } else {
        g.kind[o] = 2;
        g.arg[o] = static_cast<int8_t>(std::find(high, high + nh, q) - high);
      }
      g.gen[o] = static_cast<int8_t>(gens[o]);
      g.m[o] = m2_from(minv + 8 * o);
      g.cls[o] = m2_class(g.m[o]);
      g.slotidx[o] = 0;   // an op without a generator adds zero to slot 0
      if (gens[o]) {
        g.slotidx[o] = static_cast<int8_t>(gi);
        out.slot[gi] = slots[o];
        gi++;
      }
    }
    const uint64_t nw = 1ull << (n - 6 - nh);
    float4 *p4 = reinterpret_cast<float4 *>(psi), *l4 = reinterpret_cast<float4 *>(lam);
    cudaStream_t s = (cudaStream_t)stream;
    const Area a = area_of(ws);
    if (ngrad > 16) {   // only the compile-time tiles take more
      const int rc = qmk_adj::launch_uniform(static_cast<int>(nh), p4, l4, nw, g, out, a, s);
      return rc == 1 ? -1 : rc;
    }
    const int ng = ngrad == 0 ? 0 : (ngrad <= 4 ? 4 : (ngrad <= 8 ? 8 : 16));
    return qmk_adj::launch_tiles(static_cast<int>(nh), ng, p4, l4, nw, g, out, a, s);
  }
  if (nd > 3 || n - 1 < nd || nops > kMaxOps || ngrad > 16) return -1;
  std::sort(distinct, distinct + nd);
  GroupAdjArgs g{};
  OutSlots<kMaxOps> out{};
  out.p = d_grad;
  for (uint32_t k = 0; k < nd; k++) g.pos[k] = distinct[k] - 1;
  g.nops = nops;
  g.ngrad = static_cast<uint32_t>(ngrad);
  int gi = 0;
  for (uint32_t o = 0; o < nops; o++) {
    int where = -1;
    for (uint32_t k = 0; k < nd; k++)
      if (distinct[k] == wires[o]) where = static_cast<int>(k);
    g.where[o] = static_cast<int8_t>(where);
    g.gen[o] = static_cast<int8_t>(gens[o]);
    g.m[o] = m2_from(minv + 8 * o);
    if (gens[o]) {
      g.slotidx[o] = static_cast<uint8_t>(gi);
      out.slot[gi] = slots[o];
      gi++;
    }
  }
  const uint64_t nsites = 1ull << (n - 1 - nd);
  float4 *p4 = reinterpret_cast<float4 *>(psi), *l4 = reinterpret_cast<float4 *>(lam);
  cudaStream_t s = (cudaStream_t)stream;
  const Area a = area_of(ws);
  const int ng = ngrad == 0 ? 0 : (ngrad <= 4 ? 4 : (ngrad <= 8 ? 8 : 16));
#define QMK_ADJ_GROUP_CASE(KP)                                                  \
  if (nd == KP) {                                                               \
    if (ng == 0) launch_adj_group<KP, 0>(p4, l4, nsites, g, out, a, s);         \
    else if (ng == 4) launch_adj_group<KP, 4>(p4, l4, nsites, g, out, a, s);    \
    else if (ng == 8) launch_adj_group<KP, 8>(p4, l4, nsites, g, out, a, s);    \
    else launch_adj_group<KP, 16>(p4, l4, nsites, g, out, a, s);                \
  }
  QMK_ADJ_GROUP_CASE(0)
  QMK_ADJ_GROUP_CASE(1)
  QMK_ADJ_GROUP_CASE(2)
  QMK_ADJ_GROUP_CASE(3)
#undef QMK_ADJ_GROUP_CASE
  return launch_status();
}

extern "C" unsigned int *qmk_wait_counter(void *ws) {
  return ws ? area_of(ws).waits : nullptr;
}

extern "C" int qmk_set_wait_poll_limit(void *ws, size_t bytes, long long polls, void *stream) {
  if (!ok_ws(ws, bytes, 0)) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  // Stored as polls + 1 (0 keeps the kernels' full bound), capped at it.
  const unsigned int v =
      polls < 0 ? 0u : static_cast<unsigned int>(std::min<long long>(polls, 1ll << 22) + 1);
  cudaError_t e = cudaMemcpyAsync(area_of(ws).polls, &v, sizeof(v), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? 0 : static_cast<int>(e);
}

extern "C" int qmk_take_wait_timeouts(void *ws, size_t bytes, unsigned int *out, void *stream) {
  if (!out || !ok_ws(ws, bytes, 0)) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int *counter = area_of(ws).waits;
  cudaError_t e = cudaMemcpyAsync(out, counter, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && *out) {
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return e == cudaSuccess ? 0 : static_cast<int>(e);
}
