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
#include <vector>

#include "kquad.cuh"
#include "kreduce.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

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

constexpr int kMaxGen = 32;

template <int T>
struct DiagAdjArgs {
  uint32_t ngen;
  uint32_t undo;
  uint64_t fixmask[T > 0 ? T : 1];   // generator bits outside {0, 9..12}
  uint8_t vm[T > 0 ? T : 1];         // generator bits inside, as j bits
};

template <int T>
__global__ void __launch_bounds__(kThreads)
k_adj_diag(float4 *__restrict__ psi, float4 *__restrict__ lam, const DiagDesc *__restrict__ d,
           const float4 *__restrict__ table4, uint64_t ntiles, DiagAdjArgs<T> g, Area a,
           OutSlots<(T > 0 ? T : 1)> out) {
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
  __shared__ uint64_t fm[T > 0 ? T : 1];
  uint32_t own_sign = 0;
  if (T > 0) {
    const uint64_t mine = static_cast<uint64_t>(tid) << 1;
    for (int t = 0; t < T && t < static_cast<int>(g.ngen); t++)
      own_sign |= static_cast<uint32_t>(parity64(mine & g.fixmask[t])) << t;
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
    if (T > 0) {
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
      const uint32_t tile_sign =
          __ballot_sync(0xffffffffu, mine && parity64(tbits & fm[lane < T ? lane : 0]));
      const uint32_t sign = own_sign ^ tile_sign;
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

__device__ __forceinline__ float overlap(int gen, float2 p0, float2 p1, float2 l0, float2 l1) {
  float2 w0, w1;
  if (gen == 1) {
    w0 = p1; w1 = p0;
  } else if (gen == 2) {
    w0 = make_float2(p1.y, -p1.x);
    w1 = make_float2(-p0.y, p0.x);
  } else {
    w0 = p0; w1 = make_float2(-p1.x, -p1.y);
  }
  return (l0.x * w0.y - l0.y * w0.x) + (l1.x * w1.y - l1.y * w1.x);
}

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

// ---------------------------------------------------------------------------
// Wider window tiles for both states: a warp owns 32 consecutive vectors
// (lane = vector bits 0..4, i.e. wires 1..5) for every combination of up to
// KH wires >= 6 held in registers, so all accesses are full 512-byte warp
// accesses. Wire 0 pairs the lanes of a vector; a wire in 1..5 exchanges
// with the partner lane by shuffle, and each lane then takes its own half of
// the overlap (the two halves of a pair sum to the pair's term).

constexpr int kMaxWarpOps = 32;

struct WarpAdjArgs {
  uint32_t nops, ngrad;
  uint32_t hpos[4];              // wires >= 6: vector bit - 5, ascending
  int8_t kind[kMaxWarpOps];      // 0: wire 0, 1: lane bit, 2: register bit,
                                 // 3: the wire split across a warp pair
  int8_t arg[kMaxWarpOps];       // lane bit (0..4) or register index
  int8_t gen[kMaxWarpOps];
  int8_t slotidx[kMaxWarpOps];
  int8_t cls[kMaxWarpOps];       // kMat* structure of m
  M2 m[kMaxWarpOps];
};


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
  // FP32 per thread over its sites (a few dozen at most), FP64 from the warp up.
  float accf[NA];
#pragma unroll
  for (int t = 0; t < NA; t++) accf[t] = 0.0f;
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
      if (NG > 0 && gen) {
#pragma unroll
        for (int t = 0; t < NA; t++)
          if (t == g.slotidx[o]) accf[t] += ov;
      }
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
    for (int t = 0; t < NA; t++) acc[t] = accf[t];
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
  float accf[NA];
#pragma unroll
  for (int t = 0; t < NA; t++) accf[t] = 0.0f;
  // Every warp of the block runs the same number of rounds (the barriers of
  // the exchanges must match); a pair past the last tile works on zeros and
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
          __syncthreads();
        }
        const bool one = half != 0;
        switch (cls) {
          case kMatReal: ov = split_op<kMatReal>(P, L, oth_p, oth_l, one, gen, m); break;
          case kMatRx: ov = split_op<kMatRx>(P, L, oth_p, oth_l, one, gen, m); break;
          case kMatDiag: ov = split_op<kMatDiag>(P, L, oth_p, oth_l, one, gen, m); break;
          default: ov = split_op<kMatGeneral>(P, L, oth_p, oth_l, one, gen, m); break;
        }
        if (need) __syncthreads();
      } else {
        switch (cls) {
          case kMatReal: ov = warp_op<NV, kMatReal>(P, L, kind, arg, gen, m, lane); break;
          case kMatRx: ov = warp_op<NV, kMatRx>(P, L, kind, arg, gen, m, lane); break;
          case kMatDiag: ov = warp_op<NV, kMatDiag>(P, L, kind, arg, gen, m, lane); break;
          default: ov = warp_op<NV, kMatGeneral>(P, L, kind, arg, gen, m, lane); break;
        }
      }
      if (NG > 0 && gen) {
#pragma unroll
        for (int t = 0; t < NA; t++)
          if (t == g.slotidx[o]) accf[t] += ov;
      }
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
    for (int t = 0; t < NA; t++) acc[t] = accf[t];
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
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(ntiles, reduce_grid()));
  k_adj_diag<T><<<grid, kThreads, 0, s>>>(reinterpret_cast<float4 *>(psi),
                                           reinterpret_cast<float4 *>(lam), dd,
                                           reinterpret_cast<const float4 *>(table), ntiles, g,
                                           area_of(ws), out);
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
  if (ngen > kMaxGen || (ngen && (!gen_masks || !slots || !d_grad))) return -1;
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
  if (ngen <= 8)
    return launch_adj_diag<8>(psi, lam, n, dd, table, ngen, gen_masks, slots, d_grad, undo != 0, ws, s);
  if (ngen <= 16)
    return launch_adj_diag<16>(psi, lam, n, dd, table, ngen, gen_masks, slots, d_grad, undo != 0, ws, s);
  return launch_adj_diag<32>(psi, lam, n, dd, table, ngen, gen_masks, slots, d_grad, undo != 0, ws, s);
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
  bool w0 = false;
  int ngrad = 0;
  for (uint32_t o = 0; o < nops; o++) {
    if (wires[o] >= n || gens[o] < 0 || gens[o] > 3) return -1;
    if (gens[o] && (!slots || !d_grad)) return -1;
    if (gens[o]) ngrad++;
    if (wires[o] == 0) {
      w0 = true;
      continue;
    }
    bool seen = false;
    for (uint32_t k = 0; k < nd; k++) seen |= distinct[k] == wires[o];
    if (!seen) {
      distinct[nd++] = wires[o];
      if (wires[o] >= 6) high[nh++] = wires[o];
    }
  }
  if (ngrad > 16) return -1;
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
      g.slotidx[o] = -1;
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
    const int ng = ngrad == 0 ? 0 : (ngrad <= 4 ? 4 : (ngrad <= 8 ? 8 : 16));
    if (nh == 4) {
      // two warps per tile: the fourth register wire is split across the pair
      for (uint32_t o = 0; o < nops; o++)
        if (g.kind[o] == 2 && g.arg[o] == 3) g.kind[o] = 3;
      if (ng == 0) return launch_adj_pair<0>(p4, l4, nw, g, out, a, s);
      if (ng == 4) return launch_adj_pair<4>(p4, l4, nw, g, out, a, s);
      if (ng == 8) return launch_adj_pair<8>(p4, l4, nw, g, out, a, s);
      return launch_adj_pair<16>(p4, l4, nw, g, out, a, s);
    }
#define QMK_ADJ_WARP_CASE(KH)                                                   \
    if (nh == KH) {                                                             \
      if (ng == 0) launch_adj_warp<KH, 0>(p4, l4, nw, g, out, a, s);            \
      else if (ng == 4) launch_adj_warp<KH, 4>(p4, l4, nw, g, out, a, s);       \
      else if (ng == 8) launch_adj_warp<KH, 8>(p4, l4, nw, g, out, a, s);       \
      else launch_adj_warp<KH, 16>(p4, l4, nw, g, out, a, s);                   \
    }
    QMK_ADJ_WARP_CASE(0)
    QMK_ADJ_WARP_CASE(1)
    QMK_ADJ_WARP_CASE(2)
    QMK_ADJ_WARP_CASE(3)
    QMK_ADJ_WARP_CASE(4)
#undef QMK_ADJ_WARP_CASE
    return launch_status();
  }
  if (nd > 3 || n - 1 < nd || nops > kMaxOps) return -1;
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
  (void)w0;  // wire 0 is the lane pair of every vector; it needs no tile bit
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
