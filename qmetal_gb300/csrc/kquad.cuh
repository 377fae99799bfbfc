// kquad.cuh -- index-bit quadratic forms, shared by the diagonal-layer pass,
// the Z-Hamiltonian co-state and the fused adjoint of diagonal layers.
//
// A sum of Z-type terms whose masks have one or two bits is a quadratic form
// in the index bits x_q:  f(i) = g + sum_q a_q x_q + sum_{q<r} b_qr x_q x_r.
// With the index split into a W-bit tile (lo) and the tile number (hi),
//   f = [g + f_H(hi)] + sum_{r<W} x_r c_r(hi) + f_L(lo),
// where c_r(hi) sums b_rq over partners q >= W set in hi ("cross pairs").
// f_L is tabulated once per layer by a prep kernel; per tile, the FP64 sums
// c_r and g + f_H are formed once (tile_coeffs) and every amplitude then costs
// a few table reads.
#pragma once

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "kcommon.cuh"

namespace qmk {

constexpr uint32_t kWMax = 13;
constexpr uint32_t kMaxPairs = 600;  // n <= 34 has at most 561 distinct pairs

struct alignas(16) DiagDesc {
  uint32_t n, W;
  uint32_t nlow, ncross, nhigh;     // pair segments, in this order
  uint32_t coff[kWMax + 1];         // cross pairs of low bit r: nlow+coff[r] ..
  double g;
  double a[64];                     // single-bit coefficients per wire
  uint16_t pq[kMaxPairs];           // low wire | high wire << 8
  double pb[kMaxPairs];
};

// Workspace layout (qmk_workspace_bytes): [desc][low-bit table][reduction area].
constexpr size_t kDescBytes = (sizeof(DiagDesc) + 255) & ~size_t(255);
constexpr size_t kTableBytes = sizeof(float2) << kWMax;

// Merge (mask, coefficient) terms into the quadratic form. Masks of three or
// more bits are returned in wide_m / wide_c for a direct kernel. Returns -1 on
// a mask outside n bits or too many distinct pairs.
inline int build_quad_desc(uint32_t n, uint32_t nt, const uint64_t *masks, const double *coef,
                           double g, DiagDesc &d, std::vector<uint64_t> *wide_m,
                           std::vector<double> *wide_c) {
  const uint32_t W = std::min<uint32_t>(n, kWMax);
  std::memset(&d, 0, sizeof(d));
  d.n = n;
  d.W = W;
  d.g = g;
  std::map<std::pair<uint32_t, uint32_t>, double> pairs;
  for (uint32_t t = 0; t < nt; t++) {
    const uint64_t m = masks[t];
    if (n < 64 && (m >> n)) return -1;
    const int pc = __builtin_popcountll(m);
    if (pc == 0) {
      d.g += coef[t];
    } else if (pc == 1) {
      d.a[__builtin_ctzll(m)] += coef[t];
    } else if (pc == 2) {
      const uint32_t q = __builtin_ctzll(m), r = 63 - __builtin_clzll(m);
      pairs[{q, r}] += coef[t];
    } else {
      if (!wide_m || !wide_c) return -1;
      wide_m->push_back(m);
      wide_c->push_back(coef[t]);
    }
  }
  if (pairs.size() > kMaxPairs) return -1;
  std::vector<std::pair<uint32_t, double>> low, high;
  std::vector<std::vector<std::pair<uint32_t, double>>> cross(W);
  for (const auto &kv : pairs) {
    const uint32_t q = kv.first.first, r = kv.first.second;
    const uint32_t packed = q | (r << 8);
    if (r < W) low.push_back({packed, kv.second});
    else if (q < W) cross[q].push_back({packed, kv.second});
    else high.push_back({packed, kv.second});
  }
  uint32_t p = 0;
  for (auto &e : low) { d.pq[p] = uint16_t(e.first); d.pb[p] = e.second; p++; }
  d.nlow = p;
  for (uint32_t r = 0; r < W; r++) {
    d.coff[r] = p - d.nlow;
    for (auto &e : cross[r]) { d.pq[p] = uint16_t(e.first); d.pb[p] = e.second; p++; }
  }
  d.coff[W] = p - d.nlow;
  for (uint32_t r = W + 1; r <= kWMax; r++) d.coff[r] = d.coff[W];
  d.ncross = p - d.nlow;
  for (auto &e : high) { d.pq[p] = uint16_t(e.first); d.pb[p] = e.second; p++; }
  d.nhigh = p - d.nlow - d.ncross;
  return 0;
}

// Copy the descriptor into the workspace and tabulate f_L over the 2^W low
// indices: e^{i f_L} (PHASE) as float2, or f_L itself as float.
template <bool PHASE>
__global__ void k_quad_prep(const DiagDesc d, DiagDesc *__restrict__ out, void *__restrict__ table) {
  if (blockIdx.x == 0) {
    const uint64_t *src = reinterpret_cast<const uint64_t *>(&d);
    uint64_t *dst = reinterpret_cast<uint64_t *>(out);
    for (uint32_t k = threadIdx.x; k < sizeof(DiagDesc) / 8; k += blockDim.x) dst[k] = src[k];
  }
  const uint32_t lo = blockIdx.x * blockDim.x + threadIdx.x;
  if (lo >= (1u << d.W)) return;
  double f = 0.0;
  for (uint32_t r = 0; r < d.W; r++)
    if (lo >> r & 1) f += d.a[r];
  for (uint32_t p = 0; p < d.nlow; p++) {
    const uint32_t q = d.pq[p] & 255, r = d.pq[p] >> 8;
    if ((lo >> q & 1) && (lo >> r & 1)) f += d.pb[p];
  }
  if (PHASE) {
    double s, c;
    sincos(f, &s, &c);
    static_cast<float2 *>(table)[lo] = make_float2(static_cast<float>(c), static_cast<float>(s));
  } else {
    static_cast<float *>(table)[lo] = static_cast<float>(f);
  }
}

// Per-tile FP64 coefficients c[r] (threads 0..W-1) and h = g + f_H(tile)
// (warp 1), delivered as what the caller needs: PHASE writes the unit factors
// f[r] = e^{+-i c_r} and *eh = e^{+-i h} (sign -1 for conj); otherwise the
// sums themselves as floats. The caller synchronises before reading them.
template <bool PHASE>
__device__ __forceinline__ void tile_coeffs(const DiagDesc *__restrict__ d, uint64_t tile,
                                            float2 *f, float2 *eh, float *cr, float *hr,
                                            bool conj) {
  const uint32_t W = d->W, n = d->n, tid = threadIdx.x;
  const float sg = conj ? -1.0f : 1.0f;
  if (tid < W) {
    double s = 0.0;
    const uint32_t b0 = d->nlow + d->coff[tid], b1 = d->nlow + d->coff[tid + 1];
    for (uint32_t p = b0; p < b1; p++) {
      const uint32_t hq = d->pq[p] >> 8;
      if (tile >> (hq - W) & 1) s += d->pb[p];
    }
    if (PHASE) {
      const float2 e = expi_reduced(s);
      f[tid] = make_float2(e.x, sg * e.y);
    } else {
      cr[tid] = static_cast<float>(s);
    }
  } else if (tid >= 32 && tid < 64) {
    const uint32_t lane = tid - 32;
    double s = 0.0;
    for (uint32_t q = W + lane; q < n; q += 32)
      if (tile >> (q - W) & 1) s += d->a[q];
    const uint32_t p0 = d->nlow + d->ncross, p1 = p0 + d->nhigh;
    for (uint32_t p = p0 + lane; p < p1; p += 32) {
      const uint32_t q = d->pq[p] & 255, r = d->pq[p] >> 8;
      if ((tile >> (q - W) & 1) && (tile >> (r - W) & 1)) s += d->pb[p];
    }
    s = warp_sum(s);
    if (lane == 0) {
      if (PHASE) {
        const float2 e = expi_reduced(d->g + s);
        *eh = make_float2(e.x, sg * e.y);
      } else {
        *hr = static_cast<float>(d->g + s);
      }
    }
  }
}

// Factor tables of one tile: Y1[u] over low bits 0..5 (threads 0..63) and
// Y2[e] over bits 6..W-1 (threads 64..), Y2 carrying the tile constant.
// Complex products of the unit factors, or real sums.
__device__ __forceinline__ void tile_phase_tables(uint32_t W, const float2 *f, float2 eh,
                                                  float2 *Y1, float2 *Y2) {
  const uint32_t w1 = W < 6 ? W : 6, w2 = W - w1, tid = threadIdx.x;
  if (tid < (1u << w1)) {
    float2 y = make_float2(1.0f, 0.0f);
    for (uint32_t r = 0; r < w1; r++)
      if (tid >> r & 1) y = cmul(y, f[r]);
    Y1[tid] = y;
  } else if (tid >= 64 && tid - 64 < (1u << w2)) {
    const uint32_t e = tid - 64;
    float2 y = eh;
    for (uint32_t r = 0; r < w2; r++)
      if (e >> r & 1) y = cmul(y, f[w1 + r]);
    Y2[e] = y;
  }
}

__device__ __forceinline__ void tile_real_tables(uint32_t W, const float *c, float h, float *Y1,
                                                 float *Y2) {
  const uint32_t w1 = W < 6 ? W : 6, w2 = W - w1, tid = threadIdx.x;
  if (tid < (1u << w1)) {
    float y = 0.0f;
    for (uint32_t r = 0; r < w1; r++)
      if (tid >> r & 1) y += c[r];
    Y1[tid] = y;
  } else if (tid >= 64 && tid - 64 < (1u << w2)) {
    const uint32_t e = tid - 64;
    float y = h;
    for (uint32_t r = 0; r < w2; r++)
      if (e >> r & 1) y += c[w1 + r];
    Y2[e] = y;
  }
}

}  // namespace qmk
