// k_diag.cu -- the fused diagonal layer: amplitude i *= exp(i phi(i)),
//   phi(i) = g + sum_t angle_t [mask_t fully set in i].
//
// Every mask the plan builder emits has one or two bits (Z/S/T/P/RZ, CZ/CP,
// and the three terms of a ZZ coupling), so after merging equal masks phi is
// a quadratic form in the index bits:
//   phi(i) = g + sum_q a_q x_q + sum_{q<r} b_qr x_q x_r .
// The reference evaluates every term per amplitude in FP32 (kernels.metal:
// 203-218), which stops being bandwidth bound near 75 terms. Here the index
// splits into a tile of W low bits (lo) and the tile number (hi):
//   phi = [g + phi_H(hi)] + sum_{r<W} x_r c_r(hi) + phi_L(lo)
// with c_r(hi) = sum of b_rq over partners q >= W set in hi (cross pairs).
//   * phi_L (low singles + low-low pairs) is the same for every tile: a prep
//     kernel tabulates TL[lo] = e^{i phi_L(lo)} once per layer (FP64 sums,
//     double sincos).
//   * per tile, the FP64 sums c_r(hi) and g + phi_H(hi) are formed once and
//     turned into factors f_r = e^{i c_r}, eH = e^{i(g+phi_H)}; the linear
//     part splits over bits 0..5 and 6..W-1 into two small tables Y1, Y2.
//   * per amplitude: factor = TL[lo] * Y1[lo & 63] * Y2[lo >> 6], then one
//     complex multiply of the amplitude.
// Masks of three or more bits (never produced by the plan passes) go through
// a direct per-amplitude FP64 kernel.
#include <algorithm>
#include <cstring>
#include <vector>

#include "kquad.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

// Offsets shared with the reduction kernels.
size_t qmk_reduce_area_offset() { return kDescBytes + kTableBytes; }

namespace {

__global__ void __launch_bounds__(kThreads)
k_diag(float4 *__restrict__ st, const DiagDesc *__restrict__ d,
       const float4 *__restrict__ table4, uint64_t ntiles) {
  __shared__ float2 f[kWMax];
  __shared__ float2 eH;
  __shared__ __align__(16) float2 Y1[64];
  __shared__ float2 Y2[1 << (kWMax - 6)];
  const uint32_t W = d->W;
  const uint32_t tid = threadIdx.x;
  const uint32_t nv = 1u << (W - 1);
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    tile_coeffs<true>(d, tile, f, &eH, nullptr, nullptr, false);
    __syncthreads();
    tile_phase_tables(W, f, eH, Y1, Y2);
    __syncthreads();
    const uint64_t base = tile << (W - 1);
    constexpr int UU = 4;
    for (uint32_t e0 = tid; e0 < nv; e0 += kThreads * UU) {
      float4 x[UU], t[UU];
#pragma unroll
      for (int k = 0; k < UU; k++) {
        const uint32_t e = e0 + k * kThreads;
        if (e < nv) {
          x[k] = st[base + e];
          t[k] = table4[e];
        }
      }
#pragma unroll
      for (int k = 0; k < UU; k++) {
        const uint32_t e = e0 + k * kThreads;
        if (e >= nv) continue;
        const uint32_t lo = 2 * e;
        const float4 y1 = *reinterpret_cast<const float4 *>(&Y1[lo & 63]);
        const float2 y2 = Y2[lo >> 6];
        const float2 f0 = cmul(cmul(lo2(t[k]), lo2(y1)), y2);
        const float2 f1 = cmul(cmul(hi2(t[k]), hi2(y1)), y2);
        st[base + e] = pack4(cmul(f0, lo2(x[k])), cmul(f1, hi2(x[k])));
      }
    }
    __syncthreads();
  }
}

constexpr int kGenericTerms = 64;
struct GenericTerms {
  uint32_t count;
  uint64_t mask[kGenericTerms];
  double angle[kGenericTerms];
};

// Direct evaluation, one amplitude per thread: only for masks of >= 3 bits.
__global__ void k_diag_generic(float2 *__restrict__ st, uint64_t dim, GenericTerms g) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= dim) return;
  double phi = 0.0;
  for (uint32_t t = 0; t < g.count; t++)
    if ((i & g.mask[t]) == g.mask[t]) phi += g.angle[t];
  st[i] = cmul(expi_reduced(phi), st[i]);
}

}  // namespace

extern "C" size_t qmk_workspace_bytes(uint32_t n) {
  (void)n;
  // Reduction area: 1024 blocks x 32 doubles of partials, then a counter.
  return kDescBytes + kTableBytes + 1024 * 32 * sizeof(double) + 256;
}

extern "C" int qmk_workspace_init(void *ws, size_t bytes, void *stream) {
  if (!ws || bytes < qmk_workspace_bytes(0)) return -1;
  cudaError_t e = cudaMemsetAsync(ws, 0, bytes, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : static_cast<int>(e);
}

extern "C" int qmk_apply_diagonal(float *state, uint32_t n, uint32_t nt,
                                  const uint64_t *masks, const double *angles,
                                  double global_phase, void *ws,
                                  size_t ws_bytes, void *stream) {
  if (!state || n < 1 || n > 40 || (nt && (!masks || !angles))) return -1;
  if (!ws || ws_bytes < qmk_workspace_bytes(n)) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t W = std::min<uint32_t>(n, kWMax);
  DiagDesc d;
  std::vector<uint64_t> gm;
  std::vector<double> ga;
  if (build_quad_desc(n, nt, masks, angles, global_phase, d, &gm, &ga) != 0) return -1;

  uint8_t *base = static_cast<uint8_t *>(ws);
  DiagDesc *dd = reinterpret_cast<DiagDesc *>(base);
  float2 *table = reinterpret_cast<float2 *>(base + kDescBytes);
  k_quad_prep<true><<<grid_for(1u << W, kThreads), kThreads, 0, s>>>(d, dd, table);
  int rc = launch_status();
  if (rc) return rc;
  const uint64_t ntiles = 1ull << (n - W);
  const uint64_t cap = static_cast<uint64_t>(qmk_host::num_sms()) * 8;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(ntiles, cap));
  k_diag<<<grid, kThreads, 0, s>>>(reinterpret_cast<float4 *>(state), dd,
                                   reinterpret_cast<const float4 *>(table), ntiles);
  rc = launch_status();
  if (rc) return rc;
  for (size_t b = 0; b < gm.size(); b += kGenericTerms) {
    GenericTerms g{};
    g.count = static_cast<uint32_t>(std::min<size_t>(kGenericTerms, gm.size() - b));
    for (uint32_t k = 0; k < g.count; k++) {
      g.mask[k] = gm[b + k];
      g.angle[k] = ga[b + k];
    }
    const uint64_t dim = 1ull << n;
    k_diag_generic<<<grid_for(dim, kThreads), kThreads, 0, s>>>(
        reinterpret_cast<float2 *>(state), dim, g);
    rc = launch_status();
    if (rc) return rc;
  }
  return 0;
}
