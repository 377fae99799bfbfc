// k_xfield.cu -- the co-state of a transverse field: terms that each flip
// one wire with a real coefficient and nothing else (sum_w c_w X_w, the
// field of a TFIM Hamiltonian or an X mixer), up to seven wires >= 6 and any
// of wires 0..5 per pass.
//
// A site is 2^(4 + WB) rows of 32 psi vectors (one 512-byte row per warp
// load), the rows picked by the pass's wires >= 6; 2^WB warps hold a site,
// sixteen rows each. The site sits in shared memory, so the source of every
// term -- the same row on another lane (wires 1..5), the other half of the
// vector (wire 0), another row (wires >= 6) -- is one 16-byte shared-memory
// read, and psi is read from HBM once for all of the pass's terms. The
// outputs of a thread's sixteen rows stay in registers while the next
// site's rows stream in by cp.async; then lambda is read (unless the pass
// overwrites it), added to and stored, one 512-byte row per warp access.
//
// The same pass adds sum_w c_w <psi|X_w|psi> = sum_v Re(conj(psi_v) out_v)
// to the energy, so a Hamiltonian of short Z strings (its own pass) and a
// transverse field needs no separate energy pass.
#include <algorithm>
#include <atomic>
#include <vector>

#include "kreduce.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

namespace {

struct XFieldArgs {
  uint32_t pos[7];   // vector bits (wire - 1) of the site's wires >= 6, ascending
  float ch[7];       // their coefficients (0 for a wire that only shapes the site)
  float c0;          // wire 0
  float cl[5];       // wires 1..5
  uint32_t overwrite;
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(smem))),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void axpy4(float4 &s, float c, const float4 &x) {
  s.x = fmaf(c, x.x, s.x);
  s.y = fmaf(c, x.y, s.y);
  s.z = fmaf(c, x.z, s.z);
  s.w = fmaf(c, x.w, s.w);
}

template <int WB, bool LOW, bool ENERGY>
__global__ void __launch_bounds__(kThreads, 2)
k_xfield_blk(float4 *__restrict__ lam, const float4 *__restrict__ psi, uint64_t nsites,
             XFieldArgs c, Area a, OutContig out) {
  constexpr int NV = 16;
  constexpr int KB = 4 + WB;                  // wires >= 6 in the site
  constexpr int NW = 1 << WB;                 // warps per site
  constexpr int SPB = (kThreads / 32) / NW;   // sites per block
  constexpr int ROWS = NV * NW;
  static_assert(SPB >= 1 && SPB * NW == kThreads / 32, "whole sites per block");
  extern __shared__ __align__(16) float4 xf[];   // [site][row][32 lanes]
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t sib = warp / NW, wsl = warp % NW;
  float4 *site = xf + static_cast<size_t>(sib) * ROWS * 32;
  const uint64_t per_round = static_cast<uint64_t>(gridDim.x) * SPB;
  const uint64_t rounds = (nsites + per_round - 1) / per_round;
  // Row l of this warp is site row l | wsl << 4; its vector offset (the
  // row's wire bits) is worked out once.
  __shared__ uint64_t row_off[kThreads / 32][NV];
  if (lane < NV) {
    const uint32_t row = lane | (wsl << 4);
    uint64_t v = 0;
#pragma unroll
    for (int j = 0; j < KB; j++)
      if ((row >> j) & 1u) v |= 1ull << c.pos[j];
    row_off[warp][lane] = v;
  }
  __syncwarp();
  auto site_of = [&](uint64_t r) {
    return r * per_round + static_cast<uint64_t>(blockIdx.x) * SPB + sib;
  };
  auto base_of = [&](uint64_t sidx) {
    uint64_t b = sidx * 32 + lane;
#pragma unroll
    for (int j = 0; j < KB; j++) b = ins0(b, c.pos[j]);
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
        cp_async16(site + ((l | (wsl << 4)) * 32 + lane), psi + (base | row_off[warp][l]));
    }
    cp_async_commit();
  };
  double acc[1] = {0.0};
  prefetch(0);
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t sidx = site_of(r);
    const bool active = sidx < nsites;   // uniform over the site's warps
    cp_async_wait_all();
    site_sync();   // every warp's rows of this site have landed
    float4 o[NV];
    float part = 0.0f;
    if (active) {
#pragma unroll
      for (int l = 0; l < NV; l++) {
        const uint32_t row = l | (wsl << 4);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 4; j++) axpy4(s, c.ch[j], site[(row ^ (1u << j)) * 32 + lane]);
#pragma unroll
        for (int j = 0; j < WB; j++)
          axpy4(s, c.ch[4 + j], site[(row ^ (16u << j)) * 32 + lane]);
        if constexpr (LOW || ENERGY) {
          const float4 own = site[row * 32 + lane];
          if constexpr (LOW) {
            axpy4(s, c.c0, make_float4(own.z, own.w, own.x, own.y));
#pragma unroll
            for (int k = 0; k < 5; k++)
              axpy4(s, c.cl[k], site[row * 32 + (lane ^ (1u << k))]);
          }
          if constexpr (ENERGY)
            part = fmaf(own.x, s.x, fmaf(own.y, s.y, fmaf(own.z, s.z, fmaf(own.w, s.w, part))));
        }
        o[l] = s;
      }
    }
    site_sync();   // every warp has read the site: its slots take the next one
    prefetch(r + 1);
    if (active) {
      const uint64_t base = base_of(sidx);
      constexpr int Q = 4;   // lambda rows in flight per thread
#pragma unroll
      for (int h = 0; h < NV / Q; h++) {
        if (!c.overwrite) {
          float4 x[Q];
#pragma unroll
          for (int l = 0; l < Q; l++) x[l] = lam[base | row_off[warp][h * Q + l]];
#pragma unroll
          for (int l = 0; l < Q; l++) {
            float4 &y = o[h * Q + l];
            y = make_float4(y.x + x[l].x, y.y + x[l].y, y.z + x[l].z, y.w + x[l].w);
          }
        }
#pragma unroll
        for (int l = 0; l < Q; l++) lam[base | row_off[warp][h * Q + l]] = o[h * Q + l];
      }
      acc[0] += part;
    }
  }
  if constexpr (ENERGY) finish<1>(acc, 1, a, out);
}

template <int WB, bool LOW, bool ENERGY>
int launch_xfield(float4 *lam, const float4 *psi, uint64_t nsites, const XFieldArgs &c, Area a,
                  OutContig out, cudaStream_t s) {
  constexpr int SPB = (kThreads / 32) >> WB;
  unsigned grid = grid_for(nsites, SPB);
  grid = std::min<unsigned>(grid, static_cast<unsigned>(qmk_host::num_sms()) * 2);
  const size_t smem = static_cast<size_t>(kThreads / 32) * 16 * 32 * sizeof(float4);
  // The opt-in above 48 KiB is per device; set it once on each.
  static std::atomic<bool> opted[64];   // zero-initialised: false
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
  if (!opted[dev]) {
    const cudaError_t e = cudaFuncSetAttribute(k_xfield_blk<WB, LOW, ENERGY>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(smem));
    if (e != cudaSuccess) return static_cast<int>(e);
    opted[dev] = true;
  }
  k_xfield_blk<WB, LOW, ENERGY><<<grid, kThreads, smem, s>>>(lam, psi, nsites, c, a, out);
  return launch_status();
}

template <int WB>
int launch_xfield_wb(bool low, bool energy, float4 *lam, const float4 *psi, uint64_t nsites,
                     const XFieldArgs &c, Area a, OutContig out, cudaStream_t s) {
  if (low)
    return energy ? launch_xfield<WB, true, true>(lam, psi, nsites, c, a, out, s)
                  : launch_xfield<WB, true, false>(lam, psi, nsites, c, a, out, s);
  return energy ? launch_xfield<WB, false, true>(lam, psi, nsites, c, a, out, s)
                : launch_xfield<WB, false, false>(lam, psi, nsites, c, a, out, s);
}

bool ok_ws(void *ws, size_t bytes, uint32_t n) {
  return ws && bytes >= qmk_workspace_bytes(n);
}

}  // namespace

extern "C" int qmk_xfield_costate(float *lam, const float *psi, uint32_t n, uint32_t num_wires,
                                  const uint32_t *wires, const double *coeffs, int overwrite,
                                  double *d_energy, int energy, void *ws, size_t ws_bytes,
                                  void *stream) {
  if (!lam || !psi || n < 10 || n > 40 || num_wires < 1 || num_wires > 13 || !wires || !coeffs ||
      energy < 0 || energy > 2 || (energy && (!d_energy || !ok_ws(ws, ws_bytes, n))))
    return -1;
  XFieldArgs c{};
  c.overwrite = overwrite ? 1u : 0u;
  std::vector<uint32_t> high;
  std::vector<double> hc;
  uint32_t seen_low = 0;
  bool low = false;
  for (uint32_t t = 0; t < num_wires; t++) {
    const uint32_t w = wires[t];
    if (w >= n) return -1;
    if (w < 6) {
      if ((seen_low >> w) & 1u) return -1;   // each wire once
      seen_low |= 1u << w;
      low = true;
      if (w == 0) c.c0 = static_cast<float>(coeffs[t]);
      else c.cl[w - 1] = static_cast<float>(coeffs[t]);
    } else {
      if (std::find(high.begin(), high.end(), w) != high.end()) return -1;
      high.push_back(w);
      hc.push_back(coeffs[t]);
    }
  }
  if (high.size() > 7) return -1;
  // A site holds at least four wires >= 6, and six rather than five where the
  // width allows (the five-wire form spills at two blocks per multiprocessor):
  // wires without a term (the lowest free ones) shape it with coefficient 0.
  std::vector<double> coef_of(n, 0.0);
  for (size_t j = 0; j < high.size(); j++) coef_of[high[j]] = hc[j];
  const size_t want = high.size() <= 4 ? 4 : std::max<size_t>(6, high.size());
  for (uint32_t w = 6; w < n && high.size() < want; w++)
    if (std::find(high.begin(), high.end(), w) == high.end()) high.push_back(w);
  if (high.size() < 4) return -1;
  std::sort(high.begin(), high.end());
  const uint32_t kb = static_cast<uint32_t>(high.size());
  for (uint32_t j = 0; j < kb; j++) {
    c.pos[j] = high[j] - 1;
    c.ch[j] = static_cast<float>(coef_of[high[j]]);
  }
  const uint64_t nsites = 1ull << (n - 6 - kb);
  float4 *l4 = reinterpret_cast<float4 *>(lam);
  const float4 *p4 = reinterpret_cast<const float4 *>(psi);
  const Area a = energy ? area_of(ws) : Area{};
  const OutContig out{d_energy, energy == 2};
  cudaStream_t s = (cudaStream_t)stream;
  const bool e = energy != 0;
  switch (kb) {
    case 4: return launch_xfield_wb<0>(low, e, l4, p4, nsites, c, a, out, s);
    case 5: return launch_xfield_wb<1>(low, e, l4, p4, nsites, c, a, out, s);
    case 6: return launch_xfield_wb<2>(low, e, l4, p4, nsites, c, a, out, s);
    default: return launch_xfield_wb<3>(low, e, l4, p4, nsites, c, a, out, s);
  }
}
