// k_sample.cu -- measurement sampling without collapsing or copying the state.
//
// Same algorithm as the reference sampler (src/metal/simulator.mm:677-763):
// |a|^2 summed per 1024-amplitude block, a CDF over the blocks, a splitmix64
// uniform per shot scaled by the actual total, a binary search for the block
// and a walk inside it. Everything here stays on the device: the block sums
// and the CDF are FP64 (device prefix scan), the walk is one warp per shot
// with an FP64 warp scan, and only the drawn indices travel to the host.
#include <algorithm>

#include "kcommon.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

namespace {

constexpr uint32_t kBlock = 1024;      // amplitudes per sampling block
constexpr uint32_t kScanItems = 8;     // entries per thread in the local scan
constexpr uint32_t kScanTile = kThreads * kScanItems;

uint64_t blocks_of(uint32_t n) {
  const uint64_t dim = 1ull << n;
  return (dim + kBlock - 1) / kBlock;
}

// One warp per block.
__global__ void __launch_bounds__(kThreads)
k_block_sums(const float2 *__restrict__ st, uint64_t dim, uint64_t nb, double *__restrict__ sums) {
  const uint64_t b = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (b >= nb) return;
  const uint64_t s = b * kBlock, e = min(s + kBlock, dim);
  float acc = 0.0f;
  for (uint64_t i = s + lane; i < e; i += 32) {
    const float2 a = st[i];
    acc = fmaf(a.x, a.x, fmaf(a.y, a.y, acc));
  }
  const double t = warp_sum(static_cast<double>(acc));
  if (lane == 0) sums[b] = t;
}

// FP64 inclusive warp scan.
__device__ __forceinline__ double warp_scan(double v, uint32_t lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= static_cast<uint32_t>(o)) v += u;
  }
  return v;
}

// Inclusive scan of one kScanTile slice in place; slice total to aux[tile].
__global__ void __launch_bounds__(kThreads)
k_scan_local(double *__restrict__ x, uint64_t count, double *__restrict__ aux) {
  __shared__ double wsum[kThreads / 32];
  const uint64_t base = static_cast<uint64_t>(blockIdx.x) * kScanTile + threadIdx.x * kScanItems;
  double v[kScanItems];
  double run = 0.0;
#pragma unroll
  for (int k = 0; k < static_cast<int>(kScanItems); k++) {
    const uint64_t i = base + k;
    run += (i < count) ? x[i] : 0.0;
    v[k] = run;
  }
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double inc = warp_scan(run, lane);
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  double woff = 0.0;
  for (uint32_t k = 0; k < w; k++) woff += wsum[k];
  const double off = woff + inc - run;
#pragma unroll
  for (int k = 0; k < static_cast<int>(kScanItems); k++) {
    const uint64_t i = base + k;
    if (i < count) x[i] = v[k] + off;
  }
  if (threadIdx.x == kThreads - 1 && aux) aux[blockIdx.x] = off + run;
}

// Single-CTA inclusive scan of the slice totals.
__global__ void __launch_bounds__(kThreads) k_scan_aux(double *__restrict__ aux, uint64_t count) {
  __shared__ double wsum[kThreads / 32];
  __shared__ double carry;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint64_t c0 = 0; c0 < count; c0 += kThreads) {
    const uint64_t i = c0 + threadIdx.x;
    const double v = (i < count) ? aux[i] : 0.0;
    const double inc = warp_scan(v, lane);
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    double woff = 0.0;
    for (uint32_t k = 0; k < w; k++) woff += wsum[k];
    if (i < count) aux[i] = carry + woff + inc;
    __syncthreads();
    if (threadIdx.x == kThreads - 1) carry += woff + inc;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads)
k_scan_add(double *__restrict__ x, uint64_t count, const double *__restrict__ aux) {
  const uint64_t tile = blockIdx.x + 1;  // slice 0 needs no offset
  const double off = aux[tile - 1];
  const uint64_t base = tile * kScanTile;
  for (uint32_t k = threadIdx.x; k < kScanTile; k += kThreads) {
    const uint64_t i = base + k;
    if (i < count) x[i] += off;
  }
}

__device__ __forceinline__ uint64_t splitmix_at(uint64_t seed, uint64_t k) {
  // The (k+1)-th output of splitmix64 seeded with `seed`: the state advances
  // by the golden gamma before every output, so it is counter based.
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One warp per shot.
__global__ void __launch_bounds__(kThreads)
k_draw(const float2 *__restrict__ st, uint64_t dim, const double *__restrict__ cdf, uint64_t nb,
       uint64_t shots, uint64_t seed, uint64_t *__restrict__ out) {
  const uint64_t k = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (k >= shots) return;
  const double total = cdf[nb - 1];
  if (!(total > 0.0)) {
    if (lane == 0) out[k] = 0;
    return;
  }
  uint64_t b = 0;
  double rem = 0.0;
  if (lane == 0) {
    const double u = static_cast<double>(splitmix_at(seed, k) >> 11) *
                     (1.0 / 9007199254740992.0) * total;
    uint64_t lo = 0, hi = nb - 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    b = lo;
    rem = u - (lo > 0 ? cdf[lo - 1] : 0.0);
  }
  b = __shfl_sync(0xffffffffu, b, 0);
  rem = __shfl_sync(0xffffffffu, rem, 0);
  const uint64_t s = b * kBlock, e = min(s + kBlock, dim);
  double acc = 0.0;
  int64_t last_nz = -1;
  for (uint64_t c0 = s; c0 < e; c0 += 32) {
    const uint64_t i = c0 + lane;
    double pr = 0.0;
    if (i < e) {
      const float2 a = st[i];
      const double re = a.x, im = a.y;
      pr = re * re + im * im;
    }
    const double pre = warp_scan(pr, lane);
    const unsigned hit = __ballot_sync(0xffffffffu, i < e && acc + pre > rem);
    if (hit) {
      if (lane == 0) out[k] = c0 + (__ffs(hit) - 1);
      return;
    }
    const unsigned nz = __ballot_sync(0xffffffffu, pr > 0.0);
    if (nz) last_nz = static_cast<int64_t>(c0 + (31 - __clz(nz)));
    acc += __shfl_sync(0xffffffffu, pre, 31);
  }
  if (lane == 0) out[k] = last_nz >= 0 ? static_cast<uint64_t>(last_nz) : e - 1;
}

}  // namespace

extern "C" size_t qmk_sample_workspace_bytes(uint32_t n) {
  const uint64_t nb = blocks_of(n);
  const uint64_t na = (nb + kScanTile - 1) / kScanTile;
  return static_cast<size_t>((nb + na + 32) * sizeof(double));
}

extern "C" int qmk_sample(const float *state, uint32_t n, uint64_t shots, uint64_t seed,
                          uint64_t *d_out, void *ws, size_t ws_bytes, void *stream) {
  if (!state || n < 1 || n > 40 || !ws || ws_bytes < qmk_sample_workspace_bytes(n)) return -1;
  if (shots == 0) return 0;
  if (!d_out) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t dim = 1ull << n, nb = blocks_of(n);
  const uint64_t na = (nb + kScanTile - 1) / kScanTile;
  double *cdf = static_cast<double *>(ws);
  double *aux = cdf + nb;
  k_block_sums<<<grid_for(nb * 32, kThreads), kThreads, 0, s>>>(
      reinterpret_cast<const float2 *>(state), dim, nb, cdf);
  int rc = launch_status();
  if (rc) return rc;
  k_scan_local<<<static_cast<unsigned>(na), kThreads, 0, s>>>(cdf, nb, na > 1 ? aux : nullptr);
  if ((rc = launch_status())) return rc;
  if (na > 1) {
    k_scan_aux<<<1, kThreads, 0, s>>>(aux, na);
    if ((rc = launch_status())) return rc;
    k_scan_add<<<static_cast<unsigned>(na - 1), kThreads, 0, s>>>(cdf, nb, aux);
    if ((rc = launch_status())) return rc;
  }
  k_draw<<<grid_for(shots * 32, kThreads), kThreads, 0, s>>>(
      reinterpret_cast<const float2 *>(state), dim, cdf, nb, shots, seed, d_out);
  return launch_status();
}
