// kreduce.cuh -- the deterministic device-wide reduction used by every
// kernel that returns numbers (norms, expectations, energies, gradients).
//
// Each block reduces its FP64 accumulators (warp shuffles, then shared
// memory) into per-block partials in the workspace; the last block to finish
// (atomic ticket) sums the partials in block order and hands each total to an
// output functor. A result depends only on the grid size, never on timing.
#pragma once

#include <algorithm>

#include "kcommon.cuh"

size_t qmk_reduce_area_offset();  // k_diag.cu

namespace qmk {

constexpr uint32_t kMaxBlocks = 1024;

struct Area {
  double *partials;   // kMaxBlocks x 32
  unsigned *counter;  // last-block ticket, back to 0 after each reduction
  unsigned *waits;    // bounded waits that gave up in passes on this workspace
  unsigned *polls;    // 0: waits take the full bound; k > 0: they give up after k - 1 polls
};

inline Area area_of(void *ws) {
  uint8_t *b = static_cast<uint8_t *>(ws) + qmk_reduce_area_offset();
  Area a;
  a.partials = reinterpret_cast<double *>(b);
  a.counter = reinterpret_cast<unsigned *>(b + kMaxBlocks * 32 * sizeof(double));
  a.waits = a.counter + 16;  // 64 bytes into the 256-byte tail, its own line
  a.polls = a.counter + 32;  // 128 bytes in: a test's poll limit for those waits
  return a;
}

inline unsigned reduce_grid() {
  return std::min<unsigned>(kMaxBlocks, static_cast<unsigned>(qmk_host::num_sms()) * 4);
}

// out[t] = s (or out[t] += s).
struct OutContig {
  double *p;
  bool add;
  __device__ void operator()(int t, double s) const { p[t] = add ? p[t] + s : s; }
};

// out[slot[t]] = s: results scattered to their gate's gradient entry.
template <int T>
struct OutSlots {
  double *p;
  uint32_t slot[T];
  __device__ void operator()(int t, double s) const { p[slot[t]] = s; }
};

__host__ __device__ constexpr int pow2_at_least(int t) {
  return t <= 1 ? 1 : 2 * pow2_at_least((t + 1) / 2);
}

// Transposed butterfly over P = 2^k slots: each step halves the slots a lane
// carries and trades the other half with its partner, so lane l ends with
// slot l % P summed over the warp: P - 1 exchanges for P slots instead of
// 5 P (FP64 adds run at a small fraction of the FP32 rate on this part).
template <int P>
__device__ __forceinline__ double warp_slot_sums(double (&v)[P], int l) {
#pragma unroll
  for (int h = P / 2; h >= 1; h >>= 1) {
    const bool upper = (l & h) != 0;
#pragma unroll
    for (int j = 0; j < h; j++) {
      const double send = upper ? v[j] : v[j + h];
      const double keep = upper ? v[j + h] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
#pragma unroll
  for (int o = P; o < 32; o <<= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
  return v[0];
}

// Partials per block: 32 doubles, or 64 for reductions of more than 32
// results (their grids stay within kMaxBlocks / 2 blocks).
template <int T>
constexpr int partial_stride() {
  return T > 32 ? 64 : 32;
}

template <int T, typename Out>
__device__ __forceinline__ void finish(double (&acc)[T], int nt, Area a, const Out &out) {
  static_assert(T >= 1 && T <= 64, "at most 64 results per reduction");
  constexpr int kStride = partial_stride<T>();
  __shared__ double red[kThreads / 32][T > 0 ? T : 1];
  __shared__ unsigned ticket;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if constexpr (T == 1) {
    const double v = warp_sum(acc[0]);
    if (l == 0) red[w][0] = v;
  } else {
    // Slots 0..31, then 32..T-1, one butterfly each.
    constexpr int T0 = T < 32 ? T : 32;
    {
      constexpr int P = pow2_at_least(T0);
      double v[P];
#pragma unroll
      for (int t = 0; t < P; t++) v[t] = t < T0 ? acc[t] : 0.0;
      const double sum = warp_slot_sums<P>(v, l);
      if (l < T0) red[w][l] = sum;
    }
    if constexpr (T > 32) {
      constexpr int T1 = T - 32;
      constexpr int P = pow2_at_least(T1);
      double v[P];
#pragma unroll
      for (int t = 0; t < P; t++) v[t] = t < T1 ? acc[32 + t] : 0.0;
      const double sum = warp_slot_sums<P>(v, l);
      if (l < T1) red[w][32 + l] = sum;
    }
  }
  __syncthreads();
  if (threadIdx.x < static_cast<unsigned>(nt)) {
    double s = 0.0;
    for (int k = 0; k < kThreads / 32; k++) s += red[k][threadIdx.x];
    a.partials[blockIdx.x * kStride + threadIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(a.counter, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  if (threadIdx.x < static_cast<unsigned>(nt)) {
    double s = 0.0;
    for (unsigned b = 0; b < gridDim.x; b++) s += __ldcg(&a.partials[b * kStride + threadIdx.x]);
    out(static_cast<int>(threadIdx.x), s);
  }
  if (threadIdx.x == 0) *a.counter = 0u;
}

}  // namespace qmk
