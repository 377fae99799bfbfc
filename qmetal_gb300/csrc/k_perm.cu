// k_perm.cu -- basis permutations that are affine over GF(2) (runs of CX and
// SWAP gates) applied in one out-of-place gather pass.
//
// A CX flips bit t of the basis index where bit c is set, a SWAP exchanges
// two bits, an X flips one: each maps index x to A x ^ b with A invertible
// over GF(2), and so does any run of them. The reference applies such a run
// one gate at a time (Controlled1q / Swap plan ops, src/metal/simulator.mm:
// 526-558, one pass over half or all of the state per gate); here the whole
// run is one gather, dst[y] = src[G(y)] with G(y) = off ^ XOR_{j : y_j = 1}
// col_j, i.e. 2S of traffic however many gates the run holds. Writes are
// whole 512-byte warp stores; reads follow G, which for the runs the executor
// fuses keeps a warp's sources within a few 32-byte sectors.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "kcommon.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::launch_status;

namespace {

constexpr int kTileBits = 13;     // amplitude bits resolved by the shared tables
constexpr int kMaxBits = 40;

struct PermArgs {
  uint64_t off;                   // G(0)
  uint64_t lo[kTileBits];         // images of amplitude bits 0..12
  uint64_t hi[kMaxBits - kTileBits];
  uint32_t n;
  uint32_t pair;                  // 1: G maps bit 0 to bit 0 only
};

// Shared XOR tables of a map's images of amplitude bits 0..6 and 7..12.
__device__ __forceinline__ void build_tables(const PermArgs &a, uint64_t *T0, uint64_t *T1) {
  for (uint32_t i = threadIdx.x; i < 128; i += kThreads) {
    uint64_t v = 0;
    for (int j = 0; j < 7; j++)
      if ((i >> j) & 1) v ^= a.lo[j];
    T0[i] = v;
  }
  for (uint32_t i = threadIdx.x; i < 64; i += kThreads) {
    uint64_t v = 0;
    for (int j = 0; j < 6; j++)
      if ((i >> j) & 1) v ^= a.lo[7 + j];
    T1[i] = v;
  }
  __syncthreads();
}

// The map's value at the tile's first amplitude: off ^ images of its high bits.
__device__ __forceinline__ uint64_t tile_base(const PermArgs &a, uint64_t tile, uint32_t W) {
  uint64_t H = a.off;
  for (uint32_t b = 0; b + W < a.n; b++)
    if ((tile >> b) & 1) H ^= a.hi[b];
  return H;
}

// Gather form: dst[y] = src[G(y)], G in a. Writes are whole warp stores.
__global__ void __launch_bounds__(kThreads)
k_permute(float4 *__restrict__ dst, const float2 *__restrict__ src, uint64_t ntiles, PermArgs a) {
  __shared__ uint64_t T0[128], T1[64];     // XOR sums of lo[0..6], lo[7..12]
  build_tables(a, T0, T1);
  const uint32_t tid = threadIdx.x;
  const uint32_t W = a.n < kTileBits ? a.n : kTileBits;
  const uint32_t nv = 1u << (W - 1);                // vectors per tile
  const float4 *src4 = reinterpret_cast<const float4 *>(src);
  constexpr int UU = 8;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t H = tile_base(a, tile, W);
    for (uint32_t e0 = tid; e0 < nv; e0 += kThreads * UU) {
      float4 r[UU];
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const uint32_t e = e0 + u * kThreads;
        if (e >= nv) continue;
        const uint32_t y = 2 * e;
        const uint64_t x0 = H ^ T0[y & 127] ^ T1[(y >> 7) & 63];
        if (a.pair) {
          const float4 v = src4[x0 >> 1];
          r[u] = (x0 & 1) ? make_float4(v.z, v.w, v.x, v.y) : v;
        } else {
          const float2 p = src[x0], q = src[x0 ^ a.lo[0]];
          r[u] = make_float4(p.x, p.y, q.x, q.y);
        }
      }
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const uint32_t e = e0 + u * kThreads;
        if (e < nv) dst[tile * nv + e] = r[u];
      }
    }
  }
}

// Scatter form of the same permutation: dst[M(x)] = src[x] with M = G^-1
// in a. Reads are whole warp loads issued at once, with no address that
// waits on a table; the stores follow M.
__global__ void __launch_bounds__(kThreads)
k_permute_scatter(float2 *__restrict__ dst, const float4 *__restrict__ src, uint64_t ntiles,
                  PermArgs a) {
  __shared__ uint64_t T0[128], T1[64];
  build_tables(a, T0, T1);
  const uint32_t tid = threadIdx.x;
  const uint32_t W = a.n < kTileBits ? a.n : kTileBits;
  const uint32_t nv = 1u << (W - 1);
  constexpr int UU = 8;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t H = tile_base(a, tile, W);
    for (uint32_t e0 = tid; e0 < nv; e0 += kThreads * UU) {
      float4 r[UU];
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const uint32_t e = e0 + u * kThreads;
        if (e < nv) r[u] = src[tile * nv + e];
      }
#pragma unroll
      for (int u = 0; u < UU; u++) {
        const uint32_t e = e0 + u * kThreads;
        if (e >= nv) continue;
        const uint32_t x = 2 * e;
        const uint64_t y0 = H ^ T0[x & 127] ^ T1[(x >> 7) & 63];
        dst[y0] = make_float2(r[u].x, r[u].y);
        dst[y0 ^ a.lo[0]] = make_float2(r[u].z, r[u].w);
      }
    }
  }
}

// Rank of the columns over GF(2): the map is a bijection iff rank == n.
uint32_t gf2_rank(const uint64_t *cols, uint32_t n) {
  std::vector<uint64_t> v(cols, cols + n);
  uint32_t rank = 0;
  for (uint32_t bit = 0; bit < n && rank < n; bit++) {
    const uint64_t m = 1ull << bit;
    uint32_t piv = rank;
    while (piv < n && !(v[piv] & m)) piv++;
    if (piv == n) continue;
    std::swap(v[rank], v[piv]);
    for (uint32_t r = 0; r < n; r++)
      if (r != rank && (v[r] & m)) v[r] ^= v[rank];
    rank++;
  }
  return rank;
}

// Inverse of a bijective map x -> A x ^ off over GF(2): columns of A^-1 and
// A^-1 off. Pairs (v, w) with A w = v are reduced until every v is a unit
// vector e_k, whose paired w is then column k of A^-1.
void gf2_inverse(const uint64_t *cols, uint64_t off, uint32_t n, uint64_t *inv, uint64_t *inv_off) {
  std::vector<uint64_t> v(cols, cols + n), w(n);
  for (uint32_t j = 0; j < n; j++) w[j] = 1ull << j;
  for (uint32_t bit = 0, row = 0; bit < n; bit++) {
    const uint64_t m = 1ull << bit;
    uint32_t piv = row;
    while (piv < n && !(v[piv] & m)) piv++;
    if (piv == n) continue;
    std::swap(v[row], v[piv]);
    std::swap(w[row], w[piv]);
    for (uint32_t r = 0; r < n; r++)
      if (r != row && (v[r] & m)) {
        v[r] ^= v[row];
        w[r] ^= w[row];
      }
    row++;
  }
  for (uint32_t j = 0; j < n; j++) inv[__builtin_ctzll(v[j])] = w[j];
  uint64_t o = 0;
  for (uint32_t j = 0; j < n; j++)
    if ((off >> j) & 1) o ^= inv[j];
  *inv_off = o;
}

// How far a map spreads a warp's lanes: the bits above the 64-amplitude
// warp window in the images of amplitude bits 0..5.
uint32_t spread(const uint64_t *cols, uint32_t n) {
  uint32_t s = 0;
  for (uint32_t j = 0; j < n && j < 6; j++) s += static_cast<uint32_t>(__builtin_popcountll(cols[j] >> 6));
  return s;
}

}  // namespace

extern "C" int qmk_apply_permutation(float *dst, const float *src, uint32_t n,
                                     const uint64_t *cols, uint64_t offset, void *stream) {
  if (!dst || !src || !cols || n < 1 || n > kMaxBits) return -1;
  if ((reinterpret_cast<uintptr_t>(dst) & 15u) || (reinterpret_cast<uintptr_t>(src) & 15u))
    return -1;
  if (dst == src) return -1;                        // out of place only
  const uint64_t all = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  if (offset & ~all) return -1;
  for (uint32_t j = 0; j < n; j++)
    if (!cols[j] || (cols[j] & ~all)) return -1;
  if (gf2_rank(cols, n) != n) return -1;            // not a bijection
  // Gather through G, or scatter through M = G^-1: whichever map spreads a
  // warp's lanes further. Measured live at 26-28 qubits on a CX ladder:
  // through its spread map (prefix XOR) either form runs at 1.00-1.04 of the
  // copy rate; through its local map (bit j to bits j and j+1) a gather runs
  // at 0.71 and a scatter at 0.40. A map that spreads neither way and keeps
  // amplitude bit 0 in place (the identity) runs at 1.04 as a scatter, whose
  // two stores fill each 16-byte vector, against 0.81 as a gather.
  uint64_t inv[kMaxBits], inv_off = 0;
  gf2_inverse(cols, offset, n, inv, &inv_off);
  const uint32_t sg = spread(cols, n), sm = spread(inv, n);
  const bool scatter = sm > sg || (sm == sg && cols[0] == 1ull);
  const uint64_t *m = scatter ? inv : cols;
  PermArgs a{};
  a.off = scatter ? inv_off : offset;
  a.n = n;
  for (uint32_t j = 0; j < n; j++) {
    if (j < kTileBits) a.lo[j] = m[j];
    else a.hi[j - kTileBits] = m[j];
  }
  a.pair = m[0] == 1ull ? 1u : 0u;
  const uint32_t W = n < kTileBits ? n : kTileBits;
  const uint64_t ntiles = 1ull << (n - W);
  // One block per tile (measured 4-8% faster than a grid of 8 blocks per SM
  // looping over tiles); the loop stays for grids above the launch limit.
  const uint64_t cap = (1ull << 31) - 1;
  const unsigned grid = static_cast<unsigned>(ntiles < cap ? ntiles : cap);
  if (scatter)
    k_permute_scatter<<<grid, kThreads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<float2 *>(dst), reinterpret_cast<const float4 *>(src), ntiles, a);
  else
    k_permute<<<grid, kThreads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<float4 *>(dst), reinterpret_cast<const float2 *>(src), ntiles, a);
  return launch_status();
}
