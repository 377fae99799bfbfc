// kadjoint.cuh -- pieces the two adjoint translation units share: the
// window-tile argument block, the pair overlap, and the launcher of the
// window-tile kernels (k_adjoint_tiles.cu) that the host entry points of
// k_adjoint.cu call.
#pragma once

#include "kreduce.cuh"

namespace qmk_adj {

using qmk::M2;

constexpr int kMaxGen = 32;   // gradient slots one backward pass may write
constexpr int kMaxDiagGen = 48;   // ... and one diagonal-block pass

constexpr int kMaxWarpOps = 32;

struct WarpAdjArgs {
  uint32_t nops, ngrad;
  uint32_t hpos[6];              // wires >= 6: vector bit - 5, ascending (up to
                                 // four in a warp tile, six in a block tile)
  int8_t kind[kMaxWarpOps];      // 0: wire 0, 1: lane bit, 2: register bit,
                                 // 3: the wire split across a warp pair
  int8_t arg[kMaxWarpOps];       // lane bit (0..4) or register index
  int8_t gen[kMaxWarpOps];
  int8_t slotidx[kMaxWarpOps];   // gradient slot of op o (0 when gen[o] is 0)
  int8_t cls[kMaxWarpOps];       // kMat* structure of m
  M2 m[kMaxWarpOps];
};

// Im(conj(l0) (P psi)_0 + conj(l1) (P psi)_1) for a pair (wire bit 0 / 1)
// and the generator P = X, Y, Z (gen 1, 2, 3).
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

// The backward pass of a window tile whose wires all carry the same short
// rotation sequence (k_adjoint_uniform.cu). Returns 1 with nothing launched
// when the tile is not of that form, else 0 or a CUDA error code.
// kh is the tile's number of wires >= 6: 1..4 (warp and warp-pair tiles,
// nwsites = 2^(n - 6 - kh) warp sites) or 5..6 (block tiles of four or eight
// warps per site, wires >= 6 only; nwsites counts their sites the same way).
int launch_uniform(int kh, float4 *psi, float4 *lam, uint64_t nwsites, const WarpAdjArgs &g,
                   const qmk::OutSlots<kMaxGen> &slots, qmk::Area a, cudaStream_t s);

// Launch the backward pass of one window tile: kh wires >= 6 in registers
// (four: a warp pair), ng gradient slots (0, 4, 8 or 16). Returns 0 or a CUDA
// error code.
int launch_tiles(int kh, int ng, float4 *psi, float4 *lam, uint64_t nwsites,
                 WarpAdjArgs &g, const qmk::OutSlots<kMaxGen> &slots, qmk::Area a,
                 cudaStream_t s);

}  // namespace qmk_adj
