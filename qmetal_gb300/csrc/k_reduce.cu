// k_reduce.cu -- reductions over the state (norm, Pauli expectations, dot),
// the co-state build and the fused adjoint step.
//
// Precision: each thread sums a short run (a chunk of vectors) in FP32, adds
// the chunk into an FP64 accumulator, and everything from the warp up is
// FP64. Blocks write FP64 partials; the last block to finish adds them in
// block order, so a result depends only on the grid size, never on timing.
#include <algorithm>
#include <cstring>
#include <vector>

#include "kreduce.cuh"
#include "../../include/qmetal/qmetal_kernels.h"

using namespace qmk;
using qmk_host::grid_for;
using qmk_host::launch_status;

namespace {

constexpr int kMaxT = 16;

constexpr int kChunk = 4;  // vectors per FP32 run and per thread iteration

__global__ void __launch_bounds__(kThreads)
k_abs2(const float4 *__restrict__ st, uint64_t nvec, Area a, double *out) {
  double acc[1] = {0.0};
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kThreads;
  for (uint64_t v0 = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x; v0 < nvec;
       v0 += stride * kChunk) {
    float4 x[kChunk];
#pragma unroll
    for (int k = 0; k < kChunk; k++) {
      const uint64_t v = v0 + k * stride;
      x[k] = (v < nvec) ? st[v] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kChunk; k++)
      s = fmaf(x[k].x, x[k].x, fmaf(x[k].y, x[k].y, fmaf(x[k].z, x[k].z, fmaf(x[k].w, x[k].w, s))));
    acc[0] += s;
  }
  finish<1>(acc, 1, a, OutContig{out, false});
}

__global__ void __launch_bounds__(kThreads)
k_dot_re(const float4 *__restrict__ x4, const float4 *__restrict__ y4, uint64_t nvec,
         Area a, double *out) {
  double acc[1] = {0.0};
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kThreads;
  for (uint64_t v0 = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x; v0 < nvec;
       v0 += stride * kChunk) {
    float4 x[kChunk], y[kChunk];
#pragma unroll
    for (int k = 0; k < kChunk; k++) {
      const uint64_t v = v0 + k * stride;
      x[k] = (v < nvec) ? x4[v] : make_float4(0.f, 0.f, 0.f, 0.f);
      y[k] = (v < nvec) ? y4[v] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kChunk; k++)
      s = fmaf(x[k].x, y[k].x, fmaf(x[k].y, y[k].y, fmaf(x[k].z, y[k].z, fmaf(x[k].w, y[k].w, s))));
    acc[0] += s;
  }
  finish<1>(acc, 1, a, OutContig{out, false});
}

struct PauliArgs {
  uint64_t flip;
  uint32_t hbit;      // highest bit of flip (pairs have it clear)
  uint32_t nt;
  uint32_t useim;     // bit t: term t reads Im z (odd Y count)
  uint64_t sign[kMaxT];
};

// flip == 0: sum_i s_t(i) |psi_i|^2, two amplitudes per float4.
template <int T>
__global__ void __launch_bounds__(kThreads)
k_pauli_z(const float4 *__restrict__ st, uint64_t nvec, PauliArgs p, Area a, double *out) {
  double acc[T];
#pragma unroll
  for (int t = 0; t < T; t++) acc[t] = 0.0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kThreads;
  for (uint64_t v0 = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x; v0 < nvec;
       v0 += stride * kChunk) {
    float part[T];
#pragma unroll
    for (int t = 0; t < T; t++) part[t] = 0.0f;
#pragma unroll
    for (int k = 0; k < kChunk; k++) {
      const uint64_t v = v0 + k * stride;
      if (v >= nvec) break;
      const float4 x = st[v];
      const float p0 = x.x * x.x + x.y * x.y, p1 = x.z * x.z + x.w * x.w;
      const uint64_t i0 = 2 * v;
#pragma unroll
      for (int t = 0; t < T; t++) {
        const int s0 = parity64(i0 & p.sign[t]);
        const int s1 = s0 ^ static_cast<int>(p.sign[t] & 1);
        part[t] += (s0 ? -p0 : p0) + (s1 ? -p1 : p1);
      }
    }
#pragma unroll
    for (int t = 0; t < T; t++) acc[t] += part[t];
  }
  finish<T>(acc, p.nt, a, OutContig{out, false});
}

// flip != 0: over pairs (i, j = i ^ flip) with bit hbit of i clear,
// sum s_t(i) * (Re or Im of conj(psi_i) psi_j); the host applies +-2.
template <int T>
__global__ void __launch_bounds__(kThreads)
k_pauli_x(const float2 *__restrict__ st, uint64_t npairs, PauliArgs p, Area a, double *out) {
  double acc[T];
#pragma unroll
  for (int t = 0; t < T; t++) acc[t] = 0.0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kThreads;
  constexpr int C = 2 * kChunk;
  for (uint64_t u0 = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x; u0 < npairs;
       u0 += stride * C) {
    float part[T];
#pragma unroll
    for (int t = 0; t < T; t++) part[t] = 0.0f;
#pragma unroll
    for (int k = 0; k < C; k++) {
      const uint64_t u = u0 + k * stride;
      if (u >= npairs) break;
      const uint64_t i = ins0(u, p.hbit), j = i ^ p.flip;
      const float2 x = st[i], y = st[j];
      const float re = x.x * y.x + x.y * y.y, im = x.x * y.y - x.y * y.x;
#pragma unroll
      for (int t = 0; t < T; t++) {
        const float v = (p.useim >> t & 1) ? im : re;
        part[t] += parity64(i & p.sign[t]) ? -v : v;
      }
    }
#pragma unroll
    for (int t = 0; t < T; t++) acc[t] += part[t];
  }
  finish<T>(acc, p.nt, a, OutContig{out, false});
}

struct AccumArgs {
  uint64_t flip;
  uint32_t nt;
  uint64_t sign[kMaxT];
  float2 kappa[kMaxT];  // coeff * i^ny
};

// lambda_i (+)= sum_t kappa_t s_t(i ^ flip) psi_{i ^ flip}
template <int T, bool OVERWRITE>
__global__ void __launch_bounds__(kThreads)
k_accum(float2 *__restrict__ lam, const float2 *__restrict__ psi, uint64_t dim, AccumArgs c) {
  constexpr int UU = 2;
#pragma unroll
  for (int k = 0; k < UU; k++) {
    const uint64_t i = (static_cast<uint64_t>(blockIdx.x) * UU + k) * kThreads + threadIdx.x;
    if (i >= dim) continue;
    const uint64_t j = i ^ c.flip;
    const float2 x = psi[j];
    float2 K = make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < T; t++) {
      if (t >= static_cast<int>(c.nt)) break;
      const float sg = parity64(j & c.sign[t]) ? -1.0f : 1.0f;
      K.x += sg * c.kappa[t].x;
      K.y += sg * c.kappa[t].y;
    }
    const float2 v = cmul(K, x);
    if (OVERWRITE) {
      lam[i] = v;
    } else {
      const float2 o = lam[i];
      lam[i] = make_float2(o.x + v.x, o.y + v.y);
    }
  }
}

// Im(conj(l0) (P psi)_0 + conj(l1) (P psi)_1) for a pair (bit q = 0 / 1).
template <int GEN>
__device__ __forceinline__ float gen_overlap(float2 p0, float2 p1, float2 l0, float2 l1) {
  float2 w0, w1;
  if (GEN == 1) {          // X
    w0 = p1; w1 = p0;
  } else if (GEN == 2) {   // Y: (-i p1, i p0)
    w0 = make_float2(p1.y, -p1.x);
    w1 = make_float2(-p0.y, p0.x);
  } else {                 // Z
    w0 = p0; w1 = make_float2(-p1.x, -p1.y);
  }
  return (l0.x * w0.y - l0.y * w0.x) + (l1.x * w1.y - l1.y * w1.x);
}

// One backward step on wire q for both states. Q0: q == 0 (pair in lanes).
template <bool Q0, int GEN>
__global__ void __launch_bounds__(kThreads)
k_adj1q(float4 *__restrict__ psi, float4 *__restrict__ lam, uint64_t nsites, uint32_t pos,
        M2 minv, Area a, double *out) {
  double acc[1] = {0.0};
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kThreads;
  const uint64_t tb = 1ull << pos;
  for (uint64_t s = static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x; s < nsites;
       s += stride) {
    float part = 0.0f;
    if (Q0) {
      const float4 P = psi[s], L = lam[s];
      float2 p0 = lo2(P), p1 = hi2(P), l0 = lo2(L), l1 = hi2(L);
      if (GEN) part += gen_overlap<GEN>(p0, p1, l0, l1);
      apply2(minv, p0, p1);
      apply2(minv, l0, l1);
      psi[s] = pack4(p0, p1);
      lam[s] = pack4(l0, l1);
    } else {
      const uint64_t v0 = ins0(s, pos), v1 = v0 | tb;
      const float4 P0 = psi[v0], P1 = psi[v1], L0 = lam[v0], L1 = lam[v1];
      float2 pa = lo2(P0), pb = lo2(P1), la = lo2(L0), lb = lo2(L1);
      float2 qa = hi2(P0), qb = hi2(P1), ma = hi2(L0), mb = hi2(L1);
      if (GEN) part += gen_overlap<GEN>(pa, pb, la, lb) + gen_overlap<GEN>(qa, qb, ma, mb);
      apply2(minv, pa, pb);
      apply2(minv, qa, qb);
      apply2(minv, la, lb);
      apply2(minv, ma, mb);
      psi[v0] = pack4(pa, qa);
      psi[v1] = pack4(pb, qb);
      lam[v0] = pack4(la, ma);
      lam[v1] = pack4(lb, mb);
    }
    acc[0] += part;
  }
  if (GEN) finish<1>(acc, 1, a, OutContig{out, false});
}

template <int T>
void launch_pauli(const float *state, uint32_t n, const PauliArgs &p, Area a,
                  double *out, cudaStream_t s) {
  const unsigned g = reduce_grid();
  if (p.flip == 0) {
    k_pauli_z<T><<<g, kThreads, 0, s>>>(reinterpret_cast<const float4 *>(state),
                                        1ull << (n - 1), p, a, out);
  } else {
    k_pauli_x<T><<<g, kThreads, 0, s>>>(reinterpret_cast<const float2 *>(state),
                                        1ull << (n - 1), p, a, out);
  }
}

template <int T>
void launch_accum(float *lam, const float *psi, uint32_t n, const AccumArgs &c,
                  bool overwrite, cudaStream_t s) {
  const uint64_t dim = 1ull << n;
  const unsigned g = grid_for(dim, kThreads * 2);
  if (overwrite)
    k_accum<T, true><<<g, kThreads, 0, s>>>(reinterpret_cast<float2 *>(lam),
                                            reinterpret_cast<const float2 *>(psi), dim, c);
  else
    k_accum<T, false><<<g, kThreads, 0, s>>>(reinterpret_cast<float2 *>(lam),
                                             reinterpret_cast<const float2 *>(psi), dim, c);
}

bool ok_ws(void *ws, size_t bytes, uint32_t n) {
  return ws && bytes >= qmk_workspace_bytes(n);
}

// ---------------------------------------------------------------------------
// Co-state terms that each flip a single wire (a transverse field, X_a Z_b
// ...), many wires per pass. A warp owns 32 consecutive vectors (lane =
// vector bits 0..4, i.e. wires 1..5) for every combination of up to KH wires
// >= 6 held in registers; the flipped source of an output amplitude is the
// other half of its vector (wire 0), the partner lane's vector (wires 1..5)
// or another register (wires >= 6), so psi is read once for all the terms.

constexpr int kLocalTerms = 16;

struct LocalAccumArgs {
  uint32_t nt;
  uint32_t hpos[4];               // wires >= 6 of the tile: vector bit - 5
  int8_t kind[kLocalTerms];       // 0: wire 0, 1: lane bit, 2: register bit
  int8_t arg[kLocalTerms];        // lane bit or register index
  uint64_t sign[kLocalTerms];     // sign mask at the source index
  uint32_t lpar[kLocalTerms];     // bit l: parity of the register bits of vector l & sign
  uint32_t fpar;                  // bit t: parity(flip_t & sign_t)
  float2 kappa[kLocalTerms];      // coeff * i^ny
};

template <int NV, int J>
__device__ __forceinline__ float4 reg_source(const float4 (&P)[NV], int l) {
  float4 r = P[0];
#pragma unroll
  for (int k = 0; k < NV; k++)
    if (k == (l ^ (1 << J))) r = P[k];
  return r;
}

template <int KH, bool OVERWRITE>
__global__ void __launch_bounds__(kThreads)
k_accum_local(float4 *__restrict__ lam, const float4 *__restrict__ psi, uint64_t nwsites,
              LocalAccumArgs c) {
  constexpr int NV = 1 << KH;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gw = (static_cast<uint64_t>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
  const uint64_t nwarps = static_cast<uint64_t>(gridDim.x) * (kThreads / 32);
  for (uint64_t ws = gw; ws < nwsites; ws += nwarps) {
    uint64_t b = ws;
#pragma unroll
    for (int j = 0; j < KH; j++) b = ins0(b, c.hpos[j]);
    const uint64_t base = (b << 5) | lane;
    auto vec_of = [&](int l) {
      uint64_t v = base;
#pragma unroll
      for (int j = 0; j < KH; j++)
        if ((l >> j) & 1) v |= 1ull << (c.hpos[j] + 5);
      return v;
    };
    float4 P[NV], L[NV];
#pragma unroll
    for (int l = 0; l < NV; l++) {
      const uint64_t v = vec_of(l);
      P[l] = psi[v];
      L[l] = OVERWRITE ? make_float4(0.f, 0.f, 0.f, 0.f) : lam[v];
    }
    for (uint32_t t = 0; t < c.nt; t++) {
      const int kind = c.kind[t], arg = c.arg[t];
      const uint64_t sg = c.sign[t];
      // parity of (output index ^ flip) & sign, for amplitude 0 of vector l:
      // the site's bits, the register bits of l, and the flip's own bits.
      const uint32_t p0 = parity64((base << 1) & sg) ^ ((c.fpar >> t) & 1u);
      const uint32_t p1 = p0 ^ static_cast<uint32_t>(sg & 1ull);
      const float2 k = c.kappa[t];
      const uint32_t lpar = c.lpar[t];
#pragma unroll
      for (int l = 0; l < NV; l++) {
        float4 q;
        if (kind == 0) {
          q = make_float4(P[l].z, P[l].w, P[l].x, P[l].y);
        } else if (kind == 1) {
          q = shfl4(P[l], 1 << arg);
        } else {
          q = P[l];
          if (KH > 0 && arg == 0) q = reg_source<NV, 0>(P, l);
          if (KH > 1 && arg == 1) q = reg_source<NV, (KH > 1 ? 1 : 0)>(P, l);
          if (KH > 2 && arg == 2) q = reg_source<NV, (KH > 2 ? 2 : 0)>(P, l);
          if (KH > 3 && arg == 3) q = reg_source<NV, (KH > 3 ? 3 : 0)>(P, l);
        }
        const uint32_t lp = (lpar >> l) & 1u;
        const float2 k0 = (p0 ^ lp) ? make_float2(-k.x, -k.y) : k;
        const float2 k1 = (p1 ^ lp) ? make_float2(-k.x, -k.y) : k;
        const float2 a = cmul(k0, lo2(q)), d = cmul(k1, hi2(q));
        L[l] = make_float4(L[l].x + a.x, L[l].y + a.y, L[l].z + d.x, L[l].w + d.y);
      }
    }
#pragma unroll
    for (int l = 0; l < NV; l++) lam[vec_of(l)] = L[l];
  }
}

}  // namespace

extern "C" int qmk_abs2sum(const float *state, uint32_t n, double *d_out,
                           void *ws, size_t ws_bytes, void *stream) {
  if (!state || !d_out || n < 1 || n > 40 || !ok_ws(ws, ws_bytes, n)) return -1;
  k_abs2<<<reduce_grid(), kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4 *>(state), 1ull << (n - 1), area_of(ws), d_out);
  return launch_status();
}

extern "C" int qmk_dot_re(const float *x, const float *y, uint32_t n, double *d_out,
                          void *ws, size_t ws_bytes, void *stream) {
  if (!x || !y || !d_out || n < 1 || n > 40 || !ok_ws(ws, ws_bytes, n)) return -1;
  k_dot_re<<<reduce_grid(), kThreads, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4 *>(x), reinterpret_cast<const float4 *>(y),
      1ull << (n - 1), area_of(ws), d_out);
  return launch_status();
}

extern "C" int qmk_pauli_expect(const float *state, uint32_t n, uint64_t flip,
                                uint32_t nt, const uint64_t *signs,
                                const uint32_t *ny, double *d_out, void *ws,
                                size_t ws_bytes, void *stream) {
  if (!state || !d_out || n < 1 || n > 40 || nt < 1 || nt > kMaxT || !signs || !ny ||
      !ok_ws(ws, ws_bytes, n))
    return -1;
  if (n < 64 && (flip >> n)) return -1;
  PauliArgs p{};
  p.flip = flip;
  p.hbit = flip ? 63 - __builtin_clzll(flip) : 0;
  p.nt = nt;
  for (uint32_t t = 0; t < nt; t++) {
    p.sign[t] = signs[t];
    if (ny[t] & 1) p.useim |= 1u << t;
  }
  const Area a = area_of(ws);
  cudaStream_t s = (cudaStream_t)stream;
  if (nt == 1) launch_pauli<1>(state, n, p, a, d_out, s);
  else if (nt <= 2) launch_pauli<2>(state, n, p, a, d_out, s);
  else if (nt <= 4) launch_pauli<4>(state, n, p, a, d_out, s);
  else if (nt <= 8) launch_pauli<8>(state, n, p, a, d_out, s);
  else launch_pauli<16>(state, n, p, a, d_out, s);
  return launch_status();
}

extern "C" int qmk_pauli_accum(float *lam, const float *psi, uint32_t n, uint64_t flip,
                               uint32_t nt, const uint64_t *signs, const uint32_t *ny,
                               const double *coeffs, int overwrite, void *stream) {
  if (!lam || !psi || n < 1 || n > 40 || nt < 1 || nt > kMaxT || !signs || !ny || !coeffs)
    return -1;
  if (n < 64 && (flip >> n)) return -1;
  AccumArgs c{};
  c.flip = flip;
  c.nt = nt;
  for (uint32_t t = 0; t < nt; t++) {
    c.sign[t] = signs[t];
    const double k = coeffs[t];
    switch (ny[t] & 3u) {  // coeff * i^ny, exact
      case 0: c.kappa[t] = make_float2(float(k), 0.f); break;
      case 1: c.kappa[t] = make_float2(0.f, float(k)); break;
      case 2: c.kappa[t] = make_float2(float(-k), 0.f); break;
      default: c.kappa[t] = make_float2(0.f, float(-k)); break;
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  const bool ow = overwrite != 0;
  if (nt == 1) launch_accum<1>(lam, psi, n, c, ow, s);
  else if (nt <= 2) launch_accum<2>(lam, psi, n, c, ow, s);
  else if (nt <= 4) launch_accum<4>(lam, psi, n, c, ow, s);
  else if (nt <= 8) launch_accum<8>(lam, psi, n, c, ow, s);
  else launch_accum<16>(lam, psi, n, c, ow, s);
  return launch_status();
}

extern "C" int qmk_pauli_accum_local(float *lam, const float *psi, uint32_t n, uint32_t nt,
                                     const uint32_t *wires, const uint64_t *signs,
                                     const uint32_t *ny, const double *coeffs, int overwrite,
                                     void *stream) {
  if (!lam || !psi || n < 6 || n > 40 || nt < 1 || nt > kLocalTerms || !wires || !signs || !ny ||
      !coeffs)
    return -1;
  const uint64_t all = (1ull << n) - 1;
  std::vector<uint32_t> high;
  for (uint32_t t = 0; t < nt; t++) {
    if (wires[t] >= n || (signs[t] & ~all)) return -1;
    if (wires[t] >= 6 && std::find(high.begin(), high.end(), wires[t]) == high.end())
      high.push_back(wires[t]);
  }
  if (high.size() > 4 || n < 6 + high.size()) return -1;
  std::sort(high.begin(), high.end());
  const uint32_t nh = static_cast<uint32_t>(high.size());
  LocalAccumArgs c{};
  c.nt = nt;
  for (uint32_t j = 0; j < nh; j++) c.hpos[j] = high[j] - 6;
  for (uint32_t t = 0; t < nt; t++) {
    const uint32_t w = wires[t];
    if (w == 0) {
      c.kind[t] = 0;
    } else if (w <= 5) {
      c.kind[t] = 1;
      c.arg[t] = static_cast<int8_t>(w - 1);
    } else {
      c.kind[t] = 2;
      c.arg[t] = static_cast<int8_t>(std::find(high.begin(), high.end(), w) - high.begin());
    }
    c.sign[t] = signs[t];
    for (uint32_t l = 0; l < (1u << nh); l++) {
      uint64_t bits = 0;
      for (uint32_t j = 0; j < nh; j++)
        if ((l >> j) & 1) bits |= 1ull << high[j];      // amplitude bits of register l
      c.lpar[t] |= static_cast<uint32_t>(__builtin_popcountll(bits & signs[t]) & 1) << l;
    }
    c.fpar |= static_cast<uint32_t>(__builtin_popcountll((1ull << w) & signs[t]) & 1) << t;
    const double k = coeffs[t];
    switch (ny[t] & 3u) {  // coeff * i^ny, exact
      case 0: c.kappa[t] = make_float2(float(k), 0.f); break;
      case 1: c.kappa[t] = make_float2(0.f, float(k)); break;
      case 2: c.kappa[t] = make_float2(float(-k), 0.f); break;
      default: c.kappa[t] = make_float2(0.f, float(-k)); break;
    }
  }
  const uint64_t nw = 1ull << (n - 6 - nh);
  const unsigned grid = grid_for(nw, kThreads / 32);
  float4 *l4 = reinterpret_cast<float4 *>(lam);
  const float4 *p4 = reinterpret_cast<const float4 *>(psi);
  cudaStream_t s = (cudaStream_t)stream;
  const bool ow = overwrite != 0;
#define QMK_LOCAL_CASE(KH)                                                           \
  if (nh == KH) {                                                                    \
    if (ow) k_accum_local<KH, true><<<grid, kThreads, 0, s>>>(l4, p4, nw, c);        \
    else k_accum_local<KH, false><<<grid, kThreads, 0, s>>>(l4, p4, nw, c);          \
  }
  QMK_LOCAL_CASE(0)
  QMK_LOCAL_CASE(1)
  QMK_LOCAL_CASE(2)
  QMK_LOCAL_CASE(3)
  QMK_LOCAL_CASE(4)
#undef QMK_LOCAL_CASE
  return launch_status();
}

template <bool Q0>
static void launch_adj(float4 *psi, float4 *lam, uint64_t nsites, uint32_t pos, const M2 &m,
                       int gen, Area a, double *out, cudaStream_t s) {
  const unsigned g = std::min<unsigned>(reduce_grid(), grid_for(nsites, kThreads));
  switch (gen) {
    case 1: k_adj1q<Q0, 1><<<g, kThreads, 0, s>>>(psi, lam, nsites, pos, m, a, out); break;
    case 2: k_adj1q<Q0, 2><<<g, kThreads, 0, s>>>(psi, lam, nsites, pos, m, a, out); break;
    case 3: k_adj1q<Q0, 3><<<g, kThreads, 0, s>>>(psi, lam, nsites, pos, m, a, out); break;
    default: {
      const unsigned g2 = grid_for(nsites, kThreads);
      k_adj1q<Q0, 0><<<g2, kThreads, 0, s>>>(psi, lam, nsites, pos, m, a, out);
    }
  }
}

extern "C" int qmk_adjoint_1q(float *psi, float *lam, uint32_t n, uint32_t q,
                              const float minv[8], int gen, double *d_grad, void *ws,
                              size_t ws_bytes, void *stream) {
  if (!psi || !lam || n < 1 || n > 40 || q >= n || gen < 0 || gen > 3 ||
      !ok_ws(ws, ws_bytes, n) || (gen && !d_grad))
    return -1;
  const M2 m = m2_from(minv);
  float4 *p4 = reinterpret_cast<float4 *>(psi), *l4 = reinterpret_cast<float4 *>(lam);
  cudaStream_t s = (cudaStream_t)stream;
  if (q == 0)
    launch_adj<true>(p4, l4, 1ull << (n - 1), 0, m, gen, area_of(ws), d_grad, s);
  else
    launch_adj<false>(p4, l4, 1ull << (n - 2), q - 1, m, gen, area_of(ws), d_grad, s);
  return launch_status();
}
