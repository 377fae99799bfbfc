/*
 * qsim_oracle.c -- complex128 CPU restatement of qmetal's statevector oracle.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it. Nothing in
 * the shipped library links it, and no product code path may fall back to it.
 *
 * What it restates (the reference project's own CPU oracle, "Reference"):
 *   - gate matrices ............ src/reference.cpp:60-98 (gate_matrix_1q)
 *   - 1q / controlled / diag2q / swap / ccx
 *                                 src/reference.cpp:113-159
 *   - gate dispatch + fail-closed src/reference.cpp:161-201
 *   - plan-op execution ......... src/reference.cpp:208-243
 *   - norm, expectation ......... src/reference.cpp:250-284
 * and two algorithms the reference only has in its GPU host, restated here
 * in double so the GPU results have something to be compared against:
 *   - sampling (block sums, CDF, splitmix64, in-block walk)
 *                                 src/metal/simulator.mm:73-80, 677-763
 *   - adjoint energy + gradient . src/metal/simulator.mm:782-963
 *
 * Conventions: LSB-first (qubit q is bit q of the basis index); states are
 * complex128 stored interleaved (re, im). Gate kinds use the qm_gate_kind
 * numbering of the C ABI (X=0 ... CCX=17, and U3=18, which the library
 * appends to the ABI: its matrix is the OpenQASM U(theta, phi, lambda)).
 *
 * Plan ops arrive in the flat serialisation produced by the library's plan
 * builder (and by the reference shim): see qo_run_plan for the layout.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

/* Gate loops write disjoint elements, so splitting them across threads does
 * not change a single bit of the result; small states stay serial. */
#define PAR_MIN ((uint64_t)1 << 16)
#define PARALLEL_FOR(count)                                                  \
  const uint64_t par_n = (count);                                            \
  (void)par_n;                                                               \
  _Pragma("omp parallel for schedule(static) if (par_n >= PAR_MIN)")

enum {
  K_X = 0, K_Y, K_Z, K_H, K_S, K_SDG, K_T, K_TDG,
  K_RX, K_RY, K_RZ, K_P,
  K_CX, K_CY, K_CZ, K_SWAP, K_CP, K_CCX, K_U3
};

/* Plan-op kinds, in the order of PlanOp::Kind (include/qmetal/plan.h:27-35). */
enum {
  OP_DENSE1Q = 0, OP_GROUP, OP_BLOCKED, OP_CTRL1Q, OP_DIAG, OP_SWAP, OP_CCX
};

static const double kPi = 3.14159265358979323846;

static cplx polar1(double t) { return cos(t) + I * sin(t); }

/* Row-major 2x2 for a single-qubit gate (src/reference.cpp:60-98). Returns -1
 * for a kind that is not a one-qubit gate. */
static int gate_matrix(int kind, const double *p, cplx m[4]) {
  const double s2 = 1.0 / sqrt(2.0);
  switch (kind) {
    case K_X: m[0] = 0; m[1] = 1; m[2] = 1; m[3] = 0; return 0;
    case K_Y: m[0] = 0; m[1] = -I; m[2] = I; m[3] = 0; return 0;
    case K_Z: m[0] = 1; m[1] = 0; m[2] = 0; m[3] = -1; return 0;
    case K_H: m[0] = s2; m[1] = s2; m[2] = s2; m[3] = -s2; return 0;
    case K_S: m[0] = 1; m[1] = 0; m[2] = 0; m[3] = I; return 0;
    case K_SDG: m[0] = 1; m[1] = 0; m[2] = 0; m[3] = -I; return 0;
    case K_T: m[0] = 1; m[1] = 0; m[2] = 0; m[3] = polar1(kPi / 4); return 0;
    case K_TDG: m[0] = 1; m[1] = 0; m[2] = 0; m[3] = polar1(-kPi / 4); return 0;
    case K_RX: {
      double c = cos(p[0] / 2), s = sin(p[0] / 2);
      m[0] = c; m[1] = -I * s; m[2] = -I * s; m[3] = c;
      return 0;
    }
    case K_RY: {
      double c = cos(p[0] / 2), s = sin(p[0] / 2);
      m[0] = c; m[1] = -s; m[2] = s; m[3] = c;
      return 0;
    }
    case K_RZ:
      m[0] = polar1(-p[0] / 2); m[1] = 0; m[2] = 0; m[3] = polar1(p[0] / 2);
      return 0;
    case K_P:
      m[0] = 1; m[1] = 0; m[2] = 0; m[3] = polar1(p[0]);
      return 0;
    case K_U3: {
      double c = cos(p[0] / 2), s = sin(p[0] / 2);
      m[0] = c; m[1] = -s * polar1(p[2]); m[2] = s * polar1(p[1]); m[3] = c * polar1(p[1] + p[2]);
      return 0;
    }
    default:
      return -1;
  }
}

int qo_gate_matrix(int kind, const double *params, double out[8]) {
  cplx m[4];
  double zero[3] = {0, 0, 0};
  if (gate_matrix(kind, params ? params : zero, m) != 0) return -1;
  for (int k = 0; k < 4; k++) {
    out[2 * k] = creal(m[k]);
    out[2 * k + 1] = cimag(m[k]);
  }
  return 0;
}

/* --- primitive updates (src/reference.cpp:113-159) ------------------------ */

static void apply_1q(cplx *st, uint64_t dim, uint32_t q, const cplx m[4]) {
  const uint64_t stride = (uint64_t)1 << q, pairs = dim >> 1;
  PARALLEL_FOR(pairs)
  for (uint64_t t = 0; t < pairs; t++) {
    uint64_t i = ((t >> q) << (q + 1)) | (t & (stride - 1));
    uint64_t j = i | stride;
    cplx a = st[i], b = st[j];
    st[i] = m[0] * a + m[1] * b;
    st[j] = m[2] * a + m[3] * b;
  }
}

static void apply_ctrl_1q(cplx *st, uint64_t dim, uint32_t c, uint32_t t,
                          const cplx m[4]) {
  const uint64_t cm = (uint64_t)1 << c, tm = (uint64_t)1 << t;
  PARALLEL_FOR(dim)
  for (uint64_t i = 0; i < dim; i++) {
    if (!(i & cm) || (i & tm)) continue;
    uint64_t j = i | tm;
    cplx a = st[i], b = st[j];
    st[i] = m[0] * a + m[1] * b;
    st[j] = m[2] * a + m[3] * b;
  }
}

static void apply_diag_2q(cplx *st, uint64_t dim, uint32_t a, uint32_t b,
                          cplx ph) {
  const uint64_t ma = (uint64_t)1 << a, mb = (uint64_t)1 << b;
  PARALLEL_FOR(dim)
  for (uint64_t i = 0; i < dim; i++)
    if ((i & ma) && (i & mb)) st[i] *= ph;
}

static void apply_swap(cplx *st, uint64_t dim, uint32_t a, uint32_t b) {
  if (a == b) return;
  const uint64_t ma = (uint64_t)1 << a, mb = (uint64_t)1 << b;
  PARALLEL_FOR(dim)
  for (uint64_t i = 0; i < dim; i++) {
    if ((i & ma) && !(i & mb)) {
      uint64_t j = (i ^ ma) | mb;
      cplx t = st[i]; st[i] = st[j]; st[j] = t;
    }
  }
}

static void apply_ccx(cplx *st, uint64_t dim, uint32_t c0, uint32_t c1,
                      uint32_t t) {
  const uint64_t m0 = (uint64_t)1 << c0, m1 = (uint64_t)1 << c1,
                 mt = (uint64_t)1 << t;
  PARALLEL_FOR(dim)
  for (uint64_t i = 0; i < dim; i++) {
    if ((i & m0) && (i & m1) && !(i & mt)) {
      cplx x = st[i]; st[i] = st[i | mt]; st[i | mt] = x;
    }
  }
}

/* --- gate dispatch (src/reference.cpp:161-201) ---------------------------- */

int qo_apply_gate(uint32_t n, double *state, int kind, const uint32_t *q,
                  uint32_t nq, const double *params) {
  cplx *st = (cplx *)state;
  const uint64_t dim = (uint64_t)1 << n;
  double zero[3] = {0, 0, 0};
  const double *p = params ? params : zero;
  for (uint32_t k = 0; k < nq; k++)
    if (q[k] >= n) return -1;
  cplx m[4];
  if (nq == 1) {
    if (gate_matrix(kind, p, m) != 0) return -1;
    apply_1q(st, dim, q[0], m);
    return 0;
  }
  if (nq == 2) {
    if (q[0] == q[1]) return -1;
    switch (kind) {
      case K_CX: gate_matrix(K_X, p, m); apply_ctrl_1q(st, dim, q[0], q[1], m); return 0;
      case K_CY: gate_matrix(K_Y, p, m); apply_ctrl_1q(st, dim, q[0], q[1], m); return 0;
      case K_CZ: apply_diag_2q(st, dim, q[0], q[1], -1.0); return 0;
      case K_CP: apply_diag_2q(st, dim, q[0], q[1], polar1(p[0])); return 0;
      case K_SWAP: apply_swap(st, dim, q[0], q[1]); return 0;
      default: return -1;
    }
  }
  if (nq == 3 && kind == K_CCX) {
    apply_ccx(st, dim, q[0], q[1], q[2]);
    return 0;
  }
  return -1;
}

/* Gate streams are parallel arrays: kinds[g], nq[g], qubits[3g..3g+2],
 * params[3g..3g+2]. */
int qo_run(uint32_t n, double *state, size_t ngates, const int32_t *kinds,
           const uint32_t *nq, const uint32_t *qubits, const double *params) {
  for (size_t g = 0; g < ngates; g++) {
    int rc = qo_apply_gate(n, state, kinds[g], qubits + 3 * g, nq[g],
                           params + 3 * g);
    if (rc != 0) return -1 - (int)g;
  }
  return 0;
}

/* Threads for the gate loops (OpenMP); 1 reproduces the reference's
 * single-thread oracle. */
void qo_set_threads(int threads) {
#ifdef _OPENMP
  extern void omp_set_num_threads(int);
  omp_set_num_threads(threads > 0 ? threads : 1);
#else
  (void)threads;
#endif
}

void qo_reset(uint32_t n, double *state) {
  memset(state, 0, sizeof(double) * 2 * ((size_t)1 << n));
  state[0] = 1.0;
}

/* --- plan execution (src/reference.cpp:208-243) ----------------------------
 * Flat layout, all doubles:
 *   [num_ops] then per op:
 *   kind, q0, q1, q2, block_bits, n_group, n_terms, global_phase,
 *   matrix[8] (re, im row-major),
 *   group_qubits[n_group], group_matrices[8 * n_group],
 *   masks[n_terms], angles[n_terms]
 * Masks are below 2^53, so they travel exactly.
 */
int qo_run_plan(uint32_t n, double *state, const double *plan, size_t len) {
  cplx *st = (cplx *)state;
  const uint64_t dim = (uint64_t)1 << n;
  if (len < 1) return -1;
  size_t nops = (size_t)plan[0], pos = 1;
  for (size_t o = 0; o < nops; o++) {
    if (pos + 16 > len) return -2;
    const double *h = plan + pos;
    int kind = (int)h[0];
    uint32_t q0 = (uint32_t)h[1], q1 = (uint32_t)h[2], q2 = (uint32_t)h[3];
    size_t ng = (size_t)h[5], nt = (size_t)h[6];
    double gphase = h[7];
    cplx m[4];
    for (int k = 0; k < 4; k++) m[k] = h[8 + 2 * k] + I * h[9 + 2 * k];
    const double *gq = h + 16;
    const double *gm = gq + ng;
    const double *mk = gm + 8 * ng;
    const double *an = mk + nt;
    size_t used = 16 + ng + 8 * ng + 2 * nt;
    if (pos + used > len) return -2;
    switch (kind) {
      case OP_DENSE1Q: apply_1q(st, dim, q0, m); break;
      case OP_CTRL1Q: apply_ctrl_1q(st, dim, q0, q1, m); break;
      case OP_GROUP:
      case OP_BLOCKED:
        for (size_t k = 0; k < ng; k++) {
          cplx g[4];
          for (int e = 0; e < 4; e++)
            g[e] = gm[8 * k + 2 * e] + I * gm[8 * k + 2 * e + 1];
          apply_1q(st, dim, (uint32_t)gq[k], g);
        }
        break;
      case OP_SWAP: apply_swap(st, dim, q0, q1); break;
      case OP_CCX: apply_ccx(st, dim, q0, q1, q2); break;
      case OP_DIAG:
        PARALLEL_FOR(dim)
        for (uint64_t i = 0; i < dim; i++) {
          double phi = gphase;
          for (size_t t = 0; t < nt; t++) {
            uint64_t msk = (uint64_t)mk[t];
            if ((i & msk) == msk) phi += an[t];
          }
          st[i] *= polar1(phi);
        }
        break;
      default:
        return -3;
    }
    pos += used;
  }
  return 0;
}

/* --- reductions (src/reference.cpp:250-284) ------------------------------- */

double qo_norm(uint32_t n, const double *state) {
  const cplx *st = (const cplx *)state;
  const uint64_t dim = (uint64_t)1 << n;
  double s = 0.0;
  for (uint64_t i = 0; i < dim; i++)
    s += creal(st[i]) * creal(st[i]) + cimag(st[i]) * cimag(st[i]);
  return sqrt(s);
}

static int pauli_valid(uint32_t n, uint64_t x, uint64_t y, uint64_t z) {
  uint64_t all = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
  if ((x | y | z) & ~all) return 0;
  return !((x & y) | (x & z) | (y & z));
}

/* <psi|P|psi>; the coefficient is taken at the source index j = i ^ flip and
 * the global i^ny is applied exactly at the end. Returns NAN for an invalid
 * string (the reference raises). */
double qo_expectation(uint32_t n, const double *state, uint64_t x, uint64_t y,
                      uint64_t z) {
  if (!pauli_valid(n, x, y, z)) return NAN;
  const cplx *st = (const cplx *)state;
  const uint64_t dim = (uint64_t)1 << n;
  const uint64_t flip = x | y, sign = y | z;
  const unsigned ny = (unsigned)__builtin_popcountll(y);
  cplx acc = 0;
  for (uint64_t i = 0; i < dim; i++) {
    uint64_t j = i ^ flip;
    double s = (__builtin_popcountll(j & sign) & 1) ? -1.0 : 1.0;
    acc += conj(st[i]) * st[j] * s;
  }
  switch (ny & 3u) {
    case 0: return creal(acc);
    case 1: return -cimag(acc);
    case 2: return -creal(acc);
    default: return cimag(acc);
  }
}

double qo_expectation_sum(uint32_t n, const double *state, uint32_t nterms,
                          const double *coeffs, const uint64_t *xs,
                          const uint64_t *ys, const uint64_t *zs) {
  double t = 0.0;
  for (uint32_t k = 0; k < nterms; k++)
    t += coeffs[k] * qo_expectation(n, state, xs[k], ys[k], zs[k]);
  return t;
}

/* --- sampling (src/metal/simulator.mm:73-80, 677-763) ----------------------
 * Operates on a complex64 interleaved state, like the executor it checks.
 * Block sums are taken in double here (the GPU path reduces in FP64 too). */
static uint64_t splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int qo_sample_f32(uint32_t n, const float *amps, size_t shots, uint64_t seed,
                  uint32_t block, uint64_t *out) {
  const uint64_t dim = (uint64_t)1 << n;
  if (block == 0) return -1;
  const uint64_t nblocks = (dim + block - 1) / block;
  double *cdf = (double *)malloc(sizeof(double) * nblocks);
  if (!cdf) return -1;
  double run = 0.0;
  for (uint64_t b = 0; b < nblocks; b++) {
    uint64_t s = b * block, e = s + block < dim ? s + block : dim;
    double acc = 0.0;
    for (uint64_t i = s; i < e; i++) {
      double re = amps[2 * i], im = amps[2 * i + 1];
      acc += re * re + im * im;
    }
    run += acc;
    cdf[b] = run;
  }
  const double total = run;
  if (total <= 0.0) {
    for (size_t k = 0; k < shots; k++) out[k] = 0;
    free(cdf);
    return 0;
  }
  uint64_t rng = seed;
  for (size_t k = 0; k < shots; k++) {
    double u = (double)(splitmix64(&rng) >> 11) * (1.0 / 9007199254740992.0) *
               total;
    uint64_t lo = 0, hi = nblocks - 1;
    while (lo < hi) {
      uint64_t mid = (lo + hi) >> 1;
      if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    double rem = u - (lo > 0 ? cdf[lo - 1] : 0.0);
    uint64_t s = lo * block, e = s + block < dim ? s + block : dim;
    double acc = 0.0;
    uint64_t chosen = s;
    int64_t last_nz = -1;
    int found = 0;
    for (uint64_t i = s; i < e; i++) {
      double re = amps[2 * i], im = amps[2 * i + 1];
      double pr = re * re + im * im;
      if (pr > 0.0) last_nz = (int64_t)i;
      acc += pr;
      if (acc > rem) { chosen = i; found = 1; break; }
    }
    if (!found) chosen = (last_nz >= 0) ? (uint64_t)last_nz : e - 1;
    out[k] = chosen;
  }
  free(cdf);
  return 0;
}

/* --- adjoint energy and gradient (src/metal/simulator.mm:782-963) ----------
 * complex128 throughout. The forward pass is gate by gate from |0..0>; the
 * co-state is lambda = H psi; the backward sweep takes Im<lambda|P|psi> for
 * each RX/RY/RZ (generator X/Y/Z on its wire) and then undoes the gate on
 * both states. Returns -1 if a parameterised gate has no native generator. */
static int invert_kind(int kind) {
  switch (kind) {
    case K_S: return K_SDG;
    case K_SDG: return K_S;
    case K_T: return K_TDG;
    case K_TDG: return K_T;
    default: return kind;
  }
}

static cplx ipow(unsigned ny) {
  switch (ny & 3u) {
    case 0: return 1;
    case 1: return I;
    case 2: return -1;
    default: return -I;
  }
}

/* dst += c * (P src), (P src)_i = sgn(i ^ flip) * src_{i ^ flip} */
static void pauli_accum(cplx *dst, const cplx *src, uint64_t dim,
                        uint64_t flip, uint64_t sign, cplx c) {
  PARALLEL_FOR(dim)
  for (uint64_t i = 0; i < dim; i++) {
    uint64_t j = i ^ flip;
    double s = (__builtin_popcountll(j & sign) & 1) ? -1.0 : 1.0;
    dst[i] += c * s * src[j];
  }
}

int qo_energy_and_gradient(uint32_t n, size_t ngates, const int32_t *kinds,
                           const uint32_t *nq, const uint32_t *qubits,
                           const double *params, const uint32_t *nparams,
                           uint32_t nterms, const double *coeffs,
                           const uint64_t *xs, const uint64_t *ys,
                           const uint64_t *zs, double *energy, double *grad) {
  const uint64_t dim = (uint64_t)1 << n;
  for (size_t g = 0; g < ngates; g++) {
    if (nparams[g] > 0 && kinds[g] != K_RX && kinds[g] != K_RY &&
        kinds[g] != K_RZ)
      return -1;
  }
  for (uint32_t t = 0; t < nterms; t++)
    if (!pauli_valid(n, xs[t], ys[t], zs[t])) return -2;
  cplx *psi = (cplx *)calloc(dim, sizeof(cplx));
  cplx *lam = (cplx *)calloc(dim, sizeof(cplx));
  if (!psi || !lam) { free(psi); free(lam); return -3; }
  psi[0] = 1;
  if (qo_run(n, (double *)psi, ngates, kinds, nq, qubits, params) != 0) {
    free(psi); free(lam); return -4;
  }
  for (uint32_t t = 0; t < nterms; t++) {
    unsigned ny = (unsigned)__builtin_popcountll(ys[t]);
    pauli_accum(lam, psi, dim, xs[t] | ys[t], ys[t] | zs[t],
                coeffs[t] * ipow(ny));
  }
  double e = 0.0;
  for (uint64_t i = 0; i < dim; i++) e += creal(conj(psi[i]) * lam[i]);
  *energy = e;
  for (size_t k = ngates; k-- > 0;) {
    int kind = kinds[k];
    grad[k] = 0.0;
    if (nparams[k] > 0) {
      uint64_t bit = (uint64_t)1 << qubits[3 * k];
      uint64_t x = 0, y = 0, z = 0;
      if (kind == K_RX) x = bit;
      else if (kind == K_RY) y = bit;
      else z = bit;
      uint64_t flip = x | y, sign = y | z;
      cplx acc = 0;
      for (uint64_t i = 0; i < dim; i++) {
        uint64_t j = i ^ flip;
        double s = (__builtin_popcountll(j & sign) & 1) ? -1.0 : 1.0;
        acc += conj(lam[i]) * psi[j] * s;
      }
      cplx v = acc * ipow((unsigned)__builtin_popcountll(y));
      grad[k] = cimag(v);
    }
    double inv[3] = {params[3 * k], params[3 * k + 1], params[3 * k + 2]};
    int ik = invert_kind(kind);
    if (kind == K_RX || kind == K_RY || kind == K_RZ || kind == K_P ||
        kind == K_CP)
      inv[0] = -inv[0];
    qo_apply_gate(n, (double *)psi, ik, qubits + 3 * k, nq[k], inv);
    qo_apply_gate(n, (double *)lam, ik, qubits + 3 * k, nq[k], inv);
  }
  free(psi);
  free(lam);
  return 0;
}
