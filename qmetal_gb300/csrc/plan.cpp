// plan.cpp -- Circuit -> Plan lowering and fusion.
//
// The pass pipeline is the reference project's (src/plan.cpp:187-359) and must
// emit the same plan for the same circuit: the executor's op count, the
// dispatch count and every parity fixture depend on it. The passes are:
//
//   1. mark runs of consecutive diagonal blocks (a block is one diagonal gate,
//      or a CX.RZ.CX triple that is a ZZ coupling); a run needs two blocks or
//      one ZZ triple                                   (src/plan.cpp:193-221)
//   2. emit: a marked run becomes one DiagonalLayer; a window of >= 2 unmarked
//      one-qubit gates collapses per wire into 2x2 products, drops products
//      within 1e-12 of identity, and groups surviving wires (ascending) K at a
//      time; anything else lowers one to one             (src/plan.cpp:223-298)
//   3. optional cache blocking of runs of >= 2 ops whose wires are all below
//      block_bits                                        (src/plan.cpp:300-357)
//
// The diagonal-term rules (src/plan.cpp:106-135), the ZZ expansion
// x_a ^ x_b = x_a + x_b - 2 x_a x_b (src/plan.cpp:137-183) and the identity
// test with rtol = 0 (src/plan.cpp:25-34) are the reference's algebra.
#include <algorithm>
#include <array>
#include <cmath>
#include <stdexcept>
#include <string>

#include "circuit.hpp"

namespace qmetal {
namespace {

using Mat2 = std::array<cdouble, 4>;

// later * earlier (row-major 2x2), i.e. `earlier` acts first.
Mat2 compose(const cdouble *later, const Mat2 &earlier) {
  Mat2 r;
  r[0] = later[0] * earlier[0] + later[1] * earlier[2];
  r[1] = later[0] * earlier[1] + later[1] * earlier[3];
  r[2] = later[2] * earlier[0] + later[3] * earlier[2];
  r[3] = later[2] * earlier[1] + later[3] * earlier[3];
  return r;
}

bool near_identity(const Mat2 &m) {
  constexpr double tol = 1e-12;
  return std::abs(m[0] - 1.0) <= tol && std::abs(m[1]) <= tol &&
         std::abs(m[2]) <= tol && std::abs(m[3] - 1.0) <= tol;
}

PlanOp dense_op(uint32_t q, const cdouble *m) {
  PlanOp op;
  op.kind = PlanOp::Kind::Dense1q;
  op.qubits[0] = q;
  std::copy(m, m + 4, op.matrix);
  return op;
}

double add_diagonal_term(const Gate &g, PlanOp &op) {
  return diagonal_term(g, op.masks, op.angles);
}

bool zz_at(const Circuit &c, size_t i, uint32_t *a, uint32_t *b, double *t) {
  return zz_coupling_at(c, i, a, b, t);
}

size_t block_at(const Circuit &c, size_t i, bool zz) {
  uint32_t a, b;
  double t;
  if (zz && zz_at(c, i, &a, &b, &t)) return 3;
  return is_diagonal(c.ops[i]) ? 1 : 0;
}

PlanOp lower_one(const Gate &g) {
  PlanOp op;
  if (g.num_qubits == 1) {
    cdouble m[4];
    gate_matrix_1q(g.kind, g.params, m);
    return dense_op(g.qubits[0], m);
  }
  if (g.num_qubits == 2) {
    if (g.kind == G_CX || g.kind == G_CY) {
      op.kind = PlanOp::Kind::Controlled1q;
      op.qubits[0] = g.qubits[0];
      op.qubits[1] = g.qubits[1];
      gate_matrix_1q(g.kind == G_CX ? G_X : G_Y, nullptr, op.matrix);
      return op;
    }
    if (g.kind == G_CZ || g.kind == G_CP) {
      op.kind = PlanOp::Kind::DiagonalLayer;
      op.global_phase = add_diagonal_term(g, op);
      return op;
    }
    if (g.kind == G_SWAP) {
      op.kind = PlanOp::Kind::Swap;
      op.qubits[0] = g.qubits[0];
      op.qubits[1] = g.qubits[1];
      return op;
    }
  }
  if (g.num_qubits == 3 && g.kind == G_CCX) {
    op.kind = PlanOp::Kind::CCX;
    std::copy(g.qubits, g.qubits + 3, op.qubits);
    return op;
  }
  throw std::runtime_error(std::string("build_plan: unsupported gate ") +
                           gate_name(g.kind));
}

// Pass 2 helper: a window [i, j) of one-qubit gates, collapsed per wire.
void emit_window(const Circuit &c, size_t i, size_t j, uint32_t group,
                 Plan &plan) {
  std::vector<uint32_t> first_seen;
  std::vector<Mat2> product(c.num_qubits);
  std::vector<char> seen(c.num_qubits, 0);
  for (size_t k = i; k < j; k++) {
    const Gate &g = c.ops[k];
    const uint32_t q = g.qubits[0];
    cdouble m[4];
    gate_matrix_1q(g.kind, g.params, m);
    if (q >= c.num_qubits) throw std::runtime_error("qubit index out of range");
    if (!seen[q]) {
      seen[q] = 1;
      first_seen.push_back(q);
      product[q] = {m[0], m[1], m[2], m[3]};
    } else {
      product[q] = compose(m, product[q]);
    }
  }
  std::vector<uint32_t> live;
  for (uint32_t q : first_seen)
    if (!near_identity(product[q])) live.push_back(q);
  std::sort(live.begin(), live.end());
  const size_t K = std::max<size_t>(1, group);
  for (size_t b = 0; b < live.size(); b += K) {
    const size_t take = std::min(K, live.size() - b);
    if (take == 1) {
      plan.ops.push_back(dense_op(live[b], product[live[b]].data()));
      continue;
    }
    PlanOp op;
    op.kind = PlanOp::Kind::Dense1qGroup;
    for (size_t k = 0; k < take; k++) {
      const uint32_t q = live[b + k];
      op.group_qubits.push_back(q);
      op.group_matrices.insert(op.group_matrices.end(), product[q].begin(),
                               product[q].end());
    }
    plan.ops.push_back(std::move(op));
  }
}

bool local_1q(const PlanOp &op, uint32_t bits) {
  if (op.kind == PlanOp::Kind::Dense1q) return op.qubits[0] < bits;
  if (op.kind == PlanOp::Kind::Dense1qGroup) {
    for (uint32_t q : op.group_qubits)
      if (q >= bits) return false;
    return true;
  }
  return false;
}

Plan block_pass(Plan &&in, uint32_t bits) {
  Plan out;
  out.num_qubits = in.num_qubits;
  size_t k = 0;
  while (k < in.ops.size()) {
    size_t j = k;
    while (j < in.ops.size() && local_1q(in.ops[j], bits)) j++;
    if (j - k >= 2) {
      PlanOp op;
      op.kind = PlanOp::Kind::Blocked1q;
      op.block_bits = bits;
      for (size_t m = k; m < j; m++) {
        const PlanOp &s = in.ops[m];
        if (s.kind == PlanOp::Kind::Dense1q) {
          op.group_qubits.push_back(s.qubits[0]);
          op.group_matrices.insert(op.group_matrices.end(), s.matrix, s.matrix + 4);
        } else {
          op.group_qubits.insert(op.group_qubits.end(), s.group_qubits.begin(),
                                 s.group_qubits.end());
          op.group_matrices.insert(op.group_matrices.end(),
                                   s.group_matrices.begin(), s.group_matrices.end());
        }
      }
      out.ops.push_back(std::move(op));
      k = j;
    } else {
      out.ops.push_back(std::move(in.ops[k]));
      k++;
    }
  }
  return out;
}

}  // namespace

// One diagonal gate's term; RZ(t) = e^{-it/2} diag(1, e^{it}) carries the
// only global phase.
double diagonal_term(const Gate &g, std::vector<uint64_t> &masks, std::vector<double> &angles) {
  const uint64_t b0 = 1ull << g.qubits[0];
  auto term = [&](uint64_t m, double a) {
    masks.push_back(m);
    angles.push_back(a);
  };
  switch (g.kind) {
    case G_Z: term(b0, M_PI); return 0.0;
    case G_S: term(b0, M_PI / 2); return 0.0;
    case G_SDG: term(b0, -M_PI / 2); return 0.0;
    case G_T: term(b0, M_PI / 4); return 0.0;
    case G_TDG: term(b0, -M_PI / 4); return 0.0;
    case G_P: term(b0, g.params[0]); return 0.0;
    case G_RZ: term(b0, g.params[0]); return -g.params[0] / 2.0;
    case G_CZ: term(b0 | (1ull << g.qubits[1]), M_PI); return 0.0;
    case G_CP: term(b0 | (1ull << g.qubits[1]), g.params[0]); return 0.0;
    default: throw std::runtime_error("diagonal_term: gate is not diagonal");
  }
}

bool zz_coupling_at(const Circuit &c, size_t i, uint32_t *a, uint32_t *b, double *t) {
  if (i + 2 >= c.ops.size()) return false;
  const Gate &x = c.ops[i], &r = c.ops[i + 1], &y = c.ops[i + 2];
  if (x.kind != G_CX || y.kind != G_CX || r.kind != G_RZ) return false;
  if (x.qubits[0] != y.qubits[0] || x.qubits[1] != y.qubits[1]) return false;
  if (r.qubits[0] != x.qubits[1]) return false;
  *a = x.qubits[0];
  *b = x.qubits[1];
  *t = r.params[0];
  return true;
}


bool is_diagonal(const Gate &g) {
  switch (g.kind) {
    case G_Z: case G_S: case G_SDG: case G_T: case G_TDG: case G_RZ: case G_P:
      return g.num_qubits == 1;
    case G_CZ: case G_CP:
      return g.num_qubits == 2;
    default:
      return false;
  }
}

Plan build_plan(const Circuit &c, const FusionOptions &opts) {
  Plan plan;
  plan.num_qubits = c.num_qubits;
  const size_t n = c.ops.size();

  // Pass 1: run marking. blen[k] records the block length found at each block
  // start reached by the scan; marked[k] flags gates that belong to a run.
  std::vector<uint8_t> blen(n, 0), marked(n, 0);
  if (opts.fuse_diagonals) {
    size_t i = 0;
    while (i < n) {
      if (block_at(c, i, opts.recognize_zz) == 0) {
        i++;
        continue;
      }
      size_t j = i, blocks = 0;
      for (size_t l; j < n && (l = block_at(c, j, opts.recognize_zz)) != 0; j += l) {
        blen[j] = uint8_t(l);
        blocks++;
      }
      if (blocks >= 2 || blen[i] == 3) std::fill(marked.begin() + i, marked.begin() + j, 1);
      i = j;
    }
  }

  // Pass 2: emission.
  size_t i = 0;
  while (i < n) {
    if (marked[i]) {
      PlanOp op;
      op.kind = PlanOp::Kind::DiagonalLayer;
      size_t j = i;
      while (j < n && marked[j]) {
        const size_t len = blen[j] ? blen[j] : 1;
        if (len == 3) {
          uint32_t a, b;
          double t;
          zz_at(c, j, &a, &b, &t);
          const uint64_t ma = 1ull << a, mb = 1ull << b;
          op.masks.insert(op.masks.end(), {ma, mb, ma | mb});
          op.angles.insert(op.angles.end(), {t, t, -2.0 * t});
          op.global_phase += -t / 2.0;
        } else {
          op.global_phase += add_diagonal_term(c.ops[j], op);
        }
        j += len;
      }
      plan.ops.push_back(std::move(op));
      i = j;
      continue;
    }
    if (opts.collapse_1q_windows && c.ops[i].num_qubits == 1) {
      size_t j = i;
      while (j < n && c.ops[j].num_qubits == 1 && !marked[j]) j++;
      if (j - i >= 2) {
        emit_window(c, i, j, opts.group_1q, plan);
        i = j;
        continue;
      }
    }
    plan.ops.push_back(lower_one(c.ops[i]));
    i++;
  }

  // Pass 3: cache blocking.
  if (opts.block_bits >= 2) return block_pass(std::move(plan), opts.block_bits);
  return plan;
}

}  // namespace qmetal
