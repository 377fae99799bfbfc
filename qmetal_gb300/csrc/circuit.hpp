// circuit.hpp -- gate records, Pauli strings and the fused Plan IR.
//
// The shapes follow the reference project's C++ data model so that the C ABI
// and the plan passes keep their meaning: GateKind / Gate / Circuit
// (include/qmetal/circuit.h:17-71), PauliString / Hamiltonian
// (include/qmetal/pauli.h:25-52), PlanOp / Plan / FusionOptions
// (include/qmetal/plan.h:27-109). LSB-first: qubit q is bit q of the basis
// index.
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

namespace qmetal {

using cdouble = std::complex<double>;

// Numbering is the C ABI's qm_gate_kind (append only).
enum GateKind : uint8_t {
  G_X = 0, G_Y, G_Z, G_H, G_S, G_SDG, G_T, G_TDG,
  G_RX, G_RY, G_RZ, G_P,
  G_CX, G_CY, G_CZ, G_SWAP,
  G_CP,
  G_CCX,
  G_U3,            // appended: not in the reference's GateKind
  G_KIND_COUNT
};

struct Gate {
  GateKind kind;
  uint8_t num_qubits;
  uint8_t num_params;
  uint32_t qubits[3];
  double params[3];
};

Gate g1(GateKind k, uint32_t q);
Gate g1p(GateKind k, uint32_t q, double theta);
Gate g2(GateKind k, uint32_t a, uint32_t b);
Gate g2p(GateKind k, uint32_t a, uint32_t b, double theta);
Gate g3(GateKind k, uint32_t a, uint32_t b, uint32_t c);

struct Circuit {
  uint32_t num_qubits = 0;
  std::vector<Gate> ops;
  void add(const Gate &g) { ops.push_back(g); }
  size_t size() const { return ops.size(); }
  size_t count_1q() const;   // gates by arity
  size_t count_2q() const;
};

const char *gate_name(GateKind k);

// Row-major 2x2 of a one-qubit gate, in double. Throws for other kinds.
void gate_matrix_1q(GateKind k, const double *params, cdouble m[4]);

struct PauliString {
  uint64_t x_mask = 0, y_mask = 0, z_mask = 0;
  bool valid(uint32_t num_qubits) const;
  uint32_t weight() const;
  // "IXYZ" text, qubit 0 first (at most 64 characters); throws on anything else.
  static PauliString parse(const std::string &s);
  std::string to_string(uint32_t num_qubits) const;
  static PauliString identity() { return PauliString{}; }
  static PauliString single(char axis, uint32_t q);
};

struct PauliTerm {
  double coefficient = 1.0;
  PauliString pauli;
};

struct Hamiltonian {
  std::vector<PauliTerm> terms;
  void add(double c, const PauliString &p) { terms.push_back({c, p}); }
  size_t size() const { return terms.size(); }
};

struct PlanOp {
  enum class Kind : uint8_t {
    Dense1q, Dense1qGroup, Blocked1q, Controlled1q, DiagonalLayer, Swap, CCX,
  };
  Kind kind = Kind::Dense1q;
  uint32_t qubits[3] = {0, 0, 0};
  cdouble matrix[4] = {1, 0, 0, 1};
  // DiagonalLayer: phase(i) = global_phase + sum of angles[t] over the terms
  // whose mask is fully set in i.
  std::vector<uint64_t> masks;
  std::vector<double> angles;
  double global_phase = 0.0;
  // Dense1qGroup / Blocked1q: wires (ascending for groups) and their 2x2s.
  std::vector<uint32_t> group_qubits;
  std::vector<cdouble> group_matrices;
  uint32_t block_bits = 0;
  size_t term_count() const { return masks.size(); }
};

struct Plan {
  uint32_t num_qubits = 0;
  std::vector<PlanOp> ops;
  size_t size() const { return ops.size(); }
};

struct FusionOptions {
  bool collapse_1q_windows = true;
  bool fuse_diagonals = true;
  bool recognize_zz = true;
  uint32_t group_1q = 4;
  uint32_t block_bits = 0;
  static FusionOptions none() { return FusionOptions{false, false, false, 1, 0}; }
  static FusionOptions blocked(uint32_t bits) {
    FusionOptions o;
    o.block_bits = bits;
    return o;
  }
};

Plan build_plan(const Circuit &c, const FusionOptions &opts = {});
bool is_diagonal(const Gate &g);

// Diagonal contribution of a gate: appends its (mask, angle) term and returns
// the global phase it carries (src/plan.cpp:106-135). Precondition:
// is_diagonal(g).
double diagonal_term(const Gate &g, std::vector<uint64_t> &masks, std::vector<double> &angles);

// Is c.ops[i..i+2] a CX(a,b) . RZ_b(t) . CX(a,b) coupling (src/plan.cpp:145-157)?
bool zz_coupling_at(const Circuit &c, size_t i, uint32_t *a, uint32_t *b, double *t);

// Flat serialisation of a plan, all doubles (masks are < 2^53):
//   [num_ops] then per op: kind, q0, q1, q2, block_bits, n_group, n_terms,
//   global_phase, matrix[8], group_qubits[n_group], group_matrices[8*n_group],
//   masks[n_terms], angles[n_terms].
void serialise_plan(const Plan &p, std::vector<double> &out);

}  // namespace qmetal
