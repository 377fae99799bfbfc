// circuit.cpp -- gate constructors, gate matrices, Pauli helpers.
//
// gate_matrix_1q follows src/reference.cpp:60-98 entry for entry (the
// matrices are the gates' definitions); PauliString::valid / weight / single
// follow src/pauli.cpp:9-60.
#include "circuit.hpp"

#include <cmath>
#include <stdexcept>

namespace qmetal {

Gate g1(GateKind k, uint32_t q) { return Gate{k, 1, 0, {q, 0, 0}, {0, 0, 0}}; }
Gate g1p(GateKind k, uint32_t q, double t) { return Gate{k, 1, 1, {q, 0, 0}, {t, 0, 0}}; }
Gate g2(GateKind k, uint32_t a, uint32_t b) { return Gate{k, 2, 0, {a, b, 0}, {0, 0, 0}}; }
Gate g2p(GateKind k, uint32_t a, uint32_t b, double t) {
  return Gate{k, 2, 1, {a, b, 0}, {t, 0, 0}};
}
Gate g3(GateKind k, uint32_t a, uint32_t b, uint32_t c) {
  return Gate{k, 3, 0, {a, b, c}, {0, 0, 0}};
}

const char *gate_name(GateKind k) {
  static const char *names[G_KIND_COUNT] = {
      "x", "y", "z", "h", "s", "sdg", "t", "tdg", "rx", "ry", "rz", "p",
      "cx", "cy", "cz", "swap", "cp", "ccx", "u3"};
  return (k < G_KIND_COUNT) ? names[k] : "?";
}

void gate_matrix_1q(GateKind k, const double *p, cdouble m[4]) {
  const double r = 1.0 / std::sqrt(2.0);
  const cdouble i(0, 1);
  switch (k) {
    case G_X: m[0] = 0.0; m[1] = 1.0; m[2] = 1.0; m[3] = 0.0; return;
    case G_Y: m[0] = 0.0; m[1] = -i; m[2] = i; m[3] = 0.0; return;
    case G_Z: m[0] = 1.0; m[1] = 0.0; m[2] = 0.0; m[3] = -1.0; return;
    case G_H: m[0] = r; m[1] = r; m[2] = r; m[3] = -r; return;
    case G_S: m[0] = 1.0; m[1] = 0.0; m[2] = 0.0; m[3] = i; return;
    case G_SDG: m[0] = 1.0; m[1] = 0.0; m[2] = 0.0; m[3] = -i; return;
    case G_T:
      m[0] = 1.0; m[1] = 0.0; m[2] = 0.0; m[3] = std::polar(1.0, M_PI / 4); return;
    case G_TDG:
      m[0] = 1.0; m[1] = 0.0; m[2] = 0.0; m[3] = std::polar(1.0, -M_PI / 4); return;
    case G_RX: {
      const double c = std::cos(p[0] / 2), s = std::sin(p[0] / 2);
      m[0] = c; m[1] = cdouble(0, -s); m[2] = cdouble(0, -s); m[3] = c;
      return;
    }
    case G_RY: {
      const double c = std::cos(p[0] / 2), s = std::sin(p[0] / 2);
      m[0] = c; m[1] = -s; m[2] = s; m[3] = c;
      return;
    }
    case G_RZ:
      m[0] = std::polar(1.0, -p[0] / 2); m[1] = 0.0; m[2] = 0.0;
      m[3] = std::polar(1.0, p[0] / 2);
      return;
    case G_P:
      m[0] = 1.0; m[1] = 0.0; m[2] = 0.0; m[3] = std::polar(1.0, p[0]);
      return;
    case G_U3: {
      // The appended gate; the OpenQASM definition of U(theta, phi, lambda).
      const double c = std::cos(p[0] / 2), s = std::sin(p[0] / 2);
      m[0] = c;
      m[1] = -std::polar(s, p[2]);
      m[2] = std::polar(s, p[1]);
      m[3] = std::polar(c, p[1] + p[2]);
      return;
    }
    default:
      throw std::runtime_error("gate_matrix_1q: not a 1-qubit gate");
  }
}

bool PauliString::valid(uint32_t n) const {
  const uint64_t all = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
  if ((x_mask | y_mask | z_mask) & ~all) return false;
  return ((x_mask & y_mask) | (x_mask & z_mask) | (y_mask & z_mask)) == 0;
}

uint32_t PauliString::weight() const {
  return uint32_t(__builtin_popcountll(x_mask | y_mask | z_mask));
}

PauliString PauliString::parse(const std::string &s) {
  if (s.size() > 64) throw std::runtime_error("PauliString::parse: more than 64 qubits");
  PauliString p;
  for (size_t q = 0; q < s.size(); q++) {
    const uint64_t bit = 1ull << q;
    switch (s[q]) {
      case 'I': case 'i': break;
      case 'X': case 'x': p.x_mask |= bit; break;
      case 'Y': case 'y': p.y_mask |= bit; break;
      case 'Z': case 'z': p.z_mask |= bit; break;
      default: throw std::runtime_error(std::string("PauliString::parse: bad character '") + s[q] + "'");
    }
  }
  return p;
}

std::string PauliString::to_string(uint32_t n) const {
  std::string out(n, 'I');
  for (uint32_t q = 0; q < n && q < 64; q++) {
    const uint64_t bit = 1ull << q;
    if (x_mask & bit) out[q] = 'X';
    else if (y_mask & bit) out[q] = 'Y';
    else if (z_mask & bit) out[q] = 'Z';
  }
  return out;
}

size_t Circuit::count_1q() const {
  size_t k = 0;
  for (const Gate &g : ops) k += g.num_qubits == 1;
  return k;
}

size_t Circuit::count_2q() const {
  size_t k = 0;
  for (const Gate &g : ops) k += g.num_qubits == 2;
  return k;
}

PauliString PauliString::single(char axis, uint32_t q) {
  PauliString p;
  const uint64_t bit = 1ull << q;
  switch (axis) {
    case 'X': case 'x': p.x_mask = bit; break;
    case 'Y': case 'y': p.y_mask = bit; break;
    case 'Z': case 'z': p.z_mask = bit; break;
    case 'I': case 'i': break;
    default: throw std::runtime_error("PauliString::single: bad axis");
  }
  return p;
}

void serialise_plan(const Plan &p, std::vector<double> &v) {
  v.clear();
  v.push_back(double(p.ops.size()));
  for (const PlanOp &op : p.ops) {
    v.push_back(double(static_cast<int>(op.kind)));
    for (int k = 0; k < 3; k++) v.push_back(double(op.qubits[k]));
    v.push_back(double(op.block_bits));
    v.push_back(double(op.group_qubits.size()));
    v.push_back(double(op.masks.size()));
    v.push_back(op.global_phase);
    for (int k = 0; k < 4; k++) {
      v.push_back(op.matrix[k].real());
      v.push_back(op.matrix[k].imag());
    }
    for (uint32_t q : op.group_qubits) v.push_back(double(q));
    for (const cdouble &z : op.group_matrices) {
      v.push_back(z.real());
      v.push_back(z.imag());
    }
    for (uint64_t m : op.masks) v.push_back(double(m));
    for (double a : op.angles) v.push_back(a);
  }
}

}  // namespace qmetal
