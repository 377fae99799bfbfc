// ref_shim.cpp -- a C entry layer over the reference project's own CPU code.
//
// TEST INFRASTRUCTURE ONLY. build_ref.sh compiles this file together with
// the reference's src/{reference,plan,pauli,circuits}.cpp, read where they lie,
// into oracle/_ref/libqref.so. The parity tests use it to pin the C
// restatement (qsim_oracle.c) and the library's own plan builder against the
// reference itself. It is never linked into the product.
//
// Entry points:
//   qref_run          Reference::run (src/reference.cpp:203-206), optionally
//                     from a caller-given initial state
//   qref_run_plan     build_plan (src/plan.cpp:187-359) then Reference::run(Plan)
//                     (src/reference.cpp:245-248)
//   qref_plan         build_plan, serialised in the flat layout qsim_oracle.c reads
//   qref_expectation  Reference::expectation (src/reference.cpp:264-284)
//   qref_circuit      the frozen generators (src/circuits.cpp:24-191)
//
// The reference keeps its state private and has no setter. Reference::state()
// returns a const reference to a non-const member of a non-const object, so
// writing through const_cast is well defined; that is the only access used.

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "qmetal/circuits.h"
#include "qmetal/plan.h"
#include "qmetal/reference.h"

using namespace qmetal;

namespace {

thread_local std::string g_err;

Circuit make_circuit(uint32_t n, size_t ng, const int32_t *kinds,
                     const uint32_t *nq, const uint32_t *qubits,
                     const double *params, const uint32_t *np) {
  Circuit c;
  c.num_qubits = n;
  for (size_t g = 0; g < ng; g++) {
    Gate x{};
    x.kind = static_cast<GateKind>(kinds[g]);
    x.num_qubits = static_cast<uint8_t>(nq[g]);
    x.num_params = static_cast<uint8_t>(np ? np[g] : 0);
    for (int k = 0; k < 3; k++) {
      x.qubits[k] = qubits[3 * g + k];
      x.params[k] = params[3 * g + k];
    }
    c.add(x);
  }
  return c;
}

void load_state(Reference &r, const double *init) {
  auto &st = const_cast<std::vector<cdouble> &>(r.state());
  for (size_t i = 0; i < st.size(); i++)
    st[i] = cdouble(init[2 * i], init[2 * i + 1]);
}

void store_state(const Reference &r, double *out) {
  const auto &st = r.state();
  for (size_t i = 0; i < st.size(); i++) {
    out[2 * i] = st[i].real();
    out[2 * i + 1] = st[i].imag();
  }
}

FusionOptions opts_of(int collapse, int diag, int zz, uint32_t group,
                      uint32_t block) {
  FusionOptions o;
  o.collapse_1q_windows = collapse != 0;
  o.fuse_diagonals = diag != 0;
  o.recognize_zz = zz != 0;
  o.group_1q = group;
  o.block_bits = block;
  return o;
}

void serialise(const Plan &p, std::vector<double> &v) {
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

}  // namespace

extern "C" {

const char *qref_last_error(void) { return g_err.c_str(); }

int qref_run(uint32_t n, size_t ng, const int32_t *kinds, const uint32_t *nq,
             const uint32_t *qubits, const double *params, const uint32_t *np,
             const double *init, double *out) {
  try {
    Reference r(n);
    if (init) load_state(r, init);
    r.run(make_circuit(n, ng, kinds, nq, qubits, params, np));
    store_state(r, out);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

int qref_run_plan(uint32_t n, size_t ng, const int32_t *kinds,
                  const uint32_t *nq, const uint32_t *qubits,
                  const double *params, const uint32_t *np, int collapse,
                  int diag, int zz, uint32_t group, uint32_t block,
                  const double *init, double *out) {
  try {
    Reference r(n);
    if (init) load_state(r, init);
    r.run(build_plan(make_circuit(n, ng, kinds, nq, qubits, params, np),
                     opts_of(collapse, diag, zz, group, block)));
    store_state(r, out);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

// Writes at most cap doubles; returns the full serialised length, or -1.
long qref_plan(uint32_t n, size_t ng, const int32_t *kinds, const uint32_t *nq,
               const uint32_t *qubits, const double *params,
               const uint32_t *np, int collapse, int diag, int zz,
               uint32_t group, uint32_t block, double *out, size_t cap) {
  try {
    std::vector<double> v;
    serialise(build_plan(make_circuit(n, ng, kinds, nq, qubits, params, np),
                         opts_of(collapse, diag, zz, group, block)),
              v);
    if (out) std::memcpy(out, v.data(), sizeof(double) * std::min(cap, v.size()));
    return long(v.size());
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

int qref_expectation(uint32_t n, const double *state, uint64_t x, uint64_t y,
                     uint64_t z, double *out) {
  try {
    Reference r(n);
    load_state(r, state);
    PauliString p;
    p.x_mask = x;
    p.y_mask = y;
    p.z_mask = z;
    *out = r.expectation(p);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

// Generate one of the reference's circuits. Returns the gate count (writing at
// most cap gates), or -1. Arguments a, b are the generator's extra integers
// (depth / layers / width / rounds) and seed its seed where it takes one.
long qref_circuit(const char *name, uint32_t n, uint32_t a, uint32_t b,
                  uint64_t seed, int32_t *kinds, uint32_t *nq,
                  uint32_t *qubits, double *params, uint32_t *np, size_t cap) {
  try {
    std::string s(name);
    Circuit c;
    if (s == "ghz") c = ghz(n);
    else if (s == "qft") c = qft(n);
    else if (s == "qaoa_ring") c = qaoa_ring(n, a);
    else if (s == "tfim_trotter") c = tfim_trotter(n, a);
    else if (s == "grover_proxy") c = grover_proxy(n, a);
    else if (s == "random_circuit") c = random_circuit(n, a, seed);
    else if (s == "hardware_efficient") c = hardware_efficient(n, a, seed);
    else if (s == "local_patch") c = local_patch(n, a, b, seed);
    else throw std::runtime_error("unknown circuit " + s);
    for (size_t g = 0; g < c.ops.size() && g < cap; g++) {
      const Gate &x = c.ops[g];
      kinds[g] = int32_t(x.kind);
      nq[g] = x.num_qubits;
      np[g] = x.num_params;
      for (int k = 0; k < 3; k++) {
        qubits[3 * g + k] = x.qubits[k];
        params[3 * g + k] = x.params[k];
      }
    }
    return long(c.ops.size());
  } catch (const std::exception &e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"
