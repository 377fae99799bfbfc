// capi.cpp -- the C ABI (include/qmetal/qmetal.h) over the CUDA Simulator.
//
// Contract kept from the reference boundary (src/capi.cpp:19-274): every
// entry point catches; failures return -1 (NULL for constructors, 0 for size
// queries) and leave a thread-local message in qm_last_error(); the C gate
// enum is mapped explicitly so the C++ enum may change without breaking it.
#include "../../include/qmetal/qmetal.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>

#include "circuit.hpp"
#include "batch.hpp"
#include "schedule.hpp"
#include "simulator.hpp"

using namespace qmetal;

struct qm_circuit_s {
  Circuit c;
};
struct qm_simulator_s {
  Simulator *s;
};

namespace {

thread_local std::string g_error;

void set_error(const char *what) { g_error = what ? what : "unknown error"; }

template <typename Fn>
int guarded(Fn &&fn) {
  try {
    fn();
    return 0;
  } catch (const std::exception &e) {
    set_error(e.what());
  } catch (...) {
    set_error("unknown exception");
  }
  return -1;
}

GateKind kind_of(int k) {
  if (k < QM_X || k > QM_U3) throw std::runtime_error("unknown gate code");
  static const GateKind map[] = {G_X,  G_Y,  G_Z,  G_H,  G_S,  G_SDG, G_T,    G_TDG, G_RX, G_RY,
                                 G_RZ, G_P,  G_CX, G_CY, G_CZ, G_SWAP, G_CP, G_CCX, G_U3};
  return map[k];
}

Hamiltonian hamiltonian_of(const qm_hamiltonian *h) {
  Hamiltonian out;
  if (!h) return out;
  if (h->num_terms && (!h->coeffs || !h->x_masks || !h->y_masks || !h->z_masks))
    throw std::runtime_error("hamiltonian: null array with non-zero num_terms");
  out.terms.reserve(h->num_terms);
  for (uint32_t i = 0; i < h->num_terms; i++) {
    PauliString p;
    p.x_mask = h->x_masks[i];
    p.y_mask = h->y_masks[i];
    p.z_mask = h->z_masks[i];
    out.add(h->coeffs[i], p);
  }
  return out;
}

Gate gate_of(uint32_t width, qm_gate_kind kind, const uint32_t *qubits, uint32_t nq,
             const double *params, uint32_t np) {
  if (nq == 0 || nq > 3) throw std::runtime_error("gate arity must be 1..3");
  if (np > 3) throw std::runtime_error("at most three parameters");
  if (!qubits) throw std::runtime_error("null qubit array");
  if (np && !params) throw std::runtime_error("null parameter array");
  Gate g{};
  g.kind = kind_of(kind);
  if (g.kind == G_U3 && (nq != 1 || np != 3))
    throw std::runtime_error("u3 takes one qubit and three parameters");
  g.num_qubits = static_cast<uint8_t>(nq);
  g.num_params = static_cast<uint8_t>(np);
  for (uint32_t i = 0; i < nq; i++) {
    if (qubits[i] >= width) throw std::runtime_error("qubit index out of range");
    g.qubits[i] = qubits[i];
  }
  for (uint32_t i = 0; i < np; i++) g.params[i] = params[i];
  return g;
}

FusionOptions options_of(int collapse, int diag, int zz, uint32_t group, uint32_t block) {
  FusionOptions o;
  o.collapse_1q_windows = collapse != 0;
  o.fuse_diagonals = diag != 0;
  o.recognize_zz = zz != 0;
  o.group_1q = group;
  o.block_bits = block;
  return o;
}

}  // namespace

extern "C" {

void qm_version(int *major, int *minor, int *patch) {
  if (major) *major = QMETAL_VERSION_MAJOR;
  if (minor) *minor = QMETAL_VERSION_MINOR;
  if (patch) *patch = QMETAL_VERSION_PATCH;
}

const char *qm_last_error(void) { return g_error.c_str(); }

int qm_is_available(void) {
  try {
    return Simulator::available() ? 1 : 0;
  } catch (...) {
    return 0;
  }
}

const char *qm_device_name(void) {
  static thread_local std::string name;
  try {
    name = Simulator::device_name();
  } catch (...) {
    name = "none";
  }
  return name.c_str();
}

uint64_t qm_max_buffer_length(void) {
  try {
    return Simulator::max_buffer_length();
  } catch (...) {
    return 0;
  }
}

uint64_t qm_recommended_working_set(void) {
  try {
    return Simulator::recommended_working_set();
  } catch (...) {
    return 0;
  }
}

uint32_t qm_max_qubits(void) { return kMaxQubits; }

qm_circuit qm_circuit_create(uint32_t num_qubits) {
  auto *c = new (std::nothrow) qm_circuit_s;
  if (!c) {
    set_error("out of memory");
    return nullptr;
  }
  c->c.num_qubits = num_qubits;
  return c;
}

void qm_circuit_destroy(qm_circuit c) { delete c; }

int qm_circuit_add(qm_circuit c, qm_gate_kind kind, const uint32_t *qubits, uint32_t nq,
                   const double *params, uint32_t np) {
  if (!c) {
    set_error("null circuit");
    return -1;
  }
  return guarded([&] { c->c.add(gate_of(c->c.num_qubits, kind, qubits, nq, params, np)); });
}

size_t qm_circuit_size(qm_circuit c) { return c ? c->c.size() : 0; }

size_t qm_circuit_plan_size(qm_circuit c, int fuse) {
  if (!c) return 0;
  try {
    return build_plan(c->c, fuse ? FusionOptions{} : FusionOptions::none()).size();
  } catch (const std::exception &e) {
    set_error(e.what());
    return 0;
  }
}

qm_simulator qm_create(uint32_t num_qubits) {
  auto *h = new (std::nothrow) qm_simulator_s;
  if (!h) {
    set_error("out of memory");
    return nullptr;
  }
  h->s = nullptr;
  try {
    h->s = new Simulator(num_qubits);
  } catch (const std::exception &e) {
    set_error(e.what());
    delete h;
    return nullptr;
  }
  return h;
}

void qm_destroy(qm_simulator s) {
  if (!s) return;
  delete s->s;
  delete s;
}

int qm_reset(qm_simulator s) {
  if (!s) {
    set_error("null simulator");
    return -1;
  }
  return guarded([&] { s->s->reset(); });
}

int qm_run(qm_simulator s, qm_circuit c) {
  if (!s || !c) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->run(c->c); });
}

int qm_run_cached(qm_simulator s, qm_circuit c) {
  if (!s || !c) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->run_cached(c->c); });
}

int qm_run_merged(qm_simulator s, qm_circuit c) {
  if (!s || !c) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->run_merged(c->c); });
}

int qm_permute_qubits(qm_simulator s, const uint32_t *perm, uint32_t count) {
  if (!s || (count && !perm)) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->permute_qubits(std::vector<uint32_t>(perm, perm + count)); });
}

int qm_run_unfused(qm_simulator s, qm_circuit c) {
  if (!s || !c) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->run(c->c, FusionOptions::none()); });
}

int qm_synchronize(qm_simulator s) {
  if (!s) {
    set_error("null simulator");
    return -1;
  }
  return guarded([&] { s->s->synchronize(); });
}

uint32_t qm_num_qubits(qm_simulator s) { return s ? s->s->num_qubits() : 0; }
uint64_t qm_dim(qm_simulator s) { return s ? s->s->dim() : 0; }
uint64_t qm_dispatch_count(qm_simulator s) { return s ? s->s->dispatch_count() : 0; }

const float *qm_amplitudes(qm_simulator s) {
  if (!s) {
    set_error("null simulator");
    return nullptr;
  }
  try {
    return s->s->raw();
  } catch (const std::exception &e) {
    set_error(e.what());
    return nullptr;
  }
}

int qm_norm(qm_simulator s, double *out) {
  if (!s || !out) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { *out = s->s->norm(); });
}

int qm_expectation_pauli(qm_simulator s, uint64_t x, uint64_t y, uint64_t z, double *out) {
  if (!s || !out) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    PauliString p;
    p.x_mask = x;
    p.y_mask = y;
    p.z_mask = z;
    *out = s->s->expectation(p);
  });
}

int qm_expectation(qm_simulator s, const qm_hamiltonian *h, double *out) {
  if (!s || !h || !out) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { *out = s->s->expectation(hamiltonian_of(h)); });
}

int qm_sample(qm_simulator s, size_t shots, uint64_t seed, uint64_t *out) {
  if (!s || (shots && !out)) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    auto v = s->s->sample(shots, seed);
    if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(uint64_t));
  });
}

int qm_energy_and_gradient(qm_simulator s, qm_circuit c, const qm_hamiltonian *h,
                           double *out_energy, double *out_grad) {
  if (!s || !c || !h || !out_grad) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    auto r = s->s->energy_and_gradient(c->c, hamiltonian_of(h));
    if (out_energy) *out_energy = r.first;
    if (!r.second.empty()) std::memcpy(out_grad, r.second.data(), r.second.size() * sizeof(double));
  });
}

// --- appended extensions ----------------------------------------------------

int qm_set_state(qm_simulator s, const float *in, uint64_t count) {
  if (!s || !in) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    if (count != s->s->dim()) throw std::runtime_error("set_state: count must equal qm_dim");
    s->s->set_state(in);
  });
}

int qm_get_state(qm_simulator s, float *out, uint64_t count) {
  if (!s || !out) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    if (count != s->s->dim()) throw std::runtime_error("get_state: count must equal qm_dim");
    s->s->get_state(out);
  });
}

int qm_apply_gate(qm_simulator s, qm_gate_kind kind, const uint32_t *qubits, uint32_t nq,
                  const double *params, uint32_t np) {
  if (!s) {
    set_error("null simulator");
    return -1;
  }
  return guarded([&] { s->s->apply(gate_of(s->s->num_qubits(), kind, qubits, nq, params, np)); });
}

int qm_run_options(qm_simulator s, qm_circuit c, int collapse, int diag, int zz, uint32_t group,
                   uint32_t block) {
  if (!s || !c) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->run(c->c, options_of(collapse, diag, zz, group, block)); });
}

size_t qm_circuit_plan_export(qm_circuit c, int collapse, int diag, int zz, uint32_t group,
                              uint32_t block, double *out, size_t cap) {
  if (!c) {
    set_error("null circuit");
    return 0;
  }
  try {
    std::vector<double> v;
    serialise_plan(build_plan(c->c, options_of(collapse, diag, zz, group, block)), v);
    if (out && cap) std::memcpy(out, v.data(), sizeof(double) * std::min(cap, v.size()));
    return v.size();
  } catch (const std::exception &e) {
    set_error(e.what());
    return 0;
  }
}

size_t qm_schedule_export(qm_circuit c, const qm_hamiltonian *h, int which, uint32_t tile_high,
                          double *out, size_t cap) {
  if (!c || (which == 2 && !h)) {
    set_error("null argument");
    return 0;
  }
  try {
    std::vector<double> v;
    const uint32_t n = c->c.num_qubits;
    switch (which) {
      case 0: serialise_schedule(merged_schedule(build_plan(c->c, FusionOptions{})), n, v); break;
      case 1: serialise_schedule(backward_schedule(c->c, tile_high), n, v); break;
      case 2: serialise_schedule(costate_schedule(hamiltonian_of(h), n), v); break;
      default: throw std::runtime_error("schedule: which must be 0, 1 or 2");
    }
    if (out && cap) std::memcpy(out, v.data(), sizeof(double) * std::min(cap, v.size()));
    return v.size();
  } catch (const std::exception &e) {
    set_error(e.what());
    return 0;
  }
}

int qm_expectation_terms(qm_simulator s, const qm_hamiltonian *h, double *out) {
  if (!s || !h || (h->num_terms && !out)) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->expectation_terms(hamiltonian_of(h), out); });
}

int qm_run_profiled(qm_simulator s, qm_circuit c, int fuse, double *out, size_t cap,
                    size_t *count) {
  if (!s || !c || (cap && !out)) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    std::vector<double> t;
    s->s->run_profiled(build_plan(c->c, fuse ? FusionOptions{} : FusionOptions::none()), t);
    if (out) std::memcpy(out, t.data(), sizeof(double) * std::min(cap, t.size()));
    if (count) *count = t.size();
  });
}

int qm_set_tile_high(qm_simulator s, uint32_t tile_high) {
  if (!s) {
    set_error("null argument");
    return -1;
  }
  if (tile_high < 1 || tile_high > kMaxTileHigh) {
    set_error("tile_high must be 1..6");
    return -1;
  }
  return guarded([&] { s->s->set_tile_high(tile_high); });
}

int qm_set_wait_poll_limit(qm_simulator s, int64_t polls) {
  if (!s) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { s->s->set_wait_poll_limit(static_cast<long long>(polls)); });
}

int qm_energy_and_gradient_mode(qm_simulator s, qm_circuit c, const qm_hamiltonian *h, int mode,
                                double *out_energy, double *out_grad) {
  if (!s || !c || !h || !out_grad) {
    set_error("null argument");
    return -1;
  }
  if (mode != 0 && mode != 1) {
    set_error("gradient mode must be 0 (block-wise) or 1 (gate by gate)");
    return -1;
  }
  return guarded([&] {
    auto r = s->s->energy_and_gradient(c->c, hamiltonian_of(h), mode == 0);
    if (out_energy) *out_energy = r.first;
    if (!r.second.empty()) std::memcpy(out_grad, r.second.data(), r.second.size() * sizeof(double));
  });
}

int qm_batch_serve(const qm_batch_item *items, size_t count, int mode, uint32_t lanes) {
  if (count && !items) {
    set_error("null argument");
    return -1;
  }
  if (mode < 0 || mode > 3) {
    set_error("batch mode must be 0, 1, 2 or 3");
    return -1;
  }
  return guarded([&] {
    std::vector<Hamiltonian> hams(count);
    std::vector<BatchItem> v(count);
    for (size_t i = 0; i < count; i++) {
      if (!items[i].circuit || !items[i].hamiltonian)
        throw std::runtime_error("batch: null circuit or Hamiltonian");
      hams[i] = hamiltonian_of(items[i].hamiltonian);
      v[i].circuit = &items[i].circuit->c;
      v[i].hamiltonian = &hams[i];
      v[i].shots = items[i].shots;
      v[i].seed = items[i].seed;
      v[i].energy = items[i].out_energy;
      v[i].grad = items[i].out_grad;
      v[i].samples = items[i].out_samples;
    }
    run_batch(v, static_cast<BatchMode>(mode), lanes);
  });
}

int qm_batch_graph_timing(double *out_record_s, double *out_instantiate_s,
                          double *out_execute_s, uint64_t *out_nodes) {
  const GraphTiming t = last_graph_timing();
  if (out_record_s) *out_record_s = t.record_s;
  if (out_instantiate_s) *out_instantiate_s = t.instantiate_s;
  if (out_execute_s) *out_execute_s = t.execute_s;
  if (out_nodes) *out_nodes = t.nodes;
  return 0;
}

int qm_batch_autotune(const qm_batch_item *items, size_t count, uint32_t *out_lanes,
                      uint32_t *out_tile_high, double *out_seconds) {
  if (!count || !items) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] {
    std::vector<Hamiltonian> hams(count);
    std::vector<BatchItem> v(count);
    for (size_t i = 0; i < count; i++) {
      if (!items[i].circuit || !items[i].hamiltonian)
        throw std::runtime_error("batch: null circuit or Hamiltonian");
      hams[i] = hamiltonian_of(items[i].hamiltonian);
      v[i].circuit = &items[i].circuit->c;
      v[i].hamiltonian = &hams[i];
      v[i].shots = items[i].shots;
      v[i].seed = items[i].seed;
      v[i].energy = items[i].out_energy;
      v[i].grad = items[i].out_grad;
      v[i].samples = items[i].out_samples;
    }
    const BatchTuning t = autotune_batch(v);
    if (out_lanes) *out_lanes = t.lanes;
    if (out_tile_high) std::copy(t.tile_high, t.tile_high + kMaxQubits + 1, out_tile_high);
    if (out_seconds) *out_seconds = t.seconds;
  });
}

int qm_elapsed(qm_simulator s, double *out) {
  if (!s || !out) {
    set_error("null argument");
    return -1;
  }
  return guarded([&] { *out = s->s->elapsed(); });
}

}  // extern "C"
