// simulator.cpp -- host side of the executor: plan ops to kernel launches,
// reductions, sampling and the adjoint sweep.
//
// Behaviour follows the reference host (src/metal/simulator.mm): the same
// argument checks and fail-closed errors, the same sampling stream, the same
// adjoint formula. What differs is structural: launches go on one CUDA stream
// with their parameters passed by value (no parameter pool to recycle), all
// reductions finish on the device, and results come back in one small copy.
#include "simulator.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>

#include "../../include/qmetal/qmetal_kernels.h"
#include "schedule.hpp"

namespace qmetal {
namespace {

constexpr size_t kResultSlots = 4096;
constexpr uint32_t kMaxGroup = 5;    // wires per register-group launch
constexpr uint32_t kTermsPerPass = 16;

cudaStream_t S(void *p) { return static_cast<cudaStream_t>(p); }

void narrow(const cdouble *m, float out[8]) {
  for (int k = 0; k < 4; k++) {
    out[2 * k] = static_cast<float>(m[k].real());
    out[2 * k + 1] = static_cast<float>(m[k].imag());
  }
}

// diag(1, z) exactly, after narrowing: served by the masked-phase kernel.
bool unit_diag(const float m[8]) {
  return m[0] == 1.0f && m[1] == 0.0f && m[2] == 0.0f && m[3] == 0.0f && m[4] == 0.0f &&
         m[5] == 0.0f;
}

std::string cuda_msg(int rc) {
  if (rc < 0) return "invalid kernel arguments";
  return cudaGetErrorString(static_cast<cudaError_t>(rc));
}

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

uint32_t popc(uint64_t x) { return static_cast<uint32_t>(__builtin_popcountll(x)); }

struct FlipGroup {
  uint64_t flip;
  std::vector<size_t> terms;
};

std::vector<FlipGroup> group_by_flip(const Hamiltonian &h) {
  std::vector<FlipGroup> out;
  std::map<uint64_t, size_t> where;
  for (size_t t = 0; t < h.terms.size(); t++) {
    const PauliString &p = h.terms[t].pauli;
    const uint64_t f = p.x_mask | p.y_mask;
    auto it = where.find(f);
    if (it == where.end()) {
      where[f] = out.size();
      out.push_back({f, {t}});
    } else {
      out[it->second].terms.push_back(t);
    }
  }
  return out;
}

}  // namespace

// ---------------------------------------------------------------------------

bool Simulator::available() {
  int count = 0;
  return cudaGetDeviceCount(&count) == cudaSuccess && count > 0;
}

std::string Simulator::device_name() {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
    return "none";
  return prop.name;
}

uint64_t Simulator::max_buffer_length() {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
  return free_b;
}

uint64_t Simulator::recommended_working_set() {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
  return total_b;
}

Simulator::Simulator(uint32_t n) : n_(n) {
  if (n == 0 || n > kMaxQubits)
    throw std::runtime_error("Simulator: num_qubits must be 1.." + std::to_string(kMaxQubits));
  const char *fault = std::getenv("QMETAL_FAULT");
  if (fault && std::strcmp(fault, "alloc") == 0)
    throw std::runtime_error("Simulator: state allocation failed (injected fault)");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    throw std::runtime_error("Simulator: no CUDA device");
  cuda_check(cudaGetDevice(&device_), "cudaGetDevice");
  const uint64_t bytes = (uint64_t(1) << n) * 8ull;
  ws_bytes_ = qmk_workspace_bytes(n);
  size_t free_b = 0, total_b = 0;
  cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  if (bytes + ws_bytes_ > free_b)
    throw std::runtime_error(std::to_string(n) + " qubits needs " + std::to_string(bytes >> 30) +
                             " GiB; " + std::to_string(free_b >> 30) + " GiB free on the device");
  cudaStream_t s;
  cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
  stream_ = s;
  try {
    cuda_check(cudaMalloc(&state_, bytes), "Simulator: state allocation failed");
    cuda_check(cudaMalloc(&ws_, ws_bytes_), "Simulator: workspace allocation failed");
    cuda_check(cudaMalloc(&d_results_, kResultSlots * sizeof(double)), "cudaMalloc results");
    cuda_check(cudaMallocHost(&h_results_, (kResultSlots + 1) * sizeof(double)), "cudaMallocHost");
    h_waits_ = reinterpret_cast<unsigned *>(h_results_ + kResultSlots);
    cudaEvent_t a, b;
    cuda_check(cudaEventCreate(&a), "cudaEventCreate");
    ev_start_ = a;
    cuda_check(cudaEventCreate(&b), "cudaEventCreate");
    ev_stop_ = b;
    check(qmk_workspace_init(ws_, ws_bytes_, stream_), "workspace init");
    cuda_check(cudaEventRecord(a, s), "cudaEventRecord");
    reset();
    // An injected launch fault affects calls after construction only.
    fault_launch_ = fault && std::strcmp(fault, "launch") == 0;
    // Tests cap the state checkpoints to drive the paths where only some
    // of a gradient's gathers can keep one.
    if (const char *cap = std::getenv("QMETAL_MAX_CHECKPOINTS"))
      ck_limit_ = static_cast<size_t>(std::strtoul(cap, nullptr, 10));
  } catch (...) {
    release();
    throw;
  }
}

Simulator::~Simulator() { release(); }

void Simulator::release() {
  if (stream_) cudaStreamSynchronize(S(stream_));
  for (const GraphEntry &e : graphs_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(e.exec));
  graphs_.clear();
  cudaFree(state_);
  cudaFree(costate_);
  cudaFree(scratch_);
  scratch_ = nullptr;
  for (const Checkpoint &c : ckpts_) cudaFree(c.buf);
  ckpts_.clear();
  for (float *b : ck_free_) cudaFree(b);
  ck_free_.clear();
  cudaFree(ws_);
  cudaFree(sample_ws_);
  cudaFree(d_shots_);
  cudaFree(d_results_);
  cudaFree(d_grad_);
  if (h_results_) cudaFreeHost(h_results_);
  if (mirror_) {
    if (mirror_pinned_) cudaFreeHost(mirror_);
    else std::free(mirror_);
  }
  if (ev_start_) cudaEventDestroy(static_cast<cudaEvent_t>(ev_start_));
  if (ev_stop_) cudaEventDestroy(static_cast<cudaEvent_t>(ev_stop_));
  if (stream_) cudaStreamDestroy(S(stream_));
  state_ = costate_ = nullptr;
  ws_ = sample_ws_ = nullptr;
  d_shots_ = nullptr;
  d_results_ = h_results_ = d_grad_ = nullptr;
  h_waits_ = nullptr;
  d_grad_cap_ = 0;
  mirror_ = nullptr;
  ev_start_ = ev_stop_ = stream_ = nullptr;
}

void Simulator::activate() const { cudaSetDevice(device_); }

void Simulator::check(int rc, const char *what) {
  if (fault_launch_) throw std::runtime_error(std::string(what) + ": kernel launch failed (injected fault)");
  if (rc != 0) throw std::runtime_error(std::string(what) + ": " + cuda_msg(rc));
}

void Simulator::reset() {
  activate();
  check(qmk_init_basis(state_, n_, stream_), "reset");
  dispatches_++;
}

void Simulator::synchronize() {
  activate();
  cuda_check(cudaStreamSynchronize(S(stream_)), "GPU error");
}

bool Simulator::ensure_scratch() {
  if (scratch_) return true;
  if (scratch_failed_) return false;
  const size_t bytes = dim() * 8;
  size_t free_b = 0, total_b = 0;
  // Keep 2 GiB of headroom for other simulators and the runtime.
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < bytes + (2ull << 30) ||
      cudaMalloc(&scratch_, bytes) != cudaSuccess) {
    cudaGetLastError();
    scratch_ = nullptr;
    scratch_failed_ = true;
    return false;
  }
  return true;
}

void Simulator::invalidate_graphs() {
  for (const GraphEntry &e : graphs_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(e.exec));
  graphs_.clear();
}

float *Simulator::take_buffer() {
  if (!ck_free_.empty()) {
    float *b = ck_free_.back();
    ck_free_.pop_back();
    return b;
  }
  size_t held = 0;
  for (const Checkpoint &c : ckpts_) held += c.buf != nullptr;
  if (held >= ck_limit_) return nullptr;
  const size_t bytes = dim() * 8;
  size_t free_b = 0, total_b = 0;
  float *b = nullptr;
  // Keep 4 GiB of headroom for other simulators and the runtime.
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < bytes + (4ull << 30) ||
      cudaMalloc(&b, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return b;
}

void Simulator::drop_checkpoints() {
  for (const Checkpoint &c : ckpts_)
    if (c.buf) ck_free_.push_back(c.buf);
  ckpts_.clear();
}

namespace {

// Does the undo gather (b, boff) invert the forward gather (a, aoff)?
// dst1[y] = src[A y ^ a], dst2[z] = dst1[B z ^ b] is the identity when
// A B = I and A b ^ a = 0.
bool inverts(uint32_t n, const std::vector<uint64_t> &a, uint64_t aoff,
             const std::vector<uint64_t> &b, uint64_t boff) {
  if (a.size() != n || b.size() != n) return false;
  auto apply = [&](uint64_t x) {
    uint64_t y = 0;
    for (uint32_t k = 0; k < n; k++)
      if ((x >> k) & 1ull) y ^= a[k];
    return y;
  };
  for (uint32_t j = 0; j < n; j++)
    if (apply(b[j]) != (1ull << j)) return false;
  return (apply(boff) ^ aoff) == 0;
}

}  // namespace

// The forward schedule's gathers, last first, against the backward
// schedule's undo gathers in the order the sweep meets them: the same
// number, each undoing its partner, and no CX or SWAP undone one gate at a
// time (which would leave a forward gather without its partner).
bool Simulator::checkpoints_pair(const Circuit &c, const Plan &p) const {
  std::vector<const ForwardStep *> fwd;
  const auto fs = merged_schedule(p);
  for (const ForwardStep &st : fs)
    if (st.kind == ForwardStep::Permute) fwd.push_back(&st);
  if (fwd.empty()) return false;
  size_t i = fwd.size();
  for (const BackwardStep &st : backward_schedule(c, tile_high_)) {
    if (st.kind == BackwardStep::GateUndo) {
      const GateKind k = c.ops[st.gates[0]].kind;
      if (k == G_CX || k == G_SWAP) return false;
    } else if (st.kind == BackwardStep::PermuteUndo) {
      if (i == 0) return false;
      --i;
      if (!inverts(n_, fwd[i]->cols, fwd[i]->off, st.cols, st.off)) return false;
    }
  }
  return i == 0;
}

// The top checkpoint, paired with this undo gather by checkpoints_pair:
// restores the state from it when it holds a buffer.
bool Simulator::restore_checkpoint(const std::vector<uint64_t> &cols, uint64_t off) {
  if (ckpts_.empty()) return false;
  const Checkpoint c = ckpts_.back();
  ckpts_.pop_back();
  if (!c.buf) return false;
  if (!inverts(n_, c.cols, c.off, cols, off)) {   // pairing broke: keep nothing more
    ck_free_.push_back(c.buf);
    drop_checkpoints();
    return false;
  }
  ck_free_.push_back(state_);
  state_ = c.buf;
  invalidate_graphs();   // captured graphs hold the old state pointer
  return true;
}

bool Simulator::permute(float *&buf, const std::vector<uint64_t> &cols, uint64_t off) {
  if (!ensure_scratch()) return false;
  check(qmk_apply_permutation(scratch_, buf, n_, cols.data(), off, stream_), "permutation");
  dispatches_++;
  std::swap(buf, scratch_);
  // Captured graphs hold the old state pointer.
  invalidate_graphs();
  return true;
}

// ---------------------------------------------------------------------------
// Gates and plan ops

void Simulator::apply(const Gate &g) {
  activate();
  apply_gate_to(state_, g);
}

void Simulator::apply_gate_to(float *st, const Gate &g) {
  for (int k = 0; k < g.num_qubits; k++)
    if (g.qubits[k] >= n_) throw std::runtime_error("qubit index out of range");
  if (g.num_qubits == 1) {
    cdouble m[4];
    gate_matrix_1q(g.kind, g.params, m);
    float f[8];
    narrow(m, f);
    if (unit_diag(f))
      check(qmk_apply_phase(st, n_, 1ull << g.qubits[0], f[6], f[7], stream_), "apply");
    else
      check(qmk_apply_1q(st, n_, g.qubits[0], f, stream_), "apply");
    dispatches_++;
    return;
  }
  if (g.num_qubits == 2) {
    const uint32_t a = g.qubits[0], b = g.qubits[1];
    if (a == b) throw std::runtime_error("2-qubit gate on identical wires");
    switch (g.kind) {
      case G_CX:
      case G_CY: {
        cdouble m[4];
        gate_matrix_1q(g.kind == G_CX ? G_X : G_Y, nullptr, m);
        float f[8];
        narrow(m, f);
        check(qmk_apply_controlled(st, n_, 1, &a, b, f, stream_), "apply");
        dispatches_++;
        return;
      }
      case G_CZ:
      case G_CP: {
        const cdouble ph = g.kind == G_CZ ? cdouble(-1, 0) : std::polar(1.0, g.params[0]);
        check(qmk_apply_phase(st, n_, (1ull << a) | (1ull << b), float(ph.real()),
                              float(ph.imag()), stream_),
              "apply");
        dispatches_++;
        return;
      }
      case G_SWAP:
        check(qmk_apply_swap(st, n_, a, b, stream_), "apply");
        dispatches_++;
        return;
      default:
        break;
    }
  }
  if (g.num_qubits == 3 && g.kind == G_CCX) {
    if (n_ < 3) throw std::runtime_error("CCX needs at least 3 qubits");
    const uint32_t c[2] = {g.qubits[0], g.qubits[1]}, t = g.qubits[2];
    if (c[0] == c[1] || c[0] == t || c[1] == t) throw std::runtime_error("CCX on repeated wires");
    cdouble m[4];
    gate_matrix_1q(G_X, nullptr, m);
    float f[8];
    narrow(m, f);
    check(qmk_apply_controlled(st, n_, 2, c, t, f, stream_), "apply");
    dispatches_++;
    return;
  }
  throw std::runtime_error(std::string("unsupported gate: ") + gate_name(g.kind));
}

void Simulator::run(const Circuit &c) { run(c, FusionOptions{}); }

void Simulator::run(const Circuit &c, const FusionOptions &opts) {
  if (c.num_qubits != n_) throw std::runtime_error("circuit/simulator size mismatch");
  run(build_plan(c, opts));
}

void Simulator::run(const Plan &p) {
  if (p.num_qubits != n_) throw std::runtime_error("plan/simulator size mismatch");
  activate();
  for (const PlanOp &op : p.ops) apply_op_to(state_, op);
}

void Simulator::apply(const PlanOp &op) {
  activate();
  apply_op_to(state_, op);
}

namespace {

// FNV-1a over the circuit's content (width, kinds, wires, parameter bits).
uint64_t circuit_key(const Circuit &c) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void *p, size_t n) {
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
      h ^= b[i];
      h *= 1099511628211ull;
    }
  };
  mix(&c.num_qubits, sizeof(c.num_qubits));
  const uint64_t count = c.ops.size();
  mix(&count, sizeof(count));
  for (const Gate &g : c.ops) {
    mix(&g.kind, 1);
    mix(&g.num_qubits, 1);
    mix(&g.num_params, 1);
    mix(g.qubits, sizeof(uint32_t) * g.num_qubits);
    mix(g.params, sizeof(double) * g.num_params);
  }
  return h;
}

constexpr size_t kMaxGraphs = 16;

}  // namespace

void Simulator::run_cached(const Circuit &c) {
  if (c.num_qubits != n_) throw std::runtime_error("circuit/simulator size mismatch");
  activate();
  const uint64_t key = circuit_key(c);
  for (size_t i = 0; i < graphs_.size(); i++) {
    if (graphs_[i].key != key) continue;
    GraphEntry e = graphs_[i];
    graphs_.erase(graphs_.begin() + i);
    graphs_.push_back(e);
    cuda_check(cudaGraphLaunch(static_cast<cudaGraphExec_t>(e.exec), S(stream_)), "graph launch");
    dispatches_ += e.launches;
    return;
  }
  const Plan plan = build_plan(c, FusionOptions{});
  const uint64_t before = dispatches_;
  cuda_check(cudaStreamBeginCapture(S(stream_), cudaStreamCaptureModeThreadLocal), "graph capture");
  cudaGraph_t graph = nullptr;
  try {
    for (const PlanOp &op : plan.ops) apply_op_to(state_, op);
  } catch (...) {
    cudaStreamEndCapture(S(stream_), &graph);
    if (graph) cudaGraphDestroy(graph);
    dispatches_ = before;
    throw;
  }
  cuda_check(cudaStreamEndCapture(S(stream_), &graph), "graph capture");
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  cuda_check(e, "graph instantiate");
  const uint64_t launches = dispatches_ - before;
  if (graphs_.size() == kMaxGraphs) {
    cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graphs_.front().exec));
    graphs_.erase(graphs_.begin());
  }
  graphs_.push_back({key, exec, launches});
  cuda_check(cudaGraphLaunch(exec, S(stream_)), "graph launch");
}

// The plan through merged_schedule(): one group pass per merged set of
// one-qubit ops, one gather pass per CX / SWAP run that pays, the plan's op
// kernel for everything else.
void Simulator::run_merged(const Plan &p) {
  if (p.num_qubits != n_) throw std::runtime_error("plan/simulator size mismatch");
  activate();
  for (const ForwardStep &st : merged_schedule(p)) {
    switch (st.kind) {
      case ForwardStep::Group: {
        std::vector<float> fm(2 * st.mats.size());
        for (size_t i = 0; i < st.wires.size(); i++) narrow(&st.mats[4 * i], &fm[8 * i]);
        check(qmk_apply_group(state_, n_, static_cast<uint32_t>(st.wires.size()), st.wires.data(),
                              fm.data(), stream_),
              "merged group");
        dispatches_++;
        break;
      }
      case ForwardStep::Permute: {
        if (keep_ckpts_ && ensure_scratch()) {
          if (float *dst = take_buffer()) {
            check(qmk_apply_permutation(dst, state_, n_, st.cols.data(), st.off, stream_),
                  "permutation");
            dispatches_++;
            ckpts_.push_back({state_, st.cols, st.off});
            state_ = dst;
            invalidate_graphs();
            break;
          }
        }
        if (keep_ckpts_) ckpts_.push_back({nullptr, st.cols, st.off});   // keeps the pairing
        if (!permute(state_, st.cols, st.off))
          for (size_t i : st.ops) apply_op_to(state_, p.ops[i]);
        break;
      }
      case ForwardStep::Op:
        apply_op_to(state_, p.ops[st.ops[0]]);
        break;
    }
  }
}

void Simulator::permute_qubits(const std::vector<uint32_t> &perm) {
  if (perm.size() != n_) throw std::runtime_error("permute_qubits: one target per qubit");
  std::vector<bool> seen(n_, false);
  for (uint32_t p : perm) {
    if (p >= n_ || seen[p]) throw std::runtime_error("permute_qubits: not a permutation");
    seen[p] = true;
  }
  activate();
  // new[x'] = old[x] with bit perm[q] of x' = bit q of x, i.e. a gather with
  // G(x') = sum over set bits perm[q] of x' of e_q.
  std::vector<uint64_t> cols(n_);
  for (uint32_t q = 0; q < n_; q++) cols[perm[q]] = 1ull << q;
  bool identity = true;
  for (uint32_t q = 0; q < n_; q++) identity &= perm[q] == q;
  if (identity) return;
  if (!permute(state_, cols, 0))
    throw std::runtime_error("permute_qubits: no room for the second state buffer");
}

void Simulator::run_merged(const Circuit &c) {
  if (c.num_qubits != n_) throw std::runtime_error("circuit/simulator size mismatch");
  run_merged(build_plan(c, FusionOptions{}));
}

void Simulator::run_profiled(const Plan &p, std::vector<double> &seconds) {
  if (p.num_qubits != n_) throw std::runtime_error("plan/simulator size mismatch");
  activate();
  std::vector<cudaEvent_t> ev(p.ops.size() + 1);
  for (auto &e : ev) cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  try {
    cuda_check(cudaEventRecord(ev[0], S(stream_)), "cudaEventRecord");
    for (size_t i = 0; i < p.ops.size(); i++) {
      apply_op_to(state_, p.ops[i]);
      cuda_check(cudaEventRecord(ev[i + 1], S(stream_)), "cudaEventRecord");
    }
    synchronize();
    seconds.assign(p.ops.size(), 0.0);
    for (size_t i = 0; i < p.ops.size(); i++) {
      float ms = 0.0f;
      cuda_check(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]), "cudaEventElapsedTime");
      seconds[i] = double(ms) * 1e-3;
    }
  } catch (...) {
    for (auto &e : ev) cudaEventDestroy(e);
    throw;
  }
  for (auto &e : ev) cudaEventDestroy(e);
}

void Simulator::apply_op_to(float *st, const PlanOp &op) {
  switch (op.kind) {
    case PlanOp::Kind::Dense1q: {
      if (op.qubits[0] >= n_) throw std::runtime_error("qubit index out of range");
      float f[8];
      narrow(op.matrix, f);
      if (unit_diag(f))
        check(qmk_apply_phase(st, n_, 1ull << op.qubits[0], f[6], f[7], stream_), "dense1q");
      else
        check(qmk_apply_1q(st, n_, op.qubits[0], f, stream_), "dense1q");
      dispatches_++;
      return;
    }
    case PlanOp::Kind::Dense1qGroup: {
      const size_t k = op.group_qubits.size();
      if (k < 2) throw std::runtime_error("group size must be at least 2");
      if (op.group_matrices.size() != 4 * k) throw std::runtime_error("group matrices malformed");
      for (size_t j = 0; j < k; j++) {
        if (op.group_qubits[j] >= n_) throw std::runtime_error("qubit index out of range");
        if (j && op.group_qubits[j] <= op.group_qubits[j - 1])
          throw std::runtime_error("group wires must be ascending and distinct");
      }
      // Wider groups go K wires at a time: the gates commute, so splitting
      // changes the grouping of passes, not the unitary.
      for (size_t b = 0; b < k; b += kMaxGroup) {
        const uint32_t take = static_cast<uint32_t>(std::min<size_t>(kMaxGroup, k - b));
        std::vector<float> mats(8 * take);
        for (uint32_t j = 0; j < take; j++) narrow(&op.group_matrices[4 * (b + j)], &mats[8 * j]);
        check(qmk_apply_group(st, n_, take, &op.group_qubits[b], mats.data(), stream_), "group");
        dispatches_++;
      }
      return;
    }
    case PlanOp::Kind::Blocked1q: {
      const size_t k = op.group_qubits.size();
      const uint32_t b = op.block_bits;
      if (b < 2 || b > 14) throw std::runtime_error("block_bits must be 2..14");
      if (b > n_) throw std::runtime_error("block larger than the state");
      if (op.group_matrices.size() != 4 * k) throw std::runtime_error("blocked matrices malformed");
      std::vector<float> mats(8 * k);
      for (size_t j = 0; j < k; j++) narrow(&op.group_matrices[4 * j], &mats[8 * j]);
      check(qmk_apply_blocked(st, n_, b, static_cast<uint32_t>(k), op.group_qubits.data(),
                              mats.data(), stream_),
            "blocked");
      dispatches_ += std::max<size_t>(1, (k + 95) / 96);
      return;
    }
    case PlanOp::Kind::Controlled1q: {
      const uint32_t c = op.qubits[0], t = op.qubits[1];
      if (c >= n_ || t >= n_) throw std::runtime_error("qubit index out of range");
      if (c == t) throw std::runtime_error("2-qubit gate on identical wires");
      float f[8];
      narrow(op.matrix, f);
      check(qmk_apply_controlled(st, n_, 1, &c, t, f, stream_), "controlled1q");
      dispatches_++;
      return;
    }
    case PlanOp::Kind::DiagonalLayer: {
      const size_t nt = op.masks.size();
      if (nt == 0) return;
      if (op.angles.size() != nt) throw std::runtime_error("diagonal layer malformed");
      size_t wide = 0;
      for (uint64_t m : op.masks) {
        if (n_ < 64 && (m >> n_)) throw std::runtime_error("qubit index out of range");
        if (popc(m) >= 3) wide++;
      }
      check(qmk_apply_diagonal(st, n_, static_cast<uint32_t>(nt), op.masks.data(),
                               op.angles.data(), op.global_phase, ws_, ws_bytes_, stream_),
            "diagonal layer");
      dispatches_ += 2 + (wide + 63) / 64;
      return;
    }
    case PlanOp::Kind::Swap: {
      const uint32_t a = op.qubits[0], b = op.qubits[1];
      if (a >= n_ || b >= n_) throw std::runtime_error("qubit index out of range");
      if (a == b) return;
      check(qmk_apply_swap(st, n_, a, b, stream_), "swap");
      dispatches_++;
      return;
    }
    case PlanOp::Kind::CCX: {
      const uint32_t c[2] = {op.qubits[0], op.qubits[1]}, t = op.qubits[2];
      if (c[0] >= n_ || c[1] >= n_ || t >= n_) throw std::runtime_error("qubit index out of range");
      if (c[0] == c[1] || c[0] == t || c[1] == t) throw std::runtime_error("CCX on repeated wires");
      cdouble m[4];
      gate_matrix_1q(G_X, nullptr, m);
      float f[8];
      narrow(m, f);
      check(qmk_apply_controlled(st, n_, 2, c, t, f, stream_), "ccx");
      dispatches_++;
      return;
    }
  }
  throw std::runtime_error("Simulator: unknown PlanOp kind");
}

// ---------------------------------------------------------------------------
// State access

std::vector<cdouble> Simulator::amplitudes() {
  const float *f = raw();
  std::vector<cdouble> out(dim());
  for (size_t i = 0; i < out.size(); i++) out[i] = cdouble(f[2 * i], f[2 * i + 1]);
  return out;
}

const float *Simulator::raw() {
  activate();
  const size_t bytes = dim() * 8;
  if (!mirror_) {
    if (cudaMallocHost(&mirror_, bytes) == cudaSuccess) {
      mirror_pinned_ = true;
    } else {
      cudaGetLastError();
      mirror_ = static_cast<float *>(std::malloc(bytes));
      mirror_pinned_ = false;
      if (!mirror_) throw std::runtime_error("amplitudes: host mirror allocation failed");
    }
  }
  get_state(mirror_);
  return mirror_;
}

void Simulator::get_state(float *out) {
  activate();
  cuda_check(cudaMemcpyAsync(out, state_, dim() * 8, cudaMemcpyDeviceToHost, S(stream_)),
             "state copy");
  synchronize();
}

void Simulator::set_state(const float *in) {
  activate();
  cuda_check(cudaMemcpyAsync(state_, in, dim() * 8, cudaMemcpyHostToDevice, S(stream_)),
             "state copy");
  synchronize();
}

void Simulator::fetch(size_t count, bool waits) {
  cuda_check(cudaMemcpyAsync(h_results_, d_results_, count * sizeof(double),
                             cudaMemcpyDeviceToHost, S(stream_)),
             "result copy");
  if (waits)
    cuda_check(cudaMemcpyAsync(h_waits_, qmk_wait_counter(ws_), sizeof(unsigned),
                               cudaMemcpyDeviceToHost, S(stream_)),
               "wait count copy");
  synchronize();
  // Fail closed if a window-tile pass gave up a bounded wait (its results
  // are not valid, and neither are the states it left). The counter only
  // grows; compare with the last look.
  if (waits && *h_waits_ != waits_seen_) {
    waits_seen_ = *h_waits_;
    reset();
    synchronize();
    throw std::runtime_error("adjoint window pass: a bulk-copy wait timed out");
  }
}

void Simulator::check_waits() {
  activate();
  unsigned int n = 0;
  check(qmk_take_wait_timeouts(ws_, ws_bytes_, &n, stream_), "wait check");
  waits_seen_ = 0;  // the take reset the counter
  if (n) {
    reset();
    synchronize();
    throw std::runtime_error("adjoint window pass: a bulk-copy wait timed out");
  }
}

void Simulator::set_wait_poll_limit(long long polls) {
  activate();
  check(qmk_set_wait_poll_limit(ws_, ws_bytes_, polls, stream_), "wait poll limit");
}

// ---------------------------------------------------------------------------
// Reductions

double Simulator::abs2sum() {
  activate();
  check(qmk_abs2sum(state_, n_, d_results_, ws_, ws_bytes_, stream_), "abs2sum");
  dispatches_++;
  fetch(1);
  return h_results_[0];
}

double Simulator::norm() { return std::sqrt(abs2sum()); }

// <P_t> for every term, grouped so terms that share a flip mask share a pass.
void Simulator::pauli_values(const float *st, const Hamiltonian &h, std::vector<double> &vals) {
  vals.assign(h.terms.size(), 0.0);
  const auto groups = group_by_flip(h);
  struct Slot { size_t term; size_t slot; };
  std::vector<Slot> pending;
  size_t used = 0;
  auto drain = [&]() {
    if (pending.empty()) return;
    fetch(used);
    for (const Slot &s : pending) {
      const PauliString &p = h.terms[s.term].pauli;
      const uint64_t flip = p.x_mask | p.y_mask;
      const uint32_t ny = popc(p.y_mask);
      double v = h_results_[s.slot];
      if (flip != 0) v *= ((ny & 3u) <= 1u) ? 2.0 : -2.0;
      vals[s.term] = v;
    }
    pending.clear();
    used = 0;
  };
  for (const FlipGroup &g : groups) {
    for (size_t b = 0; b < g.terms.size(); b += kTermsPerPass) {
      const uint32_t take = static_cast<uint32_t>(std::min<size_t>(kTermsPerPass, g.terms.size() - b));
      if (used + take > kResultSlots) drain();
      uint64_t signs[kTermsPerPass];
      uint32_t nys[kTermsPerPass];
      for (uint32_t j = 0; j < take; j++) {
        const PauliString &p = h.terms[g.terms[b + j]].pauli;
        signs[j] = p.y_mask | p.z_mask;
        nys[j] = popc(p.y_mask);
        pending.push_back({g.terms[b + j], used + j});
      }
      check(qmk_pauli_expect(st, n_, g.flip, take, signs, nys, d_results_ + used, ws_, ws_bytes_,
                             stream_),
            "expectation");
      dispatches_++;
      used += take;
    }
  }
  drain();
}

double Simulator::expectation(const PauliString &p) {
  if (!p.valid(n_)) throw std::runtime_error("expectation: invalid Pauli string for this width");
  Hamiltonian h;
  h.add(1.0, p);
  std::vector<double> v;
  activate();
  pauli_values(state_, h, v);
  return v[0];
}

double Simulator::expectation(const Hamiltonian &h) {
  for (const PauliTerm &t : h.terms)
    if (!t.pauli.valid(n_))
      throw std::runtime_error("expectation: invalid Pauli string for this width");
  std::vector<double> v;
  activate();
  pauli_values(state_, h, v);
  double total = 0.0;
  for (size_t t = 0; t < h.terms.size(); t++) total += h.terms[t].coefficient * v[t];
  return total;
}

void Simulator::expectation_terms(const Hamiltonian &h, double *out) {
  for (const PauliTerm &t : h.terms)
    if (!t.pauli.valid(n_))
      throw std::runtime_error("expectation: invalid Pauli string for this width");
  std::vector<double> v;
  activate();
  pauli_values(state_, h, v);
  std::copy(v.begin(), v.end(), out);
}

// ---------------------------------------------------------------------------
// Sampling

// Queue the sampler; the draws land in d_shots_.
void Simulator::launch_sample(size_t shots, uint64_t seed) {
  const size_t need = qmk_sample_workspace_bytes(n_);
  if (!sample_ws_) {
    cuda_check(cudaMalloc(&sample_ws_, need), "sampling workspace");
    sample_ws_bytes_ = need;
  }
  if (d_shots_cap_ < shots) {
    cudaFree(d_shots_);
    d_shots_ = nullptr;
    d_shots_cap_ = 0;
    cuda_check(cudaMalloc(&d_shots_, shots * sizeof(uint64_t)), "sampling output");
    d_shots_cap_ = shots;
  }
  check(qmk_sample(state_, n_, shots, seed, d_shots_, sample_ws_, sample_ws_bytes_, stream_),
        "sample");
  const uint64_t nb = ((uint64_t(1) << n_) + 1023) / 1024;
  dispatches_ += (nb > 2048) ? 5 : 3;
}

std::vector<std::pair<std::string, uint64_t>> Simulator::counts(size_t shots, uint64_t seed) {
  std::map<uint64_t, uint64_t> tally;
  for (uint64_t v : sample(shots, seed)) tally[v]++;
  std::vector<std::pair<std::string, uint64_t>> out;
  out.reserve(tally.size());
  for (const auto &kv : tally) {
    std::string bits(n_, '0');
    for (uint32_t q = 0; q < n_; q++)
      if ((kv.first >> q) & 1ull) bits[n_ - 1 - q] = '1';
    out.emplace_back(std::move(bits), kv.second);
  }
  std::stable_sort(out.begin(), out.end(),
                   [](const auto &a, const auto &b) { return a.second > b.second; });
  return out;
}

std::vector<uint64_t> Simulator::sample(size_t shots, uint64_t seed) {
  std::vector<uint64_t> out;
  if (shots == 0) return out;
  activate();
  launch_sample(shots, seed);
  out.resize(shots);
  cuda_check(cudaMemcpyAsync(out.data(), d_shots_, shots * sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, S(stream_)),
             "sample copy");
  synchronize();
  return out;
}

// ---------------------------------------------------------------------------
// Adjoint gradient (src/metal/simulator.mm:814-963)

void Simulator::costate(const Hamiltonian &h) {
  const auto groups = group_by_flip(h);
  bool first = true;
  for (const FlipGroup &g : groups) {
    for (size_t b = 0; b < g.terms.size(); b += kTermsPerPass) {
      const uint32_t take = static_cast<uint32_t>(std::min<size_t>(kTermsPerPass, g.terms.size() - b));
      uint64_t signs[kTermsPerPass];
      uint32_t nys[kTermsPerPass];
      double coeffs[kTermsPerPass];
      for (uint32_t j = 0; j < take; j++) {
        const PauliTerm &t = h.terms[g.terms[b + j]];
        signs[j] = t.pauli.y_mask | t.pauli.z_mask;
        nys[j] = popc(t.pauli.y_mask);
        coeffs[j] = t.coefficient;
      }
      check(qmk_pauli_accum(costate_, state_, n_, g.flip, take, signs, nys, coeffs, first ? 1 : 0,
                            stream_),
            "co-state");
      dispatches_++;
      first = false;
    }
  }
  if (first) cuda_check(cudaMemsetAsync(costate_, 0, dim() * 8, S(stream_)), "co-state zero");
}

void Simulator::prepare_adjoint(const Circuit &c, const Hamiltonian &h) {
  if (c.num_qubits != n_) throw std::runtime_error("circuit/simulator size mismatch");
  for (const Gate &g : c.ops) {
    if (g.num_params > 0 && !generator_of(g))
      throw std::runtime_error(std::string("gradient: ") + gate_name(g.kind) +
                               " carries a parameter but has no native generator; only rx, ry "
                               "and rz are differentiable");
    for (int k = 0; k < g.num_qubits; k++)
      if (g.qubits[k] >= n_) throw std::runtime_error("qubit index out of range");
  }
  for (const PauliTerm &t : h.terms)
    if (!t.pauli.valid(n_)) throw std::runtime_error("gradient: invalid Pauli term");
  activate();
  if (!costate_) {
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    if (dim() * 8 > free_b) throw std::runtime_error("gradient: co-state does not fit on the device");
    cuda_check(cudaMalloc(&costate_, dim() * 8), "gradient: co-state allocation failed");
  }
  const size_t G = std::max<size_t>(c.ops.size(), 1);
  if (d_grad_cap_ < G) {
    cudaFree(d_grad_);
    d_grad_ = nullptr;
    d_grad_cap_ = 0;
    cuda_check(cudaMalloc(&d_grad_, G * sizeof(double)), "gradient buffer");
    d_grad_cap_ = G;
  }
  cuda_check(cudaMemsetAsync(d_grad_, 0, G * sizeof(double), S(stream_)), "gradient zero");
}

// lambda = H psi and E = <psi|H|psi> into d_results_[0], through
// costate_schedule().
double Simulator::energy_and_costate(const Hamiltonian &h) {
  for (const CostateStep &st : costate_schedule(h, n_)) {
    const uint32_t nt = static_cast<uint32_t>(st.coeffs.size());
    switch (st.kind) {
      case CostateStep::ZDiag:
        check(qmk_zdiag_costate(costate_, state_, n_, nt, st.masks.data(), st.coeffs.data(),
                                d_results_, ws_, ws_bytes_, stream_),
              "co-state");
        dispatches_ += 2;
        break;
      case CostateStep::Local:
        check(qmk_pauli_accum_local(costate_, state_, n_, nt, st.wires.data(), st.masks.data(),
                                    st.nys.data(), st.coeffs.data(), st.overwrite ? 1 : 0,
                                    stream_),
              "co-state");
        dispatches_++;
        break;
      case CostateStep::Flip:
        check(qmk_pauli_accum(costate_, state_, n_, st.flip, nt, st.masks.data(), st.nys.data(),
                              st.coeffs.data(), st.overwrite ? 1 : 0, stream_),
              "co-state");
        dispatches_++;
        break;
      case CostateStep::XField:
        check(qmk_xfield_costate(costate_, state_, n_, nt, st.wires.data(), st.coeffs.data(),
                                 st.overwrite ? 1 : 0, d_results_, st.energy, ws_, ws_bytes_,
                                 stream_),
              "co-state");
        dispatches_++;
        break;
      case CostateStep::Zero:
        cuda_check(cudaMemsetAsync(costate_, 0, dim() * 8, S(stream_)), "co-state zero");
        break;
      case CostateStep::Dot:
        check(qmk_dot_re(state_, costate_, n_, d_results_, ws_, ws_bytes_, stream_), "energy");
        dispatches_++;
        break;
    }
  }
  return 0.0;
}

// The reference's sweep (src/metal/simulator.mm:910-960), one gate at a time:
// a fused overlap-and-undo pass per one-qubit gate, both states undone for
// the others.
void Simulator::sweep_gate_by_gate(const Circuit &c) {
  for (size_t k = c.ops.size(); k-- > 0;) {
    const Gate &g = c.ops[k];
    const Gate inv = invert(g);
    if (g.num_qubits == 1) {
      cdouble m[4];
      gate_matrix_1q(inv.kind, inv.params, m);
      float f[8];
      narrow(m, f);
      const int gen = g.num_params > 0 ? generator_of(g) : 0;
      check(qmk_adjoint_1q(state_, costate_, n_, g.qubits[0], f, gen, d_grad_ + k, ws_, ws_bytes_,
                           stream_),
            "adjoint step");
      dispatches_++;
    } else {
      apply_gate_to(state_, inv);
      apply_gate_to(costate_, inv);
    }
  }
}

// The block-wise sweep through backward_schedule(): one window-tile pass, one
// diagonal-block pass or one gather pair per step.
void Simulator::sweep_fused(const Circuit &c) {
  auto undo_gate = [&](size_t k) {
    const Gate inv = invert(c.ops[k]);
    apply_gate_to(state_, inv);
    apply_gate_to(costate_, inv);
  };
  for (const BackwardStep &st : backward_schedule(c, tile_high_)) {
    switch (st.kind) {
      case BackwardStep::Window: {
        std::vector<uint32_t> wires, slots;
        std::vector<float> mats(8 * st.tile.size());
        std::vector<int> gens;
        for (size_t i = 0; i < st.tile.size(); i++) {
          const WireOp &o = st.tile[i];
          wires.push_back(o.wire);
          narrow(o.minv, &mats[8 * i]);
          gens.push_back(o.gen);
          slots.push_back(o.slot);
        }
        check(qmk_adjoint_group(state_, costate_, n_, static_cast<uint32_t>(st.tile.size()),
                                wires.data(), mats.data(), gens.data(), slots.data(), d_grad_, ws_,
                                ws_bytes_, stream_),
              "adjoint window");
        dispatches_++;
        break;
      }
      case BackwardStep::Diag: {
        const uint32_t ng = static_cast<uint32_t>(st.gens.size());
        check(qmk_adjoint_diagonal(state_, costate_, n_, static_cast<uint32_t>(st.masks.size()),
                                   st.masks.data(), st.angles.data(), st.gphase, ng,
                                   ng ? st.gens.data() : nullptr, ng ? st.slots.data() : nullptr,
                                   d_grad_, st.undo ? 1 : 0, ws_, ws_bytes_, stream_),
              "adjoint diagonal block");
        dispatches_ += 2;
        break;
      }
      case BackwardStep::PermuteUndo:
        if (restore_checkpoint(st.cols, st.off)) {
          // the state from the forward pass's checkpoint; the co-state gathered
          if (!permute(costate_, st.cols, st.off))
            for (size_t k : st.gates) apply_gate_to(costate_, invert(c.ops[k]));
        } else if (permute(state_, st.cols, st.off)) {
          if (!permute(costate_, st.cols, st.off))
            throw std::runtime_error("permutation: scratch buffer lost");
        } else {
          for (size_t k : st.gates) undo_gate(k);
        }
        break;
      case BackwardStep::GateUndo:
        undo_gate(st.gates[0]);
        break;
    }
  }
}

std::pair<double, std::vector<double>> Simulator::energy_and_gradient(const Circuit &c,
                                                                      const Hamiltonian &h,
                                                                      bool fused) {
  prepare_adjoint(c, h);
  const size_t G = c.ops.size();
  std::vector<double> grad(G, 0.0);
  try {
    // Forward: the fused plan (merged passes) reaches the same final state as
    // the gate stream; only the backward sweep needs per-gate identity. The
    // reference's algorithm (fused = false) runs the forward gate by gate, as
    // src/metal/simulator.mm:840-845 does.
    reset();
    drop_checkpoints();
    if (fused) {
      const Plan plan = build_plan(c, FusionOptions{});
      keep_ckpts_ = checkpoints_pair(c, plan);
      run_merged(plan);
      keep_ckpts_ = false;
    } else {
      run(build_plan(c, FusionOptions::none()));
    }
    if (fused) {
      energy_and_costate(h);
      sweep_fused(c);
      drop_checkpoints();
    } else {
      // The reference's co-state: one pass per flip mask, then the energy.
      costate(h);
      check(qmk_dot_re(state_, costate_, n_, d_results_, ws_, ws_bytes_, stream_), "energy");
      dispatches_++;
      sweep_gate_by_gate(c);
    }
    if (G)
      cuda_check(cudaMemcpyAsync(grad.data(), d_grad_, G * sizeof(double), cudaMemcpyDeviceToHost,
                                 S(stream_)),
                 "gradient copy");
    fetch(1, true);
  } catch (...) {
    cudaStreamSynchronize(S(stream_));
    keep_ckpts_ = false;
    drop_checkpoints();
    throw;
  }
  return {h_results_[0], grad};
}

std::vector<double> Simulator::gradient(const Circuit &c, const Hamiltonian &h) {
  return energy_and_gradient(c, h).second;
}

// One serving request: forward once, draw the samples from the final state,
// then energy and the block-wise adjoint gradient; one synchronisation.
void Simulator::serve(const Circuit &c, const Hamiltonian &h, size_t shots, uint64_t seed,
                      double *energy, double *grad, uint64_t *samples) {
  prepare_adjoint(c, h);
  try {
    reset();
    drop_checkpoints();
    const Plan plan = build_plan(c, FusionOptions{});
    keep_ckpts_ = checkpoints_pair(c, plan);
    run_merged(plan);
    keep_ckpts_ = false;
    if (shots) launch_sample(shots, seed);
    energy_and_costate(h);
    sweep_fused(c);
    drop_checkpoints();
    if (!c.ops.empty() && grad)
      cuda_check(cudaMemcpyAsync(grad, d_grad_, c.ops.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost, S(stream_)),
                 "gradient copy");
    if (shots && samples)
      cuda_check(cudaMemcpyAsync(samples, d_shots_, shots * sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, S(stream_)),
                 "sample copy");
    fetch(1, true);
  } catch (...) {
    cudaStreamSynchronize(S(stream_));
    keep_ckpts_ = false;
    drop_checkpoints();
    throw;
  }
  if (energy) *energy = h_results_[0];
}

void Simulator::reserve(size_t max_gates, size_t max_shots) {
  activate();
  if (!costate_) {
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    if (dim() * 8 > free_b) throw std::runtime_error("gradient: co-state does not fit on the device");
    cuda_check(cudaMalloc(&costate_, dim() * 8), "gradient: co-state allocation failed");
  }
  const size_t G = std::max<size_t>(max_gates, 1);
  if (d_grad_cap_ < G) {
    cudaFree(d_grad_);
    d_grad_ = nullptr;
    d_grad_cap_ = 0;
    cuda_check(cudaMalloc(&d_grad_, G * sizeof(double)), "gradient buffer");
    d_grad_cap_ = G;
  }
  if (!sample_ws_) {
    sample_ws_bytes_ = qmk_sample_workspace_bytes(n_);
    cuda_check(cudaMalloc(&sample_ws_, sample_ws_bytes_), "sampling workspace");
  }
  if (max_shots && d_shots_cap_ < max_shots) {
    cudaFree(d_shots_);
    d_shots_ = nullptr;
    d_shots_cap_ = 0;
    cuda_check(cudaMalloc(&d_shots_, max_shots * sizeof(uint64_t)), "sampling output");
    d_shots_cap_ = max_shots;
  }
  ensure_scratch();
}

void Simulator::serve_enqueue(const Circuit &c, const Hamiltonian &h, size_t shots, uint64_t seed,
                              double *pinned_energy, double *pinned_grad,
                              uint64_t *pinned_samples) {
  if (d_grad_cap_ < std::max<size_t>(c.ops.size(), 1) || !costate_ ||
      (shots && (d_shots_cap_ < shots || !sample_ws_)))
    throw std::runtime_error("serve_enqueue: buffers not reserved for this request");
  prepare_adjoint(c, h);
  reset();
  run_merged(build_plan(c, FusionOptions{}));
  if (shots) launch_sample(shots, seed);
  energy_and_costate(h);
  sweep_fused(c);
  if (!c.ops.empty() && pinned_grad)
    cuda_check(cudaMemcpyAsync(pinned_grad, d_grad_, c.ops.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, S(stream_)),
               "gradient copy");
  if (shots && pinned_samples)
    cuda_check(cudaMemcpyAsync(pinned_samples, d_shots_, shots * sizeof(uint64_t),
                               cudaMemcpyDeviceToHost, S(stream_)),
               "sample copy");
  if (pinned_energy)
    cuda_check(cudaMemcpyAsync(pinned_energy, d_results_, sizeof(double), cudaMemcpyDeviceToHost,
                               S(stream_)),
               "energy copy");
}

double Simulator::elapsed() {
  activate();
  cudaEvent_t a = static_cast<cudaEvent_t>(ev_start_), b = static_cast<cudaEvent_t>(ev_stop_);
  cuda_check(cudaEventRecord(b, S(stream_)), "cudaEventRecord");
  cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
  float ms = 0.0f;
  cuda_check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
  cuda_check(cudaEventRecord(a, S(stream_)), "cudaEventRecord");
  return double(ms) * 1e-3;
}

}  // namespace qmetal
