// simulator.hpp -- the statevector executor on one CUDA device.
//
// Same surface as the reference's C++ Simulator (include/qmetal/simulator.h:
// 30-112) so the C ABI maps onto it one to one; the implementation owns a
// device state buffer, a stream, a scratch workspace, and launches the
// sm_103a kernels declared in include/qmetal/qmetal_kernels.h.
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "circuit.hpp"

namespace qmetal {

// 34 qubits = 128 GiB of complex64, in place, fits one GB300's HBM.
constexpr uint32_t kMaxQubits = 34;

class Simulator {
 public:
  explicit Simulator(uint32_t num_qubits);
  ~Simulator();
  Simulator(const Simulator &) = delete;
  Simulator &operator=(const Simulator &) = delete;

  void reset();
  void apply(const Gate &g);
  void run(const Circuit &c);
  void run(const Circuit &c, const FusionOptions &opts);
  void run(const Plan &p);
  void apply(const PlanOp &op);
  // run(c) through a CUDA graph: the first call for a given circuit content
  // captures the plan's launches on this simulator's stream, later calls
  // replay the graph with one launch. Same kernels, same results.
  void run_cached(const Circuit &c);
  // The plan with each window's consecutive one-qubit ops merged into as few
  // group passes as the tile allows, and runs of CX / SWAP ops applied as one
  // permutation pass where that moves fewer bytes (same unitary, fewer passes).
  void run_merged(const Plan &p);
  void run_merged(const Circuit &c);
  // Relabel the qubits of the state: afterwards wire perm[q] holds what wire
  // q held (one out-of-place permutation pass).
  void permute_qubits(const std::vector<uint32_t> &perm);
  // Runs the plan with a CUDA event between ops; seconds[i] = op i's device time.
  void run_profiled(const Plan &p, std::vector<double> &seconds);
  void synchronize();

  uint32_t num_qubits() const { return n_; }
  size_t dim() const { return size_t(1) << n_; }

  // Amplitudes widened to complex128 (a host copy of the state).
  std::vector<cdouble> amplitudes();
  const float *raw();                   // host mirror, refreshed
  void get_state(float *out);           // 2 * dim floats
  void set_state(const float *in);      // 2 * dim floats

  double abs2sum();
  double norm();
  double expectation(const PauliString &p);
  double expectation(const Hamiltonian &h);
  void expectation_terms(const Hamiltonian &h, double *out);

  std::vector<uint64_t> sample(size_t shots, uint64_t seed = 0);
  // Bitstring counts, most frequent first; qubit 0 is the rightmost character.
  std::vector<std::pair<std::string, uint64_t>> counts(size_t shots, uint64_t seed = 0);

  // Adjoint energy and per-gate gradient. fused = true runs the block-wise
  // backward sweep (commuting blocks undone in one pass each); false runs the
  // reference's gate-by-gate sweep.
  std::pair<double, std::vector<double>> energy_and_gradient(const Circuit &c,
                                                             const Hamiltonian &h,
                                                             bool fused = true);
  std::vector<double> gradient(const Circuit &c, const Hamiltonian &h);

  // Forward, samples from the final state, energy and block-wise gradient in
  // one queued sequence with a single synchronisation.
  void serve(const Circuit &c, const Hamiltonian &h, size_t shots, uint64_t seed, double *energy,
             double *grad, uint64_t *samples);
  // The same sequence queued only, with its results copied into pinned host
  // memory by the stream (energy: one double, grad: one per gate, samples:
  // shots). After reserve() it allocates and synchronises nothing, so it can
  // be recorded into a CUDA graph.
  void serve_enqueue(const Circuit &c, const Hamiltonian &h, size_t shots, uint64_t seed,
                     double *pinned_energy, double *pinned_grad, uint64_t *pinned_samples);
  // Device buffers for requests of up to max_gates gates and max_shots shots.
  void reserve(size_t max_gates, size_t max_shots);
  void *stream() const { return stream_; }

  // Tile shape of the block-wise sweep's window passes: how many wires >= 6
  // one two-state pass holds (1..6: up to four in warp tiles, besides wire 0
  // and the five lane wires; five or six in block tiles of uniform rotation
  // layers; default 6). Chosen per width by the batch autotuner.
  void set_tile_high(uint32_t k) { tile_high_ = k < 1 ? 1 : (k > 6 ? 6 : k); }
  uint32_t tile_high() const { return tile_high_; }

  uint64_t dispatch_count() const { return dispatches_; }
  double elapsed();

  // Throws if a window pass on this simulator gave up a bounded wait since
  // the last check (a copy and a synchronisation on its stream). A pass
  // that gave up leaves both states invalid, so the state is then reset to
  // |0...0> before the throw, as a successful gradient's sweep also ends.
  void check_waits();
  // Fault injection for tests: the window passes' bounded bulk-copy waits
  // give up after `polls` polls (0: at once); negative restores the bound.
  void set_wait_poll_limit(long long polls);

  static bool available();
  static std::string device_name();
  static uint64_t max_buffer_length();
  static uint64_t recommended_working_set();

 private:
  void release();
  void check(int rc, const char *what);
  void activate() const;
  void apply_gate_to(float *state, const Gate &g);
  void apply_op_to(float *state, const PlanOp &op);
  void pauli_values(const float *state, const Hamiltonian &h, std::vector<double> &vals);
  void costate(const Hamiltonian &h);
  void prepare_adjoint(const Circuit &c, const Hamiltonian &h);
  double energy_and_costate(const Hamiltonian &h);
  void sweep_gate_by_gate(const Circuit &c);
  void sweep_fused(const Circuit &c);
  // d_results_ -> h_results_, sync; with `waits`, also read the workspace's
  // wait counter in the same copy batch and throw if a window pass gave up a
  // bounded wait since the last look.
  void fetch(size_t count, bool waits = false);
  void launch_sample(size_t shots, uint64_t seed);
  // Out-of-place permutation passes need a second state-sized buffer; it is
  // allocated on first use, and only while the device has room for it.
  bool ensure_scratch();
  // buf <- buf gathered through the affine map (cols, off); buf then names
  // the gathered buffer and the old one becomes the scratch.
  bool permute(float *&buf, const std::vector<uint64_t> &cols, uint64_t off);
  // State checkpoints at permutation passes. A gradient's forward pass keeps
  // the state from before each CX / SWAP run it gathers (the gather is out
  // of place, so that state is already in a buffer of its own) while spare
  // buffers fit on the device; the backward sweep then restores the state
  // from the checkpoint instead of gathering it back, and gathers only the
  // co-state. Buffers stay with the simulator for its next gradient.
  // Checkpoints are kept only when the forward schedule's gathers and the
  // backward schedule's undo gathers pair up one to one in reverse order
  // (checkpoints_pair); a gather that finds no spare buffer leaves an empty
  // checkpoint so the positions stay paired.
  struct Checkpoint {
    float *buf;                  // the state before the forward gather (null: none kept)
    std::vector<uint64_t> cols;  // that gather's map
    uint64_t off;
  };
  float *take_buffer();
  void drop_checkpoints();
  bool checkpoints_pair(const Circuit &c, const Plan &p) const;
  bool restore_checkpoint(const std::vector<uint64_t> &cols, uint64_t off);
  void invalidate_graphs();

  uint32_t n_ = 0;
  int device_ = 0;
  void *stream_ = nullptr;
  float *state_ = nullptr;
  float *costate_ = nullptr;
  float *scratch_ = nullptr;
  bool scratch_failed_ = false;
  void *ws_ = nullptr;
  size_t ws_bytes_ = 0;
  void *sample_ws_ = nullptr;
  size_t sample_ws_bytes_ = 0;
  uint64_t *d_shots_ = nullptr;
  size_t d_shots_cap_ = 0;
  double *d_results_ = nullptr;         // kResultSlots doubles
  double *h_results_ = nullptr;         // pinned mirror, then one wait-count slot
  unsigned *h_waits_ = nullptr;         // inside h_results_'s last slot
  unsigned waits_seen_ = 0;             // wait count at the last look
  double *d_grad_ = nullptr;            // adjoint gradient slots
  size_t d_grad_cap_ = 0;
  float *mirror_ = nullptr;
  bool mirror_pinned_ = false;
  void *ev_start_ = nullptr, *ev_stop_ = nullptr;
  uint64_t dispatches_ = 0;
  uint32_t tile_high_ = 6;
  struct GraphEntry {
    uint64_t key;
    void *exec;         // cudaGraphExec_t
    uint64_t launches;  // kernels in the graph
  };
  std::vector<GraphEntry> graphs_;   // most recent last
  bool fault_launch_ = false;
  std::vector<Checkpoint> ckpts_;   // last on top
  std::vector<float *> ck_free_;    // state-sized buffers not in use
  bool keep_ckpts_ = false;         // run_merged keeps checkpoints (gradient forward passes)
  size_t ck_limit_ = 16;            // most checkpoint buffers (QMETAL_MAX_CHECKPOINTS)
};

}  // namespace qmetal
