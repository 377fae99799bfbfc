/* qmetal.h -- the stable C ABI of the qmetal statevector simulator, served by
 * a CUDA executor on one NVIDIA GB300.
 *
 * Every declaration down to qm_energy_and_gradient is the reference project's
 * ABI (include/qmetal/qmetal.h:14-113 there) with the same names, types,
 * argument meanings, return conventions and gate numbering, so a caller built
 * against the reference binds to this library unchanged. The declarations
 * after it are appended extensions; nothing above them is renumbered.
 *
 * Conventions (unchanged):
 *   - 0 on success, a negative code on failure; qm_last_error() holds the
 *     calling thread's message. Nothing throws across the boundary.
 *   - LSB-first: qubit q is bit q of the basis index.
 *   - Amplitudes are complex64, interleaved (re, im, re, im, ...).
 */
#ifndef QMETAL_H
#define QMETAL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QMETAL_VERSION_MAJOR 0
#define QMETAL_VERSION_MINOR 1
#define QMETAL_VERSION_PATCH 0

/* Gate codes; ABI, append only (reference qmetal.h:28-36). */
typedef enum {
  QM_X = 0, QM_Y = 1, QM_Z = 2, QM_H = 3,
  QM_S = 4, QM_SDG = 5, QM_T = 6, QM_TDG = 7,
  QM_RX = 8, QM_RY = 9, QM_RZ = 10, QM_P = 11,
  QM_CX = 12, QM_CY = 13, QM_CZ = 14, QM_SWAP = 15,
  QM_CP = 16,
  QM_CCX = 17,
  /* Appended here (the reference stops at QM_CCX): U3(theta, phi, lambda) =
   * [[cos(theta/2), -e^{i lambda} sin(theta/2)],
   *  [e^{i phi} sin(theta/2), e^{i(phi + lambda)} cos(theta/2)]],
   * one qubit and exactly three parameters; not differentiable. */
  QM_U3 = 18
} qm_gate_kind;

typedef struct qm_simulator_s *qm_simulator;
typedef struct qm_circuit_s *qm_circuit;

/* A Hamiltonian as parallel arrays: one coefficient and three Pauli masks per
 * term; borrowed for the duration of a call (reference qmetal.h:41-50). */
typedef struct {
  uint32_t num_terms;
  const double *coeffs;
  const uint64_t *x_masks;
  const uint64_t *y_masks;
  const uint64_t *z_masks;
} qm_hamiltonian;

/* --- diagnostics (reference qmetal.h:54-60; src/capi.cpp:92-124) --------- */
void qm_version(int *major, int *minor, int *patch);
const char *qm_last_error(void);          /* thread-local */
int qm_is_available(void);                /* 1 if a CUDA device is usable */
const char *qm_device_name(void);
uint64_t qm_max_buffer_length(void);      /* largest state buffer, bytes */
uint64_t qm_recommended_working_set(void);/* device memory, bytes */
uint32_t qm_max_qubits(void);             /* 34 on this build */

/* --- circuits (reference qmetal.h:64-73; src/capi.cpp:128-171) ----------- */
qm_circuit qm_circuit_create(uint32_t num_qubits);
void qm_circuit_destroy(qm_circuit c);
int qm_circuit_add(qm_circuit c, qm_gate_kind kind, const uint32_t *qubits,
                   uint32_t num_qubits, const double *params,
                   uint32_t num_params);
size_t qm_circuit_size(qm_circuit c);
/* GPU passes the circuit lowers to: fuse = 0 gives the gate count. */
size_t qm_circuit_plan_size(qm_circuit c, int fuse);

/* --- simulator (reference qmetal.h:77-107; src/capi.cpp:175-274) --------- */
qm_simulator qm_create(uint32_t num_qubits);
void qm_destroy(qm_simulator s);

int qm_reset(qm_simulator s);
int qm_run(qm_simulator s, qm_circuit c);         /* fused, default passes */
int qm_run_unfused(qm_simulator s, qm_circuit c); /* one op per gate */
int qm_synchronize(qm_simulator s);

uint32_t qm_num_qubits(qm_simulator s);
uint64_t qm_dim(qm_simulator s);
uint64_t qm_dispatch_count(qm_simulator s);       /* kernels launched */

/* View of the interleaved state, 2 * qm_dim() floats, valid until the next
 * mutation. Here the state lives in device memory; the returned pointer is a
 * host mirror refreshed by this call. NULL on error. */
const float *qm_amplitudes(qm_simulator s);

int qm_norm(qm_simulator s, double *out);
int qm_expectation_pauli(qm_simulator s, uint64_t x_mask, uint64_t y_mask,
                         uint64_t z_mask, double *out);
int qm_expectation(qm_simulator s, const qm_hamiltonian *h, double *out);

/* `shots` basis indices without collapsing the state; splitmix64 stream, so
 * identical seeds give identical samples. */
int qm_sample(qm_simulator s, size_t shots, uint64_t seed, uint64_t *out);

/* Adjoint gradient: `out_grad` holds qm_circuit_size(c) entries, 0 for gates
 * without a parameter. Fails if a parameterised gate is not RX, RY or RZ. */
int qm_energy_and_gradient(qm_simulator s, qm_circuit c,
                           const qm_hamiltonian *h, double *out_energy,
                           double *out_grad);

/* ======================= appended extensions ============================= */
/* None of these has a counterpart in the reference ABI. */

/* Load / read the whole state (2 * count floats, count == qm_dim(s)). */
int qm_set_state(qm_simulator s, const float *interleaved, uint64_t count);
int qm_get_state(qm_simulator s, float *interleaved, uint64_t count);

/* Apply one gate with no plan in between (the reference's C++
 * Simulator::apply(const Gate&), src/metal/simulator.mm:348-434). */
int qm_apply_gate(qm_simulator s, qm_gate_kind kind, const uint32_t *qubits,
                  uint32_t num_qubits, const double *params,
                  uint32_t num_params);

/* qm_run through a CUDA graph: the first call for a circuit's content
 * (width, gates, wires, parameter values) captures the default plan's
 * launches on the simulator's stream; later calls with the same content
 * replay that graph in one launch. Up to 16 graphs are kept per simulator,
 * least recently used evicted. The reference has no counterpart (it encodes
 * every run's dispatches into a fresh Metal command buffer,
 * src/metal/simulator.mm:189-196 and 436-448). */
int qm_run_cached(qm_simulator s, qm_circuit c);

/* qm_run with the executor's own merging on top of the default plan: a
 * window's one-qubit ops packed into passes of up to ten wires, and runs of
 * CX / SWAP ops applied as one GF(2)-affine permutation pass where that moves
 * fewer bytes (it needs a second state-sized buffer, taken on first use while
 * the device has room; otherwise the ops run one by one). Same unitary as
 * qm_run; the reference has no counterpart. */
int qm_run_merged(qm_simulator s, qm_circuit c);

/* Relabel the state's qubits: afterwards qubit perm[q] holds what qubit q
 * held (perm is a permutation of 0..n-1). One out-of-place pass through the
 * GF(2) permutation kernel; the second state buffer is taken on first use. A
 * circuit relabeled the same way then runs on the relabeled state, so a
 * caller can move frequently used qubits into a cache-blocking window (the
 * reference's untested "qubit reordering", results/S4_RESULT.md). */
int qm_permute_qubits(qm_simulator s, const uint32_t *perm, uint32_t count);

/* Run with explicit fusion options (FusionOptions, reference plan.h:76-94). */
int qm_run_options(qm_simulator s, qm_circuit c, int collapse_1q_windows,
                   int fuse_diagonals, int recognize_zz, uint32_t group_1q,
                   uint32_t block_bits);

/* The plan the options produce, in a flat double layout:
 *   [num_ops] then per op: kind, q0, q1, q2, block_bits, n_group, n_terms,
 *   global_phase, matrix[8], group_qubits[n_group],
 *   group_matrices[8 * n_group], masks[n_terms], angles[n_terms].
 * Writes at most `cap` doubles; returns the full length, or 0 on error. */
size_t qm_circuit_plan_export(qm_circuit c, int collapse_1q_windows,
                              int fuse_diagonals, int recognize_zz,
                              uint32_t group_1q, uint32_t block_bits,
                              double *out, size_t cap);

/* The executor's launch schedules, computed on the host only (no device
 * needed), in a flat double layout:
 *   which = 0: the merged forward pass of the default plan (qm_run_merged);
 *   which = 1: the block-wise backward sweep (qm_energy_and_gradient) with
 *              `tile_high` wires >= 6 per window pass (1..6);
 *   which = 2: the co-state lambda = H psi of `h` for the circuit's width.
 * Forward steps: 0 group (nw, then wire and a row-major 2x2 as re/im pairs per
 * wire), 1 gather (n, cols[n], off, nops, plan op indices), 2 plan op (index).
 * Backward steps: 0 window tile (nops, then wire, inverse 2x2, generator 0-3,
 * gradient slot per op), 1 diagonal block (undo, nt, (mask, angle) x nt,
 * global phase, ng, (Z mask, slot) x ng), 2 gather undo (n, cols[n], off,
 * ngates, gate indices), 3 gate undo (index). Co-state steps: 0 Z strings
 * (nt, (z mask, coeff) x nt), 1 one-wire flips (overwrite, nt, (wire, sign
 * mask, Y count, coeff) x nt), 2 one flip mask (overwrite, flip, nt, (sign
 * mask, Y count, coeff) x nt), 3 zero, 4 energy, 5 transverse field
 * (overwrite, energy 0/1/2, nw, (wire, coeff) x nw). A gather step computes
 * dst[y] = src[off ^ XOR of cols[j] over the set bits j of y].
 * Writes at most `cap` doubles; returns the full length, or 0 on error. */
size_t qm_schedule_export(qm_circuit c, const qm_hamiltonian *h, int which,
                          uint32_t tile_high, double *out, size_t cap);

/* Per-term expectation values <P_t> (without the coefficients), one entry
 * per Hamiltonian term, computed in grouped passes over the state. */
int qm_expectation_terms(qm_simulator s, const qm_hamiltonian *h,
                         double *out_values);

/* Device-side timing of everything queued since the last call, in seconds
 * (CUDA events on the simulator's stream). Synchronizes. */
int qm_elapsed(qm_simulator s, double *out_seconds);

/* Run the circuit's plan (fuse != 0: default fusion; 0: one op per gate) with
 * a CUDA event between consecutive ops, then report each op's device time in
 * seconds (at most `cap` entries) and the op count. Synchronizes. */
int qm_run_profiled(qm_simulator s, qm_circuit c, int fuse, double *out_seconds,
                    size_t cap, size_t *out_count);

/* qm_energy_and_gradient with the backward sweep chosen: mode 0 is the
 * block-wise sweep qm_energy_and_gradient uses (commuting blocks undone in
 * one pass each), mode 1 the reference's gate-by-gate sweep. */
int qm_energy_and_gradient_mode(qm_simulator s, qm_circuit c,
                                const qm_hamiltonian *h, int mode,
                                double *out_energy, double *out_grad);

/* Tile shape of this simulator's block-wise backward sweep: the most wires
 * >= 6 one window pass holds, 1..6 (up to four beside wire 0 and wires 1..5;
 * five or six in passes over wires >= 6 that all carry one rotation
 * sequence, a run of such wires split evenly over its passes). Default 6;
 * the batch autotuner picks it per width. */
int qm_set_tile_high(qm_simulator s, uint32_t tile_high);

/* Fault injection for tests of the fail-closed path: the bounded bulk-copy
 * waits inside this simulator's adjoint window passes give up after `polls`
 * polls (0: at once); a negative value restores the full bound. A gradient
 * whose pass gave up a wait returns -1 with "a bulk-copy wait timed out" in
 * qm_last_error() and leaves the state reset to |0...0>. */
int qm_set_wait_poll_limit(qm_simulator s, int64_t polls);

/* One serving request of a batch: the circuit's width is its qubit count. */
typedef struct {
  qm_circuit circuit;
  const qm_hamiltonian *hamiltonian;
  size_t shots;
  uint64_t seed;
  double *out_energy;      /* 1 value (may be NULL) */
  double *out_grad;        /* qm_circuit_size(circuit) values */
  uint64_t *out_samples;   /* shots values */
} qm_batch_item;

/* Energy, adjoint gradient and samples for `count` requests of any widths.
 * mode 0: concurrent lanes (`lanes` host threads, each with its own stream),
 *         block-wise adjoint, one synchronisation per request;
 * mode 1: one request after another as a per-circuit caller would run them
 *         (gate-by-gate adjoint, then run and sample);
 * mode 2: one request after another with the block-wise adjoint;
 * mode 3: every request recorded into one CUDA graph (branches per width,
 *         heavy widths split up to four ways) and launched once, results staged in
 *         pinned memory by copy nodes; one synchronisation for the batch.
 * Every mode returns the same numbers to within float round-off. In modes 0
 * and 3, lanes = 0 uses the autotuned tile shapes (and in mode 0 lane count),
 * tuning first if this set of widths has not been tuned in this process. */
int qm_batch_serve(const qm_batch_item *items, size_t count, int mode, uint32_t lanes);

/* Where the calling thread's last mode-3 batch spent its time: recording
 * (host work of every request while the graph records), instantiation, and
 * the single launch to completion; and the graph's node count. */
int qm_batch_graph_timing(double *out_record_s, double *out_instantiate_s,
                          double *out_execute_s, uint64_t *out_nodes);

/* Tune a batch on its own requests (their outputs are overwritten): per
 * width, the most wires >= 6 each backward window pass holds (1..6, as
 * qm_set_tile_high; out_tile_high[n], qm_max_qubits() + 1 entries, may be
 * NULL), then the lane count. Cached per set of widths for the process. */
int qm_batch_autotune(const qm_batch_item *items, size_t count, uint32_t *out_lanes,
                      uint32_t *out_tile_high, double *out_seconds);

#ifdef __cplusplus
}
#endif

#endif /* QMETAL_H */
