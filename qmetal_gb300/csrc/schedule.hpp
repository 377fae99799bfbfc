// schedule.hpp -- the executor's scheduling decisions as pure host functions.
//
// The merged forward pass, the co-state accumulation and the block-wise
// backward sweep each turn their input (a plan, a Hamiltonian, a circuit)
// into a list of steps, and the Simulator issues one kernel per step. The
// decisions live here, free of device state, so that a CPU-only build can
// replay every schedule in complex128 against the gate-by-gate algorithm of
// the reference (src/metal/simulator.mm:782-963) without a GPU.
#pragma once

#include <cstdint>
#include <vector>

#include "circuit.hpp"

namespace qmetal {

// x -> A x ^ off over GF(2); cols[j] = A e_j. A gather pass with this map
// computes dst[y] = src[A y ^ off].
struct Affine {
  std::vector<uint64_t> cols;
  uint64_t off = 0;
  explicit Affine(uint32_t n);
  // Compose a CX (control, target) or a SWAP (a, b) after the map.
  void then_cx(uint32_t c, uint32_t t);
  void then_swap(uint32_t a, uint32_t b);
  // Distinct 32-byte sectors a warp's 64 sources touch (16 when contiguous).
  uint32_t sectors() const;
};

// One gate of a permutation run: CX (control, target) or SWAP (a, b).
struct PermGate {
  bool swap;
  uint32_t a, b;
};

// Gather map of a run applied forward (the run maps x -> F(x), so
// dst[y] = src[F^-1(y)]) or undone (dst[y] = src[F(y)]).
Affine run_map(uint32_t n, const std::vector<PermGate> &run, bool undo);

// Does one gather pass move fewer bytes than the run's gates one by one?
bool permutation_pays(const Affine &m, size_t gates);

// --- merged forward --------------------------------------------------------

struct ForwardStep {
  enum Kind : uint8_t { Group, Permute, Op };
  Kind kind = Op;
  std::vector<uint32_t> wires;   // Group: ascending, distinct
  std::vector<cdouble> mats;     // Group: one row-major 2x2 per wire
  std::vector<uint64_t> cols;    // Permute: gather map
  uint64_t off = 0;
  // Op: the one plan op to apply. Permute: the run's plan ops, applied one
  // by one when there is no room for the gather's second buffer.
  std::vector<size_t> ops;
};

// The plan with consecutive one-qubit ops merged into group passes (wire 0,
// up to five of wires 1..5 and four wires >= 6; or wire 0 and five wires
// >= 1; or wire 0 and six or seven wires >= 6) and runs of CX / SWAP ops
// turned into one gather pass where that moves fewer bytes. Every other op
// passes through. Same unitary as the plan.
std::vector<ForwardStep> merged_schedule(const Plan &p);

// --- co-state lambda = H psi and the energy ---------------------------------

struct CostateStep {
  enum Kind : uint8_t {
    ZDiag,   // lambda = sum c_t Z_t psi over Z strings of <= 2 bits; writes the energy
    Local,   // terms that flip one wire each: lambda (+)= sum c_t P_t psi
    Flip,    // terms sharing one flip mask: lambda (+)= sum c_t P_t psi
    Zero,    // lambda = 0 (no terms)
    Dot,     // energy = Re <psi | lambda>
    XField,  // terms c_w X_w, one per wire: lambda (+)= sum c_w X_w psi
  };
  Kind kind = Zero;
  bool overwrite = false;        // Local / Flip / XField: first write of lambda
  uint8_t energy = 0;            // XField: 1 writes, 2 adds sum c_w <psi|X_w|psi> to the energy
  uint64_t flip = 0;             // Flip
  std::vector<uint32_t> wires;   // Local / XField: the wire each term flips
  std::vector<uint64_t> masks;   // ZDiag: Z masks; Local / Flip: sign masks (y | z)
  std::vector<uint32_t> nys;     // Local / Flip: Y count of each term
  std::vector<double> coeffs;
};

// Terms per Flip / Local pass.
constexpr uint32_t kCostateTermsPerPass = 16;
// Wires >= 6 per XField pass (any of wires 0..5 ride along), and the least
// width it serves (a pass holds at least four wires >= 6).
constexpr uint32_t kXFieldHighPerPass = 7;
constexpr uint32_t kXFieldMinQubits = 10;

std::vector<CostateStep> costate_schedule(const Hamiltonian &h, uint32_t n);

// --- block-wise backward sweep -----------------------------------------------

// One one-qubit gate of a window tile, undone with minv = U^-1; gen is 1/2/3
// for an RX/RY/RZ whose gradient goes to slot, 0 for none.
struct WireOp {
  uint32_t wire;
  cdouble minv[4];
  int gen;
  uint32_t slot;
};

struct BackwardStep {
  enum Kind : uint8_t {
    Window,       // tile: each op's gradient, then its undo, in order
    Diag,         // gradients of a diagonal block's Z strings, then undo if asked
    PermuteUndo,  // a run of CX / SWAP undone on both states by one gather each
    GateUndo,     // one gate undone on both states
  };
  Kind kind = GateUndo;
  std::vector<WireOp> tile;      // Window
  // Diag: the block's forward phase (global_phase + the angles of the fully
  // set masks), its generators' Z masks and gradient slots.
  std::vector<uint64_t> masks;
  std::vector<double> angles;
  double gphase = 0.0;
  std::vector<uint64_t> gens;
  std::vector<uint32_t> slots;
  bool undo = false;
  std::vector<uint64_t> cols;    // PermuteUndo: gather map
  uint64_t off = 0;
  // GateUndo: the gate. PermuteUndo: the run's gates in undo order, undone
  // one by one when there is no room for the gather's second buffer.
  std::vector<size_t> gates;
};

// Generators per diagonal-block pass (the kernel's largest slot count).
constexpr uint32_t kDiagGensPerPass = 48;

// Most wires >= 6 one window pass may hold: four in a warp tile, five or
// six in a block tile (wires >= 6 only, one rotation sequence on every wire).
constexpr uint32_t kMaxTileHigh = 6;

// The sweep from the final state back to the first parameterised block.
// tile_high: wires >= 6 one window pass holds (1..6; above four only in block
// tiles).
std::vector<BackwardStep> backward_schedule(const Circuit &c, uint32_t tile_high);

// Inverse gate (src/metal/simulator.mm:786-799) and the generator code of a
// natively differentiable rotation (1 X, 2 Y, 3 Z; 0 for anything else).
Gate invert(const Gate &g);
int generator_of(const Gate &g);

// Flat double encodings of the three schedules, for tests and tools:
//   forward:  [steps] then per step
//     0 (Group)   nw, (wire, m00.re, m00.im, m01.re, m01.im, m10.., m11..) x nw
//     1 (Permute) n, cols[n], off, nops, ops[nops]
//     2 (Op)      op
//   co-state: [steps] then per step
//     0 (ZDiag)   nt, (zmask, coeff) x nt
//     1 (Local)   overwrite, nt, (wire, sign, ny, coeff) x nt
//     2 (Flip)    overwrite, flip, nt, (sign, ny, coeff) x nt
//     3 (Zero)    4 (Dot)
//   backward: [steps] then per step
//     0 (Window)  nops, (wire, minv[8], gen, slot) x nops
//     1 (Diag)    undo, nt, (mask, angle) x nt, gphase, ng, (gen, slot) x ng
//     2 (PermuteUndo) n, cols[n], off, ngates, gates[ngates]
//     3 (GateUndo) gate
void serialise_schedule(const std::vector<ForwardStep> &s, uint32_t n, std::vector<double> &out);
void serialise_schedule(const std::vector<CostateStep> &s, std::vector<double> &out);
void serialise_schedule(const std::vector<BackwardStep> &s, uint32_t n, std::vector<double> &out);

}  // namespace qmetal
