// schedule.cpp -- merged forward, co-state and backward-sweep schedules.
#include "schedule.hpp"

#include <algorithm>
#include <cstdint>
#include <map>
#include <stdexcept>

namespace qmetal {
namespace {

uint32_t popc(uint64_t x) { return static_cast<uint32_t>(__builtin_popcountll(x)); }

constexpr uint32_t kWindowOps = 16;     // ops per window pass below 6 qubits
constexpr uint32_t kWideWindowOps = 32;  // ops per warp-tile window pass
constexpr uint32_t kWindowGrads = 16;   // gradients per window pass
// ... and in the compile-time tile of wire 0, wires 1..5 and four wires >= 6
// that all carry RZ then RY (undo order): the first tile of a
// hardware-efficient layer.
constexpr uint32_t kWideUniformGrads = 20;
constexpr uint32_t kSigRzRy = 6;          // uniform_signature of RZ then RY

// The structure the kernel layer finds in a 2x2 once narrowed to float (the
// kMat* classes of kcommon.cuh): 3 diagonal, 1 real, 2 RX-like, 0 general.
int narrowed_class(const cdouble m[4]) {
  float f[8];
  for (int k = 0; k < 4; k++) {
    f[2 * k] = static_cast<float>(m[k].real());
    f[2 * k + 1] = static_cast<float>(m[k].imag());
  }
  if (f[2] == 0.0f && f[3] == 0.0f && f[4] == 0.0f && f[5] == 0.0f) return 3;
  if (f[1] == 0.0f && f[3] == 0.0f && f[5] == 0.0f && f[7] == 0.0f) return 1;
  if (f[1] == 0.0f && f[7] == 0.0f && f[2] == 0.0f && f[4] == 0.0f) return 2;
  return 0;
}

}  // namespace

Affine::Affine(uint32_t n) : cols(n) {
  for (uint32_t j = 0; j < n; j++) cols[j] = 1ull << j;
}

void Affine::then_cx(uint32_t c, uint32_t t) {
  auto f = [&](uint64_t v) { return v ^ (((v >> c) & 1ull) << t); };
  for (uint64_t &v : cols) v = f(v);
  off = f(off);
}

void Affine::then_swap(uint32_t a, uint32_t b) {
  auto f = [&](uint64_t v) {
    const uint64_t d = ((v >> a) ^ (v >> b)) & 1ull;
    return v ^ (d << a) ^ (d << b);
  };
  for (uint64_t &v : cols) v = f(v);
  off = f(off);
}

uint32_t Affine::sectors() const {
  std::vector<uint64_t> s;
  for (uint64_t y = 0; y < 64 && y < (1ull << cols.size()); y++) {
    uint64_t x = off;
    for (uint32_t j = 0; j < cols.size() && j < 6; j++)
      if ((y >> j) & 1) x ^= cols[j];
    s.push_back(x >> 2);
  }
  std::sort(s.begin(), s.end());
  return static_cast<uint32_t>(std::unique(s.begin(), s.end()) - s.begin());
}

// Every gate of a run is an involution, so undoing the run composes its gates
// first to last, and applying it composes them last to first.
Affine run_map(uint32_t n, const std::vector<PermGate> &run, bool undo) {
  Affine m(n);
  auto step = [&](const PermGate &g) {
    if (g.swap) m.then_swap(g.a, g.b);
    else m.then_cx(g.a, g.b);
  };
  if (undo) {
    for (const PermGate &g : run) step(g);
  } else {
    for (size_t k = run.size(); k-- > 0;) step(run[k]);
  }
  return m;
}

// A gather pass moves 2S, more when the warp's sources scatter; the run's
// gates move S each (half the state read and written per CX, all of it
// crossing for a SWAP, counted as S by the roofline model).
bool permutation_pays(const Affine &m, size_t gates) {
  const double pass = 2.0 * std::max(1.0, m.sectors() / 16.0);
  return pass * 1.25 < static_cast<double>(gates);
}

Gate invert(const Gate &g) {
  Gate inv = g;
  switch (g.kind) {
    case G_RX: case G_RY: case G_RZ: case G_P: case G_CP:
      inv.params[0] = -g.params[0];
      break;
    case G_S: inv.kind = G_SDG; break;
    case G_SDG: inv.kind = G_S; break;
    case G_T: inv.kind = G_TDG; break;
    case G_TDG: inv.kind = G_T; break;
    case G_U3:   // U3(t, f, l)^-1 = U3(-t, -l, -f)
      inv.params[0] = -g.params[0];
      inv.params[1] = -g.params[2];
      inv.params[2] = -g.params[1];
      break;
    default: break;
  }
  return inv;
}

int generator_of(const Gate &g) {
  switch (g.kind) {
    case G_RX: return 1;
    case G_RY: return 2;
    case G_RZ: return 3;
    default: return 0;
  }
}

// ---------------------------------------------------------------------------

std::vector<ForwardStep> merged_schedule(const Plan &p) {
  const uint32_t n = p.num_qubits;
  std::vector<ForwardStep> out;
  std::vector<uint32_t> wires;
  std::vector<cdouble> mats;
  auto fits = [&](const std::vector<uint32_t> &w) {
    uint32_t lane = 0, high = 0, zero = 0;
    for (uint32_t q : w) {
      if (q == 0) zero++;
      else if (q <= 5) lane++;
      else high++;
    }
    if (zero > 1) return false;
    if (lane >= 1 && lane <= 5 && high <= 4 && n >= 6 + high) return true;
    if (lane == 0 && high >= 6 && high <= 7 && n >= 6 + high) return true;   // block groups
    return lane + high <= 5;
  };
  // One pass for the given entries of the pending run, wires ascending.
  auto emit = [&](std::vector<size_t> idx) {
    if (idx.empty()) return;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return wires[a] < wires[b]; });
    ForwardStep s;
    s.kind = ForwardStep::Group;
    for (size_t i : idx) {
      s.wires.push_back(wires[i]);
      s.mats.insert(s.mats.end(), mats.begin() + 4 * i, mats.begin() + 4 * i + 4);
    }
    out.push_back(std::move(s));
  };
  // A run of one-wire ops on distinct wires (they all commute) in the fewest
  // passes: wires 0..5 take k wires >= 6 along, the rest go up to seven a
  // pass in order. Where a lane wire's matrix is general, the pass of the
  // lane wires is bound by its multiply-adds: of the k that give the fewest
  // passes the least is kept, but at least one where there is one (a pass of
  // the lane wires alone has too little work per thread to hide its loads),
  // so an HEA layer at 28 qubits goes as 6 + 1, 7, 7, 7 wires instead of
  // 6 + 4, 7, 7, 4. Otherwise the greatest is kept.
  auto flush = [&]() {
    if (wires.empty()) return;
    std::vector<size_t> low, high;
    for (size_t i = 0; i < wires.size(); i++) (wires[i] < 6 ? low : high).push_back(i);
    auto wires_of = [&](const std::vector<size_t> &idx) {
      std::vector<uint32_t> w;
      for (size_t i : idx) w.push_back(wires[i]);
      return w;
    };
    // Wires >= 6 in passes of their own, greedily in order.
    auto chunks = [&](size_t from) {
      std::vector<std::vector<size_t>> c;
      for (size_t j = from; j < high.size(); j++) {
        if (c.empty()) {
          c.push_back({high[j]});
          continue;
        }
        std::vector<uint32_t> trial = wires_of(c.back());
        trial.push_back(wires[high[j]]);
        if (fits(trial)) c.back().push_back(high[j]);
        else c.push_back({high[j]});
      }
      return c;
    };
    // Narrow matrices (real, RX-like, diagonal) halve the lane pass's
    // multiply-adds: it then keeps as many wires >= 6 as fit.
    bool general = false;
    for (size_t i : low) general = general || narrowed_class(&mats[4 * i]) == 0;
    size_t best_k = 0, best = SIZE_MAX;
    for (size_t k = low.empty() ? 0 : std::min<size_t>(1, high.size()); k <= high.size(); k++) {
      std::vector<size_t> first = low;
      first.insert(first.end(), high.begin(), high.begin() + k);
      if (!first.empty() && !fits(wires_of(first))) break;
      const size_t passes = (first.empty() ? 0 : 1) + chunks(k).size();
      if (passes < best || (!general && passes == best)) {
        best = passes;
        best_k = k;
      }
    }
    std::vector<size_t> first = low;
    first.insert(first.end(), high.begin(), high.begin() + best_k);
    emit(first);
    for (const auto &c : chunks(best_k)) emit(c);
    wires.clear();
    mats.clear();
  };
  std::vector<PermGate> run;
  std::vector<size_t> run_ops;
  auto flush_run = [&]() {
    if (run.empty()) return;
    const Affine map = run.size() >= 2 ? run_map(n, run, false) : Affine(0);
    if (run.size() >= 2 && permutation_pays(map, run.size())) {
      ForwardStep s;
      s.kind = ForwardStep::Permute;
      s.cols = map.cols;
      s.off = map.off;
      s.ops = run_ops;
      out.push_back(std::move(s));
    } else {
      for (size_t i : run_ops) {
        ForwardStep s;
        s.ops = {i};
        out.push_back(std::move(s));
      }
    }
    run.clear();
    run_ops.clear();
  };
  for (size_t i = 0; i < p.ops.size(); i++) {
    const PlanOp &op = p.ops[i];
    const bool cx = op.kind == PlanOp::Kind::Controlled1q && op.matrix[0] == 0.0 &&
                    op.matrix[1] == 1.0 && op.matrix[2] == 1.0 && op.matrix[3] == 0.0;
    if ((cx || op.kind == PlanOp::Kind::Swap) && op.qubits[0] < n && op.qubits[1] < n &&
        op.qubits[0] != op.qubits[1]) {
      flush();
      run.push_back({op.kind == PlanOp::Kind::Swap, op.qubits[0], op.qubits[1]});
      run_ops.push_back(i);
      continue;
    }
    flush_run();
    std::vector<uint32_t> w;
    std::vector<cdouble> m;
    if (op.kind == PlanOp::Kind::Dense1q) {
      w.push_back(op.qubits[0]);
      m.assign(op.matrix, op.matrix + 4);
    } else if (op.kind == PlanOp::Kind::Dense1qGroup) {
      w = op.group_qubits;
      m = op.group_matrices;
    } else {
      flush();
      ForwardStep s;
      s.ops = {i};
      out.push_back(std::move(s));
      continue;
    }
    for (uint32_t q : w)
      if (q >= n) throw std::runtime_error("qubit index out of range");
    bool overlap = false;
    for (uint32_t q : w)
      if (std::find(wires.begin(), wires.end(), q) != wires.end()) overlap = true;
    if (overlap) flush();
    // The group's wires commute with each other and with the pending ones:
    // they join the pending run, which is split into passes when it ends.
    for (size_t j = 0; j < w.size(); j++) {
      wires.push_back(w[j]);
      mats.insert(mats.end(), m.begin() + 4 * j, m.begin() + 4 * j + 4);
    }
  }
  flush();
  flush_run();
  return out;
}

// ---------------------------------------------------------------------------

namespace {

struct FlipGroup {
  uint64_t flip;
  std::vector<size_t> terms;
};

std::vector<FlipGroup> group_by_flip(const std::vector<const PauliTerm *> &terms) {
  std::vector<FlipGroup> out;
  std::map<uint64_t, size_t> where;
  for (size_t t = 0; t < terms.size(); t++) {
    const PauliString &p = terms[t]->pauli;
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

// Z strings of <= 2 bits go as one quadratic-form pass; plain X_w terms
// (a transverse field) go as block passes of up to seven wires >= 6 with any
// of wires 0..5, the terms on one wire summed; other terms that flip one wire
// pack many wires per pass (wires 0..5 ride along in every pass, at most
// four wires >= 6 and 16 terms a pass); anything else goes one pass per flip
// mask, 16 terms at a time. When every term is of the first two kinds their
// passes also sum the energy, and no separate energy pass follows.
std::vector<CostateStep> costate_schedule(const Hamiltonian &h, uint32_t n) {
  std::vector<CostateStep> out;
  std::vector<const PauliTerm *> zpart, xfield, local, rest;
  for (const PauliTerm &t : h.terms) {
    const uint64_t flip = t.pauli.x_mask | t.pauli.y_mask;
    if (!flip && popc(t.pauli.z_mask) <= 2) zpart.push_back(&t);
    else if (popc(flip) == 1 && !t.pauli.y_mask && !t.pauli.z_mask && n >= kXFieldMinQubits)
      xfield.push_back(&t);
    else if (popc(flip) == 1 && n >= 6) local.push_back(&t);
    else rest.push_back(&t);
  }
  const bool fused_energy = local.empty() && rest.empty() && !h.terms.empty();
  bool first = true;
  if (!zpart.empty()) {
    CostateStep s;
    s.kind = CostateStep::ZDiag;
    s.overwrite = true;
    for (const PauliTerm *t : zpart) {
      s.masks.push_back(t->pauli.z_mask);
      s.coeffs.push_back(t->coefficient);
    }
    out.push_back(std::move(s));
    first = false;
  }
  if (!xfield.empty()) {
    std::map<uint32_t, double> coef;   // wire -> summed coefficient, ascending
    for (const PauliTerm *t : xfield)
      coef[static_cast<uint32_t>(__builtin_ctzll(t->pauli.x_mask))] += t->coefficient;
    std::vector<uint32_t> low, high;
    for (const auto &wc : coef) (wc.first < 6 ? low : high).push_back(wc.first);
    // ceil(H / 7) passes, as even as possible (22 wires: 6, 6, 5, 5); wires
    // 0..5 join the last, which is among the smallest.
    const size_t passes = std::max<size_t>(
        1, (high.size() + kXFieldHighPerPass - 1) / kXFieldHighPerPass);
    size_t at = 0;
    for (size_t p = 0; p < passes; p++) {
      const size_t take = high.size() / passes + (p < high.size() % passes ? 1 : 0);
      CostateStep s;
      s.kind = CostateStep::XField;
      s.overwrite = first;
      if (fused_energy) s.energy = first ? 1 : 2;
      first = false;
      if (p + 1 == passes)
        for (uint32_t w : low) {
          s.wires.push_back(w);
          s.coeffs.push_back(coef[w]);
        }
      for (size_t j = 0; j < take; j++, at++) {
        s.wires.push_back(high[at]);
        s.coeffs.push_back(coef[high[at]]);
      }
      out.push_back(std::move(s));
    }
  }
  if (fused_energy) return out;
  if (!local.empty()) {
    auto wire_of = [&](const PauliTerm *t) {
      return static_cast<uint32_t>(__builtin_ctzll(t->pauli.x_mask | t->pauli.y_mask));
    };
    std::stable_sort(local.begin(), local.end(),
                     [&](const PauliTerm *a, const PauliTerm *b) { return wire_of(a) < wire_of(b); });
    const uint32_t max_high = std::min<uint32_t>(4, n - 6);
    CostateStep s;
    std::vector<uint32_t> highs;
    auto flush = [&]() {
      if (s.wires.empty()) return;
      s.kind = CostateStep::Local;
      s.overwrite = first;
      first = false;
      out.push_back(std::move(s));
      s = CostateStep{};
      highs.clear();
    };
    for (const PauliTerm *t : local) {
      const uint32_t w = wire_of(t);
      const bool new_high = w >= 6 && std::find(highs.begin(), highs.end(), w) == highs.end();
      if (s.wires.size() == kCostateTermsPerPass || (new_high && highs.size() == max_high)) flush();
      if (w >= 6 && std::find(highs.begin(), highs.end(), w) == highs.end()) highs.push_back(w);
      s.wires.push_back(w);
      s.masks.push_back(t->pauli.y_mask | t->pauli.z_mask);
      s.nys.push_back(popc(t->pauli.y_mask));
      s.coeffs.push_back(t->coefficient);
    }
    flush();
  }
  for (const FlipGroup &g : group_by_flip(rest)) {
    for (size_t b = 0; b < g.terms.size(); b += kCostateTermsPerPass) {
      const size_t take = std::min<size_t>(kCostateTermsPerPass, g.terms.size() - b);
      CostateStep s;
      s.kind = CostateStep::Flip;
      s.overwrite = first;
      s.flip = g.flip;
      for (size_t j = 0; j < take; j++) {
        const PauliTerm &t = *rest[g.terms[b + j]];
        s.masks.push_back(t.pauli.y_mask | t.pauli.z_mask);
        s.nys.push_back(popc(t.pauli.y_mask));
        s.coeffs.push_back(t.coefficient);
      }
      out.push_back(std::move(s));
      first = false;
    }
  }
  if (first) out.push_back(CostateStep{});
  CostateStep dot;
  dot.kind = CostateStep::Dot;
  out.push_back(std::move(dot));
  return out;
}

// ---------------------------------------------------------------------------

namespace {

// A run of the circuit that the sweep undoes as a unit.
struct Segment {
  enum Kind { Window, Diag, Single } kind = Single;
  size_t begin = 0, end = 0;
  bool has_param = false;
  // Diag: the block's forward phase terms and its Z-string generators.
  std::vector<uint64_t> masks;
  std::vector<double> angles;
  double gphase = 0.0;
  std::vector<uint64_t> gens;
  std::vector<uint32_t> slots;
};

// Forward segmentation: a maximal run of one-qubit gates is a window; a run
// of ZZ couplings (CX.RZ.CX) and two-qubit diagonal gates is a diagonal block;
// anything else stands alone.
std::vector<Segment> segment_circuit(const Circuit &c) {
  std::vector<Segment> segs;
  const size_t G = c.ops.size();
  size_t i = 0;
  while (i < G) {
    const Gate &g = c.ops[i];
    Segment s;
    s.begin = i;
    uint32_t a, b;
    double t;
    if (g.num_qubits == 1) {
      s.kind = Segment::Window;
      size_t j = i;
      for (; j < G && c.ops[j].num_qubits == 1; j++)
        if (c.ops[j].num_params) s.has_param = true;
      s.end = j;
    } else if (zz_coupling_at(c, i, &a, &b, &t) || (g.num_qubits == 2 && is_diagonal(g))) {
      s.kind = Segment::Diag;
      size_t j = i;
      while (j < G) {
        if (zz_coupling_at(c, j, &a, &b, &t)) {
          const uint64_t ma = 1ull << a, mb = 1ull << b;
          s.masks.insert(s.masks.end(), {ma, mb, ma | mb});
          s.angles.insert(s.angles.end(), {t, t, -2.0 * t});
          s.gphase += -t / 2.0;
          if (c.ops[j + 1].num_params) {
            s.gens.push_back(ma | mb);   // exp(-i t/2 Z_a Z_b)
            s.slots.push_back(static_cast<uint32_t>(j + 1));
            s.has_param = true;
          }
          j += 3;
        } else if (c.ops[j].num_qubits == 2 && is_diagonal(c.ops[j])) {
          s.gphase += diagonal_term(c.ops[j], s.masks, s.angles);
          if (c.ops[j].num_params) s.has_param = true;
          j++;
        } else {
          break;
        }
      }
      s.end = j;
    } else {
      s.kind = Segment::Single;
      s.end = i + 1;
      s.has_param = g.num_params > 0;
    }
    i = s.end;
    segs.push_back(std::move(s));
  }
  return segs;
}

}  // namespace

// Every gradient of a commuting block is read at the block boundary and the
// block is undone on both states in the same pass. Blocks before the first
// parameterised one are never undone.
namespace {

// A wire's ops (in undo order) as one of the rotation sequences the block
// tiles compile in: one RX, RY or RZ, or RZ then RY, or RY then RZ. Returns
// a nonzero code for each such sequence, 0 for any other.
uint32_t uniform_signature(const std::vector<WireOp> &ops) {
  if (ops.empty() || ops.size() > 2) return 0;
  int kind[2];
  for (size_t k = 0; k < ops.size(); k++) {
    const int cls = narrowed_class(ops[k].minv), gen = ops[k].gen;
    if (cls == 2 && gen == 1) kind[k] = 0;        // RX
    else if (cls == 1 && gen == 2) kind[k] = 1;   // RY
    else if (cls == 3 && gen == 3) kind[k] = 2;   // RZ
    else return 0;
  }
  if (ops.size() == 1) return 1 + kind[0];
  if ((kind[0] == 2 && kind[1] == 1) || (kind[0] == 1 && kind[1] == 2))
    return 4 + kind[0];
  return 0;
}

}  // namespace

std::vector<BackwardStep> backward_schedule(const Circuit &c, uint32_t tile_high) {
  const uint32_t n = c.num_qubits;
  tile_high = std::min<uint32_t>(std::max<uint32_t>(tile_high, 1), kMaxTileHigh);
  std::vector<BackwardStep> out;
  const auto segs = segment_circuit(c);
  size_t first = segs.size();
  for (size_t s = 0; s < segs.size(); s++)
    if (segs[s].has_param) {
      first = s;
      break;
    }
  for (size_t s = segs.size(); s-- > first;) {
    const Segment &seg = segs[s];
    const bool undo = s > first;
    if (seg.kind == Segment::Single) {
      // A run of CX / SWAP gates, all undone here, goes as one gather pass
      // per state when that moves fewer bytes.
      auto perm_gate = [&](size_t k) {
        const Gate &g = c.ops[segs[k].begin];
        return segs[k].kind == Segment::Single && (g.kind == G_CX || g.kind == G_SWAP) &&
               g.qubits[0] < n && g.qubits[1] < n && g.qubits[0] != g.qubits[1];
      };
      if (undo && perm_gate(s)) {
        size_t lo = s;
        while (lo - 1 > first && perm_gate(lo - 1)) lo--;
        if (s > lo) {
          std::vector<PermGate> run;
          for (size_t k = lo; k <= s; k++) {
            const Gate &g = c.ops[segs[k].begin];
            run.push_back({g.kind == G_SWAP, g.qubits[0], g.qubits[1]});
          }
          const Affine map = run_map(n, run, true);
          if (permutation_pays(map, run.size())) {
            BackwardStep st;
            st.kind = BackwardStep::PermuteUndo;
            st.cols = map.cols;
            st.off = map.off;
            for (size_t k = s + 1; k-- > lo;) st.gates.push_back(segs[k].begin);
            out.push_back(std::move(st));
            s = lo;
            continue;
          }
        }
      }
      if (undo) {
        BackwardStep st;
        st.gates = {seg.begin};
        out.push_back(std::move(st));
      }
      continue;
    }
    if (seg.kind == Segment::Diag) {
      const uint32_t ng = static_cast<uint32_t>(seg.gens.size());
      if (ng == 0 && !undo) continue;
      uint32_t done = 0;
      do {
        const uint32_t take = std::min(kDiagGensPerPass, ng - done);
        BackwardStep st;
        st.kind = BackwardStep::Diag;
        st.masks = seg.masks;
        st.angles = seg.angles;
        st.gphase = seg.gphase;
        st.gens.assign(seg.gens.begin() + done, seg.gens.begin() + done + take);
        st.slots.assign(seg.slots.begin() + done, seg.slots.begin() + done + take);
        st.undo = done + take == ng && undo;
        out.push_back(std::move(st));
        done += take;
      } while (done < ng);
      continue;
    }
    // Window: each wire's gates last to first, a few wires per pass. Gates
    // on different wires commute, and a generator on one wire commutes with
    // every gate on the others, so the order across wires is free.
    std::vector<std::vector<size_t>> per_wire(n);
    for (size_t k = seg.begin; k < seg.end; k++) per_wire[c.ops[k].qubits[0]].push_back(k);
    std::vector<WireOp> tile;
    uint32_t others = 0, highs = 0, grads = 0;
    bool tile_has_param = false;
    bool tile_low = false;     // the tile holds a wire below 6
    uint32_t tile_sig = 0;     // the rotation sequence all its wires share (0: none)
    const bool wide = n >= 6;
    const uint32_t max_ops = wide ? kWideWindowOps : kWindowOps;
    // Up to four wires >= 6 per pass in a warp tile; five or six in a block
    // tile, which holds only wires >= 6 that all carry one rotation sequence.
    const uint32_t max_high = wide ? std::min<uint32_t>(std::min<uint32_t>(tile_high, 4), n - 6) : 0;
    const uint32_t max_high_blk = wide ? std::min<uint32_t>(tile_high, n - 6) : 0;
    auto flush = [&]() {
      if (tile.empty()) return;
      if (undo || tile_has_param) {
        BackwardStep st;
        st.kind = BackwardStep::Window;
        st.tile = tile;
        out.push_back(std::move(st));
      }
      tile.clear();
      others = highs = grads = 0;
      tile_has_param = false;
      tile_low = false;
      tile_sig = 0;
    };
    // Each wire's ops in undo order, and the rotation sequence they form.
    std::vector<std::vector<WireOp>> wire_ops(n);
    std::vector<uint32_t> wire_sig(n, 0);
    for (uint32_t w = 0; w < n; w++) {
      for (size_t r = per_wire[w].size(); r-- > 0;) {
        const size_t k = per_wire[w][r];
        const Gate &g = c.ops[k];
        const Gate inv = invert(g);
        WireOp o{};
        o.wire = w;
        gate_matrix_1q(inv.kind, inv.params, o.minv);
        o.gen = g.num_params > 0 ? generator_of(g) : 0;
        o.slot = static_cast<uint32_t>(k);
        wire_ops[w].push_back(o);
      }
      wire_sig[w] = uniform_signature(wire_ops[w]);
    }
    // The block tiles of a run of wires sharing one rotation sequence split
    // it evenly: a run of R wires takes ceil(R / tile_high) passes of at most
    // ceil(R / passes) wires each (twenty wires: five passes of four become
    // four of five, not three of six and one of two).
    uint32_t blk_cap = max_high_blk;
    auto balanced_cap = [&](uint32_t w) {
      uint32_t run = 0;
      for (uint32_t v = w; v < n; v++) {
        if (wire_ops[v].empty()) continue;
        if (wire_sig[v] != wire_sig[w]) break;
        run++;
      }
      if (run == 0 || max_high_blk == 0) return max_high_blk;
      const uint32_t passes = (run + max_high_blk - 1) / max_high_blk;
      return (run + passes - 1) / passes;
    };
    // When every wire >= 6 of the window carries one rotation (one op per
    // wire), the block tiles take them more cheaply than the tile of wires
    // 0..5 (whose lane wires trade by shuffle): that first tile keeps only as
    // many wires >= 6 as leave the number of passes at its least, and at
    // least one, so it stays a compile-time tile (measured: 379 -> 394
    // MaxCut requests/s). With two ops per wire the first tile's share
    // moved to the block tiles costs more than it saves (the 28-qubit HEA
    // gradient 0.108 -> 0.120 s), so there it keeps what fits.
    uint32_t first_high = max_high;
    bool wide_first = false;
    {
      uint32_t run = 0, sig0 = 0, low_grads = 0, high_grads = 0;
      bool uniform = true, low = false;
      for (uint32_t w = 0; w < n; w++) {
        if (per_wire[w].empty()) continue;
        uint32_t g = 0;
        for (const WireOp &o : wire_ops[w]) g += o.gen != 0;
        if (w < 6) {
          low = true;
          low_grads += g;
          continue;
        }
        if (run == 0) {
          sig0 = wire_sig[w];
          high_grads = g;
        }
        uniform &= wire_sig[w] != 0 && wire_sig[w] == sig0;
        run++;
      }
      // The first tile of an RZ-then-RY layer takes four wires >= 6 (twenty
      // gradients, where sixteen allow two) when that saves a block pass: at
      // 28 qubits 2 + 5, 5, 5, 5 wires >= 6 become 4 + 6, 6, 6.
      bool low_rzry = n >= 10;
      for (uint32_t w = 0; w < 6 && w < n; w++) low_rzry &= wire_sig[w] == kSigRzRy;
      if (low_rzry && uniform && sig0 == kSigRzRy && run >= 4 && max_high >= 4 &&
          max_high_blk >= 5) {
        const uint32_t before = (run - 2 + max_high_blk - 1) / max_high_blk;
        const uint32_t after = (run - 4 + max_high_blk - 1) / max_high_blk;
        wide_first = after < before;
      }
      if (low && uniform && run > 0 && max_high_blk >= 5 && high_grads <= 1) {
        // as many as the first tile's gradient slots allow
        uint32_t room = max_high;
        if (high_grads > 0)
          room = low_grads >= kWindowGrads ? 0 : std::min(room, (kWindowGrads - low_grads) / high_grads);
        uint32_t best = ~0u;
        for (uint32_t k = std::min<uint32_t>(1, std::min(room, run)); k <= std::min(room, run);
             k++) {
          const uint32_t passes = (run - k + max_high_blk - 1) / max_high_blk;
          if (passes < best) {
            best = passes;
            first_high = k;
          }
        }
      }
    }
    for (uint32_t w = 0; w < n; w++) {
      if (per_wire[w].empty()) continue;
      const std::vector<WireOp> &ops = wire_ops[w];
      uint32_t wgrads = 0;
      for (const WireOp &o : ops) wgrads += o.gen != 0;
      const uint32_t need_other = w != 0 ? 1u : 0u, need_high = w >= 6 ? 1u : 0u;
      if (ops.size() > max_ops || wgrads > kWindowGrads) {
        flush();
        for (size_t b = 0; b < ops.size(); b += kWindowOps) {
          const size_t e = std::min<size_t>(ops.size(), b + kWindowOps);
          tile.assign(ops.begin() + b, ops.begin() + e);
          for (const WireOp &o : tile) tile_has_param |= o.gen != 0;
          flush();
        }
        continue;
      }
      bool full;
      const uint32_t sig = wire_sig[w];
      if (wide) {
        // Warp tiles: wire 0, wires 1..5 in the lanes, up to four wires >= 6;
        // block tiles: five or six wires >= 6 of one rotation sequence.
        const bool blk = !tile_low && w >= 6 && sig != 0 && (tile.empty() || sig == tile_sig);
        if (blk && tile.empty()) blk_cap = balanced_cap(w);
        // A tile of wire 0 and wires 1..5 that all carry RZ then RY takes four
        // wires >= 6 with the same ops (twenty gradients) where that saves a pass.
        const bool wide_rzry = wide_first && tile_low && others == 5 + highs &&
                               tile.size() == 12 + 2 * highs && tile_sig == kSigRzRy &&
                               sig == kSigRzRy;
        full = tile.size() + ops.size() > max_ops ||
               highs + need_high >
                   (blk ? std::max(blk_cap, max_high) : (tile_low ? first_high : max_high)) ||
               grads + wgrads > (wide_rzry ? kWideUniformGrads : kWindowGrads);
        if (!full && !blk && highs > max_high) full = true;   // a block tile takes no other wire
      } else {
        const uint32_t cap = (others + need_other >= 3) ? 8u : 16u;
        full = tile.size() + ops.size() > kWindowOps || others + need_other > 3 ||
               grads + wgrads > cap;
      }
      if (full) flush();
      if (tile.empty() && w >= 6 && sig != 0) blk_cap = balanced_cap(w);   // a new tile opens
      tile_sig = tile.empty() ? sig : (sig == tile_sig ? sig : 0);
      tile_low |= w < 6;
      tile.insert(tile.end(), ops.begin(), ops.end());
      others += need_other;
      highs += need_high;
      grads += wgrads;
      tile_has_param |= wgrads > 0;
    }
    flush();
  }
  return out;
}

// ---------------------------------------------------------------------------

namespace {

void put_map(std::vector<double> &v, uint32_t n, const std::vector<uint64_t> &cols, uint64_t off) {
  v.push_back(n);
  for (uint32_t j = 0; j < n; j++) v.push_back(static_cast<double>(cols[j]));
  v.push_back(static_cast<double>(off));
}

void put_mat(std::vector<double> &v, const cdouble *m) {
  for (int k = 0; k < 4; k++) {
    v.push_back(m[k].real());
    v.push_back(m[k].imag());
  }
}

}  // namespace

void serialise_schedule(const std::vector<ForwardStep> &s, uint32_t n, std::vector<double> &v) {
  v.push_back(static_cast<double>(s.size()));
  for (const ForwardStep &st : s) {
    v.push_back(st.kind);
    if (st.kind == ForwardStep::Group) {
      v.push_back(static_cast<double>(st.wires.size()));
      for (size_t i = 0; i < st.wires.size(); i++) {
        v.push_back(st.wires[i]);
        put_mat(v, &st.mats[4 * i]);
      }
    } else if (st.kind == ForwardStep::Permute) {
      put_map(v, n, st.cols, st.off);
      v.push_back(static_cast<double>(st.ops.size()));
      for (size_t i : st.ops) v.push_back(static_cast<double>(i));
    } else {
      v.push_back(static_cast<double>(st.ops.at(0)));
    }
  }
}

void serialise_schedule(const std::vector<CostateStep> &s, std::vector<double> &v) {
  v.push_back(static_cast<double>(s.size()));
  for (const CostateStep &st : s) {
    v.push_back(st.kind);
    switch (st.kind) {
      case CostateStep::ZDiag:
        v.push_back(static_cast<double>(st.masks.size()));
        for (size_t i = 0; i < st.masks.size(); i++) {
          v.push_back(static_cast<double>(st.masks[i]));
          v.push_back(st.coeffs[i]);
        }
        break;
      case CostateStep::Local:
        v.push_back(st.overwrite ? 1.0 : 0.0);
        v.push_back(static_cast<double>(st.wires.size()));
        for (size_t i = 0; i < st.wires.size(); i++) {
          v.push_back(st.wires[i]);
          v.push_back(static_cast<double>(st.masks[i]));
          v.push_back(st.nys[i]);
          v.push_back(st.coeffs[i]);
        }
        break;
      case CostateStep::Flip:
        v.push_back(st.overwrite ? 1.0 : 0.0);
        v.push_back(static_cast<double>(st.flip));
        v.push_back(static_cast<double>(st.masks.size()));
        for (size_t i = 0; i < st.masks.size(); i++) {
          v.push_back(static_cast<double>(st.masks[i]));
          v.push_back(st.nys[i]);
          v.push_back(st.coeffs[i]);
        }
        break;
      case CostateStep::XField:
        v.push_back(st.overwrite ? 1.0 : 0.0);
        v.push_back(st.energy);
        v.push_back(static_cast<double>(st.wires.size()));
        for (size_t i = 0; i < st.wires.size(); i++) {
          v.push_back(st.wires[i]);
          v.push_back(st.coeffs[i]);
        }
        break;
      default:
        break;
    }
  }
}

void serialise_schedule(const std::vector<BackwardStep> &s, uint32_t n, std::vector<double> &v) {
  v.push_back(static_cast<double>(s.size()));
  for (const BackwardStep &st : s) {
    v.push_back(st.kind);
    switch (st.kind) {
      case BackwardStep::Window:
        v.push_back(static_cast<double>(st.tile.size()));
        for (const WireOp &o : st.tile) {
          v.push_back(o.wire);
          put_mat(v, o.minv);
          v.push_back(o.gen);
          v.push_back(o.slot);
        }
        break;
      case BackwardStep::Diag:
        v.push_back(st.undo ? 1.0 : 0.0);
        v.push_back(static_cast<double>(st.masks.size()));
        for (size_t i = 0; i < st.masks.size(); i++) {
          v.push_back(static_cast<double>(st.masks[i]));
          v.push_back(st.angles[i]);
        }
        v.push_back(st.gphase);
        v.push_back(static_cast<double>(st.gens.size()));
        for (size_t i = 0; i < st.gens.size(); i++) {
          v.push_back(static_cast<double>(st.gens[i]));
          v.push_back(st.slots[i]);
        }
        break;
      case BackwardStep::PermuteUndo:
        put_map(v, n, st.cols, st.off);
        v.push_back(static_cast<double>(st.gates.size()));
        for (size_t g : st.gates) v.push_back(static_cast<double>(g));
        break;
      case BackwardStep::GateUndo:
        v.push_back(static_cast<double>(st.gates.at(0)));
        break;
    }
  }
}

}  // namespace qmetal
