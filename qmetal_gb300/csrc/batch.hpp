// batch.hpp -- many serving requests (energy, adjoint gradient, samples) of
// uneven widths in one call.
#pragma once

#include <cstdint>
#include <vector>

#include "simulator.hpp"

namespace qmetal {

struct BatchItem {
  const Circuit *circuit = nullptr;
  const Hamiltonian *hamiltonian = nullptr;
  size_t shots = 0;
  uint64_t seed = 0;
  double *energy = nullptr;
  double *grad = nullptr;        // circuit->size() entries
  uint64_t *samples = nullptr;   // shots entries
};

enum class BatchMode {
  Lanes = 0,       // concurrent lanes, block-wise adjoint, one sync per request
  PlainLoop = 1,   // one request after another, gate-by-gate adjoint, then run + sample
  FusedLoop = 2,   // one request after another, block-wise adjoint
  Graph = 3,       // every request recorded into one CUDA graph, launched once
};

// Time split of the last Graph-mode batch served by this thread.
struct GraphTiming {
  double record_s = 0.0;        // host: building and recording every request
  double instantiate_s = 0.0;   // cudaGraphInstantiate
  double execute_s = 0.0;       // one launch to completion
  size_t nodes = 0;
  size_t branches = 0;
};
GraphTiming last_graph_timing();

// Choices the autotuner makes for a batch: how many lanes run at once, and per
// width the tile shape of the backward window passes (wires >= 6 held in
// registers per pass).
struct BatchTuning {
  uint32_t lanes = 8;
  uint32_t tile_high[kMaxQubits + 1];
  double seconds = 0.0;   // time spent measuring
  BatchTuning() {
    for (auto &t : tile_high) t = 6;   // the simulator default
  }
};

// Measure candidates on the batch's own requests: per width, one request
// served with each tile shape; then a quarter of the batch served with each
// lane count. Results are cached per set of widths for the process.
BatchTuning autotune_batch(const std::vector<BatchItem> &items);

// lanes == 0 in Lanes mode: use (and if needed compute) the autotuned choices.
void run_batch(const std::vector<BatchItem> &items, BatchMode mode, uint32_t lanes);

}  // namespace qmetal
