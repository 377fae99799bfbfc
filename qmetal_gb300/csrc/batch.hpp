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
};

void run_batch(const std::vector<BatchItem> &items, BatchMode mode, uint32_t lanes);

}  // namespace qmetal
