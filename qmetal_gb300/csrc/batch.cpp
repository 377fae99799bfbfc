// batch.cpp -- serving many circuits of uneven widths together.
//
// A request is (circuit, Hamiltonian, shots, seed) -> energy, per-gate adjoint
// gradient, samples. The reference has no batched path; callers loop over
// circuits (forward, energy_and_gradient, sample each). Here L lanes run
// requests concurrently, each lane a host thread with its own CUDA stream and
// one Simulator per width it has met, so small requests overlap on the GPU
// instead of leaving it idle between tiny launches, while wide requests keep
// the full-bandwidth kernels. Requests are taken widest first from a shared
// counter (no waiting between lanes); each request is one queued sequence with
// a single synchronisation (Simulator::serve).
//
// The autotuner picks, from measurements on the batch's own requests, the
// tile shape of the backward window passes per width and the lane count.
#include "batch.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>

namespace qmetal {
namespace {

std::vector<size_t> widest_first(const std::vector<BatchItem> &items) {
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return items[a].circuit->num_qubits > items[b].circuit->num_qubits;
  });
  return order;
}

void validate(const BatchItem &it) {
  if (!it.circuit || !it.hamiltonian) throw std::runtime_error("batch: null circuit or Hamiltonian");
  if (it.circuit->num_qubits == 0 || it.circuit->num_qubits > kMaxQubits)
    throw std::runtime_error("batch: circuit width out of range");
  if (!it.grad && !it.circuit->ops.empty()) throw std::runtime_error("batch: null gradient output");
  if (it.shots && !it.samples) throw std::runtime_error("batch: null sample output");
}

// One request the way a caller of the per-circuit API does it: the reference's
// gradient (gate-by-gate forward and sweep), then the forward run again, then
// the samples.
void plain_request(Simulator &sim, const BatchItem &it) {
  auto r = sim.energy_and_gradient(*it.circuit, *it.hamiltonian, false);
  if (it.energy) *it.energy = r.first;
  std::copy(r.second.begin(), r.second.end(), it.grad);
  if (it.shots) {
    sim.reset();
    sim.run(*it.circuit);
    auto s = sim.sample(it.shots, it.seed);
    std::copy(s.begin(), s.end(), it.samples);
  }
}

Simulator &simulator_for(std::map<uint32_t, std::unique_ptr<Simulator>> &sims, uint32_t n,
                         const BatchTuning *tuning) {
  auto &sim = sims[n];
  if (!sim) {
    sim.reset(new Simulator(n));
    if (tuning) sim->set_tile_high(tuning->tile_high[n]);
  }
  return *sim;
}

void serve_lanes(const std::vector<BatchItem> &items, const std::vector<size_t> &order,
                 uint32_t lanes, const BatchTuning *tuning, int device) {
  lanes = std::max<uint32_t>(1, std::min<uint32_t>(lanes, 64));
  std::atomic<size_t> next{0};
  std::atomic<bool> failed{false};
  std::mutex err_lock;
  std::string first_error;
  auto lane = [&]() {
    try {
      if (cudaSetDevice(device) != cudaSuccess) throw std::runtime_error("batch: cudaSetDevice");
      std::map<uint32_t, std::unique_ptr<Simulator>> sims;
      for (;;) {
        if (failed.load()) return;
        const size_t k = next.fetch_add(1);
        if (k >= order.size()) return;
        const BatchItem &it = items[order[k]];
        simulator_for(sims, it.circuit->num_qubits, tuning)
            .serve(*it.circuit, *it.hamiltonian, it.shots, it.seed, it.energy, it.grad, it.samples);
      }
    } catch (const std::exception &e) {
      std::lock_guard<std::mutex> g(err_lock);
      if (!failed.exchange(true)) first_error = e.what();
    }
  };
  const uint32_t nthreads = static_cast<uint32_t>(std::min<size_t>(lanes, order.size()));
  std::vector<std::thread> pool;
  for (uint32_t t = 0; t < nthreads; t++) pool.emplace_back(lane);
  for (auto &t : pool) t.join();
  if (failed.load()) throw std::runtime_error("batch: " + first_error);
}

std::mutex g_tuning_lock;
std::map<std::vector<uint32_t>, BatchTuning> g_tuning_cache;

}  // namespace

BatchTuning autotune_batch(const std::vector<BatchItem> &items) {
  for (const BatchItem &it : items) validate(it);
  std::vector<uint32_t> widths;
  for (const BatchItem &it : items) widths.push_back(it.circuit->num_qubits);
  std::sort(widths.begin(), widths.end());
  widths.erase(std::unique(widths.begin(), widths.end()), widths.end());
  {
    std::lock_guard<std::mutex> g(g_tuning_lock);
    auto it = g_tuning_cache.find(widths);
    if (it != g_tuning_cache.end()) return it->second;
  }
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) throw std::runtime_error("batch: no CUDA device");
  const auto t0 = std::chrono::steady_clock::now();
  BatchTuning best;
  // Tile shape, per width: device time of one of its requests per candidate.
  for (uint32_t n : widths) {
    if (n < 7) continue;
    const BatchItem *req = nullptr;
    for (const BatchItem &it : items)
      if (it.circuit->num_qubits == n) {
        req = &it;
        break;
      }
    Simulator sim(n);
    double best_t = 1e300;
    for (uint32_t kh = 1; kh <= std::min<uint32_t>(4, n - 6); kh++) {
      sim.set_tile_high(kh);
      sim.serve(*req->circuit, *req->hamiltonian, req->shots, req->seed, req->energy, req->grad,
                req->samples);
      sim.elapsed();
      for (int r = 0; r < 2; r++)
        sim.serve(*req->circuit, *req->hamiltonian, req->shots, req->seed, req->energy,
                  req->grad, req->samples);
      const double t = sim.elapsed();
      if (t < best_t) {
        best_t = t;
        best.tile_high[n] = kh;
      }
    }
  }
  // Lane count: a quarter of the batch (every fourth request), wall clock.
  std::vector<BatchItem> sample;
  for (size_t i = 0; i < items.size(); i += 4) sample.push_back(items[i]);
  const std::vector<size_t> order = widest_first(sample);
  double best_lanes_t = 1e300;
  for (uint32_t lanes : {2u, 4u, 8u, 16u}) {
    const auto s0 = std::chrono::steady_clock::now();
    serve_lanes(sample, order, lanes, &best, device);
    const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
    if (t < best_lanes_t) {
      best_lanes_t = t;
      best.lanes = lanes;
    }
  }
  best.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::lock_guard<std::mutex> g(g_tuning_lock);
  g_tuning_cache[widths] = best;
  return best;
}

void run_batch(const std::vector<BatchItem> &items, BatchMode mode, uint32_t lanes) {
  for (const BatchItem &it : items) validate(it);
  if (items.empty()) return;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) throw std::runtime_error("batch: no CUDA device");
  const std::vector<size_t> order = widest_first(items);

  if (mode != BatchMode::Lanes) {
    std::map<uint32_t, std::unique_ptr<Simulator>> sims;
    for (size_t idx : order) {
      const BatchItem &it = items[idx];
      Simulator &sim = simulator_for(sims, it.circuit->num_qubits, nullptr);
      if (mode == BatchMode::PlainLoop)
        plain_request(sim, it);
      else
        sim.serve(*it.circuit, *it.hamiltonian, it.shots, it.seed, it.energy, it.grad,
                  it.samples);
    }
    return;
  }
  if (lanes == 0) {
    const BatchTuning tuned = autotune_batch(items);
    serve_lanes(items, order, tuned.lanes, &tuned, device);
    return;
  }
  serve_lanes(items, order, lanes, nullptr, device);
}

}  // namespace qmetal
