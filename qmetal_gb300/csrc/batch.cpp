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
#include "schedule.hpp"

#include "../../include/qmetal/qmetal_kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
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

thread_local GraphTiming g_graph_timing;

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Every request recorded into one CUDA graph and launched once. Requests of a
// width share a simulator (its requests follow each other in the graph); the
// widths are parallel branches forked from and joined into one origin stream,
// and a heavy width is split over up to four simulators, about one per eighth
// of the batch's state traffic. Results land in pinned staging memory through
// copy nodes and are handed out after the single synchronisation.
void serve_graph(const std::vector<BatchItem> &items, const std::vector<size_t> &order,
                 const BatchTuning *tuning) {
  GraphTiming timing;
  const auto t_record = std::chrono::steady_clock::now();
  // Branches: per width, weighted by its state traffic (2^n x ops).
  std::map<uint32_t, std::vector<size_t>> by_width;
  double total = 0.0;
  std::map<uint32_t, double> weight;
  for (size_t i : order) {
    const uint32_t n = items[i].circuit->num_qubits;
    by_width[n].push_back(i);
    const double w = std::ldexp(1.0, static_cast<int>(n)) * (1.0 + items[i].circuit->ops.size());
    weight[n] += w;
    total += w;
  }
  std::vector<std::vector<size_t>> branches;
  std::vector<uint32_t> branch_width;
  for (auto it = by_width.rbegin(); it != by_width.rend(); ++it) {
    // about one branch per eighth of the traffic, at most four per width
    const int share = static_cast<int>(std::lround(8.0 * weight[it->first] / total));
    const int parts = static_cast<int>(std::min<size_t>(
        it->second.size(), static_cast<size_t>(std::max(1, std::min(4, share)))));
    for (int p = 0; p < parts; p++) {
      branches.emplace_back();
      branch_width.push_back(it->first);
      for (size_t k = p; k < it->second.size(); k += parts) branches.back().push_back(it->second[k]);
    }
  }
  // Simulators and buffers first: nothing allocates while the graph records.
  std::vector<std::unique_ptr<Simulator>> sims;
  size_t staging = 0;
  std::vector<size_t> offset(items.size());
  for (size_t b = 0; b < branches.size(); b++) {
    size_t max_gates = 1, max_shots = 0;
    for (size_t i : branches[b]) {
      max_gates = std::max(max_gates, items[i].circuit->ops.size());
      max_shots = std::max(max_shots, items[i].shots);
      offset[i] = staging;
      staging += 1 + items[i].circuit->ops.size() + items[i].shots;
    }
    sims.emplace_back(new Simulator(branch_width[b]));
    if (tuning) sims.back()->set_tile_high(tuning->tile_high[branch_width[b]]);
    sims.back()->reserve(max_gates, max_shots);
  }
  uint64_t *pinned = nullptr;
  if (cudaMallocHost(&pinned, std::max<size_t>(staging, 1) * sizeof(uint64_t)) != cudaSuccess)
    throw std::runtime_error("batch: pinned staging allocation failed");
  cudaStream_t origin = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> events;
  auto cleanup = [&]() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    if (origin) cudaStreamDestroy(origin);
    cudaFreeHost(pinned);
  };
  try {
    if (cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking) != cudaSuccess)
      throw std::runtime_error("batch: stream creation failed");
    for (size_t k = 0; k < branches.size() + 1; k++) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
        throw std::runtime_error("batch: event creation failed");
      events.push_back(e);
    }
    for (auto &s : sims) s->synchronize();
    if (cudaStreamBeginCapture(origin, cudaStreamCaptureModeRelaxed) != cudaSuccess)
      throw std::runtime_error("batch: graph capture failed to start");
    try {
      cudaEventRecord(events[0], origin);
      for (size_t b = 0; b < branches.size(); b++) {
        cudaStream_t s = static_cast<cudaStream_t>(sims[b]->stream());
        cudaStreamWaitEvent(s, events[0], 0);
        for (size_t i : branches[b]) {
          const BatchItem &it = items[i];
          uint64_t *slot = pinned + offset[i];
          sims[b]->serve_enqueue(*it.circuit, *it.hamiltonian, it.shots, it.seed,
                                 reinterpret_cast<double *>(slot),
                                 reinterpret_cast<double *>(slot + 1), slot + 1 +
                                     it.circuit->ops.size());
        }
        cudaEventRecord(events[b + 1], s);
        cudaStreamWaitEvent(origin, events[b + 1], 0);
      }
    } catch (...) {
      cudaStreamEndCapture(origin, &graph);
      throw;
    }
    if (cudaStreamEndCapture(origin, &graph) != cudaSuccess || !graph)
      throw std::runtime_error("batch: graph capture failed");
    timing.record_s = seconds_since(t_record);
    cudaGraphGetNodes(graph, nullptr, &timing.nodes);
    timing.branches = branches.size();
    const auto t_inst = std::chrono::steady_clock::now();
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
      throw std::runtime_error("batch: graph instantiation failed");
    timing.instantiate_s = seconds_since(t_inst);
    const auto t_exec = std::chrono::steady_clock::now();
    if (cudaGraphLaunch(exec, origin) != cudaSuccess)
      throw std::runtime_error("batch: graph launch failed");
    const cudaError_t e = cudaStreamSynchronize(origin);
    if (e != cudaSuccess) throw std::runtime_error(std::string("batch: ") + cudaGetErrorString(e));
    timing.execute_s = seconds_since(t_exec);
    for (auto &sim : sims) sim->check_waits();
    for (const BatchItem &it : items) {
      const uint64_t *slot = pinned + offset[&it - items.data()];
      if (it.energy) std::memcpy(it.energy, slot, sizeof(double));
      if (!it.circuit->ops.empty())
        std::memcpy(it.grad, slot + 1, it.circuit->ops.size() * sizeof(double));
      if (it.shots)
        std::memcpy(it.samples, slot + 1 + it.circuit->ops.size(), it.shots * sizeof(uint64_t));
    }
  } catch (...) {
    cudaStreamSynchronize(origin);
    cleanup();
    throw;
  }
  cleanup();
  g_graph_timing = timing;
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
    for (uint32_t kh = 1; kh <= std::min<uint32_t>(kMaxTileHigh, n - 6); kh++) {
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

  if (mode == BatchMode::PlainLoop || mode == BatchMode::FusedLoop) {
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
  if (mode == BatchMode::Graph) {
    if (lanes == 0) {
      const BatchTuning tuned = autotune_batch(items);
      serve_graph(items, order, &tuned);
    } else {
      serve_graph(items, order, nullptr);
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

GraphTiming last_graph_timing() { return g_graph_timing; }

}  // namespace qmetal
