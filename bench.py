#!/usr/bin/env python
"""Fused-plan statevector benchmark on GB300.

Workload (one "step"): the four fused circuits of the 30-qubit configuration,
each from |0...0> on an 8 GiB complex64 state -- QAOA ring p=6, TFIM Trotter
20 steps (J=1, h=0.7, dt=0.05), hardware-efficient ansatz depth 3, and random
depth-10 U3 + CZ layers -- with seeded synthetic angles (qmetal_gb300/
workloads.py). The metric is algorithmic HBM bytes per second: every plan op
is charged 16 B per amplitude it must read and write (2S for dense, group,
blocked and diagonal ops, S for controlled and swap ops, S/2 for CCX, S for
the |0> reset, where S = 8 * 2^n bytes), over device time.

Output: one JSON line (rank 0). `value` is device-timed with the state resident
in HBM; `e2e` repeats the step through the C ABI from host gate arrays
(circuit build, reset, run, 1024 samples and the norm read back), wall-clock;
`roofline` is the dominant kernel's achieved bandwidth from CUDA events around
each op inside the timed region; `cpu_baseline` is the complex128 oracle on
the host cores on a bounded sample (the same fused plans at 20 qubits).

Two more keys carry the other configurations of the metric, each measured in
the same run after the timed region: `grad` (adjoint gradients of the HEA
depth-8 problem at 28 and 33 qubits, block-wise and gate-by-gate sweeps on
the same GPU, their difference, and the error against the complex128 oracle
at 22 qubits) and `batch` (512 QAOA MaxCut requests served together, against
the per-circuit loops, with the batch's roofline fraction and its error
against the oracle).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: the statevector path does not shard here; N GPUs run N independent
replicas (weak scaling), one process per GPU under torchrun.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30
N_CPU = 20
OP_NAMES = ["dense1q", "group", "blocked", "controlled1q", "diagonal", "swap", "ccx"]
# DRAM bytes (read + write) per algorithmic byte of one launch, from ncu's
# dram__bytes_read.sum + dram__bytes_write.sum on single launches: the group
# kernel at 28 qubits (k_group<4,0,2>: 2147.5 + 2085.9 MB against 2S =
# 4295.0 MB), the diagonal layer at 26 (k_diag: 537.0 + 477.4 MB against
# 1073.7 MB). The traffic grows with the state, so a launch at n qubits is
# charged this fraction of its 2S.
DRAM_PER_ALGO_BYTE = {1: (2147.5 + 2085.9) / 4295.0, 4: (537.0 + 477.4) / 1073.7}
DRAM_CAPTURE_QUBITS = {1: 28, 4: 26}
OP_STATE_PASSES = {0: 2.0, 1: 2.0, 2: 2.0, 3: 1.0, 4: 2.0, 5: 1.0, 6: 0.5}  # x S


def workload(n):
    from qmetal_gb300 import workloads as W
    return [("qaoa_ring_p6", W.qaoa_ring_seeded(n, 6, seed=1)),
            ("tfim_trotter_20", W.tfim_chain(n, 20, 1.0, 0.7, 0.05)),
            ("hea_d3", W.hea(n, 3, seed=3)),
            ("random_u3_d10", W.random_u3(n, 10, seed=4))]


def plan_kinds(flat):
    """Op kinds of a flat exported plan."""
    out, pos = [], 1
    for _ in range(int(flat[0])):
        kind, ng, nt = int(flat[pos]), int(flat[pos + 5]), int(flat[pos + 6])
        out.append(kind)
        pos += 16 + 9 * ng + 2 * nt
    return out


def op_bytes(kind, n):
    return OP_STATE_PASSES[kind] * 8.0 * (1 << n)


def circuit_bytes(kinds, n):
    """Reset (one state write) plus every plan op."""
    return 8.0 * (1 << n) + sum(op_bytes(k, n) for k in kinds)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during a region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.proc = None
        self.device = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    return world, rank, local, dist


def max_over_ranks(x, dist, world):
    if world <= 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, world):
    if world > 1:
        dist.barrier()


def torch_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except Exception:
        pass


def cpu_sample(threads, copies=1, repeats=1, executor="plan"):
    """The complex128 oracle (a restatement of the reference's CPU Reference)
    on the workload's circuits at N_CPU qubits, one instance per thread,
    `threads` instances concurrently. executor "plan" runs the fused plan op
    by op (Reference::run(const Plan&), src/reference.cpp:208-248) -- the
    same plans whose bytes are charged -- and "gates" the gate stream one gate
    at a time. Returns (GB/s-equivalent, secs)."""
    import oracle
    import qmetal_gb300 as qm  # noqa: F401  (plans come from the library)
    from qmetal_gb300 import workloads as W
    oracle.set_threads(1)
    jobs, total_bytes = [], 0.0
    for _name, gates in workload(N_CPU):
        plan = W.to_circuit(N_CPU, gates).plan_export()
        for _ in range(copies * repeats):
            jobs.append(plan if executor == "plan" else gates)
            total_bytes += circuit_bytes(plan_kinds(plan), N_CPU)
    run = oracle.run_plan if executor == "plan" else oracle.run
    t0 = time.perf_counter()
    if threads == 1:
        for job in jobs:
            run(N_CPU, job)
    else:
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda job: run(N_CPU, job), jobs))
    dt = time.perf_counter() - t0
    return total_bytes / dt / 1e9, dt


def run_reference(args, world, rank, dist):
    """The reference's CPU implementation of the path (the oracle port of its
    complex128 Reference; its own sources are not on this machine), all host
    threads, each step a bounded sample: every workload circuit's fused plan at
    N_CPU qubits executed op by op, cores/4 copies of each run concurrently.
    The gate-by-gate form of the same circuits is timed once beside it."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    copies = max(1, threads // 4)
    for _ in range(args.warmup):
        cpu_sample(threads, copies)
    rates, secs = [], 0.0
    for _ in range(args.steps):
        r, dt = cpu_sample(threads, copies)
        rates.append(r)
        secs += dt
    value = args.steps / sum(1.0 / r for r in rates)   # total bytes / total time
    gbg_rate, gbg_secs = cpu_sample(threads, copies, executor="gates")
    kind = "reference" if oracle.ref_available() else "port"
    line = {
        "impl": "reference", "metric": "fused_plan_hbm_gbs", "value": round(value, 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": f"fused plans of the 30-qubit config, run at {N_CPU} "
                               "qubits on the host (bounded sample)",
                   "num_qubits": N_CPU, "circuits": [c for c, _ in workload(4)],
                   "copies_per_circuit": copies},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                         "kind": kind,
                         "sample": f"4 fused plans x {copies} copies at n={N_CPU}, complex128, "
                                   f"plan op by op, {threads} threads"},
        "gate_by_gate": {"value": round(gbg_rate, 3), "unit": "GB/s",
                         "seconds": round(gbg_secs, 3),
                         "what": "the same circuits gate by gate (no fusion), same bytes charged"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --- algorithmic bytes of one serving request -------------------------------
# Each launch is charged 16 B per amplitude it must read and write, as the
# plan ops are: a one-qubit group pass or a permutation pass 2S, a window-tile
# or diagonal-block undo pass over both states 4S (a diagonal block without
# its undo 2S), one gate undone on both states twice that gate's bytes, the
# co-state passes 2S (written from psi) or 3S (accumulated), the energy dot
# product 2S, the |0> reset S and the sampler's block sums S.
GATE_STATE_PASSES = {12: 1.0, 13: 1.0, 14: 0.5, 15: 1.0, 16: 0.5, 17: 0.5}  # else 2S


def _forward_bytes(flat, plan_kinds_, S):
    total, pos = 0.0, 1
    for _ in range(int(flat[0])):
        kind = int(flat[pos])
        if kind == 0:
            nw = int(flat[pos + 1])
            total += 2 * S
            pos += 2 + 9 * nw
        elif kind == 1:
            n = int(flat[pos + 1])
            nops = int(flat[pos + 3 + n])
            total += 2 * S
            pos += 4 + n + nops
        else:
            total += OP_STATE_PASSES[plan_kinds_[int(flat[pos + 1])]] * S
            pos += 2
    assert pos == len(flat), "schedule layout"
    return total


def _costate_bytes(flat, S):
    total, pos = 0.0, 1
    for _ in range(int(flat[0])):
        kind = int(flat[pos])
        if kind == 0:
            nt = int(flat[pos + 1])
            total += 2 * S
            pos += 2 + 2 * nt
        elif kind == 1:
            overwrite, nt = int(flat[pos + 1]), int(flat[pos + 2])
            total += (2 if overwrite else 3) * S
            pos += 3 + 4 * nt
        elif kind == 2:
            overwrite, nt = int(flat[pos + 1]), int(flat[pos + 3])
            total += (2 if overwrite else 3) * S
            pos += 4 + 3 * nt
        elif kind == 5:
            overwrite, nw = int(flat[pos + 1]), int(flat[pos + 3])
            total += (2 if overwrite else 3) * S
            pos += 4 + 2 * nw
        else:
            total += (1 if kind == 3 else 2) * S
            pos += 1
    assert pos == len(flat), "schedule layout"
    return total


def _backward_bytes(flat, gates, S):
    total, pos = 0.0, 1
    for _ in range(int(flat[0])):
        kind = int(flat[pos])
        if kind == 0:
            nops = int(flat[pos + 1])
            total += 4 * S
            pos += 2 + 11 * nops
        elif kind == 1:
            undo, nt = int(flat[pos + 1]), int(flat[pos + 2])
            ng = int(flat[pos + 4 + 2 * nt])
            total += (4 if undo else 2) * S
            pos += 5 + 2 * nt + 2 * ng
        elif kind == 2:
            n = int(flat[pos + 1])
            ng = int(flat[pos + 3 + n])
            total += 4 * S
            pos += 4 + n + ng
        else:
            k = gates[int(flat[pos + 1])][0]
            total += 2 * GATE_STATE_PASSES.get(k, 2.0) * S
            pos += 2
    assert pos == len(flat), "schedule layout"
    return total


def request_bytes(n, gates, circuit, hamiltonian, shots, tile_high):
    """Algorithmic HBM bytes of one request served by Simulator::serve:
    reset, merged forward, samples, co-state and energy, block-wise sweep."""
    S = 8.0 * (1 << n)
    kinds = plan_kinds(circuit.plan_export())
    total = S + _forward_bytes(circuit.schedule_export("forward"), kinds, S)
    if shots:
        total += S
    total += _costate_bytes(circuit.schedule_export("costate", hamiltonian), S)
    total += _backward_bytes(circuit.schedule_export("backward", tile_high=tile_high), gates, S)
    return total


def batch_results(requests=512, steps=3, warmup=3, lanes=0, widths=None, loops=True,
                  oracle_max_n=16, dist=None, world=1, rank=0):
    """512 QAOA MaxCut requests (n uniform over the even widths 12..26, p in
    1..8, random 3-regular graphs, angles ~ U[0, pi]), each energy + adjoint
    gradient + 4096 samples. A step serves the whole batch with concurrent
    lanes (wall clock, host buffers). Beside it, once each: the same batch as
    one CUDA graph, the per-circuit loop with the same block-wise sweep, and
    the per-circuit loop a caller of the reference API would write
    (gate-by-gate gradient, run, sample). Returns a dict."""
    import numpy as np
    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    insts = W.maxcut_instances(requests, seed=6)
    if widths:
        insts = [i for i in insts if i["n"] in widths]
    reqs, streams = [], []
    for k, inst in enumerate(insts):
        gates = W.maxcut_qaoa(inst["n"], inst["edges"], inst["gammas"], inst["betas"])
        reqs.append((W.to_circuit(inst["n"], gates),
                     W.to_hamiltonian(W.maxcut_hamiltonian(inst["edges"])), 4096, 7000 + k))
        streams.append(gates)
    params = sum(len(c) for c, _h, _s, _seed in reqs)

    tuning = qm.batch_autotune(reqs) if lanes == 0 else None
    tile_of = (tuning or {}).get("tile_high", {})
    batch_bytes = sum(request_bytes(c.num_qubits, g, c, h, s, tile_of.get(c.num_qubits, 4))
                      for (c, h, s, _seed), g in zip(reqs, streams))
    h2d = sum(sum(4 + 4 * len(q) + 8 * len(p) for _k, q, p in g) for g in streams)
    d2h = sum(8 + 8 * len(c) + 8 * s for c, _h, s, _seed in reqs)

    def serve(mode):
        torch_sync()
        t0 = time.perf_counter()
        out = qm.batch_serve(reqs, mode=mode, lanes=lanes)
        return out, time.perf_counter() - t0

    for _ in range(max(warmup, 3)):
        serve(qm.BATCH_LANES)
    barrier(dist, world)
    with ClockSampler(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        times = []
        for _ in range(steps):
            lanes_out, dt = serve(qm.BATCH_LANES)
            times.append(dt)
    wall = max_over_ranks(sum(times), dist, world)
    per_batch = wall / steps
    peak, peak_src = peaks()
    # The same batch recorded into one CUDA graph and launched once (tile
    # shapes from the tuning above); wall clock includes recording.
    graph_runs = []
    for _ in range(2):
        graph_out, graph_t = serve(qm.BATCH_GRAPH)
        graph_runs.append((graph_t, qm.batch_graph_timing()))
    graph_t, graph_timing = min(graph_runs, key=lambda r: r[0])
    graph_diff = max(float(np.max(np.abs(np.array(a[1]) - np.array(b[1])))) for a, b in
                     zip(lanes_out, graph_out))
    out = {
        "value": round(len(reqs) / per_batch, 2), "unit": "requests/s",
        "s_per_batch": round(per_batch, 4), "steps": steps, "warmup": max(warmup, 3),
        "requests": len(reqs), "widths": sorted({i["n"] for i in insts}), "gate_params": params,
        "lanes": tuning["lanes"] if tuning else lanes, "autotuned": tuning,
        "roofline": {"bound": "hbm", "algorithmic_bytes_per_batch": batch_bytes,
                     "achieved": round(batch_bytes / per_batch / 1e9, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(batch_bytes / per_batch / 1e9 / peak, 4),
                     "peak_source": peak_src,
                     "what": "every launch's algorithmic bytes summed over the batch, over "
                             "the batch's wall-clock time (host buffers, all lanes)"},
        "e2e": {"value": round(len(reqs) / per_batch, 2), "unit": "requests/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "graph": {"value": round(len(reqs) / graph_t, 2), "unit": "requests/s",
                  "seconds": round(graph_t, 3),
                  "record_s": round(graph_timing["record_s"], 3),
                  "instantiate_s": round(graph_timing["instantiate_s"], 3),
                  "execute_s": round(graph_timing["execute_s"], 3),
                  "nodes": graph_timing["nodes"], "max_grad_diff_vs_lanes": graph_diff,
                  "what": "every request recorded into one CUDA graph, one launch"},
        "clocks": clocks.summary(),
    }
    if loops:
        fused_out, fused_t = serve(qm.BATCH_FUSED_LOOP)
        plain_out, plain_t = serve(qm.BATCH_PLAIN_LOOP)
        out["blockwise_loop"] = {
            "value": round(len(reqs) / fused_t, 2), "unit": "requests/s",
            "seconds": round(fused_t, 3),
            "what": "per-circuit loop with the same block-wise sweep, one request at a time"}
        out["plain_loop"] = {
            "value": round(len(reqs) / plain_t, 2), "unit": "requests/s",
            "seconds": round(plain_t, 3),
            "what": "per-circuit loop as a caller of the reference API writes it: "
                    "gate-by-gate adjoint, run, sample"}
        out["speedup_vs_blockwise_loop"] = round(fused_t / per_batch, 3)
        out["speedup_vs_plain_loop"] = round(plain_t / per_batch, 2)
        out["max_grad_diff_vs_plain"] = max(
            float(np.max(np.abs(np.array(a[1]) - np.array(b[1]))))
            for a, b in zip(lanes_out, plain_out))
        out["max_energy_diff_vs_plain"] = max(abs(a[0] - b[0])
                                              for a, b in zip(lanes_out, plain_out))
    if rank == 0 and oracle_max_n:
        import oracle
        oracle.build()
        e_worst = e_rel = g_worst = g_rel = 0.0
        checked = 0
        for inst, gates, got in zip(insts, streams, lanes_out):
            if inst["n"] > oracle_max_n:
                continue
            e0, g0 = oracle.energy_and_gradient(inst["n"], gates,
                                                W.maxcut_hamiltonian(inst["edges"]))
            gd = float(np.max(np.abs(np.array(got[1]) - g0)))
            e_worst = max(e_worst, abs(got[0] - e0))
            e_rel = max(e_rel, abs(got[0] - e0) / max(abs(e0), 1e-30))
            g_worst = max(g_worst, gd)
            g_rel = max(g_rel, gd / max(float(np.max(np.abs(g0))), 1e-30))
            checked += 1
        out["err_vs_complex128_oracle"] = {
            "requests_checked": checked, "widths": f"n <= {oracle_max_n}",
            "max_abs_energy_err": e_worst, "max_rel_energy_err": e_rel,
            "max_abs_grad_err": g_worst, "max_grad_err_rel_to_max_grad": g_rel}
    return out


def run_batch_workload(args, world, rank, dist):
    """The batched-serving configuration as its own line (see batch_results)."""
    r = batch_results(args.requests, args.steps, args.warmup, args.lanes, args.widths,
                      loops=not args.no_loops, oracle_max_n=0 if args.no_loops else 16,
                      dist=dist, world=world, rank=rank)
    if rank == 0:
        line = {
            "metric": "batched_adjoint_requests_per_s", "value": round(world * r["value"], 2),
            "unit": "requests/s", "n_gpus": world, "steps": args.steps,
            "warmup": r["warmup"], "ms_per_step": round(1e3 * r["s_per_batch"], 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic",
            "config": {"workload": f"{r['requests']} QAOA MaxCut requests (energy + adjoint "
                                   "gradient + 4096 samples each)",
                       "widths": r["widths"], "gate_params": r["gate_params"],
                       "lanes": r["lanes"], "autotuned": r["autotuned"]},
            **{k: v for k, v in r.items() if k not in ("value", "unit", "steps", "warmup")},
        }
        print(json.dumps(line), flush=True)
    barrier(dist, world)


def grad_results(qubits, reps=5, gate_by_gate=True, oracle_qubits=22):
    """Adjoint gradients of the HEA depth-8 problem (RY + RZ per wire per
    layer, CX ladder; H = -sum Z_i Z_{i+1} - 0.7 sum X_i on a ring): device
    seconds per gradient with the block-wise sweep (the default) and with the
    reference's gate-by-gate sweep on the same GPU, the largest difference
    between the two gradients at each width, and, at oracle_qubits, every
    entry against the complex128 oracle's adjoint gradient."""
    import numpy as np
    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    results = {}
    for n in qubits:
        gates, terms = W.hea_gradient_problem(n, depth=8, seed=5)
        c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
        nparams = sum(1 for g in gates if g[2])
        sim = qm.Simulator(n)
        entry = {"gates": len(gates), "params": nparams}
        sim.energy_and_gradient(c, h)      # warm-up (first use takes the co-state)
        sim.elapsed()
        for _ in range(reps):
            e, g = sim.energy_and_gradient(c, h)
        t = sim.elapsed() / reps
        entry["blockwise"] = {"s_per_gradient": round(t, 4), "grad_per_s": round(1.0 / t, 3),
                              "param_grads_per_s": round(nparams / t, 1), "reps": reps}
        entry["energy"] = e
        if gate_by_gate:
            sim.elapsed()
            e1, g1 = sim.energy_and_gradient(c, h, fused=False)
            t1 = sim.elapsed()
            entry["gate_by_gate"] = {"s_per_gradient": round(t1, 4),
                                     "grad_per_s": round(1.0 / t1, 3),
                                     "param_grads_per_s": round(nparams / t1, 1), "reps": 1}
            entry["speedup"] = round(t1 / t, 2)
            entry["max_abs_grad_diff_vs_gate_by_gate"] = float(
                np.max(np.abs(np.array(g) - np.array(g1))))
            entry["abs_energy_diff_vs_gate_by_gate"] = abs(e - e1)
        results[f"n{n}"] = entry
        sim.close()
        del sim
    if oracle_qubits:
        import oracle
        oracle.build()
        n = oracle_qubits
        gates, terms = W.hea_gradient_problem(n, depth=8, seed=5)
        sim = qm.Simulator(n)
        e, g = sim.energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
        sim.close()
        e0, g0 = oracle.energy_and_gradient(n, gates, terms)
        results["err_vs_complex128_oracle"] = {
            "n": n, "params": sum(1 for x in gates if x[2]),
            "max_abs_grad_err": float(np.max(np.abs(np.array(g) - g0))),
            "abs_energy_err": abs(e - e0)}
    return results


def run_grad_workload(args, world, rank, dist):
    """The gradient configuration as its own line (see grad_results)."""
    results = grad_results(args.grad_qubits, args.steps, gate_by_gate=not args.no_loops,
                           oracle_qubits=0 if args.no_loops else 22)
    if rank == 0:
        first = results[f"n{args.grad_qubits[0]}"]
        line = {
            "metric": "adjoint_gradients_per_s", "value": first["blockwise"]["grad_per_s"],
            "unit": "gradients/s", "n_gpus": world, "steps": args.steps, "warmup": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic",
            "config": {"workload": "HEA depth 8 (RY+RZ per wire per layer, CX ladder), ring "
                                   "TFIM Hamiltonian hx=0.7", "qubits": args.grad_qubits},
            "results": results,
        }
        print(json.dumps(line), flush=True)


def benchmark_set(n, extended=False):
    """The reference's frozen benchmark set at width n (src/circuits.cpp:
    171-191): the five closed-form generators restated in workloads.py and
    the mt19937-seeded members from the committed fixtures of the
    reference's own generators (tests/golden/circuits.json)."""
    from qmetal_gb300 import workloads as W
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                        "circuits.json")
    with open(path) as f:
        fixtures = json.load(f)

    def fixture(key):
        return [(k, tuple(q), tuple(p)) for k, q, p in fixtures[key]]

    out = [("ghz", W.ghz(n)), ("qft", W.qft(n)), ("qaoa_ring_p6", W.qaoa_ring(n, 6)),
           ("tfim_trotter_20", W.tfim_trotter(n, 20)), ("grover_proxy_4", W.grover_proxy(n, 4)),
           ("random_d10", fixture(f"random_circuit_{n}_10_0x5eed")),
           ("hea_d3", fixture(f"hardware_efficient_{n}_3_0x5eed"))]
    if extended:
        patch = fixture(f"local_patch_{n}_8_12_0x10ca1")
        out.append(("local_patch_w8", patch))
        # the same work register on the highest wires, where blocking cannot
        # reach it unless the qubits are reordered
        out.append(("local_patch_w8_high", W.relabel(patch, [n - 1 - q for q in range(n)])))
    return out


def time_plan(sim, circuit, reps, **opts):
    """Best device time of reps runs of one option set (reset excluded), as
    the reference's benches take the best of their repetitions."""
    best = float("inf")
    for _ in range(reps + 1):
        sim.reset()
        sim.elapsed()
        if opts.get("unfused"):
            sim.run(circuit, fuse=False)
        else:
            sim.run_options(circuit, **{k: v for k, v in opts.items() if k != "unfused"})
        best = min(best, sim.elapsed())
    return best


def run_fusion_workload(args, world, rank, dist):
    """Port of the reference's fusion_bench (bench/fusion_bench.mm): the
    frozen set at --ablation-qubits, unfused (one pass per gate) against the
    default fused plan; speedup and pass ratio per circuit, geometric mean."""
    import math
    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    n = args.ablation_qubits
    sim = qm.Simulator(n)
    rows, logsum = {}, 0.0
    with ClockSampler(0) as clocks:
        for name, gates in benchmark_set(n):
            c = W.to_circuit(n, gates)
            p0, p1 = c.plan_size(fuse=False), c.plan_size(fuse=True)
            t0 = time_plan(sim, c, args.steps, unfused=True)
            t1 = time_plan(sim, c, args.steps)
            t0 = min(t0, time_plan(sim, c, args.steps, unfused=True))
            t1 = min(t1, time_plan(sim, c, args.steps))
            rows[name] = {"gates": len(gates), "passes_unfused": p0, "passes_fused": p1,
                          "unfused_s": round(t0, 5), "fused_s": round(t1, 5),
                          "speedup": round(t0 / t1, 2), "pass_ratio": round(p0 / p1, 2)}
            logsum += math.log(t0 / t1)
    if rank == 0:
        print(json.dumps({
            "metric": "fusion_speedup_geomean", "value": round(math.exp(logsum / len(rows)), 3),
            "unit": "x", "n_gpus": world, "steps": args.steps, "higher_is_better": True,
            "dtype": "c64", "data": "synthetic",
            "config": {"workload": f"reference frozen benchmark set at n={n}, unfused vs fused "
                                   "plan, best of steps", "num_qubits": n},
            "circuits": rows, "clocks": clocks.summary()}), flush=True)


def run_ablation_workload(args, world, rank, dist):
    """Port of the reference's ablation (bench/ablation.mm): four arms --
    no fusion, fusion, blocking alone, fusion + blocking (2^bits amplitude
    blocks) -- interleaved, on the extended set; F/base, B/base and FB/F per
    circuit and their geometric means. A fifth arm, FBR, tests the qubit
    reordering the reference left untested (results/S4_RESULT.md): the
    wires with the most one-qubit gates are relabeled into the block window,
    the relabeled circuit runs fused and blocked, and one permutation pass
    restores the qubit order (timed)."""
    import math
    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    n, bits = args.ablation_qubits, args.block_bits
    none = dict(collapse=False, diagonals=False, zz=False, group=1, block_bits=0)
    arms = {"base": none, "F": dict(), "B": dict(none, block_bits=bits),
            "FB": dict(block_bits=bits)}
    sim = qm.Simulator(n)
    rows = {}
    logs = {"F/base": 0.0, "B/base": 0.0, "FB/F": 0.0, "FBR/F": 0.0}
    with ClockSampler(0) as clocks:
        for name, gates in benchmark_set(n, extended=True):
            c = W.to_circuit(n, gates)
            sizes = {a: int(c.plan_export(**o)[0]) for a, o in arms.items()}
            perm = W.hot_wires_first(n, gates)
            back = [0] * n
            for q, p in enumerate(perm):
                back[p] = q
            cr = W.to_circuit(n, W.relabel(gates, perm))
            sizes["FBR"] = int(cr.plan_export(block_bits=bits)[0]) + 1

            def remap_arm():
                best = float("inf")
                for _ in range(args.steps + 1):
                    sim.reset()
                    sim.elapsed()
                    sim.run_options(cr, block_bits=bits)
                    sim.permute_qubits(back)
                    best = min(best, sim.elapsed())
                return best

            t = {a: time_plan(sim, c, args.steps, **o) for a, o in arms.items()}
            t["FBR"] = remap_arm()
            for a, o in arms.items():      # second interleaved round, best of both
                t[a] = min(t[a], time_plan(sim, c, args.steps, **o))
            t["FBR"] = min(t["FBR"], remap_arm())
            r = {"F/base": t["base"] / t["F"], "B/base": t["base"] / t["B"],
                 "FB/F": t["F"] / t["FB"], "FBR/F": t["F"] / t["FBR"]}
            for k in logs:
                logs[k] += math.log(r[k])
            rows[name] = {"plan_ops": sizes, "seconds": {a: round(v, 5) for a, v in t.items()},
                          **{k: round(v, 2) for k, v in r.items()}}
    if rank == 0:
        geo = {k: round(math.exp(v / len(rows)), 3) for k, v in logs.items()}
        print(json.dumps({
            "metric": "blocking_on_top_of_fusion_geomean", "value": geo["FB/F"], "unit": "x",
            "n_gpus": world, "steps": args.steps, "higher_is_better": True, "dtype": "c64",
            "data": "synthetic",
            "config": {"workload": f"reference extended benchmark set at n={n}, four arms, "
                                   f"block 2^{bits} amplitudes", "num_qubits": n,
                       "block_bits": bits},
            "geomean": geo, "circuits": rows, "clocks": clocks.summary()}), flush=True)


def main():
    global N_CPU
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=N_QUBITS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scale", action="store_true",
                    help="skip the GHZ / QFT runs at 33 and 34 qubits")
    ap.add_argument("--workload", default="fused30",
                    choices=["fused30", "batch", "grad", "fusion", "ablation"])
    ap.add_argument("--ablation-qubits", type=int, default=26,
                    help="width of the fusion / ablation bench ports")
    ap.add_argument("--block-bits", type=int, default=10,
                    help="ablation: cache-blocking window, log2 amplitudes")
    ap.add_argument("--grad-qubits", type=int, nargs="+", default=[28, 33])
    ap.add_argument("--grad-reps", type=int, default=3,
                    help="timed block-wise gradients per width in the default run's grad key")
    ap.add_argument("--batch-steps", type=int, default=3,
                    help="timed batches in the default run's batch key")
    ap.add_argument("--no-grad", action="store_true",
                    help="default run: leave out the gradient configuration (grad key)")
    ap.add_argument("--no-batch", action="store_true",
                    help="default run: leave out the batched-serving configuration (batch key)")
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--lanes", type=int, default=0,
                    help="batch lanes; 0 = autotuned on the batch's own requests")
    ap.add_argument("--widths", type=int, nargs="+", default=None,
                    help="batch: keep only the requests of these widths (profiling cases)")
    ap.add_argument("--no-loops", action="store_true",
                    help="batch / grad: time the block-wise path only (no per-circuit loops, "
                         "no gate-by-gate sweep, no oracle or difference checks)")
    ap.add_argument("--cpu-qubits", type=int, default=N_CPU,
                    help="width of the bounded CPU sample (reference arm, cpu_baseline)")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    N_CPU = args.cpu_qubits
    if args.workload == "batch" and args.impl != "reference":
        run_batch_workload(args, world, rank, dist)
        return
    if args.workload == "grad" and args.impl != "reference":
        run_grad_workload(args, world, rank, dist)
        return
    if args.workload == "fusion" and args.impl != "reference":
        run_fusion_workload(args, world, rank, dist)
        return
    if args.workload == "ablation" and args.impl != "reference":
        run_ablation_workload(args, world, rank, dist)
        return
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        barrier(dist, world)
        return

    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    n = args.qubits
    S = 8.0 * (1 << n)
    circuits, kinds, gate_streams = [], [], []
    for name, gates in workload(n):
        c = W.to_circuit(n, gates)
        circuits.append((name, c))
        kinds.append(plan_kinds(c.plan_export()))
        gate_streams.append(gates)
    step_bytes = sum(circuit_bytes(k, n) for k in kinds)
    sim = qm.Simulator(n)

    def step():
        for _name, c in circuits:
            sim.reset()
            sim.run(c)

    for _ in range(max(args.warmup, 3)):
        step()
    sim.synchronize()
    torch_sync()
    barrier(dist, world)

    # --- device-timed region: per-op CUDA events on the simulator's stream ---
    per_kind_time = {k: 0.0 for k in range(7)}
    per_kind_count = {k: 0 for k in range(7)}
    d0 = sim.dispatch_count
    with ClockSampler(0 if world == 1 else local) as clocks:
        sim.elapsed()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for (name, c), ks in zip(circuits, kinds):
                sim.reset()
                secs = sim.run_profiled(c)
                for k, s in zip(ks, secs):
                    per_kind_time[k] += s
                    per_kind_count[k] += 1
        dev = sim.elapsed()
        wall = time.perf_counter() - t0
    launches = sim.dispatch_count - d0
    torch_sync()
    barrier(dist, world)
    dev_max = max_over_ranks(dev, dist, world)
    value = world * args.steps * step_bytes / dev_max / 1e9

    # --- roofline of the dominant kernel ---------------------------------------
    peak, peak_src = peaks()
    dom = max(per_kind_time, key=lambda k: per_kind_time[k])
    dom_bytes = per_kind_count[dom] * op_bytes(dom, n)
    achieved = dom_bytes / per_kind_time[dom] / 1e9 if per_kind_time[dom] > 0 else 0.0
    breakdown = {OP_NAMES[k]: {"ops": per_kind_count[k] // max(args.steps, 1),
                               "ms_per_step": round(1e3 * per_kind_time[k] / args.steps, 3),
                               "gbs": round(per_kind_count[k] * op_bytes(k, n) / per_kind_time[k] / 1e9, 1)
                               if per_kind_time[k] > 0 else None}
                 for k in range(7) if per_kind_count[k]}

    # --- end to end through the C ABI, host gate arrays ----------------------
    h2d = sum(sum(4 + 4 * len(q) + 8 * len(p) for _k, q, p in g) for g in gate_streams)
    shots = 1024
    d2h = len(circuits) * (shots * 8 + 8)
    sim.synchronize()
    torch_sync()
    barrier(dist, world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for gates in gate_streams:
            c = W.to_circuit(n, gates)
            sim.reset()
            sim.run(c)
            sim.sample(shots, 7)
            sim.norm()
    sim.synchronize()
    e2e_wall = max_over_ranks(time.perf_counter() - t0, dist, world)
    e2e_value = world * args.steps * step_bytes / e2e_wall / 1e9

    # --- the executor's merged form of the same plans (qm_run_merged): wider
    # one-qubit passes and CX / SWAP runs as one permutation pass. Outside the
    # roofline line, which is charged on the reference plan op for op.
    merged = {}
    for name, c in circuits:
        sim.reset()
        sim.run_merged(c)              # warm (takes the scratch buffer once)
        sim.reset()
        sim.elapsed()
        d0m = sim.dispatch_count
        sim.run_merged(c)
        tm = sim.elapsed()
        merged[name] = {"s": round(tm, 5), "launches": sim.dispatch_count - d0m,
                        "plan_ops": c.plan_size()}
    merged_s = sum(v["s"] for v in merged.values()) / len(merged)

    # --- scale: GHZ and QFT at 33 and 34 qubits (64 / 128 GiB in place) -------
    scale = {}
    if not args.no_scale:
        sim.close()
        del sim
        for ns in (33, 34):
            try:
                big = qm.Simulator(ns)
            except qm.QMetalError as e:
                scale[f"n{ns}"] = {"skipped": str(e)}
                continue
            for name, gates in (("ghz", W.ghz(ns)), ("qft", W.qft(ns))):
                c = W.to_circuit(ns, gates)
                ks = plan_kinds(c.plan_export())
                big.reset()
                big.run(c)
                big.synchronize()
                big.elapsed()
                big.reset()
                big.run(c)
                t = big.elapsed()
                nbytes = circuit_bytes(ks, ns)
                entry = {"gates": len(gates), "plan_ops": len(ks), "s_per_circuit": round(t, 4),
                         "gbs": round(nbytes / t / 1e9, 1),
                         "frac": round(nbytes / t / 1e9 / peaks()[0], 4),
                         "norm": big.norm(), "z0": big.expectation_pauli(z_mask=1)}
                if name == "ghz":
                    entry["z0_zlast"] = big.expectation_pauli(z_mask=1 | (1 << (ns - 1)))
                # The merged executor: GHZ's CX chain and QFT's closing
                # swaps become one permutation pass each (a second state
                # buffer, taken while the device has room).
                big.reset()
                big.run_merged(c)
                big.synchronize()
                big.elapsed()
                big.reset()
                big.run_merged(c)
                tm = big.elapsed()
                entry["merged"] = {"s_per_circuit": round(tm, 4), "norm": big.norm(),
                                   "z0": big.expectation_pauli(z_mask=1)}
                if name == "ghz":
                    entry["merged"]["z0_zlast"] = big.expectation_pauli(
                        z_mask=1 | (1 << (ns - 1)))
                scale[f"{name}_{ns}"] = entry
            big.close()
            del big

    # --- the gradient and batched-serving configurations, as sub-keys -------
    grad = None
    if not args.no_grad:
        grad = grad_results(args.grad_qubits, reps=args.grad_reps, gate_by_gate=True,
                            oracle_qubits=22)
    batch = None
    if not args.no_batch:
        batch = batch_results(args.requests, steps=args.batch_steps, warmup=3, lanes=args.lanes,
                              loops=True, oracle_max_n=16, dist=dist, world=world, rank=rank)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        rate, secs = cpu_sample(1, repeats=3)
        cpu = {"value": round(rate, 4), "unit": "GB/s", "cores": 1,
               "kind": "reference" if oracle.ref_available() else "port",
               "sample": f"the 4 fused plans 3 times at n={N_CPU}, complex128, plan op by "
                         f"op, 1 thread, {secs:.1f} s"}

    if rank == 0:
        ops_per_circuit = [len(k) for k in kinds]
        line = {
            "metric": "fused_plan_hbm_gbs", "value": round(value, 2), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": round(1e3 * dev_max / args.steps, 3),
            "s_per_circuit": round(dev_max / args.steps / len(circuits), 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64", "data": "synthetic",
            "config": {"workload": f"fused plans at n={n} from |0>: "
                                   + ", ".join(c for c, _ in circuits),
                       "num_qubits": n, "state_gib": S / 2 ** 30,
                       "plan_ops": dict(zip([c for c, _ in circuits], ops_per_circuit)),
                       "bytes_per_step": step_bytes,
                       "l2": "inputs larger than L2 (state >> 129 MB), no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "kernel": OP_NAMES[dom], "achieved": round(achieved, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "peak_source": peak_src,
                         "traffic": (round(DRAM_PER_ALGO_BYTE[dom] * op_bytes(dom, n))
                                     if dom in DRAM_PER_ALGO_BYTE else None),
                         "traffic_source": (f"ncu dram bytes per launch at "
                                            f"n={DRAM_CAPTURE_QUBITS[dom]}, scaled by units "
                                            f"to n={n}") if dom in DRAM_CAPTURE_QUBITS
                                           else None},
            "kernels": breakdown,
            "frac_of_peak_overall": round(value / world / peak, 4),
            "e2e": {"value": round(e2e_value, 2), "unit": "GB/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "scale": scale,
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
            "wall_s_timed": round(wall, 3),
            "merged": {"s_per_circuit": round(merged_s, 5),
                       "speedup_vs_plan": round(dev_max / args.steps / len(circuits) / merged_s, 3),
                       "circuits": merged},
            "grad": grad,
            "batch": batch,
        }
        print(json.dumps(line), flush=True)
    barrier(dist, world)


if __name__ == "__main__":
    main()
