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
the host cores on a bounded sample (the same circuits at 20 qubits).

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
# DRAM bytes (read + write) per algorithmic byte of one launch, from the full
# ncu captures at 26 qubits (profiles/group_diag_n26_full.md: k_group<4,0>
# 536.9 + 475.8 MB, k_diag 537.0 + 477.4 MB against 2S = 1073.7 MB). The
# traffic grows with the state, so a launch at n qubits moves this fraction
# of its 2S.
DRAM_PER_ALGO_BYTE = {1: (536.9 + 475.8) / 1073.7, 4: (537.0 + 477.4) / 1073.7}
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


def cpu_oracle_run(n, gates):
    import oracle
    t0 = time.perf_counter()
    oracle.run(n, gates)
    return time.perf_counter() - t0


def cpu_sample(threads, copies=1, repeats=1):
    """The complex128 oracle (gate by gate, the reference's CPU algorithm) on
    the workload's circuits at N_CPU qubits, each gate loop on one thread;
    `threads` instances run concurrently. Returns (GB/s-equivalent, secs)."""
    import oracle
    import qmetal_gb300 as qm  # noqa: F401  (plan kinds come from the library)
    from qmetal_gb300 import workloads as W
    oracle.set_threads(1)
    jobs, total_bytes = [], 0.0
    for _name, gates in workload(N_CPU):
        kinds = plan_kinds(W.to_circuit(N_CPU, gates).plan_export())
        for _ in range(copies * repeats):
            jobs.append(gates)
            total_bytes += circuit_bytes(kinds, N_CPU)
    t0 = time.perf_counter()
    if threads == 1:
        for g in jobs:
            cpu_oracle_run(N_CPU, g)
    else:
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda g: cpu_oracle_run(N_CPU, g), jobs))
    dt = time.perf_counter() - t0
    return total_bytes / dt / 1e9, dt


def run_reference(args, world, rank, dist):
    """The reference's CPU implementation of the path (the oracle port of its
    complex128 Reference; its own sources are not on this machine), all host
    threads, each step a bounded sample: every workload circuit at N_CPU
    qubits, cores/4 copies of each run concurrently."""
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
    kind = "reference" if oracle.ref_available() else "port"
    line = {
        "impl": "reference", "metric": "fused_plan_hbm_gbs", "value": round(value, 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": f"fused-plan circuits of the 30-qubit config, run at {N_CPU} "
                               "qubits on the host (bounded sample)",
                   "num_qubits": N_CPU, "circuits": [c for c, _ in workload(4)],
                   "copies_per_circuit": copies},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                         "kind": kind,
                         "sample": f"4 circuits x {copies} copies at n={N_CPU}, complex128, "
                                   f"gate by gate, {threads} threads"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batch_workload(args, world, rank, dist):
    """512 QAOA MaxCut requests (n uniform over the even widths 12..26, p in
    1..8, random 3-regular graphs, angles ~ U[0, pi]), each energy + adjoint
    gradient + 4096 samples. A step serves the whole batch with concurrent
    lanes; the per-circuit loop a caller of the reference API would write
    (gate-by-gate gradient, run, sample) is timed once beside it, and so is
    the loop with the block-wise gradient. Wall clock, host buffers."""
    import numpy as np
    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    insts = W.maxcut_instances(args.requests, seed=6)
    if args.widths:
        insts = [i for i in insts if i["n"] in args.widths]
    reqs = []
    for k, inst in enumerate(insts):
        gates = W.maxcut_qaoa(inst["n"], inst["edges"], inst["gammas"], inst["betas"])
        reqs.append((W.to_circuit(inst["n"], gates),
                     W.to_hamiltonian(W.maxcut_hamiltonian(inst["edges"])), 4096, 7000 + k))
    params = sum(len(c) for c, _h, _s, _seed in reqs)

    tuning = qm.batch_autotune(reqs) if args.lanes == 0 else None

    def serve(mode):
        torch_sync()
        t0 = time.perf_counter()
        out = qm.batch_serve(reqs, mode=mode, lanes=args.lanes)
        return out, time.perf_counter() - t0

    for _ in range(max(args.warmup, 3)):
        serve(qm.BATCH_LANES)
    barrier(dist, world)
    with ClockSampler(0 if world == 1 else int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        times = []
        for _ in range(args.steps):
            lanes_out, dt = serve(qm.BATCH_LANES)
            times.append(dt)
    wall = max_over_ranks(sum(times), dist, world)
    # The same batch recorded into one CUDA graph and launched once (tile
    # shapes from the tuning above); wall clock includes recording.
    graph_runs = []
    for _ in range(2):
        graph_out, graph_t = serve(qm.BATCH_GRAPH)
        graph_runs.append((graph_t, qm.batch_graph_timing()))
    graph_t, graph_timing = min(graph_runs, key=lambda r: r[0])
    graph_diff = max(float(np.max(np.abs(np.array(a[1]) - np.array(b[1])))) for a, b in
                     zip(lanes_out, graph_out))
    if args.no_loops:
        plain_out, plain_t = lanes_out, float("nan")
        fused_out, fused_t = lanes_out, float("nan")
    else:
        plain_out, plain_t = serve(qm.BATCH_PLAIN_LOOP)
        fused_out, fused_t = serve(qm.BATCH_FUSED_LOOP)
    gdiff = max(float(np.max(np.abs(np.array(a[1]) - np.array(b[1])))) for a, b in
                zip(lanes_out, plain_out))
    ediff = max(abs(a[0] - b[0]) for a, b in zip(lanes_out, plain_out))
    oracle_err = None
    if rank == 0 and not args.no_loops:
        import oracle
        oracle.build()
        e_worst = g_worst = g_rel = 0.0
        checked = 0
        for (c, _h, _s, _seed), inst, got in zip(reqs, insts, lanes_out):
            if inst["n"] > 16:
                continue
            gates = W.maxcut_qaoa(inst["n"], inst["edges"], inst["gammas"], inst["betas"])
            e0, g0 = oracle.energy_and_gradient(inst["n"], gates,
                                                W.maxcut_hamiltonian(inst["edges"]))
            gd = float(np.max(np.abs(np.array(got[1]) - g0)))
            e_worst = max(e_worst, abs(got[0] - e0))
            g_worst = max(g_worst, gd)
            g_rel = max(g_rel, gd / max(float(np.max(np.abs(g0))), 1e-30))
            checked += 1
        oracle_err = {"requests_checked": checked, "widths": "n <= 16",
                      "max_abs_energy_err": e_worst, "max_abs_grad_err": g_worst,
                      "max_grad_err_rel_to_max_grad": g_rel}
    value = world * args.steps * len(reqs) / wall
    if rank == 0:
        widths = sorted({i["n"] for i in insts})
        line = {
            "metric": "batched_adjoint_requests_per_s", "value": round(value, 2),
            "unit": "requests/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(1e3 * wall / args.steps, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "synthetic",
            "config": {"workload": f"{len(reqs)} QAOA MaxCut requests (energy + adjoint "
                                   "gradient + 4096 samples each)",
                       "widths": widths, "gate_params": params,
                       "lanes": tuning["lanes"] if tuning else args.lanes,
                       "autotuned": tuning},
            "plain_loop": {"value": round(len(reqs) / plain_t, 2), "unit": "requests/s",
                           "seconds": round(plain_t, 3),
                           "what": "per-circuit loop: gate-by-gate adjoint, run, sample"},
            "blockwise_loop": {"value": round(len(reqs) / fused_t, 2), "unit": "requests/s",
                               "seconds": round(fused_t, 3)},
            "graph": {"value": round(len(reqs) / graph_t, 2), "unit": "requests/s",
                      "seconds": round(graph_t, 3),
                      "record_s": round(graph_timing["record_s"], 3),
                      "instantiate_s": round(graph_timing["instantiate_s"], 3),
                      "execute_s": round(graph_timing["execute_s"], 3),
                      "nodes": graph_timing["nodes"],
                      "max_grad_diff_vs_lanes": graph_diff,
                      "what": "every request recorded into one CUDA graph, one launch"},
            "speedup_vs_plain_loop": round(plain_t / (wall / args.steps), 2),
            "max_grad_diff_vs_plain": gdiff, "max_energy_diff_vs_plain": ediff,
            "err_vs_complex128_oracle": oracle_err,
            "clocks": clocks.summary(),
        }
        if args.no_loops:
            for key in ("plain_loop", "blockwise_loop", "speedup_vs_plain_loop",
                        "max_grad_diff_vs_plain", "max_energy_diff_vs_plain"):
                line[key] = None
        print(json.dumps(line), flush=True)
    barrier(dist, world)


def run_grad_workload(args, world, rank, dist):
    """Adjoint gradients of the HEA depth-8 problem (RY + RZ per wire per
    layer, CX ladder; H = -sum Z_i Z_{i+1} - 0.7 sum X_i on a ring) at 28 and
    33 qubits: device time per gradient with the block-wise sweep (the
    default) and with the reference's gate-by-gate sweep, and a central
    difference check (eps = 1e-3) on a few parameters."""
    import numpy as np
    import qmetal_gb300 as qm
    from qmetal_gb300 import workloads as W
    results = {}
    for n in args.grad_qubits:
        gates, terms = W.hea_gradient_problem(n, depth=8, seed=5)
        c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
        nparams = sum(1 for g in gates if g[2])
        sim = qm.Simulator(n)
        entry = {"gates": len(gates), "params": nparams}
        modes = (("blockwise", True),) if args.no_loops else \
            (("blockwise", True), ("gate_by_gate", False))
        for label, fused in modes:
            sim.energy_and_gradient(c, h, fused=fused)      # warm-up
            sim.elapsed()
            reps = args.steps if fused else 1
            for _ in range(reps):
                e, g = sim.energy_and_gradient(c, h, fused=fused)
            t = sim.elapsed() / reps
            entry[label] = {"s_per_gradient": round(t, 4), "grad_per_s": round(1.0 / t, 3),
                            "param_grads_per_s": round(nparams / t, 1)}
            entry.setdefault("energy", e)
            entry.setdefault("_grad", g)
        g = entry.pop("_grad")
        if args.no_loops:
            results[f"n{n}"] = entry
            sim.close()
            del sim
            continue
        entry["speedup"] = round(entry["gate_by_gate"]["s_per_gradient"]
                                 / entry["blockwise"]["s_per_gradient"], 2)
        worst = 0.0
        eps = 1e-3
        for j in (0, len(gates) // 2, len(gates) - n - 2):
            while not gates[j][2]:
                j += 1
            kind, qs, ps = gates[j]
            plus = list(gates); plus[j] = (kind, qs, (ps[0] + eps,))
            minus = list(gates); minus[j] = (kind, qs, (ps[0] - eps,))
            sim.reset(); sim.run(W.to_circuit(n, plus)); ep = sim.expectation(h)
            sim.reset(); sim.run(W.to_circuit(n, minus)); em = sim.expectation(h)
            worst = max(worst, abs((ep - em) / (2 * eps) - g[j]))
        entry["max_abs_diff_vs_central_difference"] = worst
        results[f"n{n}"] = entry
        sim.close()
        del sim
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

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        rate, secs = cpu_sample(1, repeats=3)
        cpu = {"value": round(rate, 4), "unit": "GB/s", "cores": 1,
               "kind": "reference" if oracle.ref_available() else "port",
               "sample": f"the 4 circuits 3 times at n={N_CPU}, complex128 gate by gate, "
                         f"1 thread, {secs:.1f} s"}

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
                         "traffic_source": "ncu dram bytes per launch at n=26, scaled by "
                                           "units to this n"},
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
        }
        print(json.dumps(line), flush=True)
    barrier(dist, world)


if __name__ == "__main__":
    main()
