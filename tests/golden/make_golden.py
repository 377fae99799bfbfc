"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a checkout where the reference sources are available (the oracle's
build_ref.sh compiles them into oracle/_ref/libqref.so):

    python tests/golden/make_golden.py

Writes:
  circuits.json   gate streams of the reference's seeded generators
                  (random_circuit, hardware_efficient: they draw from
                  std::mt19937_64 through libstdc++'s distributions, so the
                  streams are recorded rather than regenerated), keyed
                  "<name>_<n>_<depth>_<seed>".
  reference.npz   outputs of the reference's own code for small cases:
                  final states (Reference::run from |0> or from a recorded
                  random state), flat plans (build_plan) for the frozen set,
                  and Pauli expectations (Reference::expectation).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from qmetal_gb300 import workloads as W  # noqa: E402

SEEDED = [
    ("random_circuit", 10, 4, 0xABC),        # expectation test
    ("hardware_efficient", 8, 2, 0xFEED),    # Hamiltonian-sum test
    ("random_circuit", 6, 3, 0x1234),        # sampling test
    ("hardware_efficient", 6, 2, 0xC0FFEE),  # gradient test
    ("random_circuit", 5, 4, 0xABC),
]
FROZEN_N = [4, 6, 7, 10, 11, 14, 20]
BENCH_N = [26]           # the width of the reference's fusion and ablation benches


def frozen(n):
    """The frozen benchmark set (src/circuits.cpp:171-182) at width n."""
    return {
        "ghz": W.ghz(n),
        "qft": W.qft(n),
        "qaoa_ring_p6": W.qaoa_ring(n, 6),
        "tfim_trotter_20": W.tfim_trotter(n, 20),
        "grover_proxy_4": W.grover_proxy(n, 4),
        "random_d10": oracle.ref_circuit("random_circuit", n, 10, 0, 0x5EED),
        "hea_d3": oracle.ref_circuit("hardware_efficient", n, 3, 0, 0x5EED),
    }


def main():
    if not oracle.ref_available():
        if oracle.build_ref() is None:
            raise SystemExit("reference sources not found; cannot generate fixtures")
    circuits = {}
    for name, n, d, seed in SEEDED:
        circuits[f"{name}_{n}_{d}_{seed:#x}"] = oracle.ref_circuit(name, n, d, 0, seed)
    for n in FROZEN_N + BENCH_N:
        circuits[f"random_circuit_{n}_10_0x5eed"] = oracle.ref_circuit("random_circuit", n, 10, 0, 0x5EED)
        circuits[f"hardware_efficient_{n}_3_0x5eed"] = oracle.ref_circuit("hardware_efficient", n, 3, 0, 0x5EED)
    # The ablation set's extra member, local_patch(n, 8, 12) with its default
    # seed (src/circuits.cpp:133-168, include/qmetal/circuits.h:57-58).
    for n in (14,) + tuple(BENCH_N):
        circuits[f"local_patch_{n}_8_12_0x10ca1"] = oracle.ref_circuit("local_patch", n, 8, 12, 0x10CA1)
    with open(os.path.join(HERE, "circuits.json"), "w") as f:
        json.dump({k: [[g[0], list(g[1]), list(g[2])] for g in v] for k, v in circuits.items()}, f)

    arrays = {}
    rng = np.random.default_rng(2024)
    # Final states of the reference, from |0> and from a recorded random state.
    for n in (4, 7):
        for name, gates in frozen(n).items():
            arrays[f"state/{name}/{n}"] = oracle.ref_run(n, gates)
    for n in (6, 9):
        init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        init /= np.linalg.norm(init)
        arrays[f"init/qft_swap/{n}"] = init
        arrays[f"state/qft_swap/{n}"] = oracle.ref_run(n, W.qft_swap(n), init)
    # Plans (build_plan) of the frozen set under the option sets the reference tests use.
    opts = {"all": {}, "none": dict(collapse=False, diagonals=False, zz=False, group=1),
            "diag": dict(collapse=False), "win": dict(diagonals=False, zz=False),
            "blocked8": dict(block_bits=8)}
    for n in (4, 7, 11):
        for name, gates in frozen(n).items():
            for tag, o in opts.items():
                arrays[f"plan/{name}/{n}/{tag}"] = oracle.ref_plan(n, gates, **o)
    # Pauli expectations on a state with no symmetry left.
    st = oracle.ref_run(10, circuits["random_circuit_10_4_0xabc"])
    prng = np.random.default_rng(7)
    masks = []
    for _ in range(24):
        x = y = z = 0
        for q in range(10):
            r = int(prng.integers(0, 4))
            if r == 1: x |= 1 << q
            elif r == 2: y |= 1 << q
            elif r == 3: z |= 1 << q
        masks.append((x, y, z))
    arrays["pauli/masks"] = np.array(masks, dtype=np.uint64)
    arrays["pauli/values"] = np.array([oracle.ref_expectation(10, st, *m) for m in masks])
    np.savez_compressed(os.path.join(HERE, "reference.npz"), **arrays)
    print(f"wrote {len(circuits)} circuits and {len(arrays)} arrays")


if __name__ == "__main__":
    main()
