"""The benchmark sets of the fusion and ablation bench ports (CPU only).

The reference's fusion_bench at 26 qubits lists each frozen circuit's gate
count (results/fusion_bench_n26.txt in the reference project): the set
rebuilt here from the restated generators and the recorded mt19937 streams
must have the same counts. The ablation set's extra member (local_patch,
recorded from the reference's generator) must lower to plans that reproduce
it in complex128 under every arm's options.
"""
import importlib.util
import os

import numpy as np
import pytest

import oracle
from qmetal_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_frozen_set_gate_counts_match_reference_bench():
    want = {"ghz": 26, "qft": 351, "qaoa_ring_p6": 650, "tfim_trotter_20": 2020,
            "grover_proxy_4": 450, "random_d10": 385, "hea_d3": 231}
    got = {name: len(g) for name, g in _bench().benchmark_set(26)}
    assert got == want
    ext = dict(_bench().benchmark_set(26, extended=True))
    assert set(ext) == set(want) | {"local_patch_w8", "local_patch_w8_high"}


@pytest.mark.parametrize("opts", [dict(), dict(collapse=False, diagonals=False, zz=False,
                                                group=1, block_bits=8),
                                  dict(block_bits=8)])
def test_local_patch_plans_reproduce_the_circuit(opts, golden_circuits):
    n = 14
    gates = [(k, tuple(q), tuple(p)) for k, q, p in golden_circuits["local_patch_14_8_12_0x10ca1"]]
    want = oracle.run(n, gates)
    got = oracle.run_plan(n, W.to_circuit(n, gates).plan_export(**opts))
    assert np.abs(got - want).max() <= 1e-12


def test_hot_wire_relabeling_round_trip(golden_circuits):
    """The reordering arm's relabeling on the CPU: the relabeled circuit's
    state, with its qubit axes moved back, is the original circuit's."""
    n = 14
    gates = [(k, tuple(q), tuple(p)) for k, q, p in golden_circuits["local_patch_14_8_12_0x10ca1"]]
    gates = W.relabel(gates, [n - 1 - q for q in range(n)])
    perm = W.hot_wires_first(n, gates)
    assert sorted(perm) == list(range(n))
    counts = [sum(1 for _k, qs, _p in gates if len(qs) == 1 and qs[0] == q) for q in range(n)]
    by_new = sorted(range(n), key=lambda q: perm[q])
    assert [counts[q] for q in by_new] == sorted(counts, reverse=True)
    st = oracle.run(n, W.relabel(gates, perm)).reshape([2] * n)
    back = np.moveaxis(st, [n - 1 - perm[q] for q in range(n)], [n - 1 - q for q in range(n)])
    assert np.abs(back.reshape(-1) - oracle.run(n, gates)).max() <= 1e-12
