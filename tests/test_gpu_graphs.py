"""CUDA-graph replay of repeated circuits (qm_run_cached).

The graph holds the same kernels with the same arguments as run(), so the
replayed state must be bit-identical to run()'s, every replay; the oracle
bounds both. Covers a repeat of one circuit, parameter changes (a new graph),
and more distinct circuits than the cache keeps (eviction, then recapture).
"""
import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _states(n, gates, repeats):
    c = W.to_circuit(n, gates)
    plain = qm.Simulator(n)
    plain.run(c)
    want = plain.get_state()
    sim = qm.Simulator(n)
    got = []
    for _ in range(repeats):
        sim.reset()
        sim.run_cached(c)
        got.append(sim.get_state())
    return want, got


@pytest.mark.parametrize("n", [6, 14, 20])
def test_replay_matches_run(n):
    gates = W.hea(n, 3, seed=5 + n)
    want, got = _states(n, gates, 4)
    ref = oracle.run(n, gates)
    assert np.abs(want - ref).max() <= 1e-4
    for g in got:
        assert np.array_equal(g, want)


def test_new_parameters_recapture():
    n = 12
    sim = qm.Simulator(n)
    for seed in range(3):
        gates = W.qaoa_ring_seeded(n, 2, seed=seed)
        c = W.to_circuit(n, gates)
        for _ in range(2):
            sim.reset()
            sim.run_cached(c)
            assert np.abs(sim.get_state() - oracle.run(n, gates)).max() <= 1e-4


def test_eviction_and_dispatch_count():
    n = 10
    sim = qm.Simulator(n)
    circuits = [W.random_u3(n, 2, seed=s) for s in range(20)]
    for rep in range(2):
        for gates in circuits:
            sim.reset()
            sim.run_cached(W.to_circuit(n, gates))
            assert np.abs(sim.get_state() - oracle.run(n, gates)).max() <= 1e-4
    # A replay counts the graph's kernels, like run() would.
    c = W.to_circuit(n, circuits[-1])
    before = sim.dispatch_count
    sim.run(c)
    per_run = sim.dispatch_count - before
    before = sim.dispatch_count
    sim.run_cached(c)
    assert sim.dispatch_count - before == per_run
