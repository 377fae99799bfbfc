"""Batched serving: many QAOA MaxCut requests of uneven widths in one call.

Every mode (concurrent lanes, the per-circuit loop with the reference's
gate-by-gate gradient, the loop with the block-wise gradient) must return the
same energies, gradients and samples, and they must match the complex128
oracle's adjoint gradient within 1e-5 and its energy within 1e-4 (the
reference's bound for a Hamiltonian sum, tests/test_gpu.mm:329 and 427: the
MaxCut energy sums up to 39 ZZ terms of complex64 states). Tied QAOA
parameters are chain-rule sums of the per-gate entries (RZ(2 gamma),
RX(2 beta): factor 2).
"""
ETOL = 1e-4
GTOL = 1e-5
import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def requests(count, seed, n_lo=6, n_hi=12, shots=256):
    out = []
    for k, inst in enumerate(W.maxcut_instances(count, seed=seed, n_lo=n_lo, n_hi=n_hi)):
        gates = W.maxcut_qaoa(inst["n"], inst["edges"], inst["gammas"], inst["betas"])
        terms = W.maxcut_hamiltonian(inst["edges"])
        out.append((inst, gates, terms, shots, 1000 + k))
    return out


def run_mode(reqs, mode, lanes=6):
    items = [(W.to_circuit(inst["n"], g), W.to_hamiltonian(t), shots, seed)
             for inst, g, t, shots, seed in reqs]
    return qm.batch_serve(items, mode=mode, lanes=lanes)


def test_modes_agree_and_match_oracle():
    reqs = requests(24, seed=11)
    lanes = run_mode(reqs, qm.BATCH_LANES)
    plain = run_mode(reqs, qm.BATCH_PLAIN_LOOP)
    fused = run_mode(reqs, qm.BATCH_FUSED_LOOP)
    for (inst, gates, terms, shots, seed), a, b, c in zip(reqs, lanes, plain, fused):
        n = inst["n"]
        e0, g0 = oracle.energy_and_gradient(n, gates, terms)
        for e, g, _s in (a, b, c):
            assert abs(e - e0) <= ETOL
            assert np.abs(np.array(g) - g0).max() <= GTOL
        # lanes and the block-wise loop run identical kernel sequences per request
        assert a[2] == c[2] and a[1] == c[1] and a[0] == c[0]
        # every mode samples the same forward state
        assert a[2] == b[2]


def test_tied_parameter_gradients_and_samples():
    reqs = requests(6, seed=3, n_lo=8, n_hi=10, shots=4096)
    out = run_mode(reqs, qm.BATCH_LANES, lanes=3)
    for (inst, gates, terms, shots, seed), (e, g, s) in zip(reqs, out):
        n, edges, p = inst["n"], inst["edges"], len(inst["gammas"])

        def tied(grad):
            """Chain rule over the per-gate entries: RZ(2 gamma), RX(2 beta)."""
            dgamma, dbeta = np.zeros(p), np.zeros(p)
            k = n                           # after the Hadamard layer
            for layer in range(p):
                for _ in edges:
                    dgamma[layer] += 2.0 * grad[k + 1]
                    k += 3
                for _ in range(n):
                    dbeta[layer] += 2.0 * grad[k]
                    k += 1
            assert k == len(gates)
            return {"gammas": dgamma, "betas": dbeta}

        got = tied(g)
        _e0, g0 = oracle.energy_and_gradient(n, gates, terms)
        want = tied(g0)
        # Every per-gate entry within the gradient bound; a tied value sums K
        # of them times 2, so its bound is 2 sqrt(K) GTOL (independent
        # FP32 roundings add in quadrature).
        assert np.abs(np.array(g) - g0).max() <= GTOL
        bound = {"gammas": 2.0 * np.sqrt(len(edges)) * GTOL, "betas": 2.0 * np.sqrt(n) * GTOL}

        def energy(which, layer, shift):
            par = {"gammas": list(inst["gammas"]), "betas": list(inst["betas"])}
            par[which][layer] += shift
            return oracle.expectation_sum(n, oracle.run(n, W.maxcut_qaoa(
                n, edges, par["gammas"], par["betas"])), terms)

        h = 1e-3
        for which in ("gammas", "betas"):
            for layer in range(p):
                # the GPU's tied gradient against the oracle's adjoint
                assert abs(got[which][layer] - want[which][layer]) <= bound[which]
                # and the oracle's chain rule against a fourth-order central
                # difference of the oracle energy (truncation ~ h^4)
                fd = (-energy(which, layer, 2 * h) + 8 * energy(which, layer, h)
                      - 8 * energy(which, layer, -h) + energy(which, layer, -2 * h)) / (12 * h)
                assert abs(fd - want[which][layer]) <= 1e-6
        # every qubit's marginal within 5 sigma of the exact one
        probs = np.abs(oracle.run(n, gates)) ** 2
        draws = np.array(s, dtype=np.int64)
        idx = np.arange(1 << n)
        for q in range(n):
            p1 = probs[(idx >> q) & 1 == 1].sum()
            sigma = np.sqrt(max(p1 * (1 - p1), 1e-12) / len(draws))
            assert abs(np.mean((draws >> q) & 1) - p1) <= 5 * sigma + 1e-9, q
        assert 0 <= e <= len(edges)


def test_uneven_widths_up_to_20():
    reqs = requests(16, seed=5, n_lo=12, n_hi=20, shots=64)
    lanes = run_mode(reqs, qm.BATCH_LANES, lanes=8)
    fused = run_mode(reqs, qm.BATCH_FUSED_LOOP)
    for (inst, gates, terms, _s, _seed), a, b in zip(reqs, lanes, fused):
        assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2]
    inst, gates, terms, _s, _seed = reqs[0]
    e0, g0 = oracle.energy_and_gradient(inst["n"], gates, terms)
    assert abs(lanes[0][0] - e0) <= ETOL
    assert np.abs(np.array(lanes[0][1]) - g0).max() <= GTOL


def test_batch_errors_fail_closed():
    c = qm.Circuit(3)
    c.h(0).cp(0, 1, 0.3)   # CP carries a parameter without a generator
    h = qm.Hamiltonian().add_string(1.0, "ZII")
    with pytest.raises(qm.QMetalError, match="differentiable"):
        qm.batch_serve([(c, h, 8, 1)], mode=qm.BATCH_LANES)
    with pytest.raises(qm.QMetalError, match="mode"):
        qm.batch_serve([(c, h, 8, 1)], mode=7)


def test_autotuned_lanes_and_tile_shapes():
    """lanes = 0 tunes the lane count and each width's window tile on the
    batch itself; the tuned batch must still match the oracle, and a second
    batch over the same widths reuses the cached choice."""
    reqs = requests(12, seed=21, n_lo=8, n_hi=14, shots=128)
    items = [(W.to_circuit(inst["n"], g), W.to_hamiltonian(t), shots, seed)
             for inst, g, t, shots, seed in reqs]
    tuned = qm.batch_autotune(items)
    assert tuned["lanes"] in (2, 4, 8, 16)
    assert tuned["seconds"] > 0
    for n, k in tuned["tile_high"].items():
        assert 1 <= k <= min(6, n - 6), (n, k)
    again = qm.batch_autotune(items)
    assert again["lanes"] == tuned["lanes"] and again["tile_high"] == tuned["tile_high"]
    out = qm.batch_serve(items, mode=qm.BATCH_LANES, lanes=0)
    fused = run_mode(reqs, qm.BATCH_FUSED_LOOP)
    for (inst, gates, terms, _s, _seed), (e, g, s), b in zip(reqs, out, fused):
        e0, g0 = oracle.energy_and_gradient(inst["n"], gates, terms)
        assert abs(e - e0) <= ETOL
        assert np.abs(np.array(g) - g0).max() <= GTOL
        assert s == b[2]      # the forward state, hence the draws, is unchanged


def test_graph_mode_matches_the_loop():
    """BATCH_GRAPH records every request into one CUDA graph (branches per
    width, heavy widths split up to four ways) and launches it once: the kernel
    sequence per request is the block-wise loop's, so the results are the
    same bits; the oracle bounds them too."""
    reqs = requests(20, seed=31, n_lo=8, n_hi=16, shots=256)
    graph = run_mode(reqs, qm.BATCH_GRAPH, lanes=1)
    timing = qm.batch_graph_timing()
    assert timing["nodes"] > len(reqs) and timing["execute_s"] > 0
    fused = run_mode(reqs, qm.BATCH_FUSED_LOOP)
    for (inst, gates, terms, _s, _seed), a, b in zip(reqs, graph, fused):
        assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2]
        e0, g0 = oracle.energy_and_gradient(inst["n"], gates, terms)
        assert abs(a[0] - e0) <= ETOL
        assert np.abs(np.array(a[1]) - g0).max() <= GTOL
    # a second batch reuses nothing from the first and still agrees
    again = run_mode(reqs, qm.BATCH_GRAPH, lanes=1)
    assert [x[0] for x in again] == [x[0] for x in graph]


@pytest.mark.parametrize("n,count", [(10, None), (11, None), (14, 40), (16, 48), (13, 33)])
def test_dense_cost_layers_against_the_oracle(n, count):
    """Cost layers of 33 to 55 couplings: one 48-generator diagonal pass, or
    48 and then the rest (the complete graph on 11 vertices)."""
    rng = np.random.default_rng(n)
    edges = [(a, b) for a in range(n) for b in range(a + 1, n)]
    if count is not None:
        edges = [edges[k] for k in sorted(rng.choice(len(edges), count, replace=False))]
    gates = W.maxcut_qaoa(n, edges, rng.uniform(0, np.pi, 2), rng.uniform(0, np.pi, 2))
    terms = W.maxcut_hamiltonian(edges)
    e, g = qm.Simulator(n).energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    assert abs(e - e0) <= ETOL
    assert np.abs(np.array(g) - g0).max() <= GTOL
