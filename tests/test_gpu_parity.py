"""GPU parity: every kernel path against the complex128 oracle.

Restates the reference's GPU suite (tests/test_gpu.mm:54-480) through the
C ABI: each case runs the same gate stream through the oracle and the CUDA
simulator and bounds the largest amplitude difference. Tolerances are the
reference's: 1e-5 for single gates and expectations, 1e-4 for deep circuits,
Hamiltonian sums and gradients; norms are checked beside every comparison.
"""
import math

import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W
from conftest import frozen_set

pytestmark = pytest.mark.gpu

X, Y, Z, H, S, SDG, T, TDG, RX, RY, RZ, P = range(12)
CX, CY, CZ, SWAP, CP, CCX = 12, 13, 14, 15, 16, 17
TOL1 = 1e-5


def gpu_state(n, gates, mode="fused", init=None):
    sim = qm.Simulator(n)
    if init is not None:
        sim.set_state(init)
    if mode == "gates":
        for k, qs, ps in gates:
            sim.apply(k, qs, ps)
    else:
        sim.run(W.to_circuit(n, gates), fuse=(mode == "fused"))
    return sim.get_state(), sim


def compare(n, gates, mode="fused", init=None):
    want = oracle.run(n, gates, init)
    got, sim = gpu_state(n, gates, mode, init)
    return np.abs(got - want).max(), sim


@pytest.mark.parametrize("mode", ["fused", "unfused", "gates"])
def test_single_gates_every_wire(mode):
    n = 5
    spread = [(H, (i,), ()) for i in range(n)]
    for k in (X, Y, Z, H, S, SDG, T, TDG):
        for q in range(n):
            d, _ = compare(n, spread + [(k, (q,), ())], mode)
            assert d <= TOL1, (k, q)
    for k in (RX, RY, RZ, P):
        for q in range(n):
            d, _ = compare(n, spread + [(k, (q,), (0.7853981633974483 + 0.3 * q,))], mode)
            assert d <= TOL1, (k, q)


@pytest.mark.parametrize("mode", ["fused", "unfused", "gates"])
def test_two_qubit_gates_every_pair(mode):
    n = 4
    prep = [(H, (i,), ()) for i in range(n)] + [(RZ, (0,), (0.4,)), (RY, (2,), (0.9,))]
    for k in (CX, CY, CZ, SWAP):
        for a in range(n):
            for b in range(n):
                if a != b:
                    d, _ = compare(n, prep + [(k, (a, b), ())], mode)
                    assert d <= TOL1, (k, a, b)
    for th in (0.1, math.pi / 4, math.pi / 2, math.pi, -math.pi / 3):
        d, _ = compare(n, [(H, (i,), ()) for i in range(n)] + [(CP, (1, 3), (th,))], mode)
        assert d <= TOL1


@pytest.mark.parametrize("mode", ["fused", "gates"])
def test_ccx_every_triple(mode):
    n = 4
    prep = [(H, (i,), ()) for i in range(n)] + [(RZ, (0,), (0.55,))]
    for a in range(n):
        for b in range(n):
            for t in range(n):
                if len({a, b, t}) == 3:
                    d, _ = compare(n, prep + [(CCX, (a, b, t), ())], mode)
                    assert d <= TOL1, (a, b, t)


@pytest.mark.parametrize("n", [3, 6, 9, 12])
def test_every_kernel_on_every_wire_larger_states(n):
    """Each vectorised path (wire 0 in lanes, wires 1..5 inside a warp's
    512 bytes, higher wires as vector pairs) on a random state."""
    rng = np.random.default_rng(n)
    init = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)).astype(np.complex128)
    init /= np.linalg.norm(init)
    gates = []
    for q in range(n):
        gates += [(H, (q,), ()), (RZ, (q,), (0.3 + q,)), (T, (q,), ())]
    for a in range(n):
        b = (a + 1 + a % 3) % n
        if a != b:
            gates += [(CX, (a, b), ()), (CY, (b, a), ()), (CZ, (a, b), ()), (SWAP, (a, b), ()),
                      (CP, (b, a), (0.2 * a,))]
    if n >= 3:
        gates += [(CCX, (0, n - 1, n // 2), ()), (CCX, (n - 1, 1, 0), ())]
    for mode in ("fused", "unfused", "gates"):
        d, sim = compare(n, gates, mode, init)
        assert d <= 1e-5, mode
        assert abs(sim.norm() - 1) < 1e-5


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_register_groups_all_wire_sets(k):
    n = 8
    rng = np.random.default_rng(k)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    for trial in range(12):
        wires = sorted(rng.choice(n, size=k, replace=False).tolist())
        if trial == 0:
            wires = list(range(k))
        gates = []
        for q in wires:
            gates += [(RY, (q,), (float(rng.uniform(-3, 3)),)), (RX, (q,), (float(rng.uniform(-3, 3)),))]
        c = W.to_circuit(n, gates)
        sim = qm.Simulator(n)
        sim.set_state(init)
        sim.run_options(c, group=k)
        assert c.plan_size() >= 1
        want = oracle.run(n, gates, init)
        assert np.abs(sim.get_state() - want).max() <= 1e-5, wires


@pytest.mark.parametrize("k", [2, 3, 4, 5])
def test_register_groups_with_wires_inside_a_warp(k):
    """Groups mixing wires 0..5 (lane bits and shuffles) with up to four
    wires >= 6 (registers), on states large enough for the warp-tile path."""
    rng = np.random.default_rng(50 + k)
    for n in (6, 9, 12):
        init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        init /= np.linalg.norm(init)
        for trial in range(10):
            lowq = int(rng.integers(1, 6))
            rest = [q for q in range(n) if q != lowq]
            wires = sorted([lowq] + rng.choice(rest, size=k - 1, replace=False).tolist())
            gates = [(RY, (q,), (float(rng.uniform(-3, 3)),)) for q in wires]
            gates += [(RZ, (q,), (float(rng.uniform(-3, 3)),)) for q in wires]
            sim = qm.Simulator(n)
            sim.set_state(init)
            sim.run_options(W.to_circuit(n, gates), group=k)
            want = oracle.run(n, gates, init)
            assert np.abs(sim.get_state() - want).max() <= 1e-5, (n, wires)


@pytest.mark.parametrize("bits", [2, 5, 6, 8, 9, 10, 11, 12])
def test_blocked_kernel(bits, golden_circuits):
    """Blocks of b <= 10 wires run as a warp tile, wider ones in shared
    memory; long runs with repeated wires, every matrix form."""
    n = 13
    gates = golden_circuits["hardware_efficient_14_3_0x5eed"]
    gates = [(k, qs, ps) for k, qs, ps in gates if max(qs) < n]
    local = [(RY, (q % bits,), (0.1 * q,)) for q in range(40)] + gates
    sim = qm.Simulator(n)
    sim.run_options(W.to_circuit(n, local), block_bits=bits)
    assert np.abs(sim.get_state() - oracle.run(n, local)).max() <= 1e-5
    # blocking without fusion: long uncollapsed runs (more gates than one
    # launch takes), every one-qubit kind, on a random state
    rng = np.random.default_rng(bits)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    run = []
    for k in range(150):
        q = int(rng.integers(0, bits))
        kind = int(rng.choice([X, Y, Z, H, S, SDG, T, TDG, RX, RY, RZ, P]))
        run.append((kind, (q,), (float(rng.uniform(-3, 3)),) if kind >= RX else ()))
    run += [(CX, (0, n - 1), ())] + run[:30]
    sim = qm.Simulator(n)
    sim.set_state(init)
    sim.run_options(W.to_circuit(n, run), collapse=False, diagonals=False, zz=False, group=1,
                    block_bits=bits)
    assert np.abs(sim.get_state() - oracle.run(n, run, init)).max() <= 1e-5


@pytest.mark.parametrize("n", [6, 10, 14, 20])
def test_frozen_benchmarks(n, golden_circuits):
    for name, gates in frozen_set(n, golden_circuits).items():
        want = oracle.run(n, gates)
        got, sim = gpu_state(n, gates)
        assert np.abs(got - want).max() <= 1e-4, name
        assert abs(sim.norm() - 1.0) <= 1e-4, name


def test_diagonal_layer_many_terms():
    """Wide diagonal layers: every low/cross/high split of pair masks, on a
    random state, fused into one layer (W = 13 tiles at n = 17)."""
    n = 17
    rng = np.random.default_rng(5)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    gates = []
    for _ in range(150):
        a, b = rng.choice(n, size=2, replace=False)
        gates.append((CP, (int(a), int(b)), (float(rng.uniform(-4, 4)),)))
        gates.append((RZ, (int(rng.integers(n)),), (float(rng.uniform(-4, 4)),)))
    gates += W.qaoa_ring(n, 1)[n:]          # a ring ZZ layer + mixers
    d, sim = compare(n, gates, "fused", init)
    flat = W.to_circuit(n, gates).plan_export()
    assert int(flat[1]) == 4 and int(flat[7]) == 300 + 3 * n   # one layer, every term
    assert d <= 1e-5


def test_error_growth_tfim_depth():
    n = 12
    for depth in (1, 5, 20, 50, 85, 90, 100):
        gates = W.tfim_trotter(n, depth)
        d, sim = compare(n, gates)
        assert d <= 1e-4, depth
        assert abs(sim.norm() - 1) <= 1e-4, depth


def test_results_bit_identical_across_runs_and_batches():
    """Grouping launches differently never changes the arithmetic."""
    n = 12
    gates = W.tfim_trotter(n, 90)
    c = W.to_circuit(n, gates)
    ref_state, _ = gpu_state(n, gates)
    for _ in range(3):
        sim = qm.Simulator(n)
        sim.run(c)
        assert np.array_equal(sim.get_state(), ref_state)
    sim = qm.Simulator(n)            # same circuit, split into pieces
    half = len(gates) // 2
    cut = half - (half % (3 * (n - 1) + n))
    sim.run(W.to_circuit(n, gates[:cut]))
    sim.run(W.to_circuit(n, gates[cut:]))
    assert np.array_equal(sim.get_state(), ref_state)


def test_fails_closed():
    sim = qm.Simulator(3)
    with pytest.raises(qm.QMetalError, match="identical"):
        sim.apply(CX, (1, 1))
    with pytest.raises(qm.QMetalError):
        sim.apply(X, (7,))
    with pytest.raises(qm.QMetalError):
        qm.Simulator(qm.max_qubits() + 1)
    with pytest.raises(qm.QMetalError):
        qm.Simulator(0)


def test_dispatch_count():
    c = W.to_circuit(8, W.ghz(8))
    sim = qm.Simulator(8)
    before = sim.dispatch_count
    sim.run(c)
    sim.synchronize()
    assert sim.dispatch_count - before == len(c)


def test_expectation(golden_circuits, golden_arrays):
    n = 8
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, W.ghz(n)))
    assert abs(sim.expectation("Z" + "I" * (n - 1))) <= 1e-5
    assert abs(sim.expectation_pauli(z_mask=3) - 1) <= 1e-5
    assert abs(sim.expectation_pauli(x_mask=1)) <= 1e-5
    assert abs(sim.expectation_pauli(x_mask=(1 << n) - 1) - 1) <= 1e-5
    assert abs(sim.expectation_pauli() - 1) <= 1e-5
    sim = qm.Simulator(6)
    for q in range(6):
        assert abs(sim.expectation_pauli(z_mask=1 << q) - 1) <= 1e-6
    n = 10
    gates = golden_circuits["random_circuit_10_4_0xabc"]
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, gates))
    st = oracle.run(n, gates)
    for m, v in zip(golden_arrays["pauli/masks"], golden_arrays["pauli/values"]):
        x, y, z = (int(t) for t in m)
        assert abs(sim.expectation_pauli(x, y, z) - v) <= 1e-5
        assert abs(oracle.expectation(n, st, x, y, z) - v) <= 1e-12
    n = 8
    gates = golden_circuits["hardware_efficient_8_2_0xfeed"]
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, gates))
    terms = []
    for q in range(n - 1):
        terms += [(1.0, 0, 0, 3 << q), (0.3, 1 << q, 0, 0)]
    want = oracle.expectation_sum(n, oracle.run(n, gates), terms)
    assert abs(sim.expectation(W.to_hamiltonian(terms)) - want) <= 1e-4
    assert abs(sim.norm() - 1) <= 1e-5
    with pytest.raises(qm.QMetalError, match="invalid"):
        sim.expectation_pauli(x_mask=1, z_mask=1)


def test_expectation_terms_many_groups():
    n = 11
    gates = W.qaoa_ring_seeded(n, 2, seed=9)
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, gates))
    st = oracle.run(n, gates)
    rng = np.random.default_rng(3)
    terms = []
    for _ in range(70):   # more than one 16-term pass per flip group
        x = y = z = 0
        for q in range(n):
            r = int(rng.integers(0, 6))
            if r == 1: x |= 1 << q
            elif r == 2: y |= 1 << q
            elif r >= 3: z |= 1 << q
        terms.append((float(rng.normal()), x, y, z))
    terms += [(0.5, 0, 0, 1 << q) for q in range(n)] * 2
    h = W.to_hamiltonian(terms)
    vals = sim.expectation_terms(h)
    for (c, x, y, z), v in zip(terms, vals):
        assert abs(v - oracle.expectation(n, st, x, y, z)) <= 1e-5
    assert abs(sim.expectation(h) - oracle.expectation_sum(n, st, terms)) <= 1e-4


def test_sampling_ghz_and_determinism():
    n = 6
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, W.ghz(n)))
    shots = np.array(sim.sample(20000, 12345))
    assert set(np.unique(shots)) <= {0, (1 << n) - 1}
    assert abs(np.mean(shots == 0) - 0.5) < 0.02
    sim = qm.Simulator(5)
    sim.run(W.to_circuit(5, W.qft(5)))
    a, b, c = sim.sample(500, 999), sim.sample(500, 999), sim.sample(500, 1000)
    assert a == b and a != c


def test_sampling_distribution(golden_circuits):
    n = 6
    gates = golden_circuits["random_circuit_6_3_0x1234"]
    probs = np.abs(oracle.run(n, gates)) ** 2
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, gates))
    draw = np.array(sim.sample(200000, 2024))
    hist = np.bincount(draw, minlength=1 << n) / draw.size
    assert 0.5 * np.abs(hist - probs).sum() < 0.02


@pytest.mark.parametrize("n", [6, 12, 16])
def test_sampling_matches_oracle_draw_for_draw(n):
    """Same float state, same seed: the GPU draws the oracle's indices."""
    rng = np.random.default_rng(n)
    gates = W.random_u3(n, 3, seed=n)
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, gates))
    amps = sim.get_state()
    got = np.array(sim.sample(4000, 77 + n), dtype=np.uint64)
    want = oracle.sample_f32(n, amps, 4000, 77 + n)
    assert np.mean(got == want) >= 0.999


def test_counts_format():
    n = 4
    sim = qm.Simulator(n)
    sim.run(W.to_circuit(n, [(X, (0,), ())]))
    assert sim.counts(100, 1) == {"0001": 100}


def _shift_gradient(n, gates, terms):
    out = []
    for k, (kind, qs, ps) in enumerate(gates):
        if not ps:
            out.append(0.0)
            continue
        plus = list(gates); plus[k] = (kind, qs, (ps[0] + math.pi / 2,))
        minus = list(gates); minus[k] = (kind, qs, (ps[0] - math.pi / 2,))
        out.append(0.5 * (oracle.expectation_sum(n, oracle.run(n, plus), terms)
                          - oracle.expectation_sum(n, oracle.run(n, minus), terms)))
    return np.array(out)


def test_gradients_vs_parameter_shift(golden_circuits):
    n = 6
    terms = [(1.0, 0, 0, 3 << q) for q in range(n - 1)] + [(0.4, 1 << q, 0, 0) for q in range(n)]
    terms.append((0.25, 0, 1, 0))          # a Y term, so an i^ny slip cannot hide
    cases = {"hea_d2": golden_circuits["hardware_efficient_6_2_0xc0ffee"],
             "tfim_s3": W.tfim_trotter(n, 3), "qaoa_p2": W.qaoa_ring(n, 2)}
    for name, gates in cases.items():
        sim = qm.Simulator(n)
        e, g = sim.energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
        assert abs(e - oracle.expectation_sum(n, oracle.run(n, gates), terms)) <= 1e-5, name
        want = _shift_gradient(n, gates, terms)
        assert np.abs(np.array(g) - want).max() <= 1e-5, name
        for k, (_, _, ps) in enumerate(gates):
            if not ps:
                assert g[k] == 0.0


def test_gradient_closed_form_and_fail_closed():
    for t in (0.0, 0.3, 1.1, 2.7, -0.9):
        c = qm.Circuit(2)
        c.ry(0, t)
        e, g = qm.Simulator(2).energy_and_gradient(c, qm.Hamiltonian().add_string(1.0, "ZI"))
        assert abs(e - math.cos(t)) <= 1e-5 and abs(g[0] + math.sin(t)) <= 1e-5
    bad = qm.Circuit(2)
    bad.h(0).cp(0, 1, 0.4)
    with pytest.raises(qm.QMetalError, match="differentiable"):
        qm.Simulator(2).energy_and_gradient(bad, qm.Hamiltonian().add_string(1.0, "ZI"))


def _fused_cases():
    rng = np.random.default_rng(77)
    n = 11
    zz_many = [(H, (q,), ()) for q in range(n)]
    for _ in range(40):                     # 40 couplings in one block: > 32 generators
        a, b = (int(x) for x in rng.choice(n, size=2, replace=False))
        zz_many += [(CX, (a, b), ()), (RZ, (b,), (float(rng.uniform(-2, 2)),)), (CX, (a, b), ())]
    zz_many += [(RX, (q,), (float(rng.uniform(-2, 2)),)) for q in range(n)]
    long_wire = [(H, (q,), ()) for q in range(n)]
    long_wire += [((RX, RY, RZ)[k % 3], (3,), (0.1 * k - 1.0,)) for k in range(40)]
    long_wire += [(CX, (3, 7), ()), (RY, (0,), (0.4,)), (RZ, (0,), (0.9,))]
    mixed = (W.hea(n, 2, seed=1) + W.random_u3(n, 2, seed=2)
             + [(CCX, (0, 4, 9), ()), (SWAP, (1, 8), ()), (CY, (10, 2), ()), (CZ, (3, 5), ()),
                (T, (6,), ()), (S, (7,), ())] + W.qaoa_ring_seeded(n, 2, seed=3)[n:])
    # rotations by zero are identity matrices whose X / Y generators still
    # need the partner amplitude; H, S, T, SDG mix the other matrix forms
    zero = [(H, (q,), ()) for q in range(n)] + [(T, (q,), ()) for q in range(0, n, 2)]
    for q in range(n):
        zero += [(RX, (q,), (0.0,)), (RY, (q,), (0.0 if q % 2 else 0.8,)), (RZ, (q,), (0.0,)),
                 (S, (q,), ()), (RX, (q,), (0.3 * q - 1.0,)), (SDG, (q,), ()), (H, (q,), ()),
                 (RY, (q,), (0.0,))]
    return {"qaoa_ring": W.qaoa_ring_seeded(n, 3, seed=8), "tfim": W.tfim_chain(n, 4),
            "hea_d4": W.hea(n, 4, seed=5), "zz_many": zz_many, "long_wire": long_wire,
            "mixed": mixed, "zero_angles": zero}


@pytest.mark.parametrize("name", list(_fused_cases()))
def test_fused_adjoint_matches_oracle_and_gate_by_gate(name):
    n = 11
    gates = _fused_cases()[name]
    zterms = [(-1.0, 0, 0, (1 << q) | (1 << ((q + 1) % n))) for q in range(n)]
    zterms += [(0.3, 0, 0, 1 << q) for q in range(0, n, 3)] + [(0.7, 0, 0, 0)]
    mixed_terms = W.ring_tfim_hamiltonian(n, 0.7) + [(0.25, 0, 1 << 4, 1 << 2)]
    for terms in (zterms, mixed_terms):
        e0, g0 = oracle.energy_and_gradient(n, gates, terms)
        c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
        sim = qm.Simulator(n)
        e1, g1 = sim.energy_and_gradient(c, h)                 # block-wise sweep
        e2, g2 = sim.energy_and_gradient(c, h, fused=False)    # gate by gate
        assert abs(e1 - e0) <= 1e-5 and abs(e2 - e0) <= 1e-5
        assert np.abs(np.array(g1) - g0).max() <= 1e-5, name
        assert np.abs(np.array(g2) - g0).max() <= 1e-5, name
        for k, (_, _, ps) in enumerate(gates):
            if not ps:
                assert g1[k] == 0.0


@pytest.mark.parametrize("n", [14, 18])
def test_fused_adjoint_tiles_and_lanes(n):
    """Large enough for whole 13-bit tiles plus tile bits in the generators."""
    gates, terms = W.hea_gradient_problem(n, depth=3, seed=n)
    gates = W.qaoa_ring_seeded(n, 2, seed=n) + gates
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    e1, g1 = qm.Simulator(n).energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    assert abs(e1 - e0) <= 1e-5
    assert np.abs(np.array(g1) - g0).max() <= 1e-5
    zt = [(-0.5, 0, 0, (1 << a) | (1 << b)) for a, b in W.random_3regular(n, np.random.default_rng(n))]
    e0, g0 = oracle.energy_and_gradient(n, gates, zt)
    e1, g1 = qm.Simulator(n).energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(zt))
    assert abs(e1 - e0) <= 1e-5
    assert np.abs(np.array(g1) - g0).max() <= 1e-5


@pytest.mark.parametrize("n", [10, 14])
def test_uniform_rotation_layers(n):
    """Layers of one rotation kind on every wire (RX, RY, RZ) take the
    compile-time-uniform window tiles (wire 0 + wires 1..5 + four wires >= 6,
    and four wires >= 6 alone); zero angles and a mixed layer take the
    general tiles. Both sweeps against the oracle's adjoint."""
    rng = np.random.default_rng(900 + n)
    ang = lambda: float(rng.uniform(-3, 3))
    gates = [(H, (q,), ()) for q in range(n)]
    entangle = [(CX, (q, q + 1), ()) for q in range(0, n - 1, 2)]
    entangle += [(CZ, (q, q + 1), ()) for q in range(1, n - 1, 2)]
    for kind in (RX, RY, RZ):
        gates += entangle + [(kind, (q,), (ang(),)) for q in range(n)]
    gates += entangle + [(RX, (q,), (0.0,)) for q in range(n)]             # rotations by zero
    gates += entangle + [((RY if q == 7 else RX), (q,), (ang(),)) for q in range(n)]
    terms = W.ring_tfim_hamiltonian(n, 0.7) + [(0.4, 1 << 3, 1 << 8, 0)]
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
    sim = qm.Simulator(n)
    e1, g1 = sim.energy_and_gradient(c, h)
    e2, g2 = sim.energy_and_gradient(c, h, fused=False)
    assert abs(e1 - e0) <= 1e-5 and abs(e2 - e0) <= 1e-5
    assert np.abs(np.array(g1) - g0).max() <= 1e-5
    assert np.abs(np.array(g2) - g0).max() <= 1e-5


@pytest.mark.parametrize("n", list(range(7, 16)))
def test_uniform_tile_shapes_every_width(n):
    """Every width from 7 to 15 leaves a different remainder of register
    wires for the last tile of a layer (one to four, on one warp or a warp
    pair): an RX layer, an RY.RZ layer (RZ then RY backward) and an RZ.RY
    layer, against the oracle's adjoint."""
    rng = np.random.default_rng(1300 + n)
    ang = lambda: float(rng.uniform(-3, 3))
    entangle = [(CX, (q, q + 1), ()) for q in range(n - 1)]
    gates = [(H, (q,), ()) for q in range(n)] + entangle
    gates += [(RX, (q,), (ang(),)) for q in range(n)] + entangle
    for q in range(n):
        gates += [(RY, (q,), (ang(),)), (RZ, (q,), (ang(),))]
    gates += entangle
    for q in range(n):
        gates += [(RZ, (q,), (ang(),)), (RY, (q,), (ang(),))]
    terms = W.ring_tfim_hamiltonian(n, 0.7)
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    e1, g1 = qm.Simulator(n).energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    assert abs(e1 - e0) <= 1e-5
    assert np.abs(np.array(g1) - g0).max() <= 1e-5


def test_gradient_matches_oracle_adjoint_wide():
    """All gate kinds in the backward sweep, every wire, n = 12."""
    n = 12
    rng = np.random.default_rng(11)
    gates = W.hea(n, 2, seed=2) + W.random_u3(n, 1, seed=3)
    gates += [(CCX, (0, 5, 11), ()), (SWAP, (2, 9), ()), (CY, (10, 1), ()), (H, (4,), ()),
              (S, (3,), ()), (T, (0,), ()), (CP, (1, 2), (0.3,))]
    gates += [(RX, (q,), (float(rng.uniform(-3, 3)),)) for q in range(n)]
    terms = W.ring_tfim_hamiltonian(n, 0.7) + [(0.3, 1 << 2, 1 << 5, 1 << 7)]
    # CP carries a parameter: the adjoint path fails closed on it ...
    with pytest.raises(qm.QMetalError):
        qm.Simulator(n).energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    gates = [g for g in gates if g[0] != CP]
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    e, g = qm.Simulator(n).energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    assert abs(e - e0) <= 1e-5
    assert np.abs(np.array(g) - g0).max() <= 1e-5


@pytest.mark.parametrize("mode", ["fused", "unfused", "gates"])
def test_u3_every_wire(mode):
    """The appended U3 gate (kind 18) on every wire of a 12-qubit state,
    alone and in fused windows with CX / CZ layers."""
    U3 = qm.U3
    n = 12
    rng = np.random.default_rng(31)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    gates = []
    for layer in range(3):
        for q in range(n):
            gates.append((U3, (q,), tuple(float(x) for x in rng.uniform(-3.1, 3.1, 3))))
        for q in range(layer % 2, n - 1, 2):
            gates.append((CX if layer % 2 else CZ, (q, q + 1), ()))
    d, sim = compare(n, gates, mode, init)
    assert d <= 1e-5
    assert abs(sim.norm() - 1) <= 1e-5
    # U3 carries parameters without a native generator: the gradient fails closed
    with pytest.raises(qm.QMetalError, match="differentiable"):
        sim.energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian([(1.0, 0, 0, 1)]))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7])
def test_gradients_on_the_smallest_states(n):
    """Widths below and at the edges of the tile shapes (fewer wires than a
    warp's lanes, one register wire): every sweep path, mixed Hamiltonians
    with X, Y and Z strings, CX ladders and SWAPs, against the oracle."""
    rng = np.random.default_rng(700 + n)
    gates = [(H, (q,), ()) for q in range(n)]
    for layer in range(3):
        for q in range(n):
            gates.append(((RX, RY, RZ)[(q + layer) % 3], (q,), (float(rng.uniform(-3, 3)),)))
        if n >= 2:
            gates += [(CX, (q, q + 1), ()) for q in range(n - 1)]
            gates.append((SWAP, (0, n - 1), ()))
            a, b = int(rng.integers(n)), int(rng.integers(n))
            if a != b:
                gates += [(CX, (a, b), ()), (RZ, (b,), (float(rng.uniform(-2, 2)),)),
                          (CX, (a, b), ())]
    terms = [(0.7, 1 << q, 0, 0) for q in range(n)] + [(-0.4, 0, 1 << (n - 1), 0)]
    terms += [(0.5, 0, 0, (1 << q) | (1 << ((q + 1) % n))) for q in range(n)]
    if n >= 3:
        terms.append((0.3, 1, 1 << 1, 1 << 2))          # X0 Y1 Z2
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
    for fused in (True, False):
        e, g = qm.Simulator(n).energy_and_gradient(c, h, fused=fused)
        assert abs(e - e0) <= 1e-5, fused
        assert np.abs(np.array(g) - g0).max() <= 1e-5, fused
    # and through the batch paths, widths 1..n mixed
    reqs = []
    for m in range(1, n + 1):
        gm = [(RY, (q,), (0.3 + 0.1 * q,)) for q in range(m)]
        gm += [(CX, (q, q + 1), ()) for q in range(m - 1)] + [(RX, (0,), (0.9,))]
        reqs.append((W.to_circuit(m, gm), W.to_hamiltonian([(1.0, 0, 0, 1), (0.5, 1, 0, 0)]),
                     32, m))
    for mode in (qm.BATCH_LANES, qm.BATCH_GRAPH, qm.BATCH_PLAIN_LOOP):
        out = qm.batch_serve(reqs, mode=mode, lanes=2)
        for m, (e, g, s) in zip(range(1, n + 1), out):
            gm = [(RY, (q,), (0.3 + 0.1 * q,)) for q in range(m)]
            gm += [(CX, (q, q + 1), ()) for q in range(m - 1)] + [(RX, (0,), (0.9,))]
            e1, g1 = oracle.energy_and_gradient(m, gm, [(1.0, 0, 0, 1), (0.5, 1, 0, 0)])
            assert abs(e - e1) <= 1e-5 and np.abs(np.array(g) - g1).max() <= 1e-5, (mode, m)
            assert len(s) == 32 and all(0 <= x < (1 << m) for x in s)


@pytest.mark.parametrize("tile_high", [5, 6])
@pytest.mark.parametrize("n", [11, 12, 13, 14, 15, 16])
def test_block_tiles_every_width(n, tile_high):
    """Five- and six-wire block tiles (wires >= 6 only, four or eight warps
    per site, one shared-memory transpose per round): an RX layer, an RY
    layer, an RZ layer, an RY.RZ layer (RZ then RY backward) and an RZ.RY
    layer on every wire, between CX ladders, against the oracle's adjoint;
    the block-wise sweep with tile_high 4 (no block tiles) gives the same
    gradient."""
    rng = np.random.default_rng(1600 + 10 * n + tile_high)
    ang = lambda: float(rng.uniform(-3, 3))
    entangle = [(CX, (q, q + 1), ()) for q in range(n - 1)]
    gates = [(H, (q,), ()) for q in range(n)] + entangle
    for kind in (RX, RY, RZ):
        gates += [(kind, (q,), (ang(),)) for q in range(n)] + entangle
    for q in range(n):
        gates += [(RY, (q,), (ang(),)), (RZ, (q,), (ang(),))]
    gates += entangle
    for q in range(n):
        gates += [(RZ, (q,), (ang(),)), (RY, (q,), (ang(),))]
    terms = W.ring_tfim_hamiltonian(n, 0.7) + [(0.3, 0, 1 << 2, 1 << (n - 1))]
    c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    sim = qm.Simulator(n).set_tile_high(tile_high)
    e1, g1 = sim.energy_and_gradient(c, h)
    assert abs(e1 - e0) <= 1e-5
    assert np.abs(np.array(g1) - g0).max() <= 1e-5
    e2, g2 = qm.Simulator(n).set_tile_high(4).energy_and_gradient(c, h)
    assert np.abs(np.array(g1) - np.array(g2)).max() <= 1e-5


@pytest.mark.parametrize("cap", [0, 1, 3, 16])
def test_state_checkpoints_any_number(cap, monkeypatch):
    """The gradient's forward pass keeps the state before each gathered CX
    ladder while spare buffers allow, and the sweep restores it instead of
    gathering it back. With room for none, some or all of them (the cap
    stands in for a device that is nearly full: at 33 qubits one fits), the
    gradient is the oracle's: a checkpoint is only ever restored at the undo
    it was taken for, even though every layer's ladder is the same map."""
    monkeypatch.setenv("QMETAL_MAX_CHECKPOINTS", str(cap))
    n = 14
    gates, terms = W.hea_gradient_problem(n, depth=6, seed=7)
    sim = qm.Simulator(n)
    e, g = sim.energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    assert abs(e - e0) <= 1e-5
    assert np.abs(np.array(g) - g0).max() <= 1e-5
    e1, g1 = sim.energy_and_gradient(W.to_circuit(n, gates), W.to_hamiltonian(terms))
    assert np.abs(np.array(g1) - g0).max() <= 1e-5
