"""The oracle pinned before it is trusted (CPU only).

1. Closed forms and identities, restated from the reference's oracle
   self-checks (tests/test_reference.cpp:43-323), against the C restatement.
2. The restatement against outputs of the reference's own code recorded in
   tests/golden/reference.npz (always), and against the reference compiled
   from source where it is available (oracle/_ref).
"""
import math

import numpy as np
import pytest

import oracle
from qmetal_gb300 import workloads as W
from conftest import frozen_set

TOL = 1e-12
X, Y, Z, H, S, SDG, T, TDG, RX, RY, RZ, P = range(12)
CX, CY, CZ, SWAP, CP, CCX = 12, 13, 14, 15, 16, 17


def st(n, gates, init=None):
    return oracle.run(n, gates, init)


def test_bit_convention():
    for q in range(3):
        s = st(3, [(X, (q,), ())])
        assert abs(abs(s[1 << q]) - 1.0) < TOL


def test_single_qubit_identities():
    assert abs(abs(st(1, [(H, (0,), ())] * 2)[0]) - 1) < TOL
    assert abs(abs(st(1, [(X, (0,), ())] * 2)[0]) - 1) < TOL
    a = st(1, [(X, (0,), ()), (S, (0,), ()), (S, (0,), ())])
    b = st(1, [(X, (0,), ()), (Z, (0,), ())])
    assert np.abs(a - b).max() < TOL
    assert abs(st(1, [(X, (0,), ())] + [(T, (0,), ())] * 8)[1].real - 1) < TOL
    assert abs(st(1, [(RZ, (0,), (2 * math.pi,))])[0].real + 1) < TOL
    assert abs(abs(st(1, [(RY, (0,), (math.pi,))])[1]) - 1) < TOL
    assert abs(st(1, [(RX, (0,), (math.pi,))])[1].imag + 1) < TOL
    s = st(1, [(X, (0,), ()), (S, (0,), ()), (SDG, (0,), ()), (T, (0,), ()), (TDG, (0,), ())])
    assert abs(s[1].real - 1) < TOL


def test_two_qubit_gates():
    r = 1 / math.sqrt(2)
    s = st(2, [(H, (0,), ()), (CX, (0, 1), ())])
    assert abs(s[0].real - r) < TOL and abs(s[3].real - r) < TOL
    assert abs(s[1]) < TOL and abs(s[2]) < TOL
    before = st(2, [(H, (0,), ()), (H, (1,), ())])
    after = st(2, [(H, (0,), ()), (H, (1,), ()), (CX, (0, 1), ()), (CX, (0, 1), ())])
    assert np.abs(before - after).max() < TOL
    a = st(2, [(X, (0,), ()), (CX, (0, 1), ())])
    b = st(2, [(X, (0,), ()), (CX, (1, 0), ())])
    assert np.abs(a - b).max() > 0.5 and abs(abs(a[3]) - 1) < TOL
    s = st(2, [(H, (0,), ()), (H, (1,), ()), (CZ, (0, 1), ())])
    assert abs(s[3].real + 0.5) < TOL and abs(s[0].real - 0.5) < TOL
    hh = [(H, (0,), ()), (H, (1,), ())]
    assert np.abs(st(2, hh + [(CP, (0, 1), (math.pi,))]) - st(2, hh + [(CZ, (0, 1), ())])).max() < TOL
    s = st(2, [(X, (0,), ()), (SWAP, (0, 1), ())])
    assert abs(abs(s[2]) - 1) < TOL
    s = st(2, [(X, (0,), ()), (SWAP, (0, 1), ()), (SWAP, (0, 1), ())])
    assert abs(abs(s[1]) - 1) < TOL
    s = st(3, [(X, (0,), ()), (X, (1,), ()), (CCX, (0, 1, 2), ())])
    assert abs(abs(s[7]) - 1) < TOL
    s = st(3, [(X, (0,), ()), (CCX, (0, 1, 2), ())])
    assert abs(abs(s[1]) - 1) < TOL


@pytest.mark.parametrize("n", [2, 3, 8, 12])
def test_ghz_closed_form(n):
    s = st(n, W.ghz(n))
    r = 1 / math.sqrt(2)
    assert abs(s[0].real - r) < TOL and abs(s[-1].real - r) < TOL
    assert np.sum(np.abs(s[1:-1]) ** 2) < TOL


@pytest.mark.parametrize("n", [1, 2, 5, 10])
def test_qft_uniform(n):
    s = st(n, W.qft(n))
    assert np.abs(s - 1 / math.sqrt(1 << n)).max() < 1e-12


def test_qft_phases():
    s = st(2, [(X, (0,), ())] + W.qft(2))
    want = np.array([0.5, -0.5, 0.5j, -0.5j])
    assert np.abs(s - want).max() < 1e-12
    n, N, x = 3, 8, 3
    s = st(n, [(X, (0,), ()), (X, (1,), ())] + W.qft(n))

    def rev(k):
        return sum(((k >> b) & 1) << (n - 1 - b) for b in range(n))
    for k in range(N):
        want = np.exp(2j * math.pi * x * k / N) / math.sqrt(N)
        assert abs(s[rev(k)] - want) < 1e-12


def test_pauli_closed_forms():
    s = st(1, [(H, (0,), ()), (S, (0,), ())])
    assert abs(oracle.expectation(1, s, y=1) - 1) < TOL
    assert abs(oracle.expectation(1, s, x=1)) < TOL
    assert abs(oracle.expectation(1, s, z=1)) < TOL
    s = st(1, [(H, (0,), ()), (SDG, (0,), ())])
    assert abs(oracle.expectation(1, s, y=1) + 1) < TOL
    s = st(2, [(H, (0,), ()), (CX, (0, 1), ())])
    assert abs(oracle.expectation(2, s, y=3) + 1) < TOL
    assert abs(oracle.expectation(2, s, x=3) - 1) < TOL
    assert abs(oracle.expectation(2, s, z=3) - 1) < TOL
    assert math.isnan(oracle.expectation(2, s, x=1, z=1))   # invalid string


@pytest.mark.parametrize("n", [4, 7])
def test_unitarity_frozen(n, golden_circuits):
    for name, gates in frozen_set(n, golden_circuits).items():
        s = st(n, gates)
        assert abs(oracle.norm(n, s) - 1) < 1e-11, name


def test_fails_closed():
    with pytest.raises(ValueError):
        st(2, [(CX, (0, 0), ())])
    with pytest.raises(ValueError):
        st(2, [(X, (5,), ())])


@pytest.mark.parametrize("n", [4, 7])
def test_matches_recorded_reference_states(n, golden_circuits, golden_arrays):
    for name, gates in frozen_set(n, golden_circuits).items():
        want = golden_arrays[f"state/{name}/{n}"]
        assert np.abs(st(n, gates) - want).max() < 1e-13, name


@pytest.mark.parametrize("n", [6, 9])
def test_random_initial_state_matches_reference(n, golden_arrays):
    init = golden_arrays[f"init/qft_swap/{n}"]
    want = golden_arrays[f"state/qft_swap/{n}"]
    assert np.abs(st(n, W.qft_swap(n), init) - want).max() < 1e-13


def test_expectation_matches_recorded_reference(golden_circuits, golden_arrays):
    s = st(10, golden_circuits["random_circuit_10_4_0xabc"])
    for m, v in zip(golden_arrays["pauli/masks"], golden_arrays["pauli/values"]):
        assert abs(oracle.expectation(10, s, int(m[0]), int(m[1]), int(m[2])) - v) < 1e-13


def test_gradient_matches_parameter_shift(golden_circuits):
    n = 6
    gates = golden_circuits["hardware_efficient_6_2_0xc0ffee"]
    terms = [(1.0, 0, 0, 3 << q) for q in range(n - 1)] + [(0.4, 1 << q, 0, 0) for q in range(n)]
    terms.append((0.25, 0, 1, 0))
    e, g = oracle.energy_and_gradient(n, gates, terms)
    assert abs(e - oracle.expectation_sum(n, st(n, gates), terms)) < 1e-12
    for k, (kind, qs, ps) in enumerate(gates):
        if not ps:
            assert g[k] == 0.0
            continue
        plus = list(gates); plus[k] = (kind, qs, (ps[0] + math.pi / 2,))
        minus = list(gates); minus[k] = (kind, qs, (ps[0] - math.pi / 2,))
        want = 0.5 * (oracle.expectation_sum(n, st(n, plus), terms)
                      - oracle.expectation_sum(n, st(n, minus), terms))
        assert abs(want - g[k]) < 1e-12


def test_sampler_on_ghz():
    n = 6
    s = st(n, W.ghz(n)).astype(np.complex64)
    draws = oracle.sample_f32(n, s, 20000, 12345)
    assert set(np.unique(draws)) <= {0, (1 << n) - 1}
    assert abs(np.mean(draws == 0) - 0.5) < 0.02


@pytest.mark.skipif(not oracle.ref_available(), reason="reference not compiled here")
@pytest.mark.parametrize("seed", range(5))
def test_restatement_bit_identical_to_reference(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(3, 9))
    gates = oracle.ref_circuit("random_circuit", n, 5, 0, seed) + W.qft_swap(n) + W.qaoa_ring(n, 2)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    a = oracle.run(n, gates, init)
    b = oracle.ref_run(n, gates, init)
    assert np.array_equal(a, b)
    for x, y, z in [(1, 0, 0), (0, 3, 0), (5, 0, 2), (0, 0, (1 << n) - 1)]:
        if (x | y | z) >> n:
            continue
        assert oracle.expectation(n, a, x, y, z) == oracle.ref_expectation(n, a, x, y, z)
