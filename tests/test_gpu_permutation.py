"""Runs of CX / SWAP gates as one GF(2)-affine permutation pass.

qmk_apply_permutation gathers dst[y] = src[G(y)] with G affine over GF(2);
a permutation moves amplitudes without arithmetic, so every case here is
exact: bit-identical to numpy's gather, and the merged forward / backward
paths that use it are checked against the oracle and against the plain
plan path. Singular maps and in-place calls are rejected before launch.
"""
import ctypes
from ctypes import c_int, c_uint32, c_uint64, c_void_p

import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W

pytestmark = pytest.mark.gpu
H, RX, RY, RZ, CX, CZ, SWAP = 3, 8, 9, 10, 12, 14, 15


def _lib():
    L = ctypes.CDLL(qm.library_path())
    L.qmk_apply_permutation.restype = c_int
    L.qmk_apply_permutation.argtypes = [c_void_p, c_void_p, c_uint32, c_void_p, c_uint64,
                                        c_void_p]
    return L


def _random_map(n, rng, pair):
    """A random invertible affine map, built from random CX / SWAP / X."""
    cols = [1 << j for j in range(n)]
    off = 0
    for _ in range(6 * n if n >= 2 else 0):
        a, b = (int(x) for x in rng.choice(n, size=2, replace=False))
        if pair and 0 in (a, b):
            continue
        if rng.uniform() < 0.3:
            cols = [v ^ ((((v >> a) ^ (v >> b)) & 1) * ((1 << a) | (1 << b))) for v in cols]
            off ^= (((off >> a) ^ (off >> b)) & 1) * ((1 << a) | (1 << b))
        else:
            cols = [v ^ (((v >> a) & 1) << b) for v in cols]
            off ^= ((off >> a) & 1) << b
    off ^= int(rng.integers(0, 1 << n))
    return np.array(cols, dtype=np.uint64), off


def _gather(src, cols, off):
    n = len(cols)
    y = np.arange(1 << n, dtype=np.uint64)
    x = np.full(1 << n, off, dtype=np.uint64)
    for j in range(n):
        x ^= np.where((y >> np.uint64(j)) & np.uint64(1), cols[j], np.uint64(0))
    return src[x.astype(np.int64)]


@pytest.mark.parametrize("n,pair", [(1, True), (5, False), (10, True), (10, False),
                                    (14, True), (17, False)])
def test_gather_matches_numpy(n, pair):
    torch = pytest.importorskip("torch")
    L = _lib()
    rng = np.random.default_rng(n * 2 + pair)
    src = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)).astype(np.complex64)
    cols, off = _random_map(n, rng, pair)
    if pair:
        assert cols[0] == 1
    s = torch.from_numpy(src.view(np.float32).copy()).cuda()
    d = torch.zeros_like(s)
    assert L.qmk_apply_permutation(d.data_ptr(), s.data_ptr(), n, cols.ctypes.data, off,
                                   None) == 0
    torch.cuda.synchronize()
    got = d.cpu().numpy().view(np.complex64)
    assert np.array_equal(got, _gather(src, cols, off))


def test_rejects_singular_and_in_place():
    torch = pytest.importorskip("torch")
    L = _lib()
    n = 6
    s = torch.zeros(2 << n, dtype=torch.float32, device="cuda")
    d = torch.zeros_like(s)
    good = np.array([1 << j for j in range(n)], dtype=np.uint64)
    singular = good.copy()
    singular[3] = singular[2]
    outside = good.copy()
    outside[1] = 1 << n
    assert L.qmk_apply_permutation(d.data_ptr(), s.data_ptr(), n, singular.ctypes.data, 0,
                                   None) != 0
    assert L.qmk_apply_permutation(d.data_ptr(), s.data_ptr(), n, outside.ctypes.data, 0,
                                   None) != 0
    assert L.qmk_apply_permutation(s.data_ptr(), s.data_ptr(), n, good.ctypes.data, 0,
                                   None) != 0
    assert L.qmk_apply_permutation(d.data_ptr(), s.data_ptr(), n, good.ctypes.data, 1 << n,
                                   None) != 0


def _ladders(n, depth, seed):
    """HEA-like layers whose entanglers are CX ladders, SWAP chains and
    scattered CX, so the merged paths meet long permutation runs."""
    rng = np.random.default_rng(seed)
    gates = []
    for layer in range(depth):
        for q in range(n):
            gates.append((RY, (q,), (float(rng.uniform(-3, 3)),)))
            gates.append((RZ, (q,), (float(rng.uniform(-3, 3)),)))
        if layer % 3 == 0:
            gates += [(CX, (q, q + 1), ()) for q in range(n - 1)]
        elif layer % 3 == 1:
            gates += [(CX, (q + 1, q), ()) for q in reversed(range(n - 1))]
            gates += [(SWAP, (q, n - 1 - q), ()) for q in range(n // 2)]
        else:
            for _ in range(n):
                a, b = (int(x) for x in rng.choice(n, size=2, replace=False))
                gates.append((CX, (a, b), ()))
    return gates


@pytest.mark.parametrize("n", [7, 12, 16])
def test_merged_forward_matches_plan_and_oracle(n):
    gates = _ladders(n, 5, seed=n)
    c = W.to_circuit(n, gates)
    plain = qm.Simulator(n).run(c).get_state()
    sim = qm.Simulator(n)
    before = sim.dispatch_count
    sim.run_merged(c)
    merged_launches = sim.dispatch_count - before
    got = sim.get_state()
    assert np.abs(got - oracle.run(n, gates)).max() <= 1e-5
    assert np.abs(got - plain).max() <= 1e-5
    assert merged_launches < c.plan_size()


@pytest.mark.parametrize("n", [8, 13])
def test_gradient_with_permutation_runs(n):
    gates = _ladders(n, 4, seed=100 + n)
    terms = W.ring_tfim_hamiltonian(n, 0.7)
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
    sim = qm.Simulator(n)
    e1, g1 = sim.energy_and_gradient(c, h)
    e2, g2 = sim.energy_and_gradient(c, h, fused=False)
    assert abs(e1 - e0) <= 1e-5 and abs(e2 - e0) <= 1e-5
    assert np.abs(np.array(g1) - g0).max() <= 1e-5
    assert np.abs(np.array(g2) - g0).max() <= 1e-5


def test_graph_replay_after_buffers_swapped():
    """A permutation pass swaps the state buffer; a graph captured before it
    must not replay onto the old buffer."""
    n = 11
    gates = _ladders(n, 3, seed=9)
    c = W.to_circuit(n, gates)
    sim = qm.Simulator(n)
    sim.reset()
    sim.run_cached(c)
    first = sim.get_state()
    sim.reset()
    sim.run_merged(c)                  # swaps state and scratch
    sim.reset()
    sim.run_cached(c)                  # recaptured on the current buffer
    assert np.array_equal(sim.get_state(), first)
    assert np.abs(first - oracle.run(n, gates)).max() <= 1e-5


def _relabel_numpy(state, n, perm):
    """new state with qubit perm[q] holding old qubit q (LSB-first axes)."""
    t = state.reshape([2] * n)                 # axis n-1-q is qubit q
    src_axes = [n - 1 - q for q in range(n)]
    dst_axes = [n - 1 - perm[q] for q in range(n)]
    return np.moveaxis(t, src_axes, dst_axes).reshape(-1)


@pytest.mark.parametrize("n", [2, 9, 15])
def test_permute_qubits_matches_numpy(n):
    rng = np.random.default_rng(40 + n)
    init = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)).astype(np.complex64)
    for trial in range(3):
        perm = [int(x) for x in rng.permutation(n)]
        sim = qm.Simulator(n)
        sim.set_state(init)
        sim.permute_qubits(perm)
        assert np.array_equal(sim.get_state().astype(np.complex64), _relabel_numpy(init, n, perm))
    sim = qm.Simulator(n)
    sim.set_state(init)
    sim.permute_qubits(list(range(n)))            # identity: nothing moves
    assert np.array_equal(sim.get_state().astype(np.complex64), init)
    with pytest.raises(qm.QMetalError):
        sim.permute_qubits([0] * n)
    with pytest.raises(qm.QMetalError):
        sim.permute_qubits(list(range(n - 1)))


@pytest.mark.parametrize("bits", [6, 10])
def test_relabeled_blocked_runs_restore_the_state(bits, golden_circuits):
    """The qubit-reordering arm: hot wires relabeled into the block window,
    the relabeled circuit fused and blocked, one pass restores the order."""
    n = 14
    gates = [(k, tuple(q), tuple(p)) for k, q, p in golden_circuits["local_patch_14_8_12_0x10ca1"]]
    gates = W.relabel(gates, [n - 1 - q for q in range(n)])     # the hot wires made high
    perm = W.hot_wires_first(n, gates)
    back = [0] * n
    for q, p in enumerate(perm):
        back[p] = q
    sim = qm.Simulator(n)
    sim.run_options(W.to_circuit(n, W.relabel(gates, perm)), block_bits=bits)
    sim.permute_qubits(back)
    assert np.abs(sim.get_state() - oracle.run(n, gates)).max() <= 1e-5
