"""The library's plan builder (CPU only, through qm_circuit_plan_export).

Pinned two ways: it must emit exactly the plans the reference's build_plan
emits (recorded in tests/golden/reference.npz, and live against oracle/_ref
where compiled), and every plan must reproduce the circuit in complex128 --
the reference's fusion tests (tests/test_fusion.cpp:37-163) restated.
"""
import math

import numpy as np
import pytest

import oracle
from qmetal_gb300 import workloads as W
from conftest import frozen_set

X, Y, Z, H, S, SDG, T, TDG, RX, RY, RZ, P = range(12)
CX, CY, CZ, SWAP, CP, CCX = 12, 13, 14, 15, 16, 17

OPTS = {"all": {}, "none": dict(collapse=False, diagonals=False, zz=False, group=1),
        "diag": dict(collapse=False), "win": dict(diagonals=False, zz=False),
        "blocked8": dict(block_bits=8)}


def plan(n, gates, **o):
    return np.array(W.to_circuit(n, gates).plan_export(**o))


def num_ops(p):
    return int(p[0])


def plan_ops(p):
    """Decode a flat plan into (kind, n_terms, global_phase) per op."""
    out, pos = [], 1
    for _ in range(int(p[0])):
        kind, ng, nt, gp = int(p[pos]), int(p[pos + 5]), int(p[pos + 6]), p[pos + 7]
        out.append((kind, nt, gp))
        pos += 16 + 9 * ng + 2 * nt
    return out


@pytest.mark.parametrize("n", [4, 7, 11])
@pytest.mark.parametrize("tag", list(OPTS))
def test_plan_matches_recorded_reference(n, tag, golden_circuits, golden_arrays):
    for name, gates in frozen_set(n, golden_circuits).items():
        want = golden_arrays[f"plan/{name}/{n}/{tag}"]
        got = plan(n, gates, **OPTS[tag])
        assert got.shape == want.shape, name
        assert np.abs(got - want).max() <= 1e-15, name


@pytest.mark.parametrize("n", [4, 7])
def test_every_plan_reproduces_the_circuit(n, golden_circuits):
    for name, gates in frozen_set(n, golden_circuits).items():
        want = oracle.run(n, gates)
        for tag, o in OPTS.items():
            got = oracle.run_plan(n, plan(n, gates, **o))
            assert np.abs(got - want).max() < 1e-12, (name, tag)


def test_unfused_is_one_to_one(golden_circuits):
    for n in (6, 10):
        for name, gates in frozen_set(n, golden_circuits).items():
            assert num_ops(plan(n, gates, **OPTS["none"])) == len(gates), name


def test_cancellation():
    assert num_ops(plan(3, [(H, (1,), ())] * 4)) == 0
    p = plan(2, [(RY, (0,), (1e-6,))] * 2)
    assert num_ops(p) == 1
    assert np.abs(oracle.run_plan(2, p) - oracle.run(2, [(RY, (0,), (1e-6,))] * 2)).max() < 1e-12
    assert num_ops(plan(2, [(X, (0,), ()), (H, (1,), ()), (X, (0,), ())])) == 1


def test_diagonal_algebra():
    ladder = [(CP, (k, 0), (math.pi / (1 << k),)) for k in range(1, 8)]
    p = plan(8, ladder)
    assert num_ops(p) == 1 and plan_ops(p)[0][1] == 7
    mixed = [(T, (0,), ()), (CZ, (0, 1), ()), (RZ, (2,), (0.3,)), (H, (3,), ()),
             (S, (1,), ()), (CP, (2, 3), (0.9,))]
    ops = plan_ops(plan(4, mixed))
    assert len(ops) == 3 and ops[0][1] == 3 and ops[2][1] == 2
    rz = [(H, (0,), ()), (RZ, (0,), (1.234,)), (CZ, (0, 1), ())]
    ops = plan_ops(plan(2, rz))
    assert len(ops) == 2 and abs(ops[1][2] + 0.617) < 1e-12


def test_fusion_ratio_qft16():
    c = W.to_circuit(16, W.qft(16))
    assert c.plan_size(fuse=False) == len(c)
    assert len(c) / c.plan_size(fuse=True) >= 3.0


def test_zz_recognised():
    g = [(H, (i,), ()) for i in range(4)]
    g += [(CX, (0, 1), ()), (RZ, (1,), (0.4,)), (CX, (0, 1), ())]
    ops = plan_ops(plan(4, g))
    assert ops[-1][0] == 4 and ops[-1][1] == 3      # one DiagonalLayer, 3 terms
    assert abs(ops[-1][2] + 0.2) < 1e-15


@pytest.mark.skipif(not oracle.ref_available(), reason="reference not compiled here")
@pytest.mark.parametrize("seed", range(8))
def test_plan_identical_to_live_reference(seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(4, 12))
    gates = (oracle.ref_circuit("random_circuit", n, 4, 0, seed) + W.qaoa_ring(n, 2)
             + W.random_u3(n, 2, seed) + W.qft_swap(n) + W.hea(n, 2, seed)
             + oracle.ref_circuit("local_patch", n, 4, 3, seed))
    for o in list(OPTS.values()) + [dict(group=2), dict(group=5), dict(block_bits=3)]:
        assert np.array_equal(plan(n, gates, **o), oracle.ref_plan(n, gates, **o)), o
