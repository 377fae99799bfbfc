"""The appended U3 gate (qm_gate_kind 18), on the CPU.

U3 is not in the reference's gate set (its ABI stops at CCX = 17 and asks
for new kinds to be appended). Its matrix is the OpenQASM
U(theta, phi, lambda); these tests pin it three ways: the library's matrix
(as the plan builder lowers it) against the closed form, the closed form
against e^{i(phi+lambda)/2} RZ(phi) RY(theta) RZ(lambda) in the oracle, and
fused plans containing U3 against gate-by-gate complex128 execution.
"""
import cmath
import math

import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W

RY, RZ, CX, CZ, H = 9, 10, 12, 14, 3
U3 = qm.U3


def closed_form(t, f, l):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -cmath.exp(1j * l) * s],
                     [cmath.exp(1j * f) * s, cmath.exp(1j * (f + l)) * c]])


ANGLES = [(0.3, -1.2, 2.1), (math.pi, 0.0, math.pi / 2), (0.0, 0.7, -0.2), (-2.9, 3.0, 1.4)]


@pytest.mark.parametrize("t,f,l", ANGLES)
def test_matrix_closed_form_and_decomposition(t, f, l):
    want = closed_form(t, f, l)
    assert np.abs(oracle.gate_matrix(U3, (t, f, l)) - want).max() <= 1e-15
    rz = lambda a: oracle.gate_matrix(RZ, (a,))
    ry = oracle.gate_matrix(RY, (t,))
    euler = cmath.exp(0.5j * (f + l)) * rz(f) @ ry @ rz(l)
    assert np.abs(euler - want).max() <= 1e-14
    # the plan builder lowers a lone U3 to one Dense1q op with that matrix
    c = qm.Circuit(1)
    c.u3(0, t, f, l)
    p = np.array(c.plan_export())
    assert int(p[0]) == 1 and int(p[1]) == 0
    m = (p[9:17:2] + 1j * p[10:17:2]).reshape(2, 2)
    assert np.abs(m - want).max() <= 1e-15


def test_fused_plans_with_u3_match_gate_by_gate():
    n = 7
    rng = np.random.default_rng(18)
    gates = [(H, (q,), ()) for q in range(n)]
    for layer in range(4):
        for q in range(n):
            gates.append((U3, (q,), tuple(float(x) for x in rng.uniform(-math.pi, math.pi, 3))))
        for q in range(layer % 2, n - 1, 2):
            gates.append((CX if layer % 2 else CZ, (q, q + 1), ()))
    want = oracle.run(n, gates)
    for opts in ({}, dict(group=2), dict(block_bits=4), dict(collapse=False)):
        flat = W.to_circuit(n, gates).plan_export(**opts)
        got = oracle.run_plan(n, flat)
        assert np.abs(got - want).max() <= 1e-12, opts


def test_u3_arity_and_parameter_count_fail_closed():
    c = qm.Circuit(3)
    with pytest.raises(qm.QMetalError, match="u3"):
        c.add(U3, (0,), (0.1, 0.2))
    with pytest.raises(qm.QMetalError, match="u3"):
        c.add(U3, (0, 1), (0.1, 0.2, 0.3))
    c.add(U3, (2,), (0.1, 0.2, 0.3))
    assert len(c) == 1
