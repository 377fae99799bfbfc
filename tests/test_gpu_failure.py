"""Fail-closed paths on the GPU, driven without a GPU fault.

1. The bounded bulk-copy waits of the streamed adjoint window tiles: a test
   poll limit of 0 makes every in-loop wait give up at once (the copies still
   land: the wait before each block exits keeps the full bound). The gradient
   must fail closed with the reference's error convention (-1 and a message,
   src/capi.cpp:25-38), leave the state reset to |0...0>, and the next
   gradient on the same simulator, with the bound restored, must match the
   complex128 oracle.
2. QMETAL_FAULT=launch: every kernel-layer call of a simulator reports a
   failed launch on the host; the ABI call returns -1 with the message and
   nothing raises across the boundary.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _streamed_tiles(flat):
    """Window tiles of a backward schedule that hold four wires >= 6 and two
    ops per wire: the streamed (bulk-copy pipelined) warp-pair tiles."""
    count, pos = 0, 1
    for _ in range(int(flat[0])):
        kind = int(flat[pos])
        if kind == 0:
            nops = int(flat[pos + 1])
            wires = [int(flat[pos + 2 + 11 * k]) for k in range(nops)]
            if nops == 8 and len(set(wires)) == 4 and min(wires) >= 6:
                count += 1
            pos += 2 + 11 * nops
        elif kind == 1:
            nt = int(flat[pos + 2])
            ng = int(flat[pos + 4 + 2 * nt])
            pos += 5 + 2 * nt + 2 * ng
        elif kind == 2:
            n = int(flat[pos + 1])
            pos += 4 + n + int(flat[pos + 3 + n])
        else:
            pos += 2
    assert pos == len(flat)
    return count


def test_bulk_copy_wait_give_up_fails_closed_and_recovers():
    n = 14
    gates, terms = W.hea_gradient_problem(n, depth=3, seed=5)
    c, h = W.to_circuit(n, gates), W.to_hamiltonian(terms)
    assert _streamed_tiles(c.schedule_export("backward", tile_high=4)) >= 2
    e0, g0 = oracle.energy_and_gradient(n, gates, terms)
    sim = qm.Simulator(n)
    e, g = sim.energy_and_gradient(c, h)
    assert float(np.max(np.abs(np.array(g) - g0))) <= 1e-5

    sim.set_wait_poll_limit(0)
    with pytest.raises(qm.QMetalError, match="bulk-copy wait timed out"):
        sim.energy_and_gradient(c, h)
    # the refused pass left the state reset, not half undone
    st = sim.get_state()
    assert st[0] == 1.0 and float(np.abs(st[1:]).max()) == 0.0
    # the forward path takes no bounded wait: unaffected by the limit
    sim.reset()
    sim.run(c)
    assert float(np.abs(sim.get_state() - oracle.run(n, gates)).max()) <= 1e-5

    sim.set_wait_poll_limit(-1)
    for _ in range(2):
        e, g = sim.energy_and_gradient(c, h)
        assert abs(e - e0) <= 1e-5
        assert float(np.max(np.abs(np.array(g) - g0))) <= 1e-5


def test_injected_launch_fault_fails_closed():
    code = ("import qmetal_gb300 as qm\n"
            "from qmetal_gb300 import workloads as W\n"
            "s = qm.Simulator(6)\n"
            "try:\n"
            "    s.run(W.to_circuit(6, W.ghz(6)))\n"
            "    print('NO ERROR')\n"
            "except qm.QMetalError as e:\n"
            "    print('ERR', e)\n")
    env = dict(os.environ, QMETAL_FAULT="launch", PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "ERR" in r.stdout and "injected fault" in r.stdout, r.stdout
