"""Host-side paths that need no GPU.

* The multi-process path of bench.py: two ranks over gloo on 127.0.0.1
  (torchrun), rank 0 alone prints the reference arm's JSON line and both
  ranks exit 0; the max-over-ranks helper agrees across ranks.
* Failure injection on the host (no device fault): QMETAL_FAULT=alloc makes
  simulator creation fail through the C ABI with a message.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cpu-qubits", "10"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1


WORKER = r'''
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
dist.init_process_group("gloo", init_method="env://")
import bench
rank = dist.get_rank()
v = bench.max_over_ranks(float(rank + 1) * 1.5, dist, 2)
bench.barrier(dist, 2)
print("MAX", rank, v, flush=True)
dist.destroy_process_group()
'''


def test_max_over_ranks_gloo_world2(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "w.py"
    script.write_text(WORKER.format(root=ROOT))
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port, LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
        assert "MAX" in o and o.strip().split()[-1] == "3.0"


def test_injected_allocation_fault_fails_closed():
    code = ("import qmetal_gb300 as qm\n"
            "try:\n    qm.Simulator(4)\n    print('NO ERROR')\n"
            "except qm.QMetalError as e:\n    print('ERR', e)\n")
    env = dict(os.environ, QMETAL_FAULT="alloc", PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       timeout=120, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "ERR" in r.stdout and "injected fault" in r.stdout
