"""The reference project's own clients against this library (CPU checks).

Where the reference's source tree is on this machine (oracle.reference_sources;
skipped elsewhere), its unmodified clients are pointed at this build:

* python/qmetal/__init__.py, the reference's ctypes wrapper, is loaded from
  where it lies with QMETAL_LIBRARY naming libqmetal.so. Its platform guard
  (python/qmetal/__init__.py:52-53) is satisfied in memory for the import
  only. Every symbol it declares must bind, and the checks of
  tests/test_python.py that need no device must hold: circuit building, the
  fusion visible through qm_circuit_plan_size, errors raised as its own
  QMetalError, and a failed Simulator creation reported, not crashed, where
  there is no device.
* tests/test_gpu.mm and bench/scale.mm, fusion_bench.mm and ablation.mm
  (plain C++ in .mm files) are compiled as C++ against this library's C++
  headers (include/cxx/qmetal/*.h in place of the reference's
  include/qmetal/{circuit,pauli,plan,simulator}.h), together with the
  reference's own oracle and generators (src/reference.cpp,
  src/circuits.cpp) from where they lie, and linked against libqmetal.so:
  the C++ surface of include/qmetal/simulator.h:30-112 is here, member for
  member. Outputs go to oracle/_ref/clients/ only.
"""
import importlib.util
import math
import os
import shutil
import subprocess
import sys

import pytest

import oracle
import qmetal_gb300 as qm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.reference_sources()
pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not on this machine")

WRAPPER_SYMBOLS = [
    "qm_version", "qm_last_error", "qm_is_available", "qm_device_name", "qm_max_qubits",
    "qm_circuit_create", "qm_circuit_destroy", "qm_circuit_add", "qm_circuit_size",
    "qm_circuit_plan_size", "qm_create", "qm_destroy", "qm_reset", "qm_run", "qm_run_unfused",
    "qm_synchronize", "qm_num_qubits", "qm_dim", "qm_dispatch_count", "qm_amplitudes",
    "qm_norm", "qm_expectation_pauli", "qm_expectation", "qm_sample", "qm_energy_and_gradient",
]


@pytest.fixture(scope="module")
def ref_wrapper():
    path = os.path.join(REF, "python", "qmetal", "__init__.py")
    spec = importlib.util.spec_from_file_location("qmetal_reference_wrapper", path)
    mod = importlib.util.module_from_spec(spec)
    mp = pytest.MonkeyPatch()
    mp.setenv("QMETAL_LIBRARY", qm.library_path())
    mp.setattr(sys, "platform", "darwin")
    try:
        spec.loader.exec_module(mod)     # binds every symbol at import
    finally:
        mp.undo()
    return mod


def test_wrapper_binds_every_symbol(ref_wrapper):
    text = open(os.path.join(REF, "python", "qmetal", "__init__.py")).read()
    declared = {line.split('"')[1] for line in text.splitlines() if '_decl("qm_' in line}
    assert declared == set(WRAPPER_SYMBOLS)
    lib = ref_wrapper._lib
    for name in declared:
        assert getattr(lib, name) is not None
    assert ref_wrapper.version() == qm.version()
    assert ref_wrapper.max_qubits() == 34
    assert ref_wrapper.is_available() == qm.is_available()


def test_wrapper_circuits_and_fusion(ref_wrapper):
    qmetal = ref_wrapper
    n = 6
    c = qmetal.Circuit(n)
    c.h(0)
    for i in range(n - 1):
        c.cx(i, i + 1)
    assert len(c) == n
    # tests/test_python.py: QFT-16, one pass per gate unfused, >= 3x fused
    qc = qmetal.Circuit(16)
    for j in range(15, -1, -1):
        qc.h(j)
        for k in range(j - 1, -1, -1):
            qc.cp(k, j, math.pi / (1 << (j - k)))
    assert qc.plan_size(fuse=False) == len(qc)
    assert len(qc) / qc.plan_size(fuse=True) >= 3.0
    # the same plan size as this package's own wrapper reports
    mine = qm.Circuit(16)
    for j in range(15, -1, -1):
        mine.h(j)
        for k in range(j - 1, -1, -1):
            mine.cp(k, j, math.pi / (1 << (j - k)))
    assert mine.plan_size(fuse=True) == qc.plan_size(fuse=True)
    # every gate method of the wrapper reaches qm_circuit_add
    g = qmetal.Circuit(3)
    for m in ("x", "y", "z", "h", "s", "sdg", "t", "tdg"):
        getattr(g, m)(1)
    for m in ("rx", "ry", "rz", "p"):
        getattr(g, m)(2, 0.3)
    g.cx(0, 1).cy(1, 2).cz(0, 2).swap(0, 1).cp(1, 2, 0.7).ccx(0, 1, 2)
    assert len(g) == 18


def test_wrapper_errors_cross_the_boundary(ref_wrapper):
    qmetal = ref_wrapper
    with pytest.raises(qmetal.QMetalError):
        qmetal.Circuit(2).x(5)
    with pytest.raises(qmetal.QMetalError):
        qmetal.Simulator(64)
    if not qmetal.is_available():
        # no device: creation fails closed with a message, never a crash
        with pytest.raises(qmetal.QMetalError, match="device"):
            qmetal.Simulator(4)
        return
    bad = qmetal.Circuit(2)
    bad.cp(0, 1, 0.3)
    with pytest.raises(qmetal.QMetalError):
        qmetal.Simulator(2).energy_and_gradient(bad, qmetal.Hamiltonian().add_string(1.0, "ZI"))


CXX_CLIENTS = ["tests/test_gpu.mm", "bench/scale.mm", "bench/fusion_bench.mm",
               "bench/ablation.mm"]


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
@pytest.mark.parametrize("client", CXX_CLIENTS)
def test_cpp_client_compiles_and_links(client):
    out_dir = os.path.join(ROOT, "oracle", "_ref", "clients")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, os.path.splitext(os.path.basename(client))[0])
    lib_dir = os.path.dirname(qm.library_path())
    cmd = ["g++", "-std=c++17", "-O0", "-w",
           "-include", os.path.join(ROOT, "tests", "cxx_compat", "darwin_time.h"),
           "-I", os.path.join(ROOT, "include", "cxx"), "-I", os.path.join(REF, "include"),
           "-x", "c++", os.path.join(REF, client),
           os.path.join(REF, "src", "reference.cpp"), os.path.join(REF, "src", "circuits.cpp"),
           "-x", "none", "-L", lib_dir, "-lqmetal", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    if not qm.is_available():
        # without a device the reference's GPU suite must decline, not crash
        if client == "tests/test_gpu.mm":
            run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
            assert run.returncode == 0 and "skipping" in run.stdout
