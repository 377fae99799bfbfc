"""Shared test setup.

Builds the native library (and the CPU oracle) once per session before any
test imports them, registers the ``gpu`` marker, and loads the golden
fixtures recorded from the reference (tests/golden/).
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _build_native():
    spec = importlib.util.spec_from_file_location(
        "qmetal_build", os.path.join(ROOT, "qmetal_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


_build_native()

import oracle  # noqa: E402

oracle.build()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="session")
def golden_circuits():
    with open(os.path.join(GOLDEN, "circuits.json")) as f:
        raw = json.load(f)
    return {k: [(g[0], tuple(g[1]), tuple(g[2])) for g in v] for k, v in raw.items()}


@pytest.fixture(scope="session")
def golden_arrays():
    return dict(np.load(os.path.join(GOLDEN, "reference.npz")))


def frozen_set(n, circuits):
    """The reference's frozen benchmark set at width n (src/circuits.cpp:171-182);
    the two mt19937-seeded members come from the recorded fixtures."""
    from qmetal_gb300 import workloads as W
    return {
        "ghz": W.ghz(n),
        "qft": W.qft(n),
        "qaoa_ring_p6": W.qaoa_ring(n, 6),
        "tfim_trotter_20": W.tfim_trotter(n, 20),
        "grover_proxy_4": W.grover_proxy(n, 4),
        "random_d10": circuits[f"random_circuit_{n}_10_0x5eed"],
        "hea_d3": circuits[f"hardware_efficient_{n}_3_0x5eed"],
    }
