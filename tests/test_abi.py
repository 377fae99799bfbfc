"""The C boundary, without a GPU.

The library loads, exports every symbol that include/qmetal/*.h declares,
the public header is valid C11, and every failure path reports through the
return code and qm_last_error() rather than crashing (src/capi.cpp:19-38).
"""
import ctypes
import os
import re
import subprocess

import pytest

import qmetal_gb300 as qm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "qmetal", h) for h in ("qmetal.h", "qmetal_kernels.h")]


def declared(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qmk?_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(qm.library_path())
    missing = [s for h in HEADERS for s in declared(h) if not hasattr(lib, s)]
    assert not missing, missing
    assert len(declared(HEADERS[0])) >= 30 and len(declared(HEADERS[1])) >= 15


@pytest.mark.parametrize("header", HEADERS)
def test_header_is_plain_c11(header, tmp_path):
    src = tmp_path / "t.c"
    src.write_text(f'#include "{header}"\nint main(void) {{ return 0; }}\n')
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-fsyntax-only", str(src)], check=True)


def test_gate_codes_are_the_reference_numbering():
    assert (qm.X, qm.Y, qm.Z, qm.H, qm.S, qm.SDG, qm.T, qm.TDG) == tuple(range(8))
    assert (qm.RX, qm.RY, qm.RZ, qm.P, qm.CX, qm.CY, qm.CZ, qm.SWAP, qm.CP, qm.CCX) == \
        tuple(range(8, 18))


def test_diagnostics():
    assert qm.version() == (0, 1, 0)
    assert qm.max_qubits() == 34
    assert isinstance(qm.is_available(), bool)
    assert isinstance(qm.device_name(), str)


def test_circuit_errors_cross_as_exceptions():
    with pytest.raises(qm.QMetalError, match="out of range"):
        qm.Circuit(2).x(5)
    with pytest.raises(qm.QMetalError, match="arity"):
        qm.Circuit(2).add(qm.X, ())
    with pytest.raises(qm.QMetalError, match="unknown gate"):
        qm.Circuit(2).add(99, (0,))
    c = qm.Circuit(3)
    c.h(0).cx(0, 1).ccx(0, 1, 2)
    assert len(c) == 3 and c.plan_size(fuse=False) == 3


def test_unsupported_gate_fails_plan_closed():
    c = qm.Circuit(2)
    c.add(qm.X, (0, 1))           # a one-qubit kind given two wires
    assert c.plan_size() == 0     # size query reports 0 ...
    lib = ctypes.CDLL(qm.library_path())
    lib.qm_last_error.restype = ctypes.c_char_p
    assert b"unsupported" in lib.qm_last_error()   # ... and leaves the message


@pytest.mark.skipif(qm.is_available(), reason="checks the no-device path")
def test_no_device_fails_closed():
    with pytest.raises(qm.QMetalError):
        qm.Simulator(4)


def test_null_handles_are_rejected():
    lib = ctypes.CDLL(qm.library_path())
    lib.qm_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.qm_norm.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.qm_last_error.restype = ctypes.c_char_p
    assert lib.qm_run(None, None) == -1
    assert b"null" in lib.qm_last_error()
    assert lib.qm_norm(None, None) == -1


def test_kernel_layer_rejects_bad_arguments_without_launching():
    lib = ctypes.CDLL(qm.library_path())
    f = lib.qmk_apply_1q
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
    m = (ctypes.c_float * 8)()
    assert f(None, 4, 0, m, None) == -1                      # null state
    assert f(ctypes.c_void_p(16), 4, 9, m, None) == -1       # wire out of range
    assert f(ctypes.c_void_p(18), 4, 0, m, None) == -1       # misaligned


def test_wait_counter_sits_in_the_workspace_tail():
    """The bounded-wait count of the window tiles is per workspace: an aligned
    uint32 inside the workspace's bytes, clear of the reduction area."""
    lib = ctypes.CDLL(qm.library_path())
    lib.qmk_wait_counter.restype = ctypes.c_void_p
    lib.qmk_wait_counter.argtypes = [ctypes.c_void_p]
    lib.qmk_workspace_bytes.restype = ctypes.c_size_t
    lib.qmk_workspace_bytes.argtypes = [ctypes.c_uint32]
    base = 1 << 20                     # pointer arithmetic only: nothing is dereferenced
    ws_bytes = lib.qmk_workspace_bytes(20)
    at = lib.qmk_wait_counter(ctypes.c_void_p(base)) - base
    assert at % 16 == 0 and 0 < at and at + 4 <= ws_bytes
    assert ws_bytes - at <= 256 - 64   # the tail after the 1024 x 32 FP64 partials
    assert lib.qmk_wait_counter(None) is None
    take = lib.qmk_take_wait_timeouts
    take.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    out = ctypes.c_uint32(7)
    assert take(None, ws_bytes, ctypes.byref(out), None) == -1
    assert take(ctypes.c_void_p(base), 16, ctypes.byref(out), None) == -1
    assert take(ctypes.c_void_p(base), ws_bytes, None, None) == -1
    assert out.value == 7


def test_diagonal_adjoint_argument_limits_without_launching():
    """At most 48 generators a pass, each inside the state's wires; both are
    refused before anything reaches the device."""
    lib = ctypes.CDLL(qm.library_path())
    lib.qmk_workspace_bytes.restype = ctypes.c_size_t
    lib.qmk_workspace_bytes.argtypes = [ctypes.c_uint32]
    f = lib.qmk_adjoint_diagonal
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_uint32,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    n = 12
    ws_bytes = lib.qmk_workspace_bytes(n)
    fake = ctypes.c_void_p(1 << 20)          # never dereferenced: every call is refused
    gens = (ctypes.c_uint64 * 49)(*([3] * 49))
    slots = (ctypes.c_uint32 * 49)(*range(49))
    assert f(fake, fake, n, 0, None, None, 0.0, 49, gens, slots, fake, 1, fake, ws_bytes, None) == -1
    gens[47] = 1 << n                       # a generator outside the state's wires
    assert f(fake, fake, n, 0, None, None, 0.0, 48, gens, slots, fake, 1, fake, ws_bytes, None) == -1
    assert f(fake, fake, n, 0, None, None, 0.0, 48, None, slots, fake, 1, fake, ws_bytes, None) == -1
