"""The allocation-free diagonal-layer entry point, through the C ABI.

qmk_apply_diagonal_noalloc serves callers that may not call cudaMalloc (an
application whose device memory all belongs to its own allocator, a plugin
that is only lent a state pointer and a stream): it runs the diagonal layer
with its scratch in a device array compiled into the library instead of a
caller workspace. Here it must agree with the workspace entry point
(qmk_apply_diagonal) on the same states, over two calls in a row, and reject
a state too large for its fixed scratch without launching anything.

This file is collected last so a run that stops at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes
from ctypes import c_double, c_int, c_size_t, c_uint32, c_void_p

import numpy as np
import pytest

import qmetal_gb300 as qm

pytestmark = pytest.mark.gpu
TOL = 1e-5   # the amplitude tolerance of the other GPU parity tests


def _lib():
    L = ctypes.CDLL(qm.library_path())
    L.qmk_workspace_bytes.restype = c_size_t
    L.qmk_workspace_bytes.argtypes = [c_uint32]
    L.qmk_workspace_init.restype = c_int
    L.qmk_workspace_init.argtypes = [c_void_p, c_size_t, c_void_p]
    L.qmk_apply_diagonal.restype = c_int
    L.qmk_apply_diagonal.argtypes = [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p,
                                     c_double, c_void_p, c_size_t, c_void_p]
    L.qmk_apply_diagonal_noalloc.restype = c_int
    L.qmk_apply_diagonal_noalloc.argtypes = [c_void_p, c_uint32, c_uint32, c_void_p,
                                             c_void_p, c_double, c_void_p]
    return L


def _layer(n, rng, count):
    """Random one- and two-bit masks (low, cross and high pairs at W = 13)."""
    masks, angles = [], []
    for _ in range(count):
        if rng.uniform() < 0.4:
            masks.append(1 << int(rng.integers(n)))
        else:
            a, b = rng.choice(n, size=2, replace=False)
            masks.append((1 << int(a)) | (1 << int(b)))
        angles.append(float(rng.uniform(-4, 4)))
    return (np.array(masks, dtype=np.uint64), np.array(angles, dtype=np.float64),
            float(rng.uniform(-1, 1)))


def test_noalloc_matches_workspace_entry_point_two_calls():
    torch = pytest.importorskip("torch")
    L = _lib()
    n = 20
    rng = np.random.default_rng(20)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v = (v / np.linalg.norm(v)).astype(np.complex64)
    host = torch.from_numpy(v.view(np.float32).copy())
    a = host.cuda()
    b = host.cuda()
    ws_bytes = L.qmk_workspace_bytes(n)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert L.qmk_workspace_init(ws.data_ptr(), ws_bytes, None) == 0
    for call in range(2):
        masks, angles, g = _layer(n, rng, 60 + 40 * call)
        rc_ws = L.qmk_apply_diagonal(a.data_ptr(), n, len(masks), masks.ctypes.data,
                                     angles.ctypes.data, g, ws.data_ptr(), ws_bytes, None)
        rc_na = L.qmk_apply_diagonal_noalloc(b.data_ptr(), n, len(masks), masks.ctypes.data,
                                             angles.ctypes.data, g, None)
        torch.cuda.synchronize()
        assert rc_ws == 0 and rc_na == 0, (call, rc_ws, rc_na)
        got = b.cpu().numpy().view(np.complex64)
        want = a.cpu().numpy().view(np.complex64)
        assert np.abs(got - want).max() <= TOL, call
        assert abs(np.linalg.norm(got.astype(np.complex128)) - 1.0) <= 1e-5
        # the layer did something: a phase layer moves the amplitudes
        assert np.abs(got - v).max() > 1e-3


def test_noalloc_rejects_state_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _lib()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    masks = np.array([1], dtype=np.uint64)
    angles = np.array([0.5], dtype=np.float64)
    rc = L.qmk_apply_diagonal_noalloc(buf.data_ptr(), 35, 1, masks.ctypes.data,
                                      angles.ctypes.data, 0.0, None)
    assert rc == -2      # QMK_ERR_TOO_LARGE, checked before any launch
    torch.cuda.synchronize()
    assert torch.count_nonzero(buf).item() == 0
