"""qmk_apply_group through the C ABI, on every route it takes.

One launch applies k commuting 2x2s on distinct wires: wire 0 within a
vector, wires 1..5 by warp shuffle, up to four wires >= 6 in registers
(k <= 10), wire 0 plus up to five others in registers, or wire 0 plus six or
seven wires >= 6 on a block of warps (one shared-memory transpose). Each case draws a
wire set for one route and compares the state with the same matrices applied
one wire at a time in complex128 (tolerance 1e-5, as the other amplitude
tests). Wire sets outside every route must be rejected without a launch.
"""
import ctypes
from ctypes import c_int, c_uint32, c_void_p

import numpy as np
import pytest

import qmetal_gb300 as qm

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _lib():
    L = ctypes.CDLL(qm.library_path())
    L.qmk_apply_group.restype = c_int
    L.qmk_apply_group.argtypes = [c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]
    return L


def _unitary(rng):
    z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _apply_ref(state, n, wires, mats):
    psi = state.reshape([2] * n)            # axis n-1-q is wire q (LSB first)
    for q, m in zip(wires, mats):
        ax = n - 1 - q
        psi = np.moveaxis(np.tensordot(m, psi, axes=([1], [ax])), 0, ax)
    return psi.reshape(-1)


def _route_cases(n, rng):
    """(wires) for each route the launch can take at width n."""
    cases = []
    for w0 in (False, True):
        for nlow in range(0, 6):
            for nhigh in range(0, min(4, n - 6) + 1):
                if nlow == 0 and not w0 and nhigh == 0:
                    continue
                low = sorted(rng.choice(np.arange(1, 6), size=nlow, replace=False).tolist())
                high = sorted(rng.choice(np.arange(6, n), size=nhigh, replace=False).tolist()) \
                    if nhigh else []
                cases.append(([0] if w0 else []) + low + high)
    # register route: wire 0 and up to five wires >= 1, none in 1..5
    if n >= 8:
        for k in range(1, min(5, n - 6) + 1):
            high = sorted(rng.choice(np.arange(6, n), size=k, replace=False).tolist())
            cases.append([0] + high)
    # five wires >= 1 without wire 0 (on warp pairs from n = 11), including
    # lane wires
    if n >= 11:
        cases.append(sorted(rng.choice(np.arange(6, n), size=5, replace=False).tolist()))
        cases.append([1, 3] + sorted(rng.choice(np.arange(6, n), size=3, replace=False).tolist()))
    # block route: six or seven wires >= 6, with and without wire 0
    for k in (6, 7):
        if n >= 6 + k:
            for w0 in (False, True):
                high = sorted(rng.choice(np.arange(6, n), size=k, replace=False).tolist())
                cases.append(([0] if w0 else []) + high)
    return cases


def _structured(rng, kind):
    """A 2x2 of one structure class: RX-like, real (RY-like), diagonal."""
    t = rng.uniform(-3, 3)
    c, s = np.cos(t / 2), np.sin(t / 2)
    if kind == "rx":
        return np.array([[c, -1j * s], [-1j * s, c]])
    if kind == "real":
        return np.array([[c, -s], [s, c]])
    return np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])


@pytest.mark.parametrize("n", [6, 7, 9, 10, 11, 12, 14])
def test_every_route_matches_complex128(n):
    torch = pytest.importorskip("torch")
    L = _lib()
    rng = np.random.default_rng(100 + n)
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    host = np.empty(2 << n, dtype=np.float32)
    host[0::2] = init.real
    host[1::2] = init.imag
    cases = [(w, "general") for w in _route_cases(n, rng)]
    cases += [(w, kind) for w in _route_cases(n, rng) if len(w) >= 5
              for kind in ("rx", "real", "diag")]
    for wires, kind in cases:
        mats = [_unitary(rng) if kind == "general" else _structured(rng, kind) for _ in wires]
        flat = np.empty(8 * len(wires), dtype=np.float32)
        for j, m in enumerate(mats):
            flat[8 * j:8 * j + 8] = [m[0, 0].real, m[0, 0].imag, m[0, 1].real, m[0, 1].imag,
                                     m[1, 0].real, m[1, 0].imag, m[1, 1].real, m[1, 1].imag]
        qs = np.array(wires, dtype=np.uint32)
        dev = torch.from_numpy(host.copy()).cuda()
        rc = L.qmk_apply_group(dev.data_ptr(), n, len(wires), qs.ctypes.data,
                               flat.ctypes.data, None)
        assert rc == 0, (n, wires)
        torch.cuda.synchronize()
        out = dev.cpu().numpy()
        got = out[0::2].astype(np.float64) + 1j * out[1::2]
        want = _apply_ref(init.copy(), n, wires, mats)
        assert np.abs(got - want).max() <= TOL, (n, wires)


def test_rejects_wire_sets_outside_every_route():
    torch = pytest.importorskip("torch")
    L = _lib()
    n = 12
    dev = torch.zeros(2 << n, dtype=torch.float32, device="cuda")
    flat = np.tile(np.array([1, 0, 0, 0, 0, 0, 1, 0], dtype=np.float32), 11)
    bad = [
        [1, 6, 7, 8, 9, 10],          # five wires >= 6 beside a lane wire
        [0, 1, 6, 7, 8, 9, 10, 11],   # six wires >= 6 beside a lane wire
        [3, 2],                       # not ascending
        [4, 4],                       # repeated
        [0, 12],                      # out of range
    ]
    for wires in bad:
        qs = np.array(wires, dtype=np.uint32)
        assert L.qmk_apply_group(dev.data_ptr(), n, len(wires), qs.ctypes.data,
                                 flat.ctypes.data, None) != 0, wires
    qs = np.arange(11, dtype=np.uint32)
    assert L.qmk_apply_group(dev.data_ptr(), n, 11, qs.ctypes.data, flat.ctypes.data, None) != 0


def _pauli_apply(state, n, flip, sign, ny, coeff):
    """coeff * i^ny * P psi with P given by flip (x|y) and sign (y|z) masks:
    (P psi)_i = (-1)^popcount((i ^ flip) & sign) psi_{i ^ flip}."""
    idx = np.arange(1 << n)
    src = idx ^ flip
    par = np.array([bin(int(s) & sign).count("1") & 1 for s in src])
    return coeff * (1j ** ny) * np.where(par, -1.0, 1.0) * state[src]


@pytest.mark.parametrize("n", [6, 8, 12])
def test_local_costate_terms(n):
    """qmk_pauli_accum_local: many single-flip terms (X, Y with Z signs) in
    one pass, overwrite and accumulate, against complex128."""
    torch = pytest.importorskip("torch")
    L = ctypes.CDLL(qm.library_path())
    f = L.qmk_pauli_accum_local
    f.restype = c_int
    f.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p,
                  c_void_p, c_int, c_void_p]
    rng = np.random.default_rng(300 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    lam0 = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    high = sorted(rng.choice(np.arange(6, n), size=min(4, n - 6), replace=False).tolist()) \
        if n > 6 else []
    pool = list(range(6)) + high
    for trial in range(6):
        nt = int(rng.integers(1, 17))
        wires = np.array([int(rng.choice(pool)) for _ in range(nt)], dtype=np.uint32)
        ny = np.array([int(rng.integers(0, 2)) for _ in range(nt)], dtype=np.uint32)
        signs = np.zeros(nt, dtype=np.uint64)
        coeffs = rng.uniform(-1, 1, nt)
        want = np.zeros(1 << n, dtype=complex)
        for t in range(nt):
            zmask = int(rng.integers(0, 1 << n)) & ~(1 << int(wires[t]))
            ymask = (1 << int(wires[t])) if ny[t] else 0
            signs[t] = ymask | zmask
            want += _pauli_apply(psi, n, 1 << int(wires[t]), int(signs[t]), int(ny[t]),
                                 coeffs[t])
        overwrite = trial % 2
        if not overwrite:
            want += lam0
        host_psi = np.empty(2 << n, dtype=np.float32)
        host_psi[0::2], host_psi[1::2] = psi.real, psi.imag
        host_lam = np.empty(2 << n, dtype=np.float32)
        host_lam[0::2], host_lam[1::2] = lam0.real, lam0.imag
        p = torch.from_numpy(host_psi).cuda()
        lam = torch.from_numpy(host_lam).cuda()
        assert f(lam.data_ptr(), p.data_ptr(), n, nt, wires.ctypes.data, signs.ctypes.data,
                 ny.ctypes.data, coeffs.ctypes.data, overwrite, None) == 0
        torch.cuda.synchronize()
        out = lam.cpu().numpy()
        got = out[0::2].astype(np.float64) + 1j * out[1::2]
        assert np.abs(got - want).max() <= 1e-5, (n, trial)
    # wires outside one tile, or too many terms, are refused before launch
    if n >= 12:
        wires = np.array([6, 7, 8, 9, 10], dtype=np.uint32)
        z = np.zeros(5, dtype=np.uint64)
        zi = np.zeros(5, dtype=np.uint32)
        c1 = np.ones(5)
        p = torch.zeros(2 << n, dtype=torch.float32, device="cuda")
        lam = torch.zeros_like(p)
        assert f(lam.data_ptr(), p.data_ptr(), n, 5, wires.ctypes.data, z.ctypes.data,
                 zi.ctypes.data, c1.ctypes.data, 1, None) != 0


@pytest.mark.parametrize("n", [10, 11, 12, 14, 17])
def test_xfield_costate(n):
    """qmk_xfield_costate: a transverse field on any of wires 0..5 and up to
    seven wires >= 6 per pass (sites of four to seven wires, padded with
    wires of coefficient 0), overwriting and accumulating lambda, with the
    energy left alone, written or added, against complex128."""
    torch = pytest.importorskip("torch")
    from ctypes import c_double, c_size_t
    L = ctypes.CDLL(qm.library_path())
    f = L.qmk_xfield_costate
    f.restype = c_int
    f.argtypes = [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_int, c_void_p,
                  c_int, c_void_p, c_size_t, c_void_p]
    L.qmk_workspace_bytes.restype = c_size_t
    L.qmk_workspace_bytes.argtypes = [c_uint32]
    wsb = L.qmk_workspace_bytes(n)
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(400 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    lam0 = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    idx = np.arange(1 << n)

    def dev(z):
        h = np.empty(2 << n, dtype=np.float32)
        h[0::2], h[1::2] = z.real, z.imag
        return torch.from_numpy(h).cuda()

    p = dev(psi)
    for trial in range(10):
        low = sorted(rng.choice(6, int(rng.integers(0, 7)), replace=False).tolist())
        k = int(rng.integers(0, min(7, n - 6) + 1))
        if trial == 0:
            low, k = list(range(6)), min(7, n - 6)
        high = sorted(rng.choice(np.arange(6, n), k, replace=False).tolist())
        wires = low + high
        if not wires:
            continue
        rng.shuffle(wires)
        coeffs = rng.uniform(-1, 1, len(wires))
        overwrite = trial % 2
        mode = trial % 3
        part = np.zeros(1 << n, dtype=complex)
        for w, c in zip(wires, coeffs):
            part += c * psi[idx ^ (1 << w)]
        want = part + (0 if overwrite else lam0)
        e_part = float(np.vdot(psi, part).real)
        lam = dev(lam0)
        d_e = torch.full((1,), 0.25, dtype=torch.float64, device="cuda")
        wa = np.array(wires, dtype=np.uint32)
        ca = np.array(coeffs, dtype=np.float64)
        rc = f(lam.data_ptr(), p.data_ptr(), n, len(wires), wa.ctypes.data, ca.ctypes.data,
               overwrite, d_e.data_ptr(), mode, ws.data_ptr(), wsb, None)
        assert rc == 0, (n, wires)
        torch.cuda.synchronize()
        out = lam.cpu().numpy()
        got = out[0::2].astype(np.float64) + 1j * out[1::2]
        assert np.abs(got - want).max() <= 1e-5, (n, trial, wires)
        e = float(d_e.cpu()[0])
        expect = {0: 0.25, 1: e_part, 2: 0.25 + e_part}[mode]
        assert abs(e - expect) <= 1e-5, (n, trial, mode)
    # refused before any launch: repeated, out-of-range or too many wires,
    # too narrow a state, an energy without a workspace
    lam = dev(lam0)
    d_e = torch.zeros(1, dtype=torch.float64, device="cuda")
    bad = [([3, 3], n), ([6, 6], n), ([n], n), (list(range(6, 14)), max(n, 14))]
    for wires, width in bad:
        if width != n:
            continue
        wa = np.array(wires, dtype=np.uint32)
        ca = np.ones(len(wires))
        assert f(lam.data_ptr(), p.data_ptr(), n, len(wires), wa.ctypes.data, ca.ctypes.data,
                 1, d_e.data_ptr(), 1, ws.data_ptr(), wsb, None) != 0, wires
    wa = np.array([0, 6], dtype=np.uint32)
    ca = np.ones(2)
    assert f(lam.data_ptr(), p.data_ptr(), 9, 2, wa.ctypes.data, ca.ctypes.data, 1,
             d_e.data_ptr(), 1, ws.data_ptr(), wsb, None) != 0
    assert f(lam.data_ptr(), p.data_ptr(), n, 2, wa.ctypes.data, ca.ctypes.data, 1,
             d_e.data_ptr(), 1, None, 0, None) != 0
