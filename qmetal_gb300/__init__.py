"""qmetal on GB300: Python bindings over the C ABI.

A ctypes wrapper over ``libqmetal.so`` (include/qmetal/qmetal.h). The public
names and behaviour follow the reference project's wrapper
(python/qmetal/__init__.py:27-306): ``Circuit``, ``Simulator``,
``Hamiltonian``, ``QMetalError``, ``version``, ``is_available``,
``device_name``, ``max_qubits``. Only the loader differs (a Linux ``.so``
next to this file, or ``QMETAL_LIBRARY``), plus a few appended methods.

    import qmetal_gb300 as qmetal
    c = qmetal.Circuit(4)
    c.h(0)
    for i in range(3):
        c.cx(i, i + 1)
    sim = qmetal.Simulator(4)
    sim.run(c)
    print(sim.counts(1000))

There is no CPU fallback: if the library is missing or no CUDA device is
present, creating a Simulator raises QMetalError.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (
    POINTER, byref, c_char_p, c_double, c_float, c_int, c_size_t, c_uint32,
    c_uint64, c_void_p,
)

__all__ = ["Circuit", "Simulator", "Hamiltonian", "QMetalError", "version",
           "is_available", "device_name", "max_qubits", "library_path", "batch_serve"]


class QMetalError(RuntimeError):
    """Raised when the native library reports a failure."""


_HERE = os.path.dirname(os.path.abspath(__file__))


def library_path() -> str:
    env = os.environ.get("QMETAL_LIBRARY")
    if env:
        return env
    return os.path.join(_HERE, "libqmetal.so")


def _load():
    path = library_path()
    if not os.path.exists(path):
        raise QMetalError(
            f"{path} not found. Build it with `python qmetal_gb300/build.py`, "
            "or point QMETAL_LIBRARY at it.")
    return ctypes.CDLL(path)


_lib = _load()


def _decl(name, restype, *argtypes):
    fn = getattr(_lib, name)
    fn.restype = restype
    fn.argtypes = list(argtypes)
    return fn


_u64p, _f64p, _u32p, _f32p = (POINTER(c_uint64), POINTER(c_double),
                              POINTER(c_uint32), POINTER(c_float))


class _Hamiltonian(ctypes.Structure):
    _fields_ = [
        ("num_terms", c_uint32),
        ("coeffs", _f64p),
        ("x_masks", _u64p),
        ("y_masks", _u64p),
        ("z_masks", _u64p),
    ]


_version = _decl("qm_version", None, POINTER(c_int), POINTER(c_int), POINTER(c_int))
_last_error = _decl("qm_last_error", c_char_p)
_is_available = _decl("qm_is_available", c_int)
_device_name = _decl("qm_device_name", c_char_p)
_max_qubits = _decl("qm_max_qubits", c_uint32)
_max_buffer = _decl("qm_max_buffer_length", c_uint64)
_working_set = _decl("qm_recommended_working_set", c_uint64)

_circuit_create = _decl("qm_circuit_create", c_void_p, c_uint32)
_circuit_destroy = _decl("qm_circuit_destroy", None, c_void_p)
_circuit_add = _decl("qm_circuit_add", c_int, c_void_p, c_int, _u32p, c_uint32,
                     _f64p, c_uint32)
_circuit_size = _decl("qm_circuit_size", c_size_t, c_void_p)
_plan_size = _decl("qm_circuit_plan_size", c_size_t, c_void_p, c_int)
_plan_export = _decl("qm_circuit_plan_export", c_size_t, c_void_p, c_int, c_int,
                     c_int, c_uint32, c_uint32, _f64p, c_size_t)
_schedule_export = _decl("qm_schedule_export", c_size_t, c_void_p, POINTER(_Hamiltonian), c_int,
                         c_uint32, _f64p, c_size_t)

_create = _decl("qm_create", c_void_p, c_uint32)
_destroy = _decl("qm_destroy", None, c_void_p)
_reset = _decl("qm_reset", c_int, c_void_p)
_run = _decl("qm_run", c_int, c_void_p, c_void_p)
_run_unfused = _decl("qm_run_unfused", c_int, c_void_p, c_void_p)
_run_cached = _decl("qm_run_cached", c_int, c_void_p, c_void_p)
_run_merged = _decl("qm_run_merged", c_int, c_void_p, c_void_p)
_permute_qubits = _decl("qm_permute_qubits", c_int, c_void_p, _u32p, c_uint32)
_run_options = _decl("qm_run_options", c_int, c_void_p, c_void_p, c_int, c_int,
                     c_int, c_uint32, c_uint32)
_sync = _decl("qm_synchronize", c_int, c_void_p)
_num_qubits = _decl("qm_num_qubits", c_uint32, c_void_p)
_dim = _decl("qm_dim", c_uint64, c_void_p)
_dispatch_count = _decl("qm_dispatch_count", c_uint64, c_void_p)
_amplitudes = _decl("qm_amplitudes", _f32p, c_void_p)
_set_state = _decl("qm_set_state", c_int, c_void_p, _f32p, c_uint64)
_get_state = _decl("qm_get_state", c_int, c_void_p, _f32p, c_uint64)
_apply_gate = _decl("qm_apply_gate", c_int, c_void_p, c_int, _u32p, c_uint32,
                    _f64p, c_uint32)
_norm = _decl("qm_norm", c_int, c_void_p, _f64p)
_expect_pauli = _decl("qm_expectation_pauli", c_int, c_void_p, c_uint64,
                      c_uint64, c_uint64, _f64p)
_expect = _decl("qm_expectation", c_int, c_void_p, POINTER(_Hamiltonian), _f64p)
_expect_terms = _decl("qm_expectation_terms", c_int, c_void_p,
                      POINTER(_Hamiltonian), _f64p)
_sample = _decl("qm_sample", c_int, c_void_p, c_size_t, c_uint64, _u64p)
_energy_grad = _decl("qm_energy_and_gradient", c_int, c_void_p, c_void_p,
                     POINTER(_Hamiltonian), _f64p, _f64p)
_energy_grad_mode = _decl("qm_energy_and_gradient_mode", c_int, c_void_p, c_void_p,
                          POINTER(_Hamiltonian), c_int, _f64p, _f64p)
_elapsed = _decl("qm_elapsed", c_int, c_void_p, _f64p)
_wait_poll_limit = _decl("qm_set_wait_poll_limit", c_int, c_void_p, ctypes.c_int64)
_set_tile_high = _decl("qm_set_tile_high", c_int, c_void_p, c_uint32)


class _BatchItem(ctypes.Structure):
    _fields_ = [("circuit", c_void_p), ("hamiltonian", POINTER(_Hamiltonian)),
                ("shots", c_size_t), ("seed", c_uint64), ("out_energy", _f64p),
                ("out_grad", _f64p), ("out_samples", _u64p)]


_batch_serve = _decl("qm_batch_serve", c_int, POINTER(_BatchItem), c_size_t, c_int, c_uint32)
_batch_graph_timing = _decl("qm_batch_graph_timing", c_int, POINTER(c_double), POINTER(c_double),
                            POINTER(c_double), POINTER(c_uint64))
_batch_autotune = _decl("qm_batch_autotune", c_int, POINTER(_BatchItem), c_size_t, _u32p, _u32p,
                        _f64p)
_run_profiled = _decl("qm_run_profiled", c_int, c_void_p, c_void_p, c_int, _f64p,
                      c_size_t, POINTER(c_size_t))


def _err() -> str:
    return _last_error().decode("utf-8", "replace")


def _check(rc: int) -> None:
    if rc != 0:
        raise QMetalError(_err())


# Gate codes: qm_gate_kind in qmetal.h.
X, Y, Z, H, S, SDG, T, TDG = range(8)
RX, RY, RZ, P = 8, 9, 10, 11
CX, CY, CZ, SWAP, CP, CCX = 12, 13, 14, 15, 16, 17
U3 = 18   # appended to the ABI: U3(theta, phi, lambda), not differentiable


def version() -> tuple[int, int, int]:
    a, b, c = c_int(), c_int(), c_int()
    _version(byref(a), byref(b), byref(c))
    return a.value, b.value, c.value


def is_available() -> bool:
    return bool(_is_available())


def device_name() -> str:
    return _device_name().decode()


def max_qubits() -> int:
    return int(_max_qubits())


def max_buffer_length() -> int:
    return int(_max_buffer())


def recommended_working_set() -> int:
    return int(_working_set())


class Hamiltonian:
    """A real-weighted sum of Pauli strings, given as bitmasks."""

    def __init__(self):
        self.terms: list[tuple[float, int, int, int]] = []

    def add(self, coeff: float, x_mask: int = 0, y_mask: int = 0,
            z_mask: int = 0) -> "Hamiltonian":
        self.terms.append((float(coeff), int(x_mask), int(y_mask), int(z_mask)))
        return self

    def add_string(self, coeff: float, s: str) -> "Hamiltonian":
        """`s` is "IXYZ"-style, leftmost character is qubit 0."""
        x = y = z = 0
        for q, ch in enumerate(s.upper()):
            bit = 1 << q
            if ch == "X":
                x |= bit
            elif ch == "Y":
                y |= bit
            elif ch == "Z":
                z |= bit
            elif ch != "I":
                raise ValueError(f"bad Pauli character {ch!r}")
        return self.add(coeff, x, y, z)

    def __len__(self) -> int:
        return len(self.terms)

    def _c(self):
        n = len(self.terms)
        coeffs = (c_double * n)(*[t[0] for t in self.terms])
        xs = (c_uint64 * n)(*[t[1] for t in self.terms])
        ys = (c_uint64 * n)(*[t[2] for t in self.terms])
        zs = (c_uint64 * n)(*[t[3] for t in self.terms])
        h = _Hamiltonian(n, coeffs, xs, ys, zs)
        h._keep = (coeffs, xs, ys, zs)   # the arrays must outlive the struct
        return h


class Circuit:
    def __init__(self, num_qubits: int):
        self.num_qubits = int(num_qubits)
        self._h = _circuit_create(self.num_qubits)
        if not self._h:
            raise QMetalError(_err())

    def __del__(self):
        if getattr(self, "_h", None):
            _circuit_destroy(self._h)
            self._h = None

    def __len__(self) -> int:
        return int(_circuit_size(self._h))

    def _add(self, kind, qubits, params=()):
        qs = (c_uint32 * len(qubits))(*qubits)
        ps = (c_double * len(params))(*params) if params else None
        _check(_circuit_add(self._h, kind, qs, len(qubits), ps, len(params)))
        return self

    def add(self, kind: int, qubits, params=()):
        """Append a gate by its qm_gate_kind code."""
        return self._add(int(kind), tuple(int(q) for q in qubits),
                         tuple(float(p) for p in params))

    # single-qubit
    def x(self, q): return self._add(X, (q,))
    def y(self, q): return self._add(Y, (q,))
    def z(self, q): return self._add(Z, (q,))
    def h(self, q): return self._add(H, (q,))
    def s(self, q): return self._add(S, (q,))
    def sdg(self, q): return self._add(SDG, (q,))
    def t(self, q): return self._add(T, (q,))
    def tdg(self, q): return self._add(TDG, (q,))
    def rx(self, q, theta): return self._add(RX, (q,), (theta,))
    def ry(self, q, theta): return self._add(RY, (q,), (theta,))
    def rz(self, q, theta): return self._add(RZ, (q,), (theta,))
    def p(self, q, theta): return self._add(P, (q,), (theta,))
    def u3(self, q, theta, phi, lam): return self._add(U3, (q,), (theta, phi, lam))

    # multi-qubit
    def cx(self, c, t): return self._add(CX, (c, t))
    def cy(self, c, t): return self._add(CY, (c, t))
    def cz(self, a, b): return self._add(CZ, (a, b))
    def swap(self, a, b): return self._add(SWAP, (a, b))
    def cp(self, a, b, theta): return self._add(CP, (a, b), (theta,))
    def ccx(self, c0, c1, t): return self._add(CCX, (c0, c1, t))

    def plan_size(self, fuse: bool = True) -> int:
        """GPU passes this circuit lowers to -- what execution actually costs."""
        return int(_plan_size(self._h, 1 if fuse else 0))

    def plan_export(self, collapse=True, diagonals=True, zz=True, group=4,
                    block_bits=0):
        """The fused plan as the flat double list of qm_circuit_plan_export."""
        args = (self._h, int(collapse), int(diagonals), int(zz), int(group),
                int(block_bits))
        n = int(_plan_export(*args, None, 0))
        if n == 0:
            raise QMetalError(_err())
        buf = (c_double * n)()
        _plan_export(*args, buf, n)
        return list(buf)

    def schedule_export(self, which: str, hamiltonian: "Hamiltonian | None" = None,
                        tile_high: int = 4):
        """The executor's launch schedule as the flat double list of
        qm_schedule_export: which is "forward" (merged forward pass),
        "backward" (block-wise adjoint sweep) or "costate" (lambda = H psi of
        `hamiltonian`). Host only; needs no device."""
        code = {"forward": 0, "backward": 1, "costate": 2}[which]
        h = hamiltonian._c() if hamiltonian is not None else None
        hp = byref(h) if h is not None else None
        n = int(_schedule_export(self._h, hp, code, int(tile_high), None, 0))
        if n == 0:
            raise QMetalError(_err())
        buf = (c_double * n)()
        _schedule_export(self._h, hp, code, int(tile_high), buf, n)
        return list(buf)


class Simulator:
    def __init__(self, num_qubits: int):
        self._h = _create(int(num_qubits))
        if not self._h:
            raise QMetalError(_err())

    def __del__(self):
        if getattr(self, "_h", None):
            _destroy(self._h)
            self._h = None

    def close(self):
        self.__del__()

    def __enter__(self): return self
    def __exit__(self, *exc): self.__del__()

    @property
    def num_qubits(self) -> int: return int(_num_qubits(self._h))
    @property
    def dim(self) -> int: return int(_dim(self._h))
    @property
    def dispatch_count(self) -> int: return int(_dispatch_count(self._h))

    def reset(self): _check(_reset(self._h)); return self

    def run(self, circuit: Circuit, fuse: bool = True):
        _check((_run if fuse else _run_unfused)(self._h, circuit._h))
        return self

    def run_merged(self, circuit: Circuit):
        """run() with the executor's merging on top of the plan: wider
        one-qubit passes and CX / SWAP runs as one permutation pass."""
        _check(_run_merged(self._h, circuit._h))
        return self

    def permute_qubits(self, perm):
        """Relabel the state's qubits: qubit perm[q] then holds what qubit q
        held (one permutation pass)."""
        arr = (c_uint32 * len(perm))(*[int(p) for p in perm])
        _check(_permute_qubits(self._h, arr, len(perm)))
        return self

    def run_cached(self, circuit: Circuit):
        """run() replayed from a CUDA graph captured on the first call with
        this circuit's content (same kernels and results as run())."""
        _check(_run_cached(self._h, circuit._h))
        return self

    def run_options(self, circuit: Circuit, collapse=True, diagonals=True,
                    zz=True, group=4, block_bits=0):
        _check(_run_options(self._h, circuit._h, int(collapse), int(diagonals),
                            int(zz), int(group), int(block_bits)))
        return self

    def apply(self, kind: int, qubits, params=()):
        """One gate, applied immediately (no plan)."""
        qs = (c_uint32 * len(qubits))(*[int(q) for q in qubits])
        ps = (c_double * len(params))(*[float(p) for p in params]) if params else None
        _check(_apply_gate(self._h, int(kind), qs, len(qubits), ps, len(params)))
        return self

    def synchronize(self): _check(_sync(self._h)); return self

    def amplitudes(self):
        """numpy complex64 view of the host mirror of the state (refreshed by
        this call), or a list if numpy is absent."""
        p = _amplitudes(self._h)
        if not p:
            raise QMetalError(_err())
        n = self.dim
        try:
            import numpy as np
        except ImportError:
            return [complex(p[2 * i], p[2 * i + 1]) for i in range(n)]
        return np.ctypeslib.as_array(p, shape=(2 * n,)).view(np.complex64)

    def get_state(self):
        """A fresh numpy complex64 copy of the state."""
        import numpy as np
        out = np.empty(self.dim, dtype=np.complex64)
        _check(_get_state(self._h, out.ctypes.data_as(_f32p), self.dim))
        return out

    def set_state(self, state):
        import numpy as np
        a = np.ascontiguousarray(state, dtype=np.complex64)
        if a.size != self.dim:
            raise ValueError("state size must equal dim")
        _check(_set_state(self._h, a.ctypes.data_as(_f32p), self.dim))
        return self

    def norm(self) -> float:
        out = c_double()
        _check(_norm(self._h, byref(out)))
        return out.value

    def expectation(self, observable) -> float:
        out = c_double()
        if isinstance(observable, Hamiltonian):
            h = observable._c()
            _check(_expect(self._h, byref(h), byref(out)))
        elif isinstance(observable, str):
            h = Hamiltonian().add_string(1.0, observable)._c()
            _check(_expect(self._h, byref(h), byref(out)))
        else:
            raise TypeError("observable must be a Hamiltonian or a Pauli string")
        return out.value

    def expectation_pauli(self, x_mask=0, y_mask=0, z_mask=0) -> float:
        out = c_double()
        _check(_expect_pauli(self._h, int(x_mask), int(y_mask), int(z_mask), byref(out)))
        return out.value

    def expectation_terms(self, hamiltonian: Hamiltonian):
        h = hamiltonian._c()
        buf = (c_double * max(1, len(hamiltonian)))()
        _check(_expect_terms(self._h, byref(h), buf))
        return list(buf)[:len(hamiltonian)]

    def sample(self, shots: int, seed: int = 0):
        buf = (c_uint64 * int(shots))()
        _check(_sample(self._h, int(shots), int(seed), buf))
        return list(buf)

    def counts(self, shots: int, seed: int = 0) -> dict[str, int]:
        """Bitstring counts, little-endian: qubit 0 is the rightmost character."""
        n = self.num_qubits
        out: dict[str, int] = {}
        for v in self.sample(shots, seed):
            key = format(v, f"0{n}b")
            out[key] = out.get(key, 0) + 1
        return dict(sorted(out.items(), key=lambda kv: -kv[1]))

    def energy_and_gradient(self, circuit: Circuit, hamiltonian: Hamiltonian,
                            fused: bool = True):
        """Adjoint gradient: one entry per gate, zero where unparameterised.
        fused=False runs the reference's gate-by-gate backward sweep."""
        h = hamiltonian._c()
        energy = c_double()
        grad = (c_double * max(1, len(circuit)))()
        if fused:
            _check(_energy_grad(self._h, circuit._h, byref(h), byref(energy), grad))
        else:
            _check(_energy_grad_mode(self._h, circuit._h, byref(h), 1, byref(energy), grad))
        return energy.value, list(grad)[:len(circuit)]

    def set_tile_high(self, tile_high: int):
        """Wires >= 6 per backward window pass (1..6; five and six in block
        tiles of uniform rotation layers)."""
        _check(_set_tile_high(self._h, int(tile_high)))
        return self

    def set_wait_poll_limit(self, polls: int):
        """Fault injection for tests: the adjoint window passes' bounded
        bulk-copy waits give up after `polls` polls (0: at once), so the next
        gradient fails closed; a negative value restores the full bound."""
        _check(_wait_poll_limit(self._h, int(polls)))
        return self

    def run_profiled(self, circuit: Circuit, fuse: bool = True):
        """Run with a CUDA event between plan ops; returns each op's device
        seconds, in plan order."""
        cap = max(1, circuit.plan_size(fuse))
        buf = (c_double * cap)()
        count = c_size_t()
        _check(_run_profiled(self._h, circuit._h, int(fuse), buf, cap, byref(count)))
        return list(buf)[:count.value]

    def elapsed(self) -> float:
        """Device seconds since the previous call (CUDA events); synchronizes."""
        out = c_double()
        _check(_elapsed(self._h, byref(out)))
        return out.value


BATCH_LANES, BATCH_PLAIN_LOOP, BATCH_FUSED_LOOP, BATCH_GRAPH = 0, 1, 2, 3


def batch_graph_timing():
    """Seconds the calling thread's last BATCH_GRAPH batch spent recording,
    instantiating and executing its graph, and the graph's node count."""
    r, i, e, nodes = c_double(), c_double(), c_double(), c_uint64()
    _check(_batch_graph_timing(byref(r), byref(i), byref(e), byref(nodes)))
    return {"record_s": r.value, "instantiate_s": i.value, "execute_s": e.value,
            "nodes": int(nodes.value)}


def _batch_items(requests):
    import numpy as np
    reqs = list(requests)
    items = (_BatchItem * max(1, len(reqs)))()
    keep, outs = [], []
    for i, (circ, ham, shots, seed) in enumerate(reqs):
        h = ham._c()
        e = np.zeros(1, dtype=np.float64)
        g = np.zeros(max(1, len(circ)), dtype=np.float64)
        s = np.zeros(max(1, int(shots)), dtype=np.uint64)
        keep.append((h, circ))
        outs.append((e, g, s, len(circ), int(shots)))
        items[i].circuit = circ._h
        items[i].hamiltonian = ctypes.pointer(h)
        items[i].shots = int(shots)
        items[i].seed = int(seed)
        items[i].out_energy = e.ctypes.data_as(_f64p)
        items[i].out_grad = g.ctypes.data_as(_f64p)
        items[i].out_samples = s.ctypes.data_as(_u64p)
    return items, len(reqs), keep, outs


def batch_serve(requests, mode: int = BATCH_LANES, lanes: int = 8):
    """Energy, adjoint gradient and samples for many (circuit, hamiltonian,
    shots, seed) requests of any widths in one call. Returns a list of
    (energy, gradient list, samples list), in request order. lanes=0 uses
    the autotuned lane count and tile shapes."""
    items, count, _keep, outs = _batch_items(requests)
    _check(_batch_serve(items, count, int(mode), int(lanes)))
    return [(float(e[0]), g[:ng].tolist(), s[:ns].tolist()) for e, g, s, ng, ns in outs]


def batch_autotune(requests):
    """Tune a batch on its own requests; returns {"lanes", "tile_high"
    (width -> wires >= 6 per backward pass), "seconds"}."""
    items, count, _keep, _outs = _batch_items(requests)
    lanes = c_uint32()
    tile = (c_uint32 * (max_qubits() + 1))()
    secs = c_double()
    _check(_batch_autotune(items, count, byref(lanes), tile, byref(secs)))
    widths = sorted({int(c.num_qubits) for c, _h, _s, _seed in requests})
    return {"lanes": int(lanes.value), "seconds": float(secs.value),
            "tile_high": {n: int(tile[n]) for n in widths if n >= 7}}
