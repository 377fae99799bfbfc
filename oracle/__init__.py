"""CPU oracle for the statevector hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package, and only as the checker or the timed CPU baseline; the
shipped library never calls it and has no CPU fallback.

Two backends:
  * ``libqoracle.so`` -- qsim_oracle.c, a plain-C complex128 restatement of
    the reference's CPU oracle (src/reference.cpp) plus its sampling and
    adjoint algorithms (src/metal/simulator.mm:677-763, 782-963). Built by
    ``build()`` from source on whatever machine runs the tests. Gate loops
    run on OpenMP threads above 2^16 amplitudes (bit-identical to a serial
    run: every iteration writes its own elements); OMP_NUM_THREADS=1 gives
    the reference's single-thread behaviour.
  * ``_ref/libqref.so`` -- the reference project's own CPU sources compiled
    by build_ref.sh (only where those sources exist). Used to pin the
    restatement and the library's plan builder; absent elsewhere.

Gate streams are lists of (kind, qubits, params) with qm_gate_kind codes.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_long, c_size_t, c_uint32, c_uint64

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libqoracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libqref.so")

_d, _u32, _u64, _i32 = POINTER(c_double), POINTER(c_uint32), POINTER(c_uint64), POINTER(c_int32)


def build() -> str:
    """Compile qsim_oracle.c (seconds). Returns the library path."""
    src = os.path.join(HERE, "qsim_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", src, "-o", tmp,
                    "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_where = None


def reference_sources() -> str | None:
    """The reference project's source tree, where this machine has one (the
    recipe build_ref.sh decides: QMETAL_REFERENCE_SRC, else its default), or
    None."""
    global _where
    if _where is None:
        r = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), "--where"],
                           capture_output=True, text=True)
        _where = r.stdout.strip() if r.returncode == 0 else ""
    return _where or None


def build_ref() -> str | None:
    """Compile the reference's own CPU code when its sources are present."""
    src = reference_sources()
    if src is None:
        return None
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.run(["sh", script], check=True, env=dict(os.environ, QMETAL_REFERENCE_SRC=src),
                   capture_output=True)
    return REF_LIB


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        L.qo_run.restype = c_int
        L.qo_run.argtypes = [c_uint32, _d, c_size_t, _i32, _u32, _u32, _d]
        L.qo_run_plan.restype = c_int
        L.qo_run_plan.argtypes = [c_uint32, _d, _d, c_size_t]
        L.qo_apply_gate.restype = c_int
        L.qo_apply_gate.argtypes = [c_uint32, _d, c_int, _u32, c_uint32, _d]
        L.qo_norm.restype = c_double
        L.qo_norm.argtypes = [c_uint32, _d]
        L.qo_expectation.restype = c_double
        L.qo_expectation.argtypes = [c_uint32, _d, c_uint64, c_uint64, c_uint64]
        L.qo_sample_f32.restype = c_int
        L.qo_sample_f32.argtypes = [c_uint32, POINTER(ctypes.c_float), c_size_t, c_uint64,
                                    c_uint32, _u64]
        L.qo_energy_and_gradient.restype = c_int
        L.qo_energy_and_gradient.argtypes = [c_uint32, c_size_t, _i32, _u32, _u32, _d, _u32,
                                             c_uint32, _d, _u64, _u64, _u64, _d, _d]
        L.qo_gate_matrix.restype = c_int
        L.qo_gate_matrix.argtypes = [c_int, _d, _d]
        L.qo_set_threads.restype = None
        L.qo_set_threads.argtypes = [c_int]
        _lib = L
    return _lib


def set_threads(threads: int) -> None:
    """OpenMP threads for this process's oracle gate loops (1 = serial)."""
    lib().qo_set_threads(int(threads))


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref/libqref.so not built (reference sources absent)")
        L = ctypes.CDLL(REF_LIB)
        L.qref_run.restype = c_int
        L.qref_run.argtypes = [c_uint32, c_size_t, _i32, _u32, _u32, _d, _u32, _d, _d]
        L.qref_run_plan.restype = c_int
        L.qref_run_plan.argtypes = [c_uint32, c_size_t, _i32, _u32, _u32, _d, _u32, c_int,
                                    c_int, c_int, c_uint32, c_uint32, _d, _d]
        L.qref_plan.restype = c_long
        L.qref_plan.argtypes = [c_uint32, c_size_t, _i32, _u32, _u32, _d, _u32, c_int, c_int,
                                c_int, c_uint32, c_uint32, _d, c_size_t]
        L.qref_expectation.restype = c_int
        L.qref_expectation.argtypes = [c_uint32, _d, c_uint64, c_uint64, c_uint64, _d]
        L.qref_circuit.restype = c_long
        L.qref_circuit.argtypes = [c_char_p, c_uint32, c_uint32, c_uint32, c_uint64, _i32,
                                   _u32, _u32, _d, _u32, c_size_t]
        L.qref_last_error.restype = c_char_p
        _ref = L
    return _ref


# --- gate streams ------------------------------------------------------------

class Arrays:
    """Parallel arrays of a gate stream, in the layout both C libraries take."""

    def __init__(self, gates):
        g = len(gates)
        self.count = g
        self.kinds = np.zeros(max(g, 1), dtype=np.int32)
        self.nq = np.zeros(max(g, 1), dtype=np.uint32)
        self.np = np.zeros(max(g, 1), dtype=np.uint32)
        self.qubits = np.zeros(3 * max(g, 1), dtype=np.uint32)
        self.params = np.zeros(3 * max(g, 1), dtype=np.float64)
        for i, (k, qs, ps) in enumerate(gates):
            self.kinds[i] = k
            self.nq[i] = len(qs)
            self.np[i] = len(ps)
            self.qubits[3 * i:3 * i + len(qs)] = qs
            self.params[3 * i:3 * i + len(ps)] = ps

    def ptrs(self):
        return (self.kinds.ctypes.data_as(_i32), self.nq.ctypes.data_as(_u32),
                self.qubits.ctypes.data_as(_u32), self.params.ctypes.data_as(_d))


def _state(n, init):
    if init is None:
        st = np.zeros(1 << n, dtype=np.complex128)
        st[0] = 1.0
    else:
        st = np.array(init, dtype=np.complex128)
        assert st.size == 1 << n
    return np.ascontiguousarray(st)


def run(n, gates, init=None):
    """Gate-by-gate complex128 run (src/reference.cpp:161-206)."""
    st = _state(n, init)
    a = Arrays(gates)
    rc = lib().qo_run(n, st.ctypes.data_as(_d), a.count, *a.ptrs())
    if rc != 0:
        raise ValueError(f"oracle rejected gate {-rc - 1}")
    return st


def run_plan(n, plan, init=None):
    """Execute a flat serialised plan (src/reference.cpp:208-248)."""
    st = _state(n, init)
    p = np.ascontiguousarray(plan, dtype=np.float64)
    rc = lib().qo_run_plan(n, st.ctypes.data_as(_d), p.ctypes.data_as(_d), p.size)
    if rc != 0:
        raise ValueError(f"oracle rejected plan ({rc})")
    return st


def norm(n, st):
    st = np.ascontiguousarray(st, dtype=np.complex128)
    return lib().qo_norm(n, st.ctypes.data_as(_d))


def expectation(n, st, x=0, y=0, z=0):
    st = np.ascontiguousarray(st, dtype=np.complex128)
    return lib().qo_expectation(n, st.ctypes.data_as(_d), x, y, z)


def expectation_sum(n, st, terms):
    """terms: iterable of (coeff, x, y, z)."""
    return sum(c * expectation(n, st, x, y, z) for c, x, y, z in terms)


def sample_f32(n, amps64, shots, seed, block=1024):
    a = np.ascontiguousarray(amps64, dtype=np.complex64).view(np.float32)
    out = np.zeros(max(shots, 1), dtype=np.uint64)
    rc = lib().qo_sample_f32(n, a.ctypes.data_as(POINTER(ctypes.c_float)), shots, seed, block,
                             out.ctypes.data_as(_u64))
    assert rc == 0
    return out[:shots]


def energy_and_gradient(n, gates, terms):
    """Adjoint energy and per-gate gradient in complex128. terms: (c, x, y, z)."""
    a = Arrays(gates)
    t = list(terms)
    co = np.array([x[0] for x in t] or [0.0], dtype=np.float64)
    xs = np.array([x[1] for x in t] or [0], dtype=np.uint64)
    ys = np.array([x[2] for x in t] or [0], dtype=np.uint64)
    zs = np.array([x[3] for x in t] or [0], dtype=np.uint64)
    e = c_double()
    g = np.zeros(max(a.count, 1), dtype=np.float64)
    rc = lib().qo_energy_and_gradient(n, a.count, *a.ptrs(), a.np.ctypes.data_as(_u32), len(t),
                                      co.ctypes.data_as(_d), xs.ctypes.data_as(_u64),
                                      ys.ctypes.data_as(_u64), zs.ctypes.data_as(_u64),
                                      ctypes.byref(e), g.ctypes.data_as(_d))
    if rc != 0:
        raise ValueError(f"oracle gradient failed ({rc})")
    return e.value, g[:a.count]


def gate_matrix(kind, params=(0.0,)):
    p = np.zeros(3)
    p[:len(params)] = params
    out = np.zeros(8)
    assert lib().qo_gate_matrix(kind, p.ctypes.data_as(_d), out.ctypes.data_as(_d)) == 0
    return (out[0::2] + 1j * out[1::2]).reshape(2, 2)


# --- the reference itself (where compiled) ------------------------------------

def ref_run(n, gates, init=None):
    st = _state(n, init)
    out = np.zeros_like(st)
    a = Arrays(gates)
    init_p = st.ctypes.data_as(_d) if init is not None else None
    rc = ref().qref_run(n, a.count, *a.ptrs(), a.np.ctypes.data_as(_u32), init_p,
                        out.ctypes.data_as(_d))
    if rc != 0:
        raise ValueError(ref().qref_last_error().decode())
    return out


def ref_plan(n, gates, collapse=True, diagonals=True, zz=True, group=4, block_bits=0):
    a = Arrays(gates)
    args = (n, a.count, *a.ptrs(), a.np.ctypes.data_as(_u32), int(collapse), int(diagonals),
            int(zz), group, block_bits)
    size = ref().qref_plan(*args, None, 0)
    if size < 0:
        raise ValueError(ref().qref_last_error().decode())
    buf = np.zeros(size, dtype=np.float64)
    ref().qref_plan(*args, buf.ctypes.data_as(_d), size)
    return buf


def ref_expectation(n, st, x=0, y=0, z=0):
    st = np.ascontiguousarray(st, dtype=np.complex128)
    out = c_double()
    rc = ref().qref_expectation(n, st.ctypes.data_as(_d), x, y, z, ctypes.byref(out))
    if rc != 0:
        raise ValueError(ref().qref_last_error().decode())
    return out.value


def ref_circuit(name, n, a=0, b=0, seed=0x5eed):
    cap = 1 << 16
    kinds = np.zeros(cap, np.int32)
    nq = np.zeros(cap, np.uint32)
    qs = np.zeros(3 * cap, np.uint32)
    ps = np.zeros(3 * cap, np.float64)
    npar = np.zeros(cap, np.uint32)
    g = ref().qref_circuit(name.encode(), n, a, b, seed, kinds.ctypes.data_as(_i32),
                           nq.ctypes.data_as(_u32), qs.ctypes.data_as(_u32),
                           ps.ctypes.data_as(_d), npar.ctypes.data_as(_u32), cap)
    if g < 0:
        raise ValueError(ref().qref_last_error().decode())
    return [(int(kinds[i]), tuple(int(x) for x in qs[3 * i:3 * i + nq[i]]),
             tuple(float(x) for x in ps[3 * i:3 * i + npar[i]])) for i in range(g)]
