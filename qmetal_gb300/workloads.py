"""Gate-stream generators for the benchmark workloads and tests.

A gate stream is a list of ``(kind, qubits, params)`` tuples with the C ABI's
qm_gate_kind codes. ``to_circuit`` turns one into a ``Circuit``.

Two families:
  * restatements of the reference project's deterministic generators
    (src/circuits.cpp:24-93): ``ghz``, ``qft``, ``qaoa_ring``,
    ``tfim_trotter``, ``grover_proxy`` -- same gate streams, gate for gate;
  * seeded synthetic workloads for the statevector benchmark configurations:
    ``qft_swap`` (QFT with its swap layer), ``qaoa_ring_seeded``,
    ``tfim_chain``, ``hea``, ``random_u3``, ``hea_gradient_problem`` and
    ``maxcut_instances``. Seeds go through numpy's PCG64, so a stream is
    identical on every machine.
"""
from __future__ import annotations

import math

import numpy as np

X, Y, Z, H, S, SDG, T, TDG = range(8)
RX, RY, RZ, P = 8, 9, 10, 11
CX, CY, CZ, SWAP, CP, CCX = 12, 13, 14, 15, 16, 17


def to_circuit(n, gates):
    from . import Circuit
    c = Circuit(n)
    for k, qs, ps in gates:
        c.add(k, qs, ps)
    return c


def hot_wires_first(n, gates):
    """Qubit relabeling that puts the wires with the most one-qubit gates on
    the lowest indices (ties keep their order): perm[q] is q's new index."""
    count = [0] * n
    for _k, qs, _ps in gates:
        if len(qs) == 1:
            count[qs[0]] += 1
    order = sorted(range(n), key=lambda q: -count[q])
    perm = [0] * n
    for new, q in enumerate(order):
        perm[q] = new
    return perm


def relabel(gates, perm):
    """The gate stream with every qubit q renamed perm[q]."""
    return [(k, tuple(perm[q] for q in qs), ps) for k, qs, ps in gates]


def _zz(out, a, b, theta):
    # exp(-i theta Z_a Z_b) as CX / RZ(2 theta) / CX (src/circuits.cpp:11-16)
    out += [(CX, (a, b), ()), (RZ, (b,), (2.0 * theta,)), (CX, (a, b), ())]


# --- restatements of the reference generators ---------------------------------

def ghz(n):
    """H on wire 0, then a CX chain (src/circuits.cpp:24-31)."""
    return [(H, (0,), ())] + [(CX, (i, i + 1), ()) for i in range(n - 1)]


def qft(n):
    """Descending stages: H(j) then CP(k, j, pi / 2^(j-k)) for k < j, no swap
    layer (src/circuits.cpp:33-48)."""
    g = []
    for j in range(n - 1, -1, -1):
        g.append((H, (j,), ()))
        for k in range(j - 1, -1, -1):
            g.append((CP, (k, j), (math.pi / float(1 << (j - k)),)))
    return g


def qaoa_ring(n, p):
    """Fixed-angle ring QAOA (src/circuits.cpp:50-63)."""
    g = [(H, (i,), ()) for i in range(n)]
    for layer in range(p):
        gamma = 0.3 + 0.11 * layer
        beta = 0.7 - 0.05 * layer
        for i in range(n):
            _zz(g, i, (i + 1) % n, gamma)
        g += [(RX, (i,), (2.0 * beta,)) for i in range(n)]
    return g


def tfim_trotter(n, steps):
    """First-order TFIM chain, dt = 0.1, J = 1, h = 0.8 (src/circuits.cpp:65-75)."""
    dt, J, h = 0.1, 1.0, 0.8
    g = []
    for _ in range(steps):
        for i in range(n - 1):
            _zz(g, i, i + 1, J * dt)
        g += [(RX, (i,), (2.0 * h * dt,)) for i in range(n)]
    return g


def grover_proxy(n, iters):
    """src/circuits.cpp:77-93."""
    g = [(H, (i,), ()) for i in range(n)]
    for _ in range(iters):
        g.append((CZ, (n - 2, n - 1), ()))
        g += [(H, (i,), ()) for i in range(n)]
        g += [(X, (i,), ()) for i in range(n)]
        g.append((CZ, (n - 2, n - 1), ()))
        g += [(X, (i,), ()) for i in range(n)]
        g += [(H, (i,), ()) for i in range(n)]
    return g


# --- seeded workloads ----------------------------------------------------------

def qft_swap(n):
    """QFT followed by its swap layer: n H, n(n-1)/2 CP, n//2 SWAP."""
    return qft(n) + [(SWAP, (i, n - 1 - i), ()) for i in range(n // 2)]


def qaoa_ring_seeded(n, p=6, seed=1):
    """Ring QAOA, p layers, gamma and beta ~ U[0, pi]; ZZ as CX-RZ(2 gamma)-CX,
    mixer RX(2 beta)."""
    rng = np.random.default_rng(seed)
    gammas = rng.uniform(0.0, math.pi, p)
    betas = rng.uniform(0.0, math.pi, p)
    g = [(H, (i,), ()) for i in range(n)]
    for layer in range(p):
        for i in range(n):
            _zz(g, i, (i + 1) % n, float(gammas[layer]))
        g += [(RX, (i,), (2.0 * float(betas[layer]),)) for i in range(n)]
    return g


def tfim_chain(n, steps=20, J=1.0, h=0.7, dt=0.05):
    """First-order Trotter steps of H = -J sum Z_i Z_{i+1} - h sum X_i on a
    chain, from |0...0>: per step exp(-i J dt ZZ) on each bond (CX-RZ-CX) and
    RX(2 h dt) on each wire."""
    g = []
    for _ in range(steps):
        for i in range(n - 1):
            _zz(g, i, i + 1, J * dt)
        g += [(RX, (i,), (2.0 * h * dt,)) for i in range(n)]
    return g


def hea(n, depth=3, seed=3):
    """Hardware-efficient ansatz: RY, RZ per wire with angles ~ U[-pi, pi],
    then a CX ladder, per layer."""
    rng = np.random.default_rng(seed)
    g = []
    for _ in range(depth):
        ang = rng.uniform(-math.pi, math.pi, (n, 2))
        for q in range(n):
            g.append((RY, (q,), (float(ang[q, 0]),)))
            g.append((RZ, (q,), (float(ang[q, 1]),)))
        g += [(CX, (i, i + 1), ()) for i in range(n - 1)]
    return g


def random_u3(n, depth=10, seed=4):
    """Per layer: a Haar-random U3 on every wire, emitted layer by layer as
    RZ(lambda), RY(theta), RZ(phi) (U3 up to a global phase), then CZ on a
    seeded random set of disjoint pairs (a random perfect matching)."""
    rng = np.random.default_rng(seed)
    g = []
    for _ in range(depth):
        theta = np.arccos(1.0 - 2.0 * rng.uniform(0.0, 1.0, n))
        phi = rng.uniform(0.0, 2.0 * math.pi, n)
        lam = rng.uniform(0.0, 2.0 * math.pi, n)
        g += [(RZ, (q,), (float(lam[q]),)) for q in range(n)]
        g += [(RY, (q,), (float(theta[q]),)) for q in range(n)]
        g += [(RZ, (q,), (float(phi[q]),)) for q in range(n)]
        perm = rng.permutation(n)
        for i in range(0, n - 1, 2):
            a, b = int(perm[i]), int(perm[i + 1])
            g.append((CZ, (min(a, b), max(a, b)), ()))
    return g


def ring_tfim_hamiltonian(n, hx=0.7):
    """H = -sum_i Z_i Z_{i+1 mod n} - hx sum_i X_i as (coeff, x, y, z) terms."""
    terms = [(-1.0, 0, 0, (1 << i) | (1 << ((i + 1) % n))) for i in range(n)]
    terms += [(-hx, 1 << i, 0, 0) for i in range(n)]
    return terms


def hea_gradient_problem(n, depth=8, seed=5):
    """The adjoint benchmark: HEA (RY + RZ per wire per layer, CX ladder),
    angles ~ U[-pi, pi], and the ring TFIM Hamiltonian with hx = 0.7."""
    return hea(n, depth, seed), ring_tfim_hamiltonian(n, 0.7)


def to_hamiltonian(terms):
    from . import Hamiltonian
    h = Hamiltonian()
    for c, x, y, z in terms:
        h.add(c, x, y, z)
    return h


def random_3regular(n, rng):
    """A random simple 3-regular graph on n (even) vertices by the pairing
    model with rejection."""
    if n % 2 or n < 4:
        raise ValueError("3-regular graphs need an even n >= 4")
    while True:
        stubs = np.repeat(np.arange(n), 3)
        rng.shuffle(stubs)
        edges = set()
        ok = True
        for i in range(0, len(stubs), 2):
            a, b = int(stubs[i]), int(stubs[i + 1])
            if a == b or (min(a, b), max(a, b)) in edges:
                ok = False
                break
            edges.add((min(a, b), max(a, b)))
        if ok:
            return sorted(edges)


def maxcut_qaoa(n, edges, gammas, betas):
    """QAOA for MaxCut: H layer, then per layer ZZ(gamma) on every edge (as
    CX-RZ(2 gamma)-CX) and RX(2 beta) mixers."""
    g = [(H, (i,), ()) for i in range(n)]
    for gm, bt in zip(gammas, betas):
        for a, b in edges:
            _zz(g, a, b, float(gm))
        g += [(RX, (i,), (2.0 * float(bt),)) for i in range(n)]
    return g


def maxcut_hamiltonian(edges):
    """Cost operator C = sum_edges (1 - Z_a Z_b) / 2, as terms; the constant
    goes in as an identity term."""
    terms = [(0.5 * len(edges), 0, 0, 0)]
    terms += [(-0.5, 0, 0, (1 << a) | (1 << b)) for a, b in edges]
    return terms


def maxcut_instances(count=512, seed=6, n_lo=12, n_hi=26):
    """Seeded batch: n uniform over the even values in [n_lo, n_hi] (3-regular
    graphs need even n), a random 3-regular graph, p uniform in 1..8, gammas
    and betas ~ U[0, pi]. Returns dicts with n, edges, gammas, betas."""
    rng = np.random.default_rng(seed)
    evens = [n for n in range(n_lo, n_hi + 1) if n % 2 == 0]
    out = []
    for _ in range(count):
        n = int(rng.choice(evens))
        edges = random_3regular(n, rng)
        p = int(rng.integers(1, 9))
        out.append(dict(n=n, edges=edges, gammas=rng.uniform(0, math.pi, p).tolist(),
                        betas=rng.uniform(0, math.pi, p).tolist()))
    return out
