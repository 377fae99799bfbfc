"""The executor's launch schedules, replayed in complex128 on the CPU.

qm_schedule_export hands out the exact step lists the GPU executor launches
for the merged forward pass, the co-state lambda = H psi and the block-wise
adjoint sweep. Each test interprets every step with numpy (a group pass as its
2x2s, a gather as dst[y] = src[A y ^ off], a window tile as gradient-then-undo
per op, a diagonal block as Z-string gradients then the conjugate phase) and
checks the result against the oracle's gate-by-gate algorithm -- the
reference's forward run and adjoint sweep (src/metal/simulator.mm:782-963) --
so the scheduling logic is pinned without a GPU. The structural limits the
kernels rely on (wires per tile, terms per pass) are asserted on the way.
"""
import numpy as np
import pytest

import oracle
import qmetal_gb300 as qm
from qmetal_gb300 import workloads as W
from conftest import frozen_set

X, Y, Z, H, S, SDG, T, TDG, RX, RY, RZ, P = range(12)
CX, CY, CZ, SWAP, CP, CCX = 12, 13, 14, 15, 16, 17

PAULI = {1: np.array([[0, 1], [1, 0]], dtype=complex),
         2: np.array([[0, -1j], [1j, 0]], dtype=complex),
         3: np.array([[1, 0], [0, -1]], dtype=complex)}


# --- numpy primitives ---------------------------------------------------------

def apply_1q(st, n, q, m):
    v = st.reshape(1 << (n - 1 - q), 2, 1 << q)
    return np.einsum("ab,ibj->iaj", m, v).reshape(-1)


def gather(st, n, cols, off):
    y = np.arange(1 << n, dtype=np.uint64)
    src = np.full(1 << n, off, dtype=np.uint64)
    for j, c in enumerate(cols):
        src ^= ((y >> np.uint64(j)) & np.uint64(1)) * np.uint64(c)
    return st[src.astype(np.int64)]


def pauli_apply(st, n, x, y, z):
    """P psi for P with masks (x, y, z): (P psi)[i] = i^ny (-1)^popc(j & (y|z)) psi[j], j = i ^ (x|y)."""
    idx = np.arange(1 << n, dtype=np.uint64)
    j = idx ^ np.uint64(x | y)
    par = np.zeros(1 << n, dtype=np.uint64)
    s = j & np.uint64(y | z)
    while s.any():
        par ^= s & np.uint64(1)
        s >>= np.uint64(1)
    sign = 1.0 - 2.0 * par.astype(np.float64)
    return (1j ** (bin(y).count("1") % 4)) * sign * st[j.astype(np.int64)]


def h_apply(st, n, terms):
    out = np.zeros_like(st)
    for c, x, y, z in terms:
        out += c * pauli_apply(st, n, x, y, z)
    return out


def diag_phase(n, masks, angles, gphase):
    idx = np.arange(1 << n, dtype=np.uint64)
    ph = np.full(1 << n, gphase)
    for m, a in zip(masks, angles):
        ph += np.where((idx & np.uint64(m)) == np.uint64(m), a, 0.0)
    return np.exp(1j * ph)


def plan_op(plan, k):
    """Op k of a flat plan (qm_circuit_plan_export) as a one-op flat plan."""
    pos = 1
    for i in range(int(plan[0])):
        ng, nt = int(plan[pos + 5]), int(plan[pos + 6])
        size = 16 + 9 * ng + 2 * nt
        if i == k:
            return np.concatenate([[1.0], plan[pos:pos + size]])
        pos += size
    raise IndexError(k)


def inverse_gate(g):
    kind, qs, ps = g
    if kind in (RX, RY, RZ, P, CP):
        return (kind, qs, (-ps[0],))
    return ({S: SDG, SDG: S, T: TDG, TDG: T}.get(kind, kind), qs, ps)


# --- decoders -----------------------------------------------------------------

class Reader:
    def __init__(self, v):
        self.v, self.p = v, 0

    def f(self):
        x = self.v[self.p]
        self.p += 1
        return x

    def i(self):
        return int(self.f())

    def mat(self):
        a = [self.f() for _ in range(8)]
        return np.array([[a[0] + 1j * a[1], a[2] + 1j * a[3]],
                         [a[4] + 1j * a[5], a[6] + 1j * a[7]]])

    def gather_map(self):
        n = self.i()
        cols = [self.i() for _ in range(n)]
        return cols, self.i()


def decode_forward(v):
    r, out = Reader(v), []
    for _ in range(r.i()):
        kind = r.i()
        if kind == 0:
            out.append(("group", [(r.i(), r.mat()) for _ in range(r.i())]))
        elif kind == 1:
            cols, off = r.gather_map()
            out.append(("permute", cols, off, [r.i() for _ in range(r.i())]))
        else:
            assert kind == 2
            out.append(("op", r.i()))
    assert r.p == len(v)
    return out


def decode_costate(v):
    r, out = Reader(v), []
    for _ in range(r.i()):
        kind = r.i()
        if kind == 0:
            out.append(("zdiag", [(r.i(), r.f()) for _ in range(r.i())]))
        elif kind == 1:
            ow = bool(r.i())
            out.append(("local", ow, [(r.i(), r.i(), r.i(), r.f()) for _ in range(r.i())]))
        elif kind == 2:
            ow, flip = bool(r.i()), r.i()
            out.append(("flip", ow, flip, [(r.i(), r.i(), r.f()) for _ in range(r.i())]))
        elif kind == 5:
            ow, energy = bool(r.i()), r.i()
            out.append(("xfield", ow, energy, [(r.i(), r.f()) for _ in range(r.i())]))
        else:
            assert kind in (3, 4)
            out.append(("zero",) if kind == 3 else ("dot",))
    assert r.p == len(v)
    return out


def decode_backward(v):
    r, out = Reader(v), []
    for _ in range(r.i()):
        kind = r.i()
        if kind == 0:
            out.append(("window", [(r.i(), r.mat(), r.i(), r.i()) for _ in range(r.i())]))
        elif kind == 1:
            undo = bool(r.i())
            terms = [(r.i(), r.f()) for _ in range(r.i())]
            gphase = r.f()
            gens = [(r.i(), r.i()) for _ in range(r.i())]
            out.append(("diag", undo, terms, gphase, gens))
        elif kind == 2:
            cols, off = r.gather_map()
            out.append(("permute", cols, off, [r.i() for _ in range(r.i())]))
        else:
            assert kind == 3
            out.append(("gate", r.i()))
    assert r.p == len(v)
    return out


# --- replays ------------------------------------------------------------------

def replay_forward(n, gates):
    c = W.to_circuit(n, gates)
    plan = np.array(c.plan_export())
    steps = decode_forward(c.schedule_export("forward"))
    st = np.zeros(1 << n, dtype=complex)
    st[0] = 1.0
    seen = []
    for s in steps:
        if s[0] == "group":
            wires = [w for w, _ in s[1]]
            assert wires == sorted(set(wires))
            zero = sum(w == 0 for w in wires)
            lane = sum(1 <= w <= 5 for w in wires)
            high = sum(w >= 6 for w in wires)
            assert zero <= 1
            assert ((1 <= lane <= 5 and high <= 4 and n >= 6 + high) or lane + high <= 5
                    or (lane == 0 and high <= 7 and n >= 6 + high))
            for w, m in s[1]:
                st = apply_1q(st, n, w, m)
        elif s[0] == "permute":
            assert len(s[3]) >= 2
            seen += s[3]
            st = gather(st, n, s[1], s[2])
        else:
            seen.append(s[1])
            st = oracle.run_plan(n, plan_op(plan, s[1]), init=st)
    assert seen == sorted(seen)   # plan order kept for everything but groups
    return st, steps


def replay_costate(n, psi, terms):
    """lambda = H psi by the co-state schedule, in complex128; the energy as
    the passes that carry it sum it (the ZZ pass, then each transverse-field
    pass's sum_w c_w <psi|X_w|psi>), or by the final dot. Returns lambda, the
    covered (coefficient, flip, sign, ny) terms and that energy."""
    h = W.to_hamiltonian(terms)
    steps = decode_costate(W.to_circuit(n, []).schedule_export("costate", h))
    lam = None
    covered = []
    energy = None
    assert steps[-1][0] in ("dot", "zdiag", "xfield")
    for k, s in enumerate(steps):
        if s[0] == "zdiag":
            assert k == 0 and lam is None
            lam = np.zeros_like(psi)
            for z, c in s[1]:
                assert bin(z).count("1") <= 2
                lam += c * pauli_apply(psi, n, 0, 0, z)
                covered.append((c, 0, z))
            energy = float(np.vdot(psi, lam).real)
        elif s[0] == "xfield":
            ow, emode, items = s[1], s[2], s[3]
            assert ow == (lam is None)
            if lam is None:
                lam = np.zeros_like(psi)
            wires = [w for w, _ in items]
            assert len(set(wires)) == len(wires) and n >= 10
            assert sum(w >= 6 for w in wires) <= 7
            part = np.zeros_like(psi)
            for w, c in items:
                part += c * pauli_apply(psi, n, 1 << w, 0, 0)
                covered.append((c, 1 << w, 0, 0))
            lam += part
            # the pass carries the energy exactly when no dot pass follows
            assert (emode != 0) == (steps[-1][0] != "dot")
            if emode:
                assert (emode == 1) == (energy is None)
                energy = (energy or 0.0) + float(np.vdot(psi, part).real)
        elif s[0] in ("local", "flip"):
            assert s[1] == (lam is None)   # only the first accumulation overwrites
            if lam is None:
                lam = np.zeros_like(psi)
            if s[0] == "local":
                items = s[2]
                assert 1 <= len(items) <= 16
                highs = {w for w, _, _, _ in items if w >= 6}
                assert len(highs) <= min(4, n - 6)
                for w, sign, ny, c in items:
                    flip = 1 << w
                    lam += c * (1j ** ny) * pauli_apply(psi, n, flip, 0, sign)
                    covered.append((c, flip, sign, ny))
            else:
                flip, items = s[2], s[3]
                assert 1 <= len(items) <= 16
                for sign, ny, c in items:
                    lam += c * (1j ** ny) * pauli_apply(psi, n, flip, 0, sign)
                    covered.append((c, flip, sign, ny))
        elif s[0] == "zero":
            assert lam is None
            lam = np.zeros_like(psi)
        else:
            assert k == len(steps) - 1
            energy = float(np.vdot(psi, lam).real)
    return lam, covered, energy


def assert_covers(covered, terms):
    """Every term once: coefficients summed per (flip, sign, Y count) agree
    (the transverse-field passes sum the terms on one wire)."""
    def key(x, y, z):
        return (x | y, y | z, bin(y).count("1"))
    want, got = {}, {}
    for c, x, y, z in terms:
        want[key(x, y, z)] = want.get(key(x, y, z), 0.0) + c
    for item in covered:
        if len(item) == 3:                      # a Z string of the ZZ pass
            c, _, z = item
            k = key(0, 0, z)
        else:
            c, flip, sign, ny = item
            k = (flip, sign, ny)
        got[k] = got.get(k, 0.0) + c
    assert set(got) == set(want)
    for k in want:
        assert abs(got[k] - want[k]) <= 1e-12 * max(1.0, abs(want[k])), k


def rotation_kind(minv, gen):
    """The rotation an undo matrix and generator describe, as the block tiles
    see it (after narrowing to float): rx, ry, rz, or None."""
    m = np.asarray(minv).reshape(2, 2).astype(np.complex64)
    diag = m[0, 1] == 0 and m[1, 0] == 0
    real = np.all(m.imag == 0)
    rxl = m[0, 0].imag == 0 and m[1, 1].imag == 0 and m[0, 1].real == 0 and m[1, 0].real == 0
    if diag and gen == 3:
        return "rz"
    if not diag and real and gen == 2:
        return "ry"
    if not diag and not real and rxl and gen == 1:
        return "rx"
    return None


def replay_backward(n, gates, terms, tile_high):
    c = W.to_circuit(n, gates)
    steps = decode_backward(c.schedule_export("backward", tile_high=tile_high))
    psi = oracle.run(n, gates)
    lam = h_apply(psi, n, terms)
    grad = np.zeros(len(gates))
    touched = np.zeros(len(gates), dtype=int)
    for s in steps:
        if s[0] == "window":
            ops = s[1]
            wires = {w for w, _, _, _ in ops}
            if n >= 6:
                assert len(ops) <= 32
                high = len({w for w in wires if w >= 6})
                assert high <= min(tile_high, n - 6)
                if high > 4:
                    # a block tile: wires >= 6 only, one rotation sequence each
                    assert min(wires) >= 6 and high <= 6
                    seqs = {tuple(rotation_kind(m, g) for ww, m, g, _ in ops if ww == w)
                            for w in wires}
                    assert len(seqs) == 1, seqs
                    seq = seqs.pop()
                    assert seq in {("rx",), ("ry",), ("rz",), ("rz", "ry"), ("ry", "rz")}, seq
            else:
                assert len(ops) <= 16
            ngrad = sum(g != 0 for _, _, g, _ in ops)
            if ngrad > 16:
                # only the compile-time first tile of an RZ-then-RY layer:
                # wire 0, wires 1..5 and four wires >= 6, each with RZ then
                # RY (undo order), twenty gradients
                assert ngrad <= 20 and set(range(6)) <= wires
                assert len({w for w in wires if w >= 6}) == 4
                for w in wires:
                    seq = tuple(rotation_kind(m, g) for ww, m, g, _ in ops if ww == w)
                    assert seq == ("rz", "ry"), seq
            for w, minv, gen, slot in ops:
                if gen:
                    pl = apply_1q(psi, n, w, PAULI[gen])
                    grad[slot] += np.vdot(lam, pl).imag
                    touched[slot] += 1
                psi = apply_1q(psi, n, w, minv)
                lam = apply_1q(lam, n, w, minv)
        elif s[0] == "diag":
            _, undo, tms, gphase, gens = s
            assert len(gens) <= 48
            for z, slot in gens:
                grad[slot] += np.vdot(lam, pauli_apply(psi, n, 0, 0, z)).imag
                touched[slot] += 1
            if undo:
                d = np.conj(diag_phase(n, [m for m, _ in tms], [a for _, a in tms], gphase))
                psi, lam = psi * d, lam * d
        elif s[0] == "permute":
            ks = s[3]
            assert len(ks) >= 2 and ks == sorted(ks, reverse=True)
            psi, lam = gather(psi, n, s[1], s[2]), gather(lam, n, s[1], s[2])
        else:
            inv = inverse_gate(gates[s[1]])
            psi = oracle.run(n, [inv], init=psi)
            lam = oracle.run(n, [inv], init=lam)
    return grad, touched, steps


# --- circuits -------------------------------------------------------------------

def random_mixed(n, count, seed):
    """Rotations RX/RY/RZ among fixed one-qubit gates, CX ladders and the
    other multi-qubit gates."""
    rng = np.random.default_rng(seed)
    g = []
    fixed1 = [X, Y, Z, H, S, SDG, T, TDG]
    while len(g) < count:
        r = rng.random()
        q = int(rng.integers(n))
        if r < 0.35:
            g.append((int(rng.choice([RX, RY, RZ])), (q,), (float(rng.uniform(-3, 3)),)))
        elif r < 0.5:
            g.append((int(rng.choice(fixed1)), (q,), ()))
        elif r < 0.7:
            a = int(rng.integers(n - 1))
            for i in range(a, min(n - 1, a + int(rng.integers(2, 6)))):
                g.append((CX, (i, i + 1), ()))
        elif r < 0.8:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            g.append((int(rng.choice([CY, SWAP, CZ, CX])), (a, b), ()))
        elif r < 0.9:
            a, b = (int(v) for v in rng.choice(n, 2, replace=False))
            t = float(rng.uniform(-2, 2))
            g += [(CX, (a, b), ()), (RZ, (b,), (t,)), (CX, (a, b), ())]
        else:
            a, b, c = (int(v) for v in rng.choice(n, 3, replace=False))
            g.append((CCX, (a, b, c), ()))
    return g


def random_terms(n, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        x = y = z = 0
        for q in rng.choice(n, int(rng.integers(1, min(4, n + 1))), replace=False):
            k = int(rng.integers(3))
            x |= (k == 0) << int(q)
            y |= (k == 1) << int(q)
            z |= (k == 2) << int(q)
        out.append((float(rng.normal()), x, y, z))
    return out


def one_flip_terms(n, seed):
    """Many terms that flip a single wire (X_i, Y_i Z_j, ...): the tiled path."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        for _ in range(3):
            x, y = (1 << q, 0) if rng.random() < 0.5 else (0, 1 << q)
            z = int(rng.integers(1 << n)) & ~(1 << q) & int(rng.integers(1 << n))
            out.append((float(rng.normal()), x, y, z))
    return out


def gradient_problems():
    out = []
    for n in (4, 7, 9, 11):
        out.append((f"hea{n}", n) + W.hea_gradient_problem(n, depth=3))
        out.append((f"mixed{n}", n, random_mixed(n, 90, n), random_terms(n, 12, n)))
    rng = np.random.default_rng(8)
    for n in (8, 10):
        edges = W.random_3regular(n, rng)
        out.append((f"maxcut{n}", n, W.maxcut_qaoa(n, edges, [0.4, 1.1], [0.7, 0.2]),
                    W.maxcut_hamiltonian(edges)))
    out.append(("tfim9", 9, W.tfim_chain(9, steps=4), W.ring_tfim_hamiltonian(9)))
    out.append(("u3_10", 10, W.random_u3(10, depth=3), one_flip_terms(10, 2)))
    # Wide enough for block tiles (five or six wires >= 6 of one rotation
    # sequence after the first tile of a layer).
    for n in (13, 14):
        out.append((f"hea{n}", n) + W.hea_gradient_problem(n, depth=2))
    edges = W.random_3regular(16, rng)
    out.append(("maxcut16", 16, W.maxcut_qaoa(16, edges, [0.4, 1.1], [0.7, 0.2]),
                W.maxcut_hamiltonian(edges)))
    return out


PROBLEMS = gradient_problems()


# --- tests ----------------------------------------------------------------------

@pytest.mark.parametrize("n", [4, 7, 11])
def test_forward_schedule_reproduces_the_circuit(n, golden_circuits):
    for name, gates in frozen_set(n, golden_circuits).items():
        st, _ = replay_forward(n, gates)
        assert np.abs(st - oracle.run(n, gates)).max() < 1e-12, name


@pytest.mark.parametrize("n", [6, 9, 12])
def test_forward_schedule_gathers_cx_ladders(n):
    gates = W.hea(n, depth=2) + random_mixed(n, 60, 100 + n)
    st, steps = replay_forward(n, gates)
    assert np.abs(st - oracle.run(n, gates)).max() < 1e-12
    assert any(s[0] == "permute" for s in steps)
    assert any(s[0] == "group" and len(s[1]) > 4 for s in steps)


@pytest.mark.parametrize("name,n,gates,terms", PROBLEMS, ids=[p[0] for p in PROBLEMS])
def test_costate_schedule_is_h_psi(name, n, gates, terms):
    psi = oracle.run(n, gates)
    lam, covered, energy = replay_costate(n, psi, terms)
    want = h_apply(psi, n, terms)
    assert np.abs(lam - want).max() < 1e-12
    assert abs(energy - float(np.vdot(psi, want).real)) < 1e-12
    assert_covers(covered, terms)


def transverse_field(n, hx, wires=None):
    return [(-hx, 1 << q, 0, 0) for q in (range(n) if wires is None else wires)]


@pytest.mark.parametrize("n", [8, 12])
def test_costate_schedule_edge_cases(n):
    psi = oracle.run(n, W.hea(n, depth=1))
    for terms in ([], [(0.5, 0, 0, 0)], [(1.0, 0, 0, 0b111)], one_flip_terms(n, 5),
                  [(1.0, 1 << 7, 0, 0)] * 20, random_terms(n, 40, 3),
                  transverse_field(n, 0.7), transverse_field(n, 0.3, [1, 3, 7]),
                  transverse_field(n, 0.3, [2]) + transverse_field(n, 0.1, [2]),
                  W.ring_tfim_hamiltonian(n, 0.7),
                  W.ring_tfim_hamiltonian(n, 0.7) + [(0.2, 0, 1 << 3, 1)]):
        lam, covered, energy = replay_costate(n, psi, terms)
        want = h_apply(psi, n, terms)
        assert np.abs(lam - want).max() < 1e-12, terms[:3]
        assert abs(energy - float(np.vdot(psi, want).real)) < 1e-12
        assert_covers(covered, terms)


@pytest.mark.parametrize("n,passes", [(10, 1), (13, 1), (14, 2), (20, 2), (28, 4), (34, 4)])
def test_transverse_field_passes(n, passes):
    """A transverse field on every wire: ceil((n - 6) / 7) block passes of
    as even a size as possible, wires 0..5 riding in the last; with the ZZ
    ring its passes carry the energy and no dot pass follows."""
    steps = decode_costate(W.to_circuit(n, []).schedule_export(
        "costate", W.to_hamiltonian(W.ring_tfim_hamiltonian(n, 0.7))))
    kinds = [s[0] for s in steps]
    assert kinds == ["zdiag"] + ["xfield"] * passes
    highs = [sum(w >= 6 for w, _ in s[3]) for s in steps[1:]]
    assert sum(highs) == n - 6 and max(highs) - min(highs) <= 1 and max(highs) <= 7
    assert [w for w, _ in steps[-1][3] if w < 6] == list(range(6))
    assert all(s[2] == 2 and not s[1] for s in steps[1:])
    # below ten qubits the same field goes by the per-wire tiles
    small = decode_costate(W.to_circuit(9, []).schedule_export(
        "costate", W.to_hamiltonian(W.ring_tfim_hamiltonian(9, 0.7))))
    assert "xfield" not in [s[0] for s in small] and small[-1][0] == "dot"
    # Below 6 qubits one-wire flips go by flip mask.
    steps = decode_costate(W.to_circuit(5, []).schedule_export(
        "costate", W.to_hamiltonian(one_flip_terms(5, 1))))
    assert all(s[0] != "local" for s in steps)


@pytest.mark.parametrize("name", ["hea13", "hea14", "maxcut16"])
def test_block_tiles_form_for_uniform_layers(name):
    """Rotation layers go five or six wires >= 6 per pass with tile_high 6,
    and never more than four with tile_high 4; with block tiles the first
    tile of a layer (wires 0..5) keeps no more wires >= 6 than leave the
    number of passes at its least."""
    _, n, gates, _ = next(p for p in PROBLEMS if p[0] == name)
    c = W.to_circuit(n, gates)
    passes = {}
    for th in (6, 4):
        steps = decode_backward(c.schedule_export("backward", tile_high=th))
        high = [len({w for w, _, _, _ in s[1] if w >= 6}) for s in steps if s[0] == "window"]
        assert max(high) >= 5 if th == 6 else max(high) == 4, (th, high)
        passes[th] = len(high)
    assert passes[6] <= passes[4]


@pytest.mark.parametrize("tile_high", [1, 2, 4, 5, 6])
@pytest.mark.parametrize("name,n,gates,terms", PROBLEMS, ids=[p[0] for p in PROBLEMS])
def test_backward_schedule_gradient(name, n, gates, terms, tile_high):
    grad, touched, steps = replay_backward(n, gates, terms, tile_high)
    _, want = oracle.energy_and_gradient(n, gates, terms)
    assert np.abs(grad - want).max() < 1e-10, name
    params = np.array([len(g[2]) > 0 for g in gates])
    # Every parameter read exactly once; no launch for a block that needs none.
    assert (touched == params).all()
    assert all(s[0] != "window" or s[1] for s in steps)


def test_backward_schedule_uses_every_step_kind():
    n = 9
    gates = random_mixed(n, 120, 42)
    kinds = {s[0] for s in replay_backward(n, gates, random_terms(n, 6, 1), 4)[2]}
    assert kinds == {"window", "diag", "permute", "gate"}


def test_backward_schedule_long_wire_and_tied():
    """A wire with more gates than a tile holds is split; a parameter used
    by many gates still gets one gradient slot per gate."""
    n = 7
    gates = [(H, (q,), ()) for q in range(n)]
    gates += [(RX if k % 2 else RY, (3,), (0.1 * k,)) for k in range(40)]
    gates += [(CX, (i, i + 1), ()) for i in range(n - 1)]
    gates += [(RZ, (q,), (0.3,)) for q in range(n)] * 3
    terms = W.ring_tfim_hamiltonian(n)
    grad, touched, steps = replay_backward(n, gates, terms, 2)
    _, want = oracle.energy_and_gradient(n, gates, terms)
    assert np.abs(grad - want).max() < 1e-10
    assert sum(s[0] == "window" for s in steps) >= 3


@pytest.mark.parametrize("n,split,undo", [(10, [45, 45], [True, False]),
                                          (11, [48, 7, 48, 7], [False, True, False, False])])
def test_backward_schedule_dense_cost_layer(n, split, undo):
    """Cost layers on the complete graph: 45 couplings take one diagonal
    pass, 55 a 48-generator pass and then the rest with the undo (none for
    the first layer, where the sweep ends)."""
    edges = [(a, b) for a in range(n) for b in range(a + 1, n)]
    gates = W.maxcut_qaoa(n, edges, [0.4, 1.3], [0.7, 0.2])
    terms = W.maxcut_hamiltonian(edges)
    grad, touched, steps = replay_backward(n, gates, terms, 2)
    _, want = oracle.energy_and_gradient(n, gates, terms)
    assert np.abs(grad - want).max() < 1e-10
    diag = [s for s in steps if s[0] == "diag" and s[4]]
    assert [len(s[4]) for s in diag] == split
    assert [bool(s[1]) for s in diag] == undo


def test_schedule_export_errors():
    c = W.to_circuit(3, [(H, (0,), ())])
    with pytest.raises(qm.QMetalError):
        c.schedule_export("costate")
    with pytest.raises(KeyError):
        c.schedule_export("sideways")


# --- property tests (hypothesis; skipped where it is not installed) -----------

def _gate_strategy(st, n):
    one = st.tuples(st.sampled_from([X, Y, Z, H, S, SDG, T, TDG]), st.integers(0, n - 1)).map(
        lambda t: (t[0], (t[1],), ()))
    rot = st.tuples(st.sampled_from([RX, RY, RZ]), st.integers(0, n - 1),
                    st.floats(-3.0, 3.0, allow_nan=False)).map(lambda t: (t[0], (t[1],), (t[2],)))
    pair = st.tuples(st.sampled_from([CX, CY, CZ, SWAP]), st.integers(0, n - 1),
                     st.integers(1, n - 1)).map(lambda t: (t[0], (t[1], (t[1] + t[2]) % n), ()))
    zz = st.tuples(st.integers(0, n - 1), st.integers(1, n - 1),
                   st.floats(-2.0, 2.0, allow_nan=False)).map(
        lambda t: [(CX, (t[0], (t[0] + t[1]) % n), ()), (RZ, ((t[0] + t[1]) % n,), (t[2],)),
                   (CX, (t[0], (t[0] + t[1]) % n), ())])
    ladder = st.integers(2, n).map(lambda k: [(CX, (i, i + 1), ()) for i in range(k - 1)])
    return st.lists(st.one_of(one.map(lambda g: [g]), rot.map(lambda g: [g]),
                              pair.map(lambda g: [g]), zz, ladder), min_size=4, max_size=30
                    ).map(lambda chunks: [g for c in chunks for g in c])


def test_random_circuits_replay_property():
    """Random circuits of every gate kind (rotations, fixed one-qubit gates,
    couplings, CX ladders, swaps) and random Hamiltonians: the forward
    schedule reproduces the gate-by-gate state and the backward schedule the
    adjoint gradient, for every tile shape."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=80, deadline=None, derandomize=True)
    @hyp.given(st.data())
    def check(data):
        n = data.draw(st.integers(2, 9))
        gates = data.draw(_gate_strategy(st, n))
        seed = data.draw(st.integers(0, 2**31 - 1))
        terms = random_terms(n, 5, seed) + one_flip_terms(n, seed)[:4]
        state, _ = replay_forward(n, gates)
        assert np.abs(state - oracle.run(n, gates)).max() < 1e-12
        tile_high = data.draw(st.integers(1, 6))
        grad, touched, _ = replay_backward(n, gates, terms, tile_high)
        _, want = oracle.energy_and_gradient(n, gates, terms)
        assert np.abs(grad - want).max() < 1e-10
        params = np.array([len(g[2]) > 0 for g in gates])
        assert (touched == params).all()
        lam, covered, _ = replay_costate(n, oracle.run(n, gates), terms)
        assert np.abs(lam - h_apply(oracle.run(n, gates), n, terms)).max() < 1e-12

    check()


@pytest.mark.parametrize("n,first,blocks", [(20, 2, [6, 6]), (22, 4, [6, 6]), (28, 4, [6, 6, 6]),
                                            (33, 4, [6, 6, 6, 5])])
def test_wide_first_tile_of_rzry_layers(n, first, blocks):
    """An HEA layer's first tile (wire 0, wires 1..5) takes four wires >= 6
    with their twenty gradients only where that saves a block pass (at 20
    qubits two and then 6 + 6 either way)."""
    gates, _ = W.hea_gradient_problem(n, depth=1, seed=5)
    steps = decode_backward(W.to_circuit(n, gates).schedule_export("backward", tile_high=6))
    shape = [len({w for w, _, _, _ in s[1] if w >= 6}) for s in steps if s[0] == "window"]
    assert shape == [first] + blocks, shape


def test_wide_first_tile_gradient_replay():
    n = 22
    gates, terms = W.hea_gradient_problem(n, depth=1, seed=7)
    grad, touched, steps = replay_backward(n, gates, terms, 6)
    assert max(sum(g != 0 for _, _, g, _ in s[1]) for s in steps if s[0] == "window") == 20
    _, want = oracle.energy_and_gradient(n, gates, terms)
    assert np.abs(grad - want).max() < 1e-10
    params = np.array([len(g[2]) > 0 for g in gates])
    assert (touched == params).all()


def test_wide_layers_and_fields_property():
    """Property test at 10..16 qubits, where the transverse-field co-state
    passes apply: random RY+RZ layers (on every wire or on a random subset)
    between CX ladders, and Hamiltonians of a ZZ ring, plain X fields on
    random wires (repeats summed) and sometimes other terms. The co-state
    replay gives H psi and the energy the passes carry; the backward replay
    gives the oracle's gradient. (The twenty-gradient first tile, which pays
    from 15 qubits, is pinned by the two tests above.)"""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(st.data())
    def check(data):
        n = data.draw(st.integers(10, 16))
        layers = data.draw(st.integers(1, 2))
        ang = st.floats(-3.0, 3.0, allow_nan=False)
        # (the ladder closes the Hadamard layer's window, so that each RY+RZ
        # layer is a window of its own)
        gates = [(H, (q,), ()) for q in range(n)] + [(CX, (q, q + 1), ()) for q in range(n - 1)]
        for _ in range(layers):
            full = data.draw(st.booleans())
            wires = list(range(n)) if full else sorted(
                data.draw(st.sets(st.integers(0, n - 1), min_size=1, max_size=n)))
            for q in wires:
                gates += [(RY, (q,), (data.draw(ang),)), (RZ, (q,), (data.draw(ang),))]
            gates += [(CX, (q, q + 1), ()) for q in range(n - 1)]
        field = data.draw(st.lists(st.integers(0, n - 1), min_size=1, max_size=2 * n))
        terms = [(-1.0, 0, 0, (1 << i) | (1 << ((i + 1) % n))) for i in range(n)]
        terms += [(data.draw(ang) / 3.0, 1 << w, 0, 0) for w in field]
        if data.draw(st.booleans()):
            terms += random_terms(n, 3, data.draw(st.integers(0, 2**31 - 1)))
        psi = oracle.run(n, gates)
        lam, covered, energy = replay_costate(n, psi, terms)
        want = h_apply(psi, n, terms)
        assert np.abs(lam - want).max() < 1e-12
        assert abs(energy - float(np.vdot(psi, want).real)) < 1e-12
        assert_covers(covered, terms)
        tile_high = data.draw(st.sampled_from([4, 5, 6]))
        grad, touched, _ = replay_backward(n, gates, terms, tile_high)
        _, g0 = oracle.energy_and_gradient(n, gates, terms)
        assert np.abs(grad - g0).max() < 1e-10
        params = np.array([len(g[2]) > 0 for g in gates])
        assert (touched == params).all()

    check()
