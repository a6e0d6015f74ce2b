"""Generate the golden fixtures in this folder from an independent numpy model.

The model applies each gate as its textbook 2x2 matrix on one tensor axis of
the state (no bit-flip loops), computes Born-rule probabilities with numpy,
and applies rand's WeightedIndex selection rule (running sums, first sum above
u * scale) to explicit uniform draws.  It shares no code with the C oracle or
the CUDA engine; it only shares the workload generators in
kbw_gb300/circuits.py.

    python tests/golden/make_golden.py          # rewrites *.npz here
    python tests/golden/make_golden.py OUTDIR   # writes them elsewhere
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from kbw_gb300 import circuits as C  # noqa: E402

EPS_F64 = 1e-15


def matrix(kind, angle):
    c, s = math.cos(angle / 2), math.sin(angle / 2)
    if kind == C.X:
        return np.array([[0, 1], [1, 0]], complex)
    if kind == C.Y:
        return np.array([[0, -1j], [1j, 0]], complex)
    if kind == C.Z:
        return np.array([[1, 0], [0, -1]], complex)
    if kind == C.H:
        return np.array([[1, 1], [1, -1]], complex) / math.sqrt(2)
    if kind == C.P:
        return np.array([[1, 0], [0, np.exp(1j * angle)]], complex)
    if kind == C.RX:
        return np.array([[c, -1j * s], [-1j * s, c]], complex)
    if kind == C.RY:
        return np.array([[c, -s], [s, c]], complex)
    if kind == C.RZ:
        return np.array([[np.exp(-0.5j * angle), 0], [0, np.exp(0.5j * angle)]], complex)
    raise ValueError(kind)


def apply(psi, n, gate):
    kind, t, ctrl, angle = gate
    u = matrix(kind, angle)
    axis = n - 1 - t
    tens = psi.reshape((2,) * n)
    out = np.moveaxis(np.tensordot(u, tens, axes=([1], [axis])), 0, axis).reshape(-1)
    if ctrl:
        idx = np.arange(psi.size, dtype=np.uint64)
        m = np.uint64(sum(1 << c for c in ctrl))
        on = (idx & m) == m
        out = np.where(on, out, psi)
    return out


def run(n, gates):
    psi = np.zeros(1 << n, complex)
    psi[0] = 1.0
    for g in gates:
        psi = apply(psi, n, g)
    return psi


def uniform_scale(total):
    scale = total
    while scale * (1.0 - 2.0 ** -52) + 0.0 >= total:
        scale = np.nextafter(scale, 0.0)
    return scale


def measure(psi, n, qubits, draws):
    psi = psi.copy()
    out = 0
    idx = np.arange(psi.size, dtype=np.uint64)
    for index, q in enumerate(reversed(qubits)):
        bit = ((idx >> np.uint64(q)) & np.uint64(1)).astype(bool)
        p1 = float(np.sum(np.abs(psi[bit]) ** 2))
        p0 = max(1.0 - p1, 0.0)
        chosen = draws[index] * uniform_scale(p0 + p1)
        r = 1 if p0 <= chosen else 0
        prob = p1 if r else p0
        p = 1.0 / math.sqrt(max(prob, sys.float_info.min))
        psi = np.where(bit == bool(r), psi * p, 0)
        out |= r << index
    return out, psi


def pack(idx, qubits):
    packed = np.zeros(idx.size, np.uint64)
    for i, q in enumerate(reversed(qubits)):
        packed |= ((idx >> np.uint64(q)) & np.uint64(1)) << np.uint64(i)
    return packed


def sample(psi, qubits, shots, draws):
    idx = np.arange(psi.size, dtype=np.uint64)
    keep = np.abs(psi) > EPS_F64
    w = np.abs(psi[keep]) ** 2
    states = pack(idx[keep], qubits)
    run_sum = np.cumsum(w)
    cum, total = run_sum[:-1], run_sum[-1]
    chosen = np.asarray(draws[:shots]) * uniform_scale(total)
    picks = states[np.searchsorted(cum, chosen, side="right")]
    u, cnt = np.unique(picks, return_counts=True)
    return u.astype(np.uint64), cnt.astype(np.uint64)


def pauli_matrix(p):
    return {C.PAULI_X: np.array([[0, 1], [1, 0]], complex),
            C.PAULI_Y: np.array([[0, -1j], [1j, 0]], complex),
            C.PAULI_Z: np.array([[1, 0], [0, -1]], complex)}[p]


def expectation(psi, n, hamiltonian):
    total = 0.0
    for coef, terms in hamiltonian:
        phi = psi
        for p, q in terms:
            axis = n - 1 - q
            tens = phi.reshape((2,) * n)
            phi = np.moveaxis(np.tensordot(pauli_matrix(p), tens, axes=([1], [axis])), 0, axis).reshape(-1)
        total += coef * float(np.vdot(psi, phi).real)
    return total


def encode(gates):
    kinds = np.array([g[0] for g in gates], np.int8)
    targets = np.array([g[1] for g in gates], np.int8)
    masks = np.array([sum(1 << c for c in g[2]) for g in gates], np.uint64)
    angles = np.array([g[3] for g in gates], np.float64)
    return kinds, targets, masks, angles


def main(out=HERE):
    # 1. random small circuits with every gate kind and random controls
    cases = [(1, 30, 11), (2, 40, 12), (3, 60, 13), (5, 80, 14), (7, 100, 15), (9, 120, 16)]
    blob = {}
    for i, (n, ng, seed) in enumerate(cases):
        g = C.random_circuit(n, ng, seed, max_controls=min(3, n - 1) if n > 1 else 0)
        k, t, m, a = encode(g)
        blob["c%d_n" % i] = np.int64(n)
        blob["c%d_kind" % i], blob["c%d_target" % i] = k, t
        blob["c%d_ctrl" % i], blob["c%d_angle" % i] = m, a
        blob["c%d_state" % i] = run(n, g)
    blob["count"] = np.int64(len(cases))
    np.savez_compressed(os.path.join(out, "random_small.npz"), **blob)

    # 2. Grover 12q: full probability vector for seeds 0..2, P(marked) for 0..9,
    #    and a 1024-shot histogram from seeded draws for seed 0.
    blob = {}
    pm = []
    for seed in range(10):
        m = C.grover_marked(seed)
        psi = run(12, C.grover(12, m, 50))
        pm.append((m, float(abs(psi[m]) ** 2)))
        if seed < 3:
            blob["prob_seed%d" % seed] = (np.abs(psi) ** 2).astype(np.float64)
        if seed == 0:
            draws = C.uniform_draws(1024, 1000)
            st, ct = sample(psi, list(range(12)), 1024, draws)
            blob["sample_states"], blob["sample_counts"] = st, ct
            blob["sample_draws"] = draws
    blob["marked"] = np.array([x[0] for x in pm], np.int64)
    blob["p_marked"] = np.array([x[1] for x in pm], np.float64)
    np.savez_compressed(os.path.join(out, "grover12.npz"), **blob)

    # 3. measurement with injected draws on random entangled states
    blob = {}
    for i, (n, seed) in enumerate([(4, 21), (6, 22), (8, 23)]):
        g = C.random_circuit(n, 10 * n, seed, max_controls=2)
        psi = run(n, g)
        qubits = list(range(n)) if i != 1 else [5, 0, 3, 1]
        draws = C.uniform_draws(len(qubits), 500 + i)
        res, post = measure(psi, n, qubits, draws)
        k, t, m, a = encode(g)
        blob["m%d_n" % i] = np.int64(n)
        blob["m%d_kind" % i], blob["m%d_target" % i] = k, t
        blob["m%d_ctrl" % i], blob["m%d_angle" % i] = m, a
        blob["m%d_qubits" % i] = np.array(qubits, np.int64)
        blob["m%d_draws" % i] = draws
        blob["m%d_result" % i] = np.uint64(res)
        blob["m%d_post" % i] = post
        sd = C.uniform_draws(256, 600 + i)
        st, ct = sample(psi, qubits, 256, sd)
        blob["m%d_sdraws" % i], blob["m%d_sstates" % i], blob["m%d_scounts" % i] = sd, st, ct
    blob["count"] = np.int64(3)
    np.savez_compressed(os.path.join(out, "measure.npz"), **blob)

    # 4. TFIM ring expectation after HEA circuits (and a Y-containing string set)
    blob = {}
    for i, (n, L, seed) in enumerate([(4, 2, 31), (6, 3, 32), (8, 2, 33), (10, 2, 34)]):
        params = C.hea_params(n, L, seed)
        psi = run(n, C.hea(n, L, params))
        blob["e%d_n" % i], blob["e%d_L" % i] = np.int64(n), np.int64(L)
        blob["e%d_params" % i] = params
        blob["e%d_tfim" % i] = np.float64(expectation(psi, n, C.tfim_ring(n)))
        ham_y = [(0.7, [(C.PAULI_Y, 0), (C.PAULI_X, n - 1)]), (-1.3, [(C.PAULI_Y, 1)]),
                 (0.25, [(C.PAULI_Z, 2), (C.PAULI_Y, 3), (C.PAULI_X, 0)]), (2.0, [])]
        blob["e%d_mixed" % i] = np.float64(expectation(psi, n, ham_y))
    blob["count"] = np.int64(4)
    np.savez_compressed(os.path.join(out, "expval.npz"), **blob)
    print("golden fixtures written to", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
