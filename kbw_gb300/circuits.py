"""Seeded workload generators for the dense state-vector path.

A gate is a tuple ``(kind, target, controls, angle)`` with ``kind`` one of the
QuantumExecution trait gates (kbw src/quantum_execution.rs:58-79): X, Y, Z, H,
P, RX, RY, RZ.  CNOT is X with one control and CZ is Z with one control, as in
the reference's native gate mapping (src/quantum_execution.rs:356-357).

A Hamiltonian is a list of ``(coefficient, [(pauli, qubit), ...])`` with pauli
codes PAULI_X=1, PAULI_Y=2, PAULI_Z=3 (ket's Pauli-string terms).
"""
import math

import numpy as np

X, Y, Z, H, P, RX, RY, RZ = range(8)
GATE_NAMES = ["x", "y", "z", "h", "p", "rx", "ry", "rz"]
PARAMETRIC = (P, RX, RY, RZ)
PAULI_X, PAULI_Y, PAULI_Z = 1, 2, 3


def grover(num_qubits=12, marked=0, iterations=50):
    """Plain Grover search: H on all, then `iterations` rounds of the oracle
    (X-conjugated C^{n-1}Z on the marked index) and the diffusion operator
    (H, X on all, C^{n-1}Z, X, H).  The multi-controlled Z targets the top
    qubit with every other qubit as control."""
    n = num_qubits
    top = n - 1
    ctrl = tuple(range(n - 1))
    g = [(H, q, (), 0.0) for q in range(n)]
    zero_bits = [q for q in range(n) if not (marked >> q) & 1]
    for _ in range(iterations):
        g += [(X, q, (), 0.0) for q in zero_bits]
        g.append((Z, top, ctrl, 0.0))
        g += [(X, q, (), 0.0) for q in zero_bits]
        g += [(H, q, (), 0.0) for q in range(n)]
        g += [(X, q, (), 0.0) for q in range(n)]
        g.append((Z, top, ctrl, 0.0))
        g += [(X, q, (), 0.0) for q in range(n)]
        g += [(H, q, (), 0.0) for q in range(n)]
    return g


def grover_marked(seed):
    return int(np.random.default_rng(seed).integers(0, 4096))


def grover_success_probability(num_qubits, iterations):
    """Closed form sin^2((2k+1) asin(2^{-n/2}))."""
    return math.sin((2 * iterations + 1) * math.asin(2.0 ** (-num_qubits / 2))) ** 2


def brickwork(num_qubits=30, layers=20, seed=0):
    """Random brickwork circuit: per layer, one gate per qubit drawn from
    {H, X, Y, Z, S=P(pi/2), T=P(pi/4), RX, RY, RZ} with angles U[0, 2pi), then
    CNOT(i -> i+1) on disjoint pairs starting at offset 0 on even layers and
    offset 1 on odd layers."""
    rng = np.random.default_rng(seed)
    n = num_qubits
    g = []
    for layer in range(layers):
        choice = rng.integers(0, 9, size=n)
        angles = rng.uniform(0.0, 2.0 * math.pi, size=n)
        for q in range(n):
            c = int(choice[q])
            if c == 0:
                g.append((H, q, (), 0.0))
            elif c == 1:
                g.append((X, q, (), 0.0))
            elif c == 2:
                g.append((Y, q, (), 0.0))
            elif c == 3:
                g.append((Z, q, (), 0.0))
            elif c == 4:
                g.append((P, q, (), math.pi / 2))
            elif c == 5:
                g.append((P, q, (), math.pi / 4))
            elif c == 6:
                g.append((RX, q, (), float(angles[q])))
            elif c == 7:
                g.append((RY, q, (), float(angles[q])))
            else:
                g.append((RZ, q, (), float(angles[q])))
        for i in range(layer % 2, n - 1, 2):
            g.append((X, i + 1, (i,), 0.0))
    return g


def hea(num_qubits, layers, params):
    """Hardware-efficient ansatz: per layer RY then RZ on every qubit, then a
    CZ ring (i, i+1 mod n).  `params` has 2*n*layers angles, ordered
    layer-major as [RY q0..q{n-1}, RZ q0..q{n-1}] per layer."""
    n = num_qubits
    params = np.asarray(params, dtype=np.float64)
    assert params.size == 2 * n * layers
    g = []
    k = 0
    for _ in range(layers):
        for q in range(n):
            g.append((RY, q, (), float(params[k])))
            k += 1
        for q in range(n):
            g.append((RZ, q, (), float(params[k])))
            k += 1
        if n >= 2:
            for i in range(n):
                j = (i + 1) % n
                if n == 2 and i == 1:
                    break
                g.append((Z, j, (i,), 0.0))
    return g


def hea_param_index(num_qubits, layers):
    """param_index of hea(): each RY/RZ has its own parameter, CZ gates none."""
    n = num_qubits
    idx = []
    k = 0
    for _ in range(layers):
        for _q in range(2 * n):
            idx.append(k)
            k += 1
        if n >= 2:
            idx += [-1] * (n if n > 2 else 1)
    return idx


def hea_params(num_qubits, layers, seed):
    return np.random.default_rng(seed).uniform(-math.pi, math.pi, size=2 * num_qubits * layers)


def tfim_ring(num_qubits, zz=1.0, x=0.5):
    """Ring transverse-field Ising H = zz * sum Z_i Z_{i+1} + x * sum X_i."""
    n = num_qubits
    h = []
    for i in range(n):
        j = (i + 1) % n
        if n == 2 and i == 1:
            break
        h.append((zz, [(PAULI_Z, i), (PAULI_Z, j)]))
    for i in range(n):
        h.append((x, [(PAULI_X, i)]))
    return h


def hea_batch(num_circuits=4096, seed=0, min_qubits=8, max_qubits=20, min_layers=2, max_layers=8):
    """The batched forward workload: per circuit (n, L, params)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(min_qubits, max_qubits + 1, size=num_circuits)
    ls = rng.integers(min_layers, max_layers + 1, size=num_circuits)
    out = []
    for i in range(num_circuits):
        n, L = int(ns[i]), int(ls[i])
        out.append((n, L, rng.uniform(-math.pi, math.pi, size=2 * n * L)))
    return out


def random_circuit(num_qubits, num_gates, seed, max_controls=2, kinds=None):
    """Random gates of every kind with random targets and up to
    `max_controls` distinct controls; angles U[0, 2pi)."""
    rng = np.random.default_rng(seed)
    kinds = list(range(8)) if kinds is None else list(kinds)
    g = []
    for _ in range(num_gates):
        kind = kinds[int(rng.integers(0, len(kinds)))]
        t = int(rng.integers(0, num_qubits))
        others = [q for q in range(num_qubits) if q != t]
        nc = int(rng.integers(0, min(max_controls, len(others)) + 1))
        ctrl = tuple(int(c) for c in rng.choice(others, size=nc, replace=False)) if nc else ()
        angle = float(rng.uniform(0.0, 2.0 * math.pi)) if kind in PARAMETRIC else 0.0
        g.append((kind, t, ctrl, angle))
    return g


def uniform_draws(count, seed):
    """52-bit uniform draws in [0, 1): the value rand's UniformFloat derives
    from one u64 (`(x >> 12)` as the mantissa of a float in [1, 2), minus 1)."""
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 1 << 52, size=count, dtype=np.uint64)
    return bits.astype(np.float64) * (2.0 ** -52)
