"""Pins the CPU oracle (restated kbw Dense<F>) against the golden fixtures made
by the independent numpy model and against closed-form known answers."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from kbw_gb300 import circuits as C
from conftest import decode_circuit, load_golden, rel_err


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_random_small_circuits(prec, tol):
    g = load_golden("random_small.npz")
    for i in range(int(g["count"])):
        n = int(g["c%d_n" % i])
        o = oracle.OracleDense(n, prec)
        o.apply(decode_circuit(g, "c%d" % i))
        assert rel_err(o.state(), g["c%d_state" % i]) < tol, (prec, i)


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 1e-4)])
def test_grover_probabilities(prec, tol):
    g = load_golden("grover12.npz")
    for seed in range(3):
        m = C.grover_marked(seed)
        assert m == int(g["marked"][seed])
        o = oracle.OracleDense(12, prec)
        o.apply(C.grover(12, m, 50))
        prob = np.abs(o.state()) ** 2
        assert np.max(np.abs(prob - g["prob_seed%d" % seed])) < tol
        assert abs(prob[m] - C.grover_success_probability(12, 50)) < tol


def test_grover_samples_bit_exact():
    g = load_golden("grover12.npz")
    o = oracle.OracleDense(12, "c128")
    o.apply(C.grover(12, C.grover_marked(0), 50))
    st, ct = o.sample(list(range(12)), 1024, g["sample_draws"])
    assert np.array_equal(st, g["sample_states"]) and np.array_equal(ct, g["sample_counts"])


def test_measure_and_sample_with_draws():
    g = load_golden("measure.npz")
    for i in range(int(g["count"])):
        n = int(g["m%d_n" % i])
        qubits = [int(q) for q in g["m%d_qubits" % i]]
        o = oracle.OracleDense(n, "c128")
        o.apply(decode_circuit(g, "m%d" % i))
        st, ct = o.sample(qubits, 256, g["m%d_sdraws" % i])
        assert np.array_equal(st, g["m%d_sstates" % i]) and np.array_equal(ct, g["m%d_scounts" % i])
        res = o.measure(qubits, g["m%d_draws" % i])
        assert res == int(g["m%d_result" % i])
        assert rel_err(o.state(), g["m%d_post" % i]) < 1e-12


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_exp_value(prec, tol):
    g = load_golden("expval.npz")
    for i in range(int(g["count"])):
        n, L = int(g["e%d_n" % i]), int(g["e%d_L" % i])
        o = oracle.OracleDense(n, prec)
        o.apply(C.hea(n, L, g["e%d_params" % i]))
        assert abs(o.exp_value(C.tfim_ring(n)) - float(g["e%d_tfim" % i])) < tol * n
        ham_y = [(0.7, [(C.PAULI_Y, 0), (C.PAULI_X, n - 1)]), (-1.3, [(C.PAULI_Y, 1)]),
                 (0.25, [(C.PAULI_Z, 2), (C.PAULI_Y, 3), (C.PAULI_X, 0)]), (2.0, [])]
        assert abs(o.exp_value(ham_y) - float(g["e%d_mixed" % i])) < tol * 10


def test_ghz_and_rotation_kats():
    o = oracle.OracleDense(5, "c128")
    o.hadamard(0)
    for q in range(4):
        o.pauli_x(q + 1, [q])
    st, re, im = o.dump(list(range(5)))
    assert list(st) == [0, 31]
    assert np.allclose(re, [1 / math.sqrt(2)] * 2) and np.allclose(im, 0)
    for theta in (0.3, 1.7, -2.2):
        o = oracle.OracleDense(1, "c128")
        o.ry(theta, 0)
        assert abs(o.exp_value([(1.0, [(C.PAULI_Z, 0)])]) - math.cos(theta)) < 1e-14
        o = oracle.OracleDense(1, "c128")
        o.rx(theta, 0)
        assert abs(o.exp_value([(1.0, [(C.PAULI_Y, 0)])]) + math.sin(theta)) < 1e-14


def test_gate_inverse_identity_and_norm():
    n = 6
    g = C.random_circuit(n, 60, 7, max_controls=2)
    o = oracle.OracleDense(n, "c128")
    o.apply(g)
    assert abs(np.linalg.norm(o.state()) - 1.0) < 1e-13
    inv = []
    for kind, t, c, a in reversed(g):
        if kind in (C.P, C.RX, C.RY, C.RZ):
            inv.append((kind, t, c, -a))
        else:
            inv.append((kind, t, c, a))
    o.apply(inv)
    ref = np.zeros(1 << n, complex)
    ref[0] = 1
    assert rel_err(o.state(), ref) < 1e-13


def test_swap_relabel_invariance():
    """Swapping qubits a,b, applying the gate list with a,b exchanged and
    swapping back equals the flat run (the Block wrapper's contract)."""
    n = 6
    g = C.random_circuit(n, 40, 9, max_controls=2)
    flat = oracle.OracleDense(n, "c128")
    flat.apply(g)
    a, b = 1, 5
    swap = {a: b, b: a}
    o = oracle.OracleDense(n, "c128")
    o.swap_qubits(a, b)
    o.apply([(k, swap.get(t, t), tuple(swap.get(c, c) for c in cs), ang) for k, t, cs, ang in g])
    o.swap_qubits(a, b)
    assert rel_err(o.state(), flat.state()) < 1e-14


def test_weighted_index_rule():
    assert oracle.uniform_scale(1.0) == 1.0
    # every double in [1, 2) keeps its scale (max draw * scale stays below it)
    for t in (1.5, 1.9999999999999998, 0.75, 3.0):
        s = oracle.uniform_scale(t)
        assert s <= t and s * (1 - 2.0 ** -52) < t


def test_too_many_qubits_rejected():
    with pytest.raises(ValueError):
        oracle.OracleDense(33, "c64")


def test_golden_fixtures_regenerate(tmp_path):
    """The committed fixtures are exactly what tests/golden/make_golden.py
    (the independent numpy model) produces."""
    from conftest import GOLDEN
    r = subprocess.run([sys.executable, os.path.join(GOLDEN, "make_golden.py"), str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for f in ("random_small.npz", "grover12.npz", "measure.npz", "expval.npz"):
        a = np.load(os.path.join(GOLDEN, f))
        b = np.load(os.path.join(str(tmp_path), f))
        assert set(a.files) == set(b.files), f
        for k in a.files:
            assert np.allclose(a[k], b[k], rtol=0, atol=1e-13), (f, k)


def _libm_f32():
    import ctypes
    import ctypes.util
    m = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    for f in ("cosf", "sinf"):
        getattr(m, f).restype = ctypes.c_float
        getattr(m, f).argtypes = [ctypes.c_float]
    return m


def _densev2_apply(re, im, n, gate, f32=None):
    """One gate in DenseV2's in-place form (src/dense_v2.rs:166-280) with its
    own expressions, in numpy binary64 or (f32: libm handle) binary32: pairs
    (ket0, ket1) split at the target bit, complex products as num's Mul
    (re*re' - im*im', re*im' + im*re'), constants from libm (cos/sin through
    Python's math module; cosf/sinf of the binary32 angle)."""
    kind, t, ctrl, a = gate
    if f32 is None:
        T, cos, sin = float, math.cos, math.sin
    else:
        T = np.float32
        cos = lambda x: np.float32(f32.cosf(float(np.float32(x))))  # noqa: E731
        sin = lambda x: np.float32(f32.sinf(float(np.float32(x))))  # noqa: E731
    idx = np.arange(1 << n)
    mask = 0
    for c in ctrl:
        mask |= 1 << c
    i0 = idx[((idx >> t) & 1 == 0) & ((idx & mask) == mask)]
    i1 = i0 | (1 << t)
    r0, m0, r1, m1 = re[i0].copy(), im[i0].copy(), re[i1].copy(), im[i1].copy()

    def cmul(r, m, cr, ci):
        return r * cr - m * ci, r * ci + m * cr

    if kind == C.X:
        re[i0], im[i0], re[i1], im[i1] = r1, m1, r0, m0
    elif kind == C.Y:  # swap, then ket0 *= -i, ket1 *= i
        re[i0], im[i0] = cmul(r1, m1, T(-0.0), T(-1.0))
        re[i1], im[i1] = cmul(r0, m0, T(0.0), T(1.0))
    elif kind == C.Z:  # ket1 *= -1
        re[i1], im[i1] = cmul(r1, m1, T(-1.0), T(-0.0))
    elif kind == C.H:
        s = T(0.70710678118654752440)
        re[i0], im[i0] = (r0 + r1) * s, (m0 + m1) * s
        re[i1], im[i1] = (r0 - r1) * s, (m0 - m1) * s
    elif kind == C.P:  # ket1 *= exp(i lambda)
        re[i1], im[i1] = cmul(r1, m1, cos(a), sin(a))
    elif kind == C.RX:
        c, s = cos(a / 2.0), sin(a / 2.0)
        re[i0], im[i0] = c * r0 + s * m1, c * m0 - s * r1
        re[i1], im[i1] = s * m0 + c * r1, -s * r0 + c * m1
    elif kind == C.RY:
        c, s = cos(a / 2.0), sin(a / 2.0)
        re[i0], im[i0] = c * r0 - s * r1, c * m0 - s * m1
        re[i1], im[i1] = s * r0 + c * r1, s * m0 + c * m1
    else:  # RZ: ket0 *= exp(-i theta/2), ket1 *= exp(i theta/2)
        h0, h1 = -a / 2.0, a / 2.0
        re[i0], im[i0] = cmul(r0, m0, cos(h0), sin(h0))
        re[i1], im[i1] = cmul(r1, m1, cos(h1), sin(h1))


@pytest.mark.parametrize("seed,prec", [(5, "c128"), (6, "c128"), (7, "c64")])
def test_densev2_formulas_equal_the_dense_restatement(seed, prec):
    """The C ABI's default simulator is DenseV2 (in place); the oracle
    restates Dense (double-buffered).  Their gate bodies compute the same
    products and two-term sums up to order and exact negations, so DenseV2's
    amplitudes are the oracle's bit for bit: checked on random circuits with
    every gate kind and controls, in binary64 and binary32."""
    n = 9
    circ = C.random_circuit(n, 400, seed, max_controls=2)
    f32 = _libm_f32() if prec == "c64" else None
    dt = np.float32 if f32 else np.float64
    re = np.zeros(1 << n, dt)
    im = np.zeros(1 << n, dt)
    re[0] = 1.0
    for g in circ:
        _densev2_apply(re, im, n, g, f32)
    o = oracle.OracleDense(n, prec)
    o.apply(circ)
    st = o.state()
    assert np.array_equal(st.real, re) and np.array_equal(st.imag, im)
