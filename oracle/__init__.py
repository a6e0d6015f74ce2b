"""CPU oracle for the dense state-vector path -- test infrastructure only.

``OracleDense`` wraps the C restatement of kbw's ``Dense<F>``
(src/dense.rs:42-406) and of the trait defaults built on it
(src/quantum_execution.rs:99-158, 272-292; src/convert.rs:30-73).

Parity status: unpinned against the reference itself (it has no tests and its
Rust toolchain is absent); pinned against tests/golden fixtures produced by an
independent numpy matrix model and against closed-form known answers.

Only tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline leg
import this package.
"""
import ctypes
import os

import numpy as np

from . import build as _build

X, Y, Z, H, P, RX, RY, RZ = range(8)
PAULI_X, PAULI_Y, PAULI_Z = 1, 2, 3

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        sz = ctypes.c_size_t
        szp = ctypes.POINTER(ctypes.c_size_t)
        dp = ctypes.POINTER(ctypes.c_double)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        L.od_new.restype = ctypes.c_void_p
        L.od_new.argtypes = [sz, ctypes.c_int]
        L.od_free.argtypes = [ctypes.c_void_p]
        L.od_clear.argtypes = [ctypes.c_void_p]
        L.od_gate.restype = ctypes.c_int
        L.od_gate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, sz, szp, sz]
        L.od_apply_gates.restype = ctypes.c_int
        L.od_apply_gates.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), szp, u64p, dp, sz]
        L.od_measure_p1.restype = ctypes.c_double
        L.od_measure_p1.argtypes = [ctypes.c_void_p, sz]
        L.od_measure_collapse.argtypes = [ctypes.c_void_p, sz, ctypes.c_int, ctypes.c_double]
        L.od_dump.restype = sz
        L.od_dump.argtypes = [ctypes.c_void_p, szp, sz, u64p, dp, dp]
        L.od_measure.restype = ctypes.c_uint64
        L.od_measure.argtypes = [ctypes.c_void_p, szp, sz, dp]
        L.od_sample.restype = ctypes.c_long
        L.od_sample.argtypes = [ctypes.c_void_p, szp, sz, sz, dp, u64p, u64p]
        L.od_exp_value.restype = ctypes.c_double
        L.od_exp_value.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), szp, szp, dp, sz]
        L.od_pauli_expect.restype = ctypes.c_double
        L.od_pauli_expect.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), szp, szp, dp, sz]
        L.od_z_all.argtypes = [ctypes.c_void_p, dp]
        L.od_get_state.argtypes = [ctypes.c_void_p, dp]
        L.od_set_state.argtypes = [ctypes.c_void_p, dp]
        L.od_swap_qubits.argtypes = [ctypes.c_void_p, sz, sz]
        L.od_uniform_scale.restype = ctypes.c_double
        L.od_uniform_scale.argtypes = [ctypes.c_double]
        L.od_weighted_pick.restype = sz
        L.od_weighted_pick.argtypes = [dp, sz, ctypes.c_double]
        L.od_num_threads.restype = ctypes.c_int
        L.od_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _sizes(seq):
    a = np.ascontiguousarray(np.asarray(list(seq), dtype=np.uintp))
    if a.size == 0:
        a = np.zeros(1, dtype=np.uintp)[:0]
    return a


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class OracleDense:
    """Restated ``Dense<f32>`` (prec='c64') or ``Dense<f64>`` (prec='c128')."""

    def __init__(self, num_qubits, prec="c128"):
        self.num_qubits = int(num_qubits)
        self.prec = prec
        self._h = lib().od_new(self.num_qubits, 1 if prec == "c128" else 0)
        if not self._h:
            raise ValueError("oracle: cannot create a %d-qubit state" % num_qubits)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.od_free(h)
            self._h = None

    # -- QuantumExecution trait (src/quantum_execution.rs:48-162) -------------
    def gate(self, kind, target, control=(), angle=0.0):
        c = _sizes(control)
        rc = lib().od_gate(self._h, int(kind), float(angle), int(target), _ptr(c, ctypes.c_size_t), c.size)
        if rc != 0:
            raise ValueError("oracle: bad qubit index")

    def pauli_x(self, target, control=()):
        self.gate(X, target, control)

    def pauli_y(self, target, control=()):
        self.gate(Y, target, control)

    def pauli_z(self, target, control=()):
        self.gate(Z, target, control)

    def hadamard(self, target, control=()):
        self.gate(H, target, control)

    def phase(self, angle, target, control=()):
        self.gate(P, target, control, angle)

    def rx(self, angle, target, control=()):
        self.gate(RX, target, control, angle)

    def ry(self, angle, target, control=()):
        self.gate(RY, target, control, angle)

    def rz(self, angle, target, control=()):
        self.gate(RZ, target, control, angle)

    def measure_p1(self, target):
        return lib().od_measure_p1(self._h, int(target))

    def measure_collapse(self, target, result, p):
        lib().od_measure_collapse(self._h, int(target), 1 if result else 0, float(p))

    def dump(self, qubits):
        q = _sizes(qubits)
        m = lib().od_dump(self._h, _ptr(q, ctypes.c_size_t), q.size, None, None, None)
        st = np.zeros(max(m, 1), np.uint64)
        re = np.zeros(max(m, 1), np.float64)
        im = np.zeros(max(m, 1), np.float64)
        lib().od_dump(self._h, _ptr(q, ctypes.c_size_t), q.size, _ptr(st, ctypes.c_uint64),
                      _ptr(re, ctypes.c_double), _ptr(im, ctypes.c_double))
        return st[:m], re[:m], im[:m]

    def clear(self):
        lib().od_clear(self._h)

    # -- QubitManager level ----------------------------------------------------
    def measure(self, qubits, draws):
        q = _sizes(qubits)
        d = np.ascontiguousarray(draws, dtype=np.float64)
        assert d.size >= q.size
        return int(lib().od_measure(self._h, _ptr(q, ctypes.c_size_t), q.size, _ptr(d, ctypes.c_double)))

    def sample(self, qubits, shots, draws):
        q = _sizes(qubits)
        d = np.ascontiguousarray(draws, dtype=np.float64)
        assert d.size >= shots
        st = np.zeros(max(shots, 1), np.uint64)
        ct = np.zeros(max(shots, 1), np.uint64)
        n = lib().od_sample(self._h, _ptr(q, ctypes.c_size_t), q.size, int(shots), _ptr(d, ctypes.c_double),
                            _ptr(st, ctypes.c_uint64), _ptr(ct, ctypes.c_uint64))
        if n < 0:
            raise ValueError("oracle: zero total weight")
        return st[:n], ct[:n]

    def exp_value(self, hamiltonian):
        """hamiltonian: list of (coefficient, [(pauli_code, qubit), ...])."""
        return self._expect(lib().od_exp_value, hamiltonian)

    def pauli_expect(self, hamiltonian):
        """<H> from the amplitudes directly (parity checks needing many
        energies); equals exp_value up to the dump's epsilon filter."""
        return self._expect(lib().od_pauli_expect, hamiltonian)

    def _expect(self, fn, hamiltonian):
        paulis, qubits, offsets, coefs = [], [], [0], []
        for coef, terms in hamiltonian:
            for p, q in terms:
                paulis.append(p)
                qubits.append(q)
            offsets.append(len(paulis))
            coefs.append(coef)
        pa = np.ascontiguousarray(paulis if paulis else [0], dtype=np.intc)
        qa = np.ascontiguousarray(qubits if qubits else [0], dtype=np.uintp)
        oa = np.ascontiguousarray(offsets, dtype=np.uintp)
        ca = np.ascontiguousarray(coefs if coefs else [0.0], dtype=np.float64)
        return fn(self._h, _ptr(pa, ctypes.c_int), _ptr(qa, ctypes.c_size_t), _ptr(oa, ctypes.c_size_t),
                  _ptr(ca, ctypes.c_double), len(coefs))

    def z_all(self):
        """<Z_q> for every qubit (one pass over the state)."""
        out = np.zeros(self.num_qubits, np.float64)
        lib().od_z_all(self._h, _ptr(out, ctypes.c_double))
        return out

    # -- raw access ------------------------------------------------------------
    def state(self):
        out = np.zeros(2 << self.num_qubits, np.float64)
        lib().od_get_state(self._h, _ptr(out, ctypes.c_double))
        return out.view(np.complex128)

    def set_state(self, amps):
        a = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128)).view(np.float64)
        assert a.size == 2 << self.num_qubits
        lib().od_set_state(self._h, _ptr(a, ctypes.c_double))

    def swap_qubits(self, a, b):
        lib().od_swap_qubits(self._h, int(a), int(b))

    def apply(self, circuit):
        """Apply a list of (kind, target, controls, angle) tuples (one call)."""
        n = len(circuit)
        if n == 0:
            return
        kinds, targets, ctrls, angles = zip(*circuit)
        k = np.ascontiguousarray(kinds, dtype=np.intc)
        t = np.ascontiguousarray(targets, dtype=np.uintp)
        m = np.ascontiguousarray([sum(1 << int(c) for c in cs) for cs in ctrls], dtype=np.uint64)
        a = np.ascontiguousarray(angles, dtype=np.float64)
        rc = lib().od_apply_gates(self._h, _ptr(k, ctypes.c_int), _ptr(t, ctypes.c_size_t), _ptr(m, ctypes.c_uint64),
                                  _ptr(a, ctypes.c_double), n)
        if rc != 0:
            raise ValueError("oracle: bad qubit index")


def uniform_scale(total):
    return lib().od_uniform_scale(float(total))


def set_num_threads(n):
    lib().od_set_num_threads(int(n))


def num_threads():
    return lib().od_num_threads()
