"""Python mirror of the reference's backend trait over the C ABI.

``DenseGB300`` exposes the methods of kbw's ``QuantumExecution`` trait
(src/quantum_execution.rs:48-162) with the same names and argument meaning:
gates take ``(target, control)`` or ``(angle, target, control)``,
``measure_p1`` does not collapse, ``measure_collapse`` takes
``p = 1/sqrt(P)``, ``dump`` packs ``qubits[0]`` as the most significant bit.
The ``QubitManager`` level (src/quantum_execution.rs:272-306) is ``measure``,
``sample`` and ``exp_value`` with explicit uniform draws.

Every call goes to the CUDA engine; nothing here computes amplitudes.
"""
import ctypes

import numpy as np

from . import _native as N
from .circuits import PAULI_X, PAULI_Y, PAULI_Z  # noqa: F401

_DT = {"c64": (N.C64, np.complex64), "c128": (N.C128, np.complex128)}


def _sizes(seq):
    a = np.ascontiguousarray(np.asarray(list(seq), dtype=np.uintp))
    return a


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t)) if a.size else None


class DenseGB300:
    """One state vector of 2^n amplitudes on the current CUDA device."""

    def __init__(self, num_qubits, prec="c128", fusion=True, fast_c128=False, exact_order=False, graphs=True,
                 fold=True, jit=None):
        lib = N.load()
        if prec not in _DT:
            raise ValueError("prec must be 'c64' or 'c128'")
        self.num_qubits = int(num_qubits)
        self.prec = prec
        flags = (0 if fusion else N.FLAG_NO_FUSION) | (N.FLAG_FAST_C128 if fast_c128 else 0)
        flags |= N.FLAG_EXACT_ORDER if exact_order else 0
        flags |= 0 if graphs else N.FLAG_NO_GRAPHS
        flags |= 0 if fold else N.FLAG_NO_FOLD
        h = ctypes.c_void_p()
        N.check(lib.kbwg_new(self.num_qubits, _DT[prec][0], flags, ctypes.byref(h)))
        self._h = h
        self._lib = lib
        if jit is not None:
            self.set_jit(jit)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.kbwg_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- trait gates --------------------------------------------------------------
    def _g(self, fn, target, control, angle=None):
        c = _sizes(control)
        cp = _p(c, ctypes.c_size_t)
        if angle is None:
            N.check(fn(self._h, int(target), cp, c.size))
        else:
            N.check(fn(self._h, float(angle), int(target), cp, c.size))

    def pauli_x(self, target, control=()):
        self._g(self._lib.kbwg_pauli_x, target, control)

    def pauli_y(self, target, control=()):
        self._g(self._lib.kbwg_pauli_y, target, control)

    def pauli_z(self, target, control=()):
        self._g(self._lib.kbwg_pauli_z, target, control)

    def hadamard(self, target, control=()):
        self._g(self._lib.kbwg_hadamard, target, control)

    def phase(self, angle, target, control=()):
        self._g(self._lib.kbwg_phase, target, control, angle)

    def rx(self, angle, target, control=()):
        self._g(self._lib.kbwg_rx, target, control, angle)

    def ry(self, angle, target, control=()):
        self._g(self._lib.kbwg_ry, target, control, angle)

    def rz(self, angle, target, control=()):
        self._g(self._lib.kbwg_rz, target, control, angle)

    def apply(self, circuit):
        """Queue a list of (kind, target, controls, angle) gates in one call."""
        N.check(self._lib.kbwg_apply_gates(self._h, _gate_array(circuit), len(circuit)))

    def flush(self):
        N.check(self._lib.kbwg_flush(self._h))

    # -- measurement ------------------------------------------------------------
    def measure_p1(self, target):
        out = ctypes.c_double()
        N.check(self._lib.kbwg_measure_p1(self._h, int(target), ctypes.byref(out)))
        return out.value

    def measure_collapse(self, target, result, p):
        N.check(self._lib.kbwg_measure_collapse(self._h, int(target), bool(result), float(p)))

    def measure(self, qubits, draws=None):
        q = _sizes(qubits)
        d = None if draws is None else np.ascontiguousarray(draws, dtype=np.float64)
        if d is not None and d.size < q.size:
            raise ValueError("one draw per qubit is needed")
        out = ctypes.c_uint64()
        N.check(self._lib.kbwg_measure(self._h, _p(q, ctypes.c_size_t), q.size,
                                       None if d is None else _p(d, ctypes.c_double), ctypes.byref(out)))
        return int(out.value)

    def dump(self, qubits):
        q = _sizes(qubits)
        size = ctypes.c_size_t()
        N.check(self._lib.kbwg_dump(self._h, _p(q, ctypes.c_size_t), q.size, None, None, None, 0,
                                    ctypes.byref(size)))
        m = size.value
        st = np.zeros(max(m, 1), np.uint64)
        re = np.zeros(max(m, 1), np.float64)
        im = np.zeros(max(m, 1), np.float64)
        N.check(self._lib.kbwg_dump(self._h, _p(q, ctypes.c_size_t), q.size, _p(st, ctypes.c_uint64),
                                    _p(re, ctypes.c_double), _p(im, ctypes.c_double), m, ctypes.byref(size)))
        return st[:m], re[:m], im[:m]

    def sample(self, qubits, shots, draws=None):
        q = _sizes(qubits)
        shots = int(shots)
        d = None if draws is None else np.ascontiguousarray(draws, dtype=np.float64)
        if d is not None and d.size < shots:
            raise ValueError("one draw per shot is needed")
        st = np.zeros(max(shots, 1), np.uint64)
        ct = np.zeros(max(shots, 1), np.uint64)
        n = ctypes.c_size_t()
        N.check(self._lib.kbwg_sample(self._h, _p(q, ctypes.c_size_t), q.size, shots,
                                      None if d is None else _p(d, ctypes.c_double),
                                      _p(st, ctypes.c_uint64), _p(ct, ctypes.c_uint64), max(shots, 1),
                                      ctypes.byref(n)))
        return st[:n.value], ct[:n.value]

    def exp_value(self, hamiltonian):
        """hamiltonian: list of (coefficient, [(pauli_code, qubit), ...])."""
        paulis, qubits, offsets, coefs = [], [], [0], []
        for coef, terms in hamiltonian:
            for p, q in terms:
                paulis.append(int(p))
                qubits.append(int(q))
            offsets.append(len(paulis))
            coefs.append(float(coef))
        pa = np.ascontiguousarray(paulis if paulis else [0], dtype=np.uint8)
        qa = np.ascontiguousarray(qubits if qubits else [0], dtype=np.uintp)
        oa = np.ascontiguousarray(offsets, dtype=np.uintp)
        ca = np.ascontiguousarray(coefs if coefs else [0.0], dtype=np.float64)
        out = ctypes.c_double()
        N.check(self._lib.kbwg_exp_value(self._h, _p(pa, ctypes.c_uint8), _p(qa, ctypes.c_size_t),
                                         _p(oa, ctypes.c_size_t), _p(ca, ctypes.c_double), len(coefs),
                                         ctypes.byref(out)))
        return out.value

    def clear(self):
        N.check(self._lib.kbwg_clear(self._h))

    # -- gradients ------------------------------------------------------------------
    def adjoint_gradient(self, circuit, param_index, n_params, hamiltonian, max_checkpoints=16):
        """E = <psi|H|psi> and dE/dparams by the reverse-mode adjoint kernel.
        param_index[i] is the parameter gate i's angle is (-1: constant)."""
        ga = _gate_array(circuit)
        pi = np.ascontiguousarray(param_index, dtype=np.int32)
        pa, qa, oa, ca, ns = _ham_arrays(hamiltonian)
        e = ctypes.c_double()
        g = np.zeros(max(int(n_params), 1), np.float64)
        N.check(self._lib.kbwg_adjoint_gradient(self._h, ga, len(circuit), _p(pi, ctypes.c_int32), int(n_params),
                                                _p(pa, ctypes.c_uint8), _p(qa, ctypes.c_size_t),
                                                _p(oa, ctypes.c_size_t), _p(ca, ctypes.c_double), ns,
                                                int(max_checkpoints), ctypes.byref(e), _p(g, ctypes.c_double)))
        return e.value, g[: int(n_params)]

    def param_shift_gradient(self, circuit, param_index, n_params, hamiltonian):
        """The same gradient by the parameter-shift rule on the GPU."""
        ga = _gate_array(circuit)
        pi = np.ascontiguousarray(param_index, dtype=np.int32)
        pa, qa, oa, ca, ns = _ham_arrays(hamiltonian)
        e = ctypes.c_double()
        g = np.zeros(max(int(n_params), 1), np.float64)
        N.check(self._lib.kbwg_param_shift_gradient(self._h, ga, len(circuit), _p(pi, ctypes.c_int32), int(n_params),
                                                    _p(pa, ctypes.c_uint8), _p(qa, ctypes.c_size_t),
                                                    _p(oa, ctypes.c_size_t), _p(ca, ctypes.c_double), ns,
                                                    ctypes.byref(e), _p(g, ctypes.c_double)))
        return e.value, g[: int(n_params)]

    # -- raw access -----------------------------------------------------------------
    def state(self):
        dt = _DT[self.prec][1]
        out = np.zeros(1 << self.num_qubits, dt)
        N.check(self._lib.kbwg_get_state(self._h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
        return out

    def set_state(self, amps):
        a = np.ascontiguousarray(np.asarray(amps, dtype=_DT[self.prec][1]))
        if a.size != 1 << self.num_qubits:
            raise ValueError("need 2^n amplitudes")
        N.check(self._lib.kbwg_set_state(self._h, a.ctypes.data_as(ctypes.c_void_p), a.nbytes))

    def swap_qubits(self, a, b):
        N.check(self._lib.kbwg_swap_qubits(self._h, int(a), int(b)))

    def device_info(self):
        n = ctypes.c_size_t()
        prec = ctypes.c_int32()
        ptr = ctypes.c_void_p()
        nbytes = ctypes.c_size_t()
        N.check(self._lib.kbwg_state_info(self._h, ctypes.byref(n), ctypes.byref(prec), ctypes.byref(ptr),
                                          ctypes.byref(nbytes)))
        return int(n.value), int(prec.value), int(ptr.value or 0), int(nbytes.value)

    def stream_handle(self):
        ptr = ctypes.c_void_p()
        N.check(self._lib.kbwg_stream(self._h, ctypes.byref(ptr)))
        return int(ptr.value or 0)

    def profile(self, enable=True):
        N.check(self._lib.kbwg_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        n = ctypes.c_uint64()
        ms = ctypes.c_double()
        b = ctypes.c_double()
        N.check(self._lib.kbwg_profile_read(self._h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(b)))
        return int(n.value), float(ms.value), float(b.value)

    def distance(self, other):
        """||self - other|| / ||other||, computed on the device."""
        out = ctypes.c_double()
        N.check(self._lib.kbwg_state_distance(self._h, other._h, ctypes.byref(out)))
        return out.value

    def fidelity(self, other):
        """|<self|other>|^2 / (<self|self><other|other>), on the device; the
        two handles may differ in precision."""
        out = ctypes.c_double()
        N.check(self._lib.kbwg_state_fidelity(self._h, other._h, ctypes.byref(out)))
        return out.value

    def last_flush_stats(self):
        g = ctypes.c_uint64()
        p = ctypes.c_uint64()
        N.check(self._lib.kbwg_last_flush_stats(self._h, ctypes.byref(g), ctypes.byref(p)))
        return int(g.value), int(p.value)

    def set_jit(self, mode):
        """Run-time specialised sweep kernels: N.JIT_OFF, N.JIT_AUTO or N.JIT_ALWAYS."""
        N.check(self._lib.kbwg_set_jit(self._h, int(mode)))

    def jit_wait(self):
        """Wait for the handle's background compilations of specialised
        kernels (auto mode): the next flush of each structure runs them."""
        N.check(self._lib.kbwg_jit_wait(self._h))

    def jit_info(self):
        """The handle's JIT mode, how many sweeps of its last flush ran a
        specialised kernel, and the process-wide compile statistics."""
        return N.jit_info(self._h)

    def wait_probe(self, spins=1024):
        """Run the tile kernels' bounded wait on a barrier nothing completes;
        raises KbwgError with code ETIMEOUT (the handle stays usable)."""
        N.check(self._lib.kbwg_wait_probe(self._h, int(spins)))

    # ---- sweep tuning --------------------------------------------------------
    def tile_options(self):
        """Tile sizes (qubits per tile) with a compiled sweep kernel, default first."""
        buf = (ctypes.c_uint32 * 8)()
        n = ctypes.c_size_t()
        N.check(self._lib.kbwg_tile_options(self._h, buf, 8, ctypes.byref(n)))
        return [int(buf[i]) for i in range(n.value)]

    def set_tuning(self, tile_qubits=0, fusion_depth=0):
        N.check(self._lib.kbwg_set_tuning(self._h, int(tile_qubits), int(fusion_depth)))

    def tuning(self):
        t = N.Tuning()
        N.check(self._lib.kbwg_get_tuning(self._h, ctypes.byref(t)))
        return _tuning_dict(t)

    def autotune(self, circuit, reps=1):
        """Time the circuit under every tile size x fusion depth, keep the
        fastest for this handle (the state is left unchanged)."""
        arr = _gate_array(circuit)
        t = N.Tuning()
        N.check(self._lib.kbwg_autotune(self._h, arr, len(circuit), int(reps), ctypes.byref(t)))
        return _tuning_dict(t)


def _tuning_dict(t):
    return {"tile_qubits": int(t.tile_qubits), "fusion_depth": int(t.fusion_depth),
            "source": N.TUNE_SOURCES[t.source] if t.source < len(N.TUNE_SOURCES) else int(t.source),
            "candidates": int(t.candidates), "ms_per_run": float(t.ms_per_run),
            "default_ms_per_run": float(t.default_ms_per_run)}


def batch_hea_tfim(circuits, zz=1.0, x=0.5, prec="c64", fast_c128=False):
    """Energies of many hardware-efficient-ansatz circuits in one launch.
    circuits: list of (num_qubits, layers, params) as circuits.hea_batch()."""
    lib = N.load()
    nc = len(circuits)
    nq = np.ascontiguousarray([c[0] for c in circuits], dtype=np.uint32)
    ly = np.ascontiguousarray([c[1] for c in circuits], dtype=np.uint32)
    offs = np.zeros(nc, np.uint64)
    total = 0
    for i, c in enumerate(circuits):
        offs[i] = total
        total += len(c[2])
    params = np.ascontiguousarray(np.concatenate([np.asarray(c[2], np.float64) for c in circuits])
                                  if nc else np.zeros(1), dtype=np.float64)
    out = np.zeros(max(nc, 1), np.float64)
    flags = N.FLAG_FAST_C128 if fast_c128 else 0
    N.check(lib.kbwg_batch_hea_tfim(nc, _p(nq, ctypes.c_uint32), _p(ly, ctypes.c_uint32), _p(offs, ctypes.c_uint64),
                                    _p(params, ctypes.c_double), int(total), float(zz), float(x), _DT[prec][0],
                                    flags, _p(out, ctypes.c_double)))
    return out[:nc]


def _flags(fast_c128=False, exact_order=False):
    return (N.FLAG_FAST_C128 if fast_c128 else 0) | (N.FLAG_EXACT_ORDER if exact_order else 0)


def batch_exp_value(num_qubits, circuit, hamiltonians, prec="c128", fast_c128=False, exact_order=False):
    """BatchExecution::exp_value: <H_k> for each Hamiltonian after the whole
    circuit on a fresh (pooled) register."""
    lib = N.load()
    ga = _gate_array(circuit)
    allh = [s for h in hamiltonians for s in h]
    pa, qa, oa, ca, _ = _ham_arrays(allh)
    ho = np.ascontiguousarray(np.cumsum([0] + [len(h) for h in hamiltonians]), dtype=np.uintp)
    out = np.zeros(max(len(hamiltonians), 1), np.float64)
    N.check(lib.kbwg_batch_exp_value(int(num_qubits), _DT[prec][0], _flags(fast_c128, exact_order), ga, len(circuit),
                                     _p(pa, ctypes.c_uint8), _p(qa, ctypes.c_size_t), _p(oa, ctypes.c_size_t),
                                     _p(ca, ctypes.c_double), _p(ho, ctypes.c_size_t), len(hamiltonians),
                                     _p(out, ctypes.c_double)))
    return out[: len(hamiltonians)]


def batch_sample(num_qubits, circuit, qubits, shots, draws=None, prec="c128", fast_c128=False, exact_order=False):
    """BatchExecution::sample: histogram of `shots` samples after the whole
    circuit on a fresh (pooled) register."""
    lib = N.load()
    ga = _gate_array(circuit)
    q = _sizes(qubits)
    shots = int(shots)
    d = None if draws is None else np.ascontiguousarray(draws, dtype=np.float64)
    if d is not None and d.size < shots:
        raise ValueError("one draw per shot is needed")
    st = np.zeros(max(shots, 1), np.uint64)
    ct = np.zeros(max(shots, 1), np.uint64)
    n = ctypes.c_size_t()
    N.check(lib.kbwg_batch_sample(int(num_qubits), _DT[prec][0], _flags(fast_c128, exact_order), ga, len(circuit),
                                  _p(q, ctypes.c_size_t), q.size, shots, None if d is None else _p(d, ctypes.c_double),
                                  _p(st, ctypes.c_uint64), _p(ct, ctypes.c_uint64), max(shots, 1), ctypes.byref(n)))
    return st[: n.value], ct[: n.value]


def batch_gradient(num_qubits, circuit, param_index, n_params, hamiltonian, prec="c128", fast_c128=False,
                   max_checkpoints=16):
    """BatchExecution::gradient, native: E and dE/dparams by the adjoint method."""
    lib = N.load()
    ga = _gate_array(circuit)
    pi = np.ascontiguousarray(param_index, dtype=np.int32)
    pa, qa, oa, ca, ns = _ham_arrays(hamiltonian)
    e = ctypes.c_double()
    g = np.zeros(max(int(n_params), 1), np.float64)
    N.check(lib.kbwg_batch_gradient(int(num_qubits), _DT[prec][0], _flags(fast_c128), ga, len(circuit),
                                    _p(pi, ctypes.c_int32), int(n_params), _p(pa, ctypes.c_uint8),
                                    _p(qa, ctypes.c_size_t), _p(oa, ctypes.c_size_t), _p(ca, ctypes.c_double), ns,
                                    int(max_checkpoints), ctypes.byref(e), _p(g, ctypes.c_double)))
    return e.value, g[: int(n_params)]


def batch_circuits_prepare(circuits):
    """The C arrays of kbwg_batch_circuits_exp_value for a list of
    (num_qubits, gate list, hamiltonian) (done once; see batch_circuits_run)."""
    nq = np.ascontiguousarray([int(c[0]) for c in circuits], dtype=np.uint32)
    gates = [g for c in circuits for g in c[1]]
    goff = np.zeros(len(circuits) + 1, np.uintp)
    goff[1:] = np.cumsum([len(c[1]) for c in circuits])
    paulis, qubits, toff, coefs, hoff = [], [], [0], [], [0]
    for c in circuits:
        for coef, terms in c[2]:
            for p, q in terms:
                paulis.append(p)
                qubits.append(q)
            toff.append(len(paulis))
            coefs.append(coef)
        hoff.append(len(coefs))
    return {"n": len(circuits), "nq": nq, "gates": _gate_array(gates) if gates else None, "goff": goff,
            "paulis": np.ascontiguousarray(paulis if paulis else [0], dtype=np.uint8),
            "qubits": np.ascontiguousarray(qubits if qubits else [0], dtype=np.uintp),
            "toff": np.ascontiguousarray(toff, dtype=np.uintp),
            "coefs": np.ascontiguousarray(coefs if coefs else [0.0], dtype=np.float64),
            "hoff": np.ascontiguousarray(hoff, dtype=np.uintp)}


def batch_circuits_run(packed, prec="c64", fast_c128=False):
    """One kbwg_batch_circuits_exp_value call on prepared arrays."""
    e = np.zeros(max(packed["n"], 1), np.float64)
    N.check(N.load().kbwg_batch_circuits_exp_value(
        packed["n"], _DT[prec][0], N.FLAG_FAST_C128 if fast_c128 else 0, _p(packed["nq"], ctypes.c_uint32),
        packed["gates"], _p(packed["goff"], ctypes.c_size_t), _p(packed["paulis"], ctypes.c_uint8),
        _p(packed["qubits"], ctypes.c_size_t), _p(packed["toff"], ctypes.c_size_t),
        _p(packed["coefs"], ctypes.c_double), _p(packed["hoff"], ctypes.c_size_t), _p(e, ctypes.c_double)))
    return e[: packed["n"]]


def batch_circuits_exp_value(circuits, prec="c64", fast_c128=False):
    """<H> of many circuits in one launch: circuits is a list of
    (num_qubits, gate list, hamiltonian); returns one energy per circuit."""
    return batch_circuits_run(batch_circuits_prepare(circuits), prec, fast_c128)


def batch_release():
    """Free the registers the batch entries keep between calls."""
    N.check(N.load().kbwg_batch_release())


_GATE_DT = np.dtype([("kind", "<u4"), ("target", "<u4"), ("control_mask", "<u8"), ("angle", "<f8")])
assert _GATE_DT.itemsize == ctypes.sizeof(N.Gate)


_MASKS = {}


def _mask(cs):
    """Bit mask of a control list (memoised for tuples)."""
    try:
        return _MASKS[cs]
    except KeyError:
        m = _MASKS[cs] = sum(1 << int(c) for c in cs)
        return m
    except TypeError:  # unhashable (a list)
        return sum(1 << int(c) for c in cs)


def _gate_array(circuit):
    """kbwg_gate records of a (kind, target, controls, angle) list, as a
    ctypes array over one numpy buffer (filled column by column)."""
    n = len(circuit)
    buf = np.zeros(max(n, 1), _GATE_DT)
    if n:
        kinds, targets, ctrls, angles = zip(*circuit)
        buf["kind"][:n] = kinds
        buf["target"][:n] = targets
        buf["control_mask"][:n] = [_mask(cs) for cs in ctrls]
        buf["angle"][:n] = angles
    return (N.Gate * max(n, 1)).from_buffer(buf)


def _ham_arrays(hamiltonian):
    paulis, qubits, offsets, coefs = [], [], [0], []
    for coef, terms in hamiltonian:
        for p, q in terms:
            paulis.append(int(p))
            qubits.append(int(q))
        offsets.append(len(paulis))
        coefs.append(float(coef))
    pa = np.ascontiguousarray(paulis if paulis else [0], dtype=np.uint8)
    qa = np.ascontiguousarray(qubits if qubits else [0], dtype=np.uintp)
    oa = np.ascontiguousarray(offsets, dtype=np.uintp)
    ca = np.ascontiguousarray(coefs if coefs else [0.0], dtype=np.float64)
    return pa, qa, oa, ca, len(coefs)


def plan(num_qubits, circuit, prec="c128", exact_order=False, fast_c128=False, tile_qubits=None, fusion_depth=0):
    """Host planner diagnostic: list of (tile_mask, [gate indices in execution order]).
    tile_qubits None: the arithmetic's default tile (kbwg_plan); otherwise
    kbwg_plan_tuned with that tile size (0: a handle's default) and depth."""
    lib = N.load()
    n = len(circuit)
    arr = _gate_array(circuit)
    order = (ctypes.c_uint32 * max(n, 1))()
    ends = (ctypes.c_uint32 * max(n, 1))()
    masks = (ctypes.c_uint64 * max(n, 1))()
    ns = ctypes.c_size_t()
    flags = _flags(fast_c128, exact_order)
    if tile_qubits is None:
        N.check(lib.kbwg_plan(int(num_qubits), _DT[prec][0], flags, arr, n, order, ends, masks, ctypes.byref(ns)))
    else:
        N.check(lib.kbwg_plan_tuned(int(num_qubits), _DT[prec][0], flags, int(tile_qubits), int(fusion_depth), arr, n,
                                    order, ends, masks, ctypes.byref(ns)))
    out, b = [], 0
    for k in range(ns.value):
        e = ends[k]
        out.append((int(masks[k]), [int(order[i]) for i in range(b, e)]))
        b = e
    return out
