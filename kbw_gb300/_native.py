"""ctypes binding of the engine's C ABI (include/kbwg.h).

The library is built in-tree by ``kbw_gb300/build.py`` (or
``__graft_entry__.build()``).  Loading fails loudly when it is missing: there
is no CPU fallback.
"""
import atexit
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkbwg.so")

OK, EINVAL, EQUBITS, ENOMEM, ECUDA, EWEIGHT, ECAPACITY, ETIMEOUT, EUNSUPPORTED = range(9)
C64, C128 = 0, 1
FLAG_NO_FUSION = 1
FLAG_FAST_C128 = 2
FLAG_EXACT_ORDER = 4
FLAG_NO_GRAPHS = 8
FLAG_NO_FOLD = 16


class KbwgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("kbwg error %d: %s" % (code, msg))
        self.code = code


class Gate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("target", ctypes.c_uint32),
                ("control_mask", ctypes.c_uint64), ("angle", ctypes.c_double)]


class Tuning(ctypes.Structure):
    _fields_ = [("tile_qubits", ctypes.c_uint32), ("fusion_depth", ctypes.c_uint32),
                ("source", ctypes.c_uint32), ("candidates", ctypes.c_uint32),
                ("ms_per_run", ctypes.c_double), ("default_ms_per_run", ctypes.c_double)]


TUNE_SOURCES = ("default", "set", "env", "timed", "cached")

JIT_OFF, JIT_AUTO, JIT_ALWAYS = 0, 1, 2


class JitStats(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("available", ctypes.c_int32), ("last_specialised", ctypes.c_uint64),
                ("compiled", ctypes.c_uint64), ("reused", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("compile_seconds", ctypes.c_double)]

# name -> (restype, argtypes); every function declared in include/kbwg.h
_P = ctypes.c_void_p
_U = ctypes.c_size_t  # uintptr_t
_UP = ctypes.POINTER(ctypes.c_size_t)
_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_I32 = ctypes.c_int32
SIGNATURES = {
    "kbwg_new": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(_P)]),
    "kbwg_free": (_I32, [_P]),
    "kbwg_pauli_x": (_I32, [_P, _U, _UP, _U]),
    "kbwg_pauli_y": (_I32, [_P, _U, _UP, _U]),
    "kbwg_pauli_z": (_I32, [_P, _U, _UP, _U]),
    "kbwg_hadamard": (_I32, [_P, _U, _UP, _U]),
    "kbwg_phase": (_I32, [_P, _D, _U, _UP, _U]),
    "kbwg_rx": (_I32, [_P, _D, _U, _UP, _U]),
    "kbwg_ry": (_I32, [_P, _D, _U, _UP, _U]),
    "kbwg_rz": (_I32, [_P, _D, _U, _UP, _U]),
    "kbwg_apply_gates": (_I32, [_P, ctypes.POINTER(Gate), _U]),
    "kbwg_measure_p1": (_I32, [_P, _U, _DP]),
    "kbwg_measure_collapse": (_I32, [_P, _U, ctypes.c_bool, _D]),
    "kbwg_measure": (_I32, [_P, _UP, _U, _DP, _U64P]),
    "kbwg_dump": (_I32, [_P, _UP, _U, _U64P, _DP, _DP, _U, _UP]),
    "kbwg_sample": (_I32, [_P, _UP, _U, _U, _DP, _U64P, _U64P, _U, _UP]),
    "kbwg_exp_value": (_I32, [_P, ctypes.POINTER(ctypes.c_uint8), _UP, _UP, _DP, _U, _DP]),
    "kbwg_adjoint_gradient": (_I32, [_P, ctypes.POINTER(Gate), _U, ctypes.POINTER(ctypes.c_int32), _U,
                                     ctypes.POINTER(ctypes.c_uint8), _UP, _UP, _DP, _U, ctypes.c_uint32, _DP, _DP]),
    "kbwg_param_shift_gradient": (_I32, [_P, ctypes.POINTER(Gate), _U, ctypes.POINTER(ctypes.c_int32), _U,
                                         ctypes.POINTER(ctypes.c_uint8), _UP, _UP, _DP, _U, _DP, _DP]),
    "kbwg_batch_hea_tfim": (_I32, [_U, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                                   _U64P, _DP, _U, _D, _D, _I32, ctypes.c_uint32, _DP]),
    "kbwg_clear": (_I32, [_P]),
    "kbwg_flush": (_I32, [_P]),
    "kbwg_get_state": (_I32, [_P, _P, _U]),
    "kbwg_set_state": (_I32, [_P, _P, _U]),
    "kbwg_state_info": (_I32, [_P, _UP, ctypes.POINTER(_I32), ctypes.POINTER(_P), _UP]),
    "kbwg_swap_qubits": (_I32, [_P, _U, _U]),
    "kbwg_build_info": (_I32, [ctypes.POINTER(ctypes.POINTER(ctypes.c_uint8)), _UP]),
    "kbwg_plan": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(Gate), _U, ctypes.POINTER(ctypes.c_uint32),
                         ctypes.POINTER(ctypes.c_uint32), _U64P, _UP]),
    "kbwg_plan_tuned": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(Gate), _U,
                               ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32), _U64P, _UP]),
    "kbwg_last_flush_stats": (_I32, [_P, _U64P, _U64P]),
    "kbwg_wait_probe": (_I32, [_P, ctypes.c_uint32]),
    "kbwg_stream": (_I32, [_P, ctypes.POINTER(_P)]),
    "kbwg_select_device": (_I32, [_I32]),
    "kbwg_profile": (_I32, [_P, _I32]),
    "kbwg_profile_read": (_I32, [_P, _U64P, _DP, _DP]),
    "kbwg_transfer_bytes": (_I32, [_U64P, _U64P]),
    "kbwg_state_distance": (_I32, [_P, _P, _DP]),
    "kbwg_state_fidelity": (_I32, [_P, _P, _DP]),
    "kbwg_batch_exp_value": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(Gate), _U, ctypes.POINTER(ctypes.c_uint8),
                                    _UP, _UP, _DP, _UP, _U, _DP]),
    "kbwg_batch_sample": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(Gate), _U, _UP, _U, _U, _DP, _U64P,
                                 _U64P, _U, _UP]),
    "kbwg_batch_gradient": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(Gate), _U, ctypes.POINTER(ctypes.c_int32),
                                   _U, ctypes.POINTER(ctypes.c_uint8), _UP, _UP, _DP, _U, ctypes.c_uint32, _DP, _DP]),
    "kbwg_batch_release": (_I32, []),
    "kbwg_batch_circuits_exp_value": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                                             ctypes.POINTER(Gate), _UP, ctypes.POINTER(ctypes.c_uint8), _UP, _UP,
                                             _DP, _UP, _DP]),
    "kbwg_tile_options": (_I32, [_P, ctypes.POINTER(ctypes.c_uint32), _U, _UP]),
    "kbwg_set_tuning": (_I32, [_P, ctypes.c_uint32, ctypes.c_uint32]),
    "kbwg_get_tuning": (_I32, [_P, ctypes.c_void_p]),
    "kbwg_autotune": (_I32, [_P, ctypes.POINTER(Gate), _U, ctypes.c_uint32, ctypes.c_void_p]),
    "kbwg_set_jit": (_I32, [_P, _I32]),
    "kbwg_jit_wait": (_I32, [_P]),
    "kbwg_jit_shutdown": (_I32, []),
    "kbwg_jit_info": (_I32, [_P, ctypes.c_void_p]),
    "kbwg_jit_last_error": (ctypes.c_char_p, []),
    "kbwg_jit_check": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(Gate), _U,
                              _UP, _UP]),
    "kbwg_jit_check_adjoint": (_I32, [_U, _I32, ctypes.c_uint32, ctypes.POINTER(Gate), _U, _UP, _UP]),
    "kbwg_draws": (_I32, [ctypes.c_uint64, _U, _DP]),
    "kbwg_chacha_block": (_I32, [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                 ctypes.POINTER(ctypes.c_uint32)]),
    "kbwg_masked_norm_noalloc": (_I32, [_P, _U, _I32, ctypes.c_uint64, ctypes.c_uint64, _P, _P]),
    "kbwg_last_error": (ctypes.c_char_p, []),
    "kbwg_launch_count": (ctypes.c_uint64, []),
}

_lib = None


def load(path=None):
    """Load libkbwg.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("kbw_gb300: %s is missing; build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    # background compilations must end before the C library teardown
    atexit.register(lib.kbwg_jit_shutdown)
    return lib


def check(code):
    if code != OK:
        msg = _lib.kbwg_last_error().decode(errors="replace") if _lib is not None else ""
        raise KbwgError(code, msg)
    return code


def launch_count():
    return int(load().kbwg_launch_count())


def select_device(device):
    check(load().kbwg_select_device(int(device)))


def transfer_bytes():
    h2d = ctypes.c_uint64()
    d2h = ctypes.c_uint64()
    check(load().kbwg_transfer_bytes(ctypes.byref(h2d), ctypes.byref(d2h)))
    return int(h2d.value), int(d2h.value)


def jit_info(handle=None):
    """Process-wide statistics of the run-time specialised sweep kernels (and
    the handle's mode and last flush, given a raw handle)."""
    st = JitStats()
    check(load().kbwg_jit_info(handle, ctypes.byref(st)))
    return {f: getattr(st, f) for f, _ in JitStats._fields_}


def jit_last_error():
    return load().kbwg_jit_last_error().decode(errors="replace")


def jit_check(num_qubits, prec, flags, gates, tile_qubits=0, fusion_depth=0):
    """Compile (NVRTC, no GPU) the specialised kernel of every sweep a flush
    of `gates` (a ctypes Gate array) would run; returns (sweeps, failed)."""
    ns = ctypes.c_size_t()
    nf = ctypes.c_size_t()
    check(load().kbwg_jit_check(int(num_qubits), prec, int(flags), int(tile_qubits), int(fusion_depth), gates,
                                len(gates), ctypes.byref(ns), ctypes.byref(nf)))
    return int(ns.value), int(nf.value)


def jit_check_adjoint(num_qubits, prec, flags, gates):
    """Compile (NVRTC, no GPU) the specialised reverse sweeps of an adjoint
    gradient of `gates`; returns (sweeps, failed)."""
    ns = ctypes.c_size_t()
    nf = ctypes.c_size_t()
    check(load().kbwg_jit_check_adjoint(int(num_qubits), prec, int(flags), gates, len(gates), ctypes.byref(ns),
                                        ctypes.byref(nf)))
    return int(ns.value), int(nf.value)


def draws(seed, count):
    """The first `count` draws of a register's generator seeded with `seed`
    (rand's StdRng::seed_from_u64 + UniformFloat<f64>)."""
    import numpy as np
    out = np.zeros(max(int(count), 1), np.float64)
    check(load().kbwg_draws(int(seed) & 0xFFFFFFFFFFFFFFFF, int(count),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out[: int(count)]


def chacha_block(key, counter, stream, rounds):
    k = (ctypes.c_uint32 * 8)(*key)
    out = (ctypes.c_uint32 * 16)()
    check(load().kbwg_chacha_block(k, int(counter), int(stream), int(rounds), out))
    return list(out)


def build_info():
    lib = load()
    msg = ctypes.POINTER(ctypes.c_uint8)()
    size = ctypes.c_size_t()
    check(lib.kbwg_build_info(ctypes.byref(msg), ctypes.byref(size)))
    return ctypes.string_at(msg, size.value).decode()
