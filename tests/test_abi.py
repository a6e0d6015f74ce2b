"""CPU tests of the C ABI library: it loads, exports every symbol declared in
include/kbwg.h, and its host-side fusion planner only reorders gates that
commute (checked by replaying the planned order on the oracle)."""
import os
import re

import numpy as np
import pytest

import oracle
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C
from kbw_gb300 import plan
from conftest import ROOT, rel_err


def header_functions():
    text = open(os.path.join(ROOT, "include", "kbwg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kbwg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(N.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return N.load()


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(N.SIGNATURES), set(names) ^ set(N.SIGNATURES)


def test_build_info(lib):
    assert N.build_info().startswith("kbw-gb300")


def test_new_without_gpu_fails_cleanly(lib, cuda_available):
    if cuda_available:
        pytest.skip("GPU present")
    import ctypes
    h = ctypes.c_void_p()
    code = lib.kbwg_new(4, N.C64, 0, ctypes.byref(h))
    assert code != N.OK and not h.value
    assert lib.kbwg_new(41, N.C64, 0, ctypes.byref(h)) == N.EQUBITS


def replay(n, circuit, prec):
    """Execute the planner's order on the oracle."""
    sweeps = plan(n, circuit, prec)
    order = [i for _, idx in sweeps for i in idx]
    assert sorted(order) == list(range(len(circuit)))
    o = oracle.OracleDense(n, prec)
    o.apply([circuit[i] for i in order])
    return o, sweeps


@pytest.mark.parametrize("prec", ["c64", "c128"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_planner_order_is_equivalent(lib, prec, seed):
    n = 14
    circ = C.random_circuit(n, 300, seed, max_controls=3)
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    o, sweeps = replay(n, circ, prec)
    # only commuting gates are reordered, so the states agree to rounding
    assert rel_err(o.state(), ref.state()) < (1e-12 if prec == "c128" else 1e-5)
    K = 13 if prec == "c64" else 12
    for mask, idx in sweeps:
        assert bin(mask).count("1") == K
        assert mask & 0b11111 == 0b11111
        for i in idx:
            kind, t, _, _ = circ[i]
            if kind not in (C.Z, C.P, C.RZ):
                assert (mask >> t) & 1


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_planner_exact_order_keeps_program_order(lib, prec):
    n = 15
    circ = C.random_circuit(n, 250, 4, max_controls=2)
    sweeps = plan(n, circ, prec, exact_order=True)
    order = [i for _, idx in sweeps for i in idx]
    assert order == list(range(len(circ)))
    assert len(sweeps) < len(circ) // 3


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_planner_brickwork_sweep_count(lib, prec):
    circ = C.brickwork(30, 20, 0)
    sweeps = plan(30, circ, prec)
    order = [i for _, idx in sweeps for i in idx]
    assert sorted(order) == list(range(len(circ)))
    # 25 high qubits per layer over 8 (c64) / 7 (c128) high slots per tile; the
    # window choice of the high qubits and the commutation rules pack about
    # 2.3 layers into a sweep (15 sweeps c64, 17 c128)
    assert len(sweeps) <= (16 if prec == "c64" else 18), len(sweeps)
    o16, _ = replay(16, C.brickwork(16, 6, 3), prec)
    ref = oracle.OracleDense(16, prec)
    ref.apply(C.brickwork(16, 6, 3))
    assert rel_err(o16.state(), ref.state()) < (1e-12 if prec == "c128" else 1e-5)


@pytest.mark.parametrize("prec,fast,tiles", [("c64", False, (13, 12, 11)), ("c128", False, (12, 11)),
                                             ("c128", True, (11, 12))])
def test_planner_every_tile_size_and_depth(lib, prec, fast, tiles):
    """The plans the autotuner chooses between: for every compiled tile size
    and several fusion depths, the planned order only moves commuting gates
    (replayed on the oracle), each sweep holds at most `depth` gates, and
    every tile has the requested size with the low five qubits in it."""
    n = 15
    circ = C.random_circuit(n, 220, 17, max_controls=2)
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    tol = 1e-12 if prec == "c128" else 1e-5
    for K in tiles:
        for depth in (256, 16, 1):
            sweeps = plan(n, circ, prec, fast_c128=fast, tile_qubits=K, fusion_depth=depth)
            order = [i for _, idx in sweeps for i in idx]
            assert sorted(order) == list(range(len(circ)))
            for mask, idx in sweeps:
                assert bin(mask).count("1") == K and mask & 0b11111 == 0b11111
                assert len(idx) <= depth
            o = oracle.OracleDense(n, prec)
            o.apply([circ[i] for i in order])
            assert rel_err(o.state(), ref.state()) < tol, (K, depth)
    assert len(plan(n, circ, prec, fast_c128=fast, tile_qubits=tiles[0], fusion_depth=1)) >= len(circ) // 2


def test_planner_rejects_unknown_tile_sizes(lib):
    circ = C.random_circuit(14, 20, 1)
    for prec, fast, K in (("c64", False, 10), ("c128", False, 13), ("c128", True, 13)):
        with pytest.raises(N.KbwgError) as ei:
            plan(14, circ, prec, fast_c128=fast, tile_qubits=K)
        assert ei.value.code == N.EINVAL
    with pytest.raises(N.KbwgError) as ei:
        plan(12, circ[:0], "c64", tile_qubits=13)
    assert ei.value.code == N.EQUBITS


@pytest.mark.parametrize("seed", range(4))
def test_planner_fuzz_commutation(lib, seed):
    """Random registers, gate mixes (diagonal-heavy, control-heavy), tile
    sizes and depths: the planned order must reproduce the program's state on
    the oracle (only commuting gates move) and place every gate once."""
    rng = np.random.default_rng(1000 + seed)
    for _ in range(3):
        n = int(rng.integers(13, 19))
        kinds = [C.Z, C.P, C.RZ, C.X, C.H, C.RY] if rng.random() < 0.5 else None
        circ = C.random_circuit(n, int(rng.integers(60, 260)), int(rng.integers(0, 1 << 30)),
                                max_controls=int(rng.integers(0, 4)), kinds=kinds)
        prec = "c64" if rng.random() < 0.5 else "c128"
        fast = prec == "c128" and rng.random() < 0.5
        tiles = {("c64", False): (13, 12, 11), ("c128", False): (12, 11), ("c128", True): (11, 12)}[(prec, fast)]
        K = int(rng.choice(tiles))
        depth = int(rng.choice([256, 40, 7]))
        sweeps = plan(n, circ, prec, fast_c128=fast, tile_qubits=K, fusion_depth=depth)
        order = [i for _, idx in sweeps for i in idx]
        assert sorted(order) == list(range(len(circ)))
        ref = oracle.OracleDense(n, "c128")
        ref.apply(circ)
        o = oracle.OracleDense(n, "c128")
        o.apply([circ[i] for i in order])
        assert rel_err(o.state(), ref.state()) < 1e-12, (n, K, depth)


# (precision, flags, tile size): every arithmetic's default geometry, one
# other geometry, the order-preserving mode
JIT_CASES = [(N.C128, N.FLAG_FAST_C128, 0), (N.C64, 0, 0), (N.C128, 0, 11), (N.C64, N.FLAG_EXACT_ORDER, 0)]


@pytest.mark.parametrize("prec,flags,tile", JIT_CASES)
def test_specialised_sweep_kernels_compile(lib, prec, flags, tile):
    """Every sweep of a planned circuit gets a run-time specialised kernel
    source that NVRTC compiles for sm_103a (host only; no GPU needed)."""
    from kbw_gb300.dense import _gate_array
    circ = C.random_circuit(16, 160, 21, max_controls=3)
    try:
        sweeps, failed = N.jit_check(16, prec, flags, _gate_array(circ), tile)
    except N.KbwgError as e:
        if e.code == N.EUNSUPPORTED:
            pytest.skip("NVRTC not available: %s" % e)
        raise
    assert sweeps > 0
    assert failed == 0, N.jit_last_error()


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_planner_long_lists_and_stage_limit(lib, prec):
    """Past the planner's 8192-gate selection window, and with sweeps that
    hit the 48-stage limit (gates that alternate between the two register
    layouts and do not commute): every gate placed exactly once, and the
    planned order gives the program-order state on the oracle."""
    n = 14
    circ = C.random_circuit(n, 9000, 77, max_controls=2)
    # each gate needs the other layout and shares a qubit non-diagonally with the last
    circ += [(C.X, 12, (5,), 0.0), (C.X, 5, (12,), 0.0)] * 60
    circ += C.random_circuit(n, 300, 78, max_controls=1)
    sweeps = plan(n, circ, prec)
    order = [i for _, idx in sweeps for i in idx]
    assert sorted(order) == list(range(len(circ)))
    o = oracle.OracleDense(n, prec)
    o.apply([circ[i] for i in order])
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    tol = 1e-12 if prec == "c128" else 1e-4
    assert rel_err(o.state(), ref.state()) < tol


@pytest.mark.parametrize("prec,flags", [(N.C64, 0), (N.C128, N.FLAG_FAST_C128), (N.C128, 0),
                                        (N.C128, N.FLAG_FAST_C128 | N.FLAG_NO_FUSION)])
def test_specialised_adjoint_kernels_compile(lib, prec, flags):
    """The specialised reverse sweeps of the adjoint gradient compile for
    every arithmetic (host only): a hardware-efficient ansatz and a random
    circuit with controlled parameterised gates."""
    from kbw_gb300.dense import _gate_array
    n = 14
    circ = C.hea(n, 2, C.hea_params(n, 2, 3)) + C.random_circuit(n, 60, 9, max_controls=2)
    try:
        sweeps, failed = N.jit_check_adjoint(n, prec, flags, _gate_array(circ))
    except N.KbwgError as e:
        if e.code == N.EUNSUPPORTED:
            pytest.skip("NVRTC not available: %s" % e)
        raise
    assert sweeps > 0
    assert failed == 0, N.jit_last_error()


def test_batch_circuits_validation(lib):
    """kbwg_batch_circuits_exp_value checks every circuit (on all host
    cores) before any device work: status codes for bad qubit counts, gates,
    Pauli codes and qubits, a qubit named twice in a string, and offsets that
    decrease; the first bad circuit in index order decides the code."""
    from kbw_gb300.dense import batch_circuits_prepare, batch_circuits_run
    assert len(batch_circuits_run(batch_circuits_prepare([]))) == 0
    good = (4, [(C.H, 0, (), 0.0), (C.X, 1, (0,), 0.0)], [(1.0, [(C.PAULI_Z, 1)])])
    cases = [
        ([(25, [], [])], N.EQUBITS),
        ([(0, [], [])], N.EQUBITS),
        ([good, (3, [(C.X, 3, (), 0.0)], [])], N.EINVAL),             # target out of range
        ([good, (3, [(C.X, 1, (1,), 0.0)], [])], N.EINVAL),           # target among its controls
        ([good, (3, [(C.X, 1, (5,), 0.0)], [])], N.EINVAL),           # control out of range
        ([good, (3, [(8, 1, (), 0.0)], [])], N.EINVAL),               # no such gate kind
        ([good, (3, [], [(1.0, [(4, 1)])])], N.EINVAL),               # no such Pauli code
        ([good, (3, [], [(1.0, [(C.PAULI_X, 3)])])], N.EINVAL),       # qubit out of range
        ([good, (3, [], [(1.0, [(C.PAULI_Z, 1), (C.PAULI_X, 1)])])], N.EINVAL),  # qubit twice
        ([good, (3, [(C.X, 3, (), 0.0)], []), (30, [], [])], N.EINVAL),  # circuit 1 before circuit 2
        ([good, (30, [], []), (3, [(C.X, 3, (), 0.0)], [])], N.EQUBITS),
    ]
    for circs, code in cases:
        with pytest.raises(N.KbwgError) as e:
            batch_circuits_run(batch_circuits_prepare(circs))
        assert e.value.code == code, (circs, e.value)
    # decreasing offsets (within the arrays: circuit 1's range is [2, 1))
    packed = batch_circuits_prepare([good, good])
    packed["goff"][2] = 1
    with pytest.raises(N.KbwgError) as e:
        batch_circuits_run(packed)
    assert e.value.code == N.EINVAL


@pytest.mark.parametrize("prec,flags", [(N.C128, N.FLAG_FAST_C128), (N.C64, 0)])
def test_specialised_kernels_above_32_qubits_compile(lib, prec, flags):
    """Registers above 32 qubits: the specialised sweeps index with 64 bits
    (controls and diagonal targets on qubits 32 and up compiled in as 64-bit
    masks and shifts), and so do the specialised reverse sweeps of the
    adjoint gradient; both compile for sm_103a (host only)."""
    from kbw_gb300.dense import _gate_array
    n = 34
    circ = C.random_circuit(n, 90, 23, max_controls=2)
    circ += [(C.RZ, 33, (), 0.4), (C.X, 2, (33, 32), 0.0), (C.P, 32, (1,), 0.9), (C.RY, 33, (32,), 0.3)]
    try:
        sweeps, failed = N.jit_check(n, prec, flags, _gate_array(circ))
        assert sweeps > 0 and failed == 0, N.jit_last_error()
        sweeps, failed = N.jit_check_adjoint(n, prec, flags, _gate_array(circ))
        assert sweeps > 0 and failed == 0, N.jit_last_error()
    except N.KbwgError as e:
        if e.code == N.EUNSUPPORTED:
            pytest.skip("NVRTC not available: %s" % e)
        raise


@pytest.mark.parametrize("n,prec,fast", [(33, "c128", True), (36, "c64", False), (40, "c128", False)])
def test_planner_wide_registers(lib, n, prec, fast):
    """Registers above 32 qubits, where no state fits the oracle: the
    planner places every gate once, keeps each non-diagonal gate's target in
    its sweep's tile, and never swaps two gates that share a qubit on which
    either acts non-diagonally (controls and diagonal targets commute)."""
    from kbw_gb300.dense import plan
    rng = np.random.default_rng(n)
    circ = C.random_circuit(n, 220, int(rng.integers(0, 1 << 30)), max_controls=3)
    circ += [(C.RZ, n - 1, (), 0.3), (C.X, 0, (n - 1, n - 2), 0.0), (C.H, n - 1, (5,), 0.0),
             (C.P, n - 3, (n - 1,), 0.7), (C.RY, 31, (n - 1,), 0.2), (C.RX, n - 2, (), 0.4)]
    diag = {C.Z, C.P, C.RZ}
    sweeps = plan(n, circ, prec, fast_c128=fast)
    order = [i for _, idx in sweeps for i in idx]
    assert sorted(order) == list(range(len(circ)))
    pos = {g: k for k, g in enumerate(order)}
    for mask, idx in sweeps:
        for i in idx:
            kind, t, c, a = circ[i]
            if kind not in diag:
                assert mask >> t & 1, (i, t, hex(mask))

    def acts(g):  # qubit -> True if the gate acts on it non-diagonally
        kind, t, c, a = g
        out = {q: False for q in c}
        out[t] = kind not in diag
        return out

    for i in range(len(circ)):
        ai = acts(circ[i])
        for j in range(i + 1, len(circ)):
            aj = acts(circ[j])
            if any(q in aj and (ai[q] or aj[q]) for q in ai):
                assert pos[i] < pos[j], (i, j, circ[i], circ[j])
