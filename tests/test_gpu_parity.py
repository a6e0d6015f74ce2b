"""GPU parity: the CUDA engine against the oracle (restated kbw Dense<F>).

Gate arithmetic keeps the reference's per-amplitude operation order, so with
the order-preserving planner (exact_order=True) and with fusion off the
amplitudes must equal the oracle's exactly (value equality), in both
precisions.  The default planner also reorders gates that commute, which
changes rounding only: complex128 amplitudes then agree within 1e-12
relative (the parity bar) and complex64 within 1e-5.  Reductions accumulate
in FP64, so p1 and <H> agree within 1e-12 (c128) / 1e-6 (c64); measurement
outcomes and sampled bitstrings are identical given the same draws.
"""
import math

import numpy as np
import pytest

import oracle
from kbw_gb300 import DenseGB300, KbwgError
from kbw_gb300 import circuits as C
from conftest import decode_circuit, load_golden, rel_err

pytestmark = pytest.mark.gpu

PRECS = ["c128", "c64"]


TOL = {"c128": 1e-12, "c64": 1e-5}


def both(n, circ, prec, fusion=True, exact_order=True):
    sim = DenseGB300(n, prec, fusion=fusion, exact_order=exact_order)
    sim.apply(circ)
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    return sim, ref


def assert_exact(sim, ref):
    got = sim.state().astype(np.complex128)
    want = ref.state()
    if not np.array_equal(got, want):
        bad = np.flatnonzero(got != want)
        raise AssertionError("%d amplitudes differ, first at %d: %r vs %r (rel %.3g)"
                             % (bad.size, bad[0], got[bad[0]], want[bad[0]], rel_err(got, want)))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fusion", [True, False])
def test_every_gate_kind_small_registers(prec, fusion):
    for n in range(1, 15):
        circ = C.random_circuit(n, 12 * n, 100 + n, max_controls=min(3, n - 1))
        sim, ref = both(n, circ, prec, fusion)
        assert_exact(sim, ref)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,gates,seed", [(16, 400, 1), (18, 500, 2), (20, 600, 3), (21, 300, 4)])
def test_fused_sweeps_exact(prec, n, gates, seed):
    circ = C.random_circuit(n, gates, seed, max_controls=3)
    sim, ref = both(n, circ, prec, exact_order=True)
    assert_exact(sim, ref)
    _, passes = sim.last_flush_stats()
    assert passes < gates


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,gates,seed", [(16, 400, 1), (20, 600, 3), (22, 400, 5)])
def test_fused_sweeps_reordered(prec, n, gates, seed):
    circ = C.random_circuit(n, gates, seed, max_controls=3)
    sim, ref = both(n, circ, prec, exact_order=False)
    assert rel_err(sim.state(), ref.state()) < TOL[prec]
    if prec == "c64":  # against the complex128 oracle: state infidelity (norms divided out)
        r128 = oracle.OracleDense(n, "c128")
        r128.apply(circ)
        a, b = r128.state(), sim.state().astype(np.complex128)
        ov = abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
        assert 1 - ov < 1e-8


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("exact_order", [True, False])
def test_brickwork(prec, exact_order):
    circ = C.brickwork(20, 8, 0)
    sim, ref = both(20, circ, prec, exact_order=exact_order)
    if exact_order:
        assert_exact(sim, ref)
    else:
        assert rel_err(sim.state(), ref.state()) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_single_gate_every_target_and_control(prec):
    n = 15
    rng = np.random.default_rng(7)
    base = C.random_circuit(n, 40, 8, max_controls=1)
    for kind in range(8):
        for t in range(n):
            c = int(rng.integers(0, n - 1))
            c = c if c < t else c + 1
            angle = float(rng.uniform(0, 2 * math.pi))
            circ = base + [(kind, t, (c,), angle), (kind, (t + 3) % n, (), angle)]
            sim, ref = both(n, circ, prec)
            assert_exact(sim, ref)


def test_random_small_golden():
    g = load_golden("random_small.npz")
    for i in range(int(g["count"])):
        n = int(g["c%d_n" % i])
        sim = DenseGB300(n, "c128")
        sim.apply(decode_circuit(g, "c%d" % i))
        assert rel_err(sim.state(), g["c%d_state" % i]) < 1e-12


@pytest.mark.parametrize("prec", PRECS)
def test_grover12(prec):
    g = load_golden("grover12.npz")
    tol = 1e-12 if prec == "c128" else 1e-4
    for seed in range(3):
        m = C.grover_marked(seed)
        sim = DenseGB300(12, prec)
        sim.apply(C.grover(12, m, 50))
        prob = np.abs(sim.state().astype(np.complex128)) ** 2
        assert np.max(np.abs(prob - g["prob_seed%d" % seed])) < tol
        assert abs(prob[m] - C.grover_success_probability(12, 50)) < tol
    sim = DenseGB300(12, "c128")
    sim.apply(C.grover(12, C.grover_marked(0), 50))
    st, ct = sim.sample(list(range(12)), 1024, g["sample_draws"])
    assert np.array_equal(st, g["sample_states"]) and np.array_equal(ct, g["sample_counts"])


@pytest.mark.parametrize("prec", PRECS)
def test_measure_p1_and_collapse(prec):
    n = 16
    circ = C.random_circuit(n, 200, 11, max_controls=2)
    sim, ref = both(n, circ, prec)
    tol = 1e-12 if prec == "c128" else 2e-6
    for t in (0, 3, 9, 15):
        assert abs(sim.measure_p1(t) - ref.measure_p1(t)) < tol
    p1 = ref.measure_p1(9)
    p = 1.0 / math.sqrt(p1)
    sim.measure_collapse(9, True, p)
    ref.measure_collapse(9, True, p)
    assert_exact(sim, ref)
    sim.measure_collapse(2, False, 1.25)
    ref.measure_collapse(2, False, 1.25)
    assert_exact(sim, ref)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [5, 13, 17])
def test_measure_with_draws(prec, n):
    for rep in range(4):
        circ = C.random_circuit(n, 15 * n, 40 + rep, max_controls=2)
        sim, ref = both(n, circ, prec)
        qubits = list(range(n)) if rep % 2 == 0 else [n - 1, 0, n // 2]
        draws = C.uniform_draws(len(qubits), 70 + rep)
        assert sim.measure(qubits, draws) == ref.measure(qubits, draws)
        tol = 1e-12 if prec == "c128" else 1e-5
        assert rel_err(sim.state(), ref.state()) < tol


def test_measure_golden():
    g = load_golden("measure.npz")
    for i in range(int(g["count"])):
        n = int(g["m%d_n" % i])
        qubits = [int(q) for q in g["m%d_qubits" % i]]
        sim = DenseGB300(n, "c128")
        sim.apply(decode_circuit(g, "m%d" % i))
        st, ct = sim.sample(qubits, 256, g["m%d_sdraws" % i])
        assert np.array_equal(st, g["m%d_sstates" % i]) and np.array_equal(ct, g["m%d_scounts" % i])
        assert sim.measure(qubits, g["m%d_draws" % i]) == int(g["m%d_result" % i])
        assert rel_err(sim.state(), g["m%d_post" % i]) < 1e-12


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [3, 12, 18])
def test_dump_exact(prec, n):
    circ = C.random_circuit(n, 6 * n, 21 + n, max_controls=2, kinds=[C.H, C.X, C.RY, C.P])
    sim, ref = both(n, circ, prec)
    for qubits in (list(range(n)), [n - 1, 0], list(range(n))[::-1][: max(1, n // 2)]):
        a = sim.dump(qubits)
        b = ref.dump(qubits)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [4, 14, 19])
def test_sample_bit_exact(prec, n):
    circ = C.random_circuit(n, 10 * n, 31 + n, max_controls=2)
    sim, ref = both(n, circ, prec)
    shots = 2048
    draws = C.uniform_draws(shots, 5 + n)
    for qubits in (list(range(n)), [0, n - 1]):
        st, ct = sim.sample(qubits, shots, draws)
        so, co = ref.sample(qubits, shots, draws)
        assert np.array_equal(st, so) and np.array_equal(ct, co)
        assert int(ct.sum()) == shots


@pytest.mark.parametrize("prec", PRECS)
def test_exp_value(prec):
    tol = 1e-11 if prec == "c128" else 2e-5
    for n, L, seed in [(6, 3, 1), (12, 2, 2), (16, 3, 3)]:
        params = C.hea_params(n, L, seed)
        sim, ref = both(n, C.hea(n, L, params), prec)
        h = C.tfim_ring(n)
        assert abs(sim.exp_value(h) - ref.exp_value(h)) < tol * n
        mixed = [(0.7, [(C.PAULI_Y, 0), (C.PAULI_X, n - 1)]), (-1.3, [(C.PAULI_Y, 1)]),
                 (0.25, [(C.PAULI_Z, 2), (C.PAULI_Y, 3), (C.PAULI_X, 0)]),
                 (1.1, [(C.PAULI_Y, 2), (C.PAULI_Y, 4), (C.PAULI_Y, 5)]), (2.0, [])]
        assert abs(sim.exp_value(mixed) - ref.exp_value(mixed)) < tol * 10
    g = load_golden("expval.npz")
    for i in range(int(g["count"])):
        n, L = int(g["e%d_n" % i]), int(g["e%d_L" % i])
        sim = DenseGB300(n, "c128")
        sim.apply(C.hea(n, L, g["e%d_params" % i]))
        assert abs(sim.exp_value(C.tfim_ring(n)) - float(g["e%d_tfim" % i])) < 1e-11 * n


@pytest.mark.parametrize("prec", PRECS)
def test_exp_value_tiled_passes(prec):
    """Strings with flip masks go through tiled passes (many masks per pass);
    strings too wide for one tile fall back to one pass per mask.  Mixes X/Y
    strings on low, high and scattered qubits with Z factors inside and
    outside the tile."""
    n = 17
    sim, ref = both(n, C.hea(n, 2, C.hea_params(n, 2, 91)), prec)
    rng = np.random.default_rng(92)
    h = C.tfim_ring(n)
    for _ in range(40):
        k = int(rng.integers(1, 5))
        qs = rng.choice(n, size=k, replace=False)
        h.append((float(rng.normal()), [(int(rng.integers(1, 4)), int(q)) for q in qs]))
    h.append((0.7, [(C.PAULI_X, q) for q in range(5, 16)]))            # 11 high flip bits: no tile holds it
    h.append((-0.4, [(C.PAULI_Y, q) for q in (0, 6, 9, 12, 13, 14, 15, 16)]))
    tol = 1e-11 if prec == "c128" else 2e-5
    assert abs(sim.exp_value(h) - ref.exp_value(h)) < tol * len(h)
    for term in h[-6:]:
        assert abs(sim.exp_value([term]) - ref.exp_value([term])) < tol


@pytest.mark.parametrize("prec", PRECS)
def test_swap_qubits_exact(prec):
    n = 15
    circ = C.random_circuit(n, 100, 77, max_controls=2)
    sim, ref = both(n, circ, prec)
    for a, b in [(0, 14), (3, 4), (13, 2)]:
        sim.swap_qubits(a, b)
        ref.swap_qubits(a, b)
        assert_exact(sim, ref)


def test_clear_and_state_roundtrip():
    sim = DenseGB300(10, "c128")
    sim.apply(C.random_circuit(10, 50, 3))
    sim.clear()
    s = sim.state()
    assert s[0] == 1 and np.count_nonzero(s) == 1
    rng = np.random.default_rng(0)
    v = rng.normal(size=1024) + 1j * rng.normal(size=1024)
    sim.set_state(v)
    assert np.array_equal(sim.state(), v)


def test_errors_are_status_codes():
    with pytest.raises(KbwgError) as e:
        DenseGB300(41, "c64")
    assert e.value.code == 2
    with pytest.raises(KbwgError) as e:  # 16 TiB: the device's memory refuses it
        DenseGB300(40, "c128")
    assert e.value.code == 3
    sim = DenseGB300(4, "c64")
    with pytest.raises(KbwgError):
        sim.pauli_x(4)
    with pytest.raises(KbwgError):
        sim.pauli_x(1, [1])
    with pytest.raises(KbwgError):
        sim.exp_value([(1.0, [(C.PAULI_X, 0), (C.PAULI_Z, 0)])])
    sim.pauli_x(0)
    # qubits[0] is the most significant bit of the packed result
    assert sim.measure([0, 1], [0.5, 0.5]) == 0b10


def test_zero_qubits():
    sim = DenseGB300(0, "c128")
    assert sim.state().tolist() == [1]
    assert sim.measure([], []) == 0
    st, re, im = sim.dump([])
    assert st.tolist() == [0] and re.tolist() == [1.0]


@pytest.mark.parametrize("prec", PRECS)
def test_28q_brickwork_round_trip(prec):
    """Size-independent properties at a large register: the norm stays 1 and
    the inverse circuit returns |0...0>."""
    n = 28
    circ = C.brickwork(n, 6, 5)
    inv = []
    for kind, t, c, a in reversed(circ):
        if kind in (C.P, C.RX, C.RY, C.RZ):
            inv.append((kind, t, c, -a))
        elif kind == C.Y:
            inv.append((kind, t, c, a))
        else:
            inv.append((kind, t, c, a))
    sim = DenseGB300(n, prec)
    sim.apply(circ)
    z = sim.exp_value([(1.0, [])])
    assert abs(z - 1.0) < (1e-12 if prec == "c128" else 1e-5)
    sim.apply(inv)
    st, re, im = sim.dump(list(range(n)))
    tol = 1e-12 if prec == "c128" else 1e-4
    assert st[0] == 0 and abs(re[0] - 1.0) < tol


@pytest.mark.parametrize("n,prec,fast", [(32, "c64", False), (31, "c128", True)])
def test_largest_registers(n, prec, fast):
    """The largest registers (32 GiB of amplitudes; 32 qubits is the Dense
    limit): a random circuit with controls on the top qubits keeps the norm,
    its inverse returns |0...0>, and a Bell pair between the top and bottom
    qubit reads out exactly (dump, p1, measurement with injected draws)."""
    circ = C.random_circuit(n, 120, 77, max_controls=2)
    inv = [(k, t, c, -a if k in C.PARAMETRIC else a) for (k, t, c, a) in reversed(circ)]
    sim = DenseGB300(n, prec, fast_c128=fast)
    tol = 1e-12 if prec == "c128" else 2e-5
    sim.apply(circ)
    assert abs(sim.exp_value([(1.0, [])]) - 1.0) < tol
    sim.apply(inv)
    top = n - 1
    assert sim.measure_p1(top) < tol and sim.measure_p1(0) < tol
    sim.clear()
    sim.hadamard(top)
    sim.pauli_x(0, [top])
    st, re, im = sim.dump([top, 0])
    assert st.tolist() == [0, 3]
    assert np.allclose(re, [2 ** -0.5] * 2, atol=tol) and np.allclose(im, 0.0, atol=tol)
    assert abs(sim.measure_p1(top) - 0.5) < tol
    assert sim.measure([top, 0], [0.75, 0.1]) in (0, 3)
    sim.close()


# ---- complex128 float-float fast path ------------------------------------------

@pytest.mark.parametrize("n,gates,seed", [(12, 300, 61), (16, 500, 62), (20, 800, 63), (23, 400, 64)])
def test_fast_c128_random_circuits(n, gates, seed):
    """Float-float arithmetic on binary64 storage: amplitudes within 1e-12
    relative of the restated Dense<f64>."""
    circ = C.random_circuit(n, gates, seed, max_controls=3)
    sim = DenseGB300(n, "c128", fast_c128=True)
    sim.apply(circ)
    ref = oracle.OracleDense(n, "c128")
    ref.apply(circ)
    assert rel_err(sim.state(), ref.state()) < 1e-12


def test_fast_c128_brickwork_and_readout():
    n = 20
    circ = C.brickwork(n, 20, 0)
    sim = DenseGB300(n, "c128", fast_c128=True)
    sim.apply(circ)
    ref = oracle.OracleDense(n, "c128")
    ref.apply(circ)
    assert rel_err(sim.state(), ref.state()) < 1e-12
    zs = [(1.0, [(C.PAULI_Z, q)]) for q in range(n)]
    assert abs(sim.exp_value(zs) - ref.exp_value(zs)) < 1e-11
    for t in (0, 7, 19):
        assert abs(sim.measure_p1(t) - ref.measure_p1(t)) < 1e-12
    draws = C.uniform_draws(n, 3)
    assert sim.measure(list(range(n)), draws) == ref.measure(list(range(n)), draws)


def test_fast_c128_many_hadamards_rescale():
    """More than 100 uncontrolled H in one flush forces an intermediate
    rescale of the folded 1/sqrt(2) factors."""
    n = 14
    circ = []
    for layer in range(30):
        circ += [(C.H, q, (), 0.0) for q in range(n)]
        circ += [(C.RZ, q, (), 0.3 * q + layer) for q in range(n)]
        circ += [(C.X, (q + 1) % n, (q,), 0.0) for q in range(0, n - 1, 2)]
    sim = DenseGB300(n, "c128", fast_c128=True)
    sim.apply(circ)
    ref = oracle.OracleDense(n, "c128")
    ref.apply(circ)
    assert rel_err(sim.state(), ref.state()) < 1e-12


def test_fast_c128_resident_format_transitions():
    """The float-float handle keeps its state in float-float form between
    sweeps; exp_value, measure_p1, collapse and measurement read (and
    write) that form as is, the other operations return it to binary64:
    interleave gates with every kind of read, a swap (format-agnostic), a
    collapse, a partial measurement, set_state and clear, and follow the
    restated Dense<f64> throughout."""
    n = 14
    sim = DenseGB300(n, "c128", fast_c128=True)
    ref = oracle.OracleDense(n, "c128")

    def step(circ):
        sim.apply(circ)
        ref.apply(circ)

    step(C.random_circuit(n, 150, 71, max_controls=2))
    assert rel_err(sim.state(), ref.state()) < 1e-12        # get_state converts back
    step(C.brickwork(n, 3, 72))
    sim.swap_qubits(2, 11)                                  # runs on the float-float form
    ref.swap_qubits(2, 11)
    step(C.random_circuit(n, 100, 73))
    assert abs(sim.measure_p1(5) - ref.measure_p1(5)) < 1e-12
    p = ref.measure_p1(5)
    sim.measure_collapse(5, True, 1.0 / math.sqrt(p))
    ref.measure_collapse(5, True, 1.0 / math.sqrt(p))
    step(C.random_circuit(n, 100, 74))
    draws = C.uniform_draws(4, 9)
    assert sim.measure([1, 7, 12, 3], draws) == ref.measure([1, 7, 12, 3], draws)
    step(C.random_circuit(n, 80, 76))
    assert rel_err(sim.state(), ref.state()) < 1e-12
    step(C.random_circuit(n, 40, 77))
    h = C.tfim_ring(n) + [(0.3, [(C.PAULI_Y, 1), (C.PAULI_Z, 6)])]
    assert abs(sim.exp_value(h) - ref.exp_value(h)) < 1e-11
    step(C.random_circuit(n, 60, 75))
    st, re, im = sim.dump(list(range(n)))
    rst, rre, rim = ref.dump(list(range(n)))
    assert np.array_equal(st, rst)
    assert np.max(np.abs(re - rre)) < 1e-12 and np.max(np.abs(im - rim)) < 1e-12
    # set_state replaces the resident form; gates after it start from binary64
    psi = ref.state()
    sim.set_state(psi)
    step(C.random_circuit(n, 80, 76))
    assert rel_err(sim.state(), ref.state()) < 1e-12
    # clear re-initialises in float-float form
    sim.clear()
    ref2 = oracle.OracleDense(n, "c128")
    circ = C.random_circuit(n, 120, 77)
    sim.apply(circ)
    ref2.apply(circ)
    assert rel_err(sim.state(), ref2.state()) < 1e-12
    draws = C.uniform_draws(n, 78)
    assert sim.measure(list(range(n)), draws) == ref2.measure(list(range(n)), draws)


def test_fast_c128_distance_and_gradient_after_gates():
    """state_distance and the adjoint gradient on a handle whose state was
    left in float-float form by earlier gates."""
    n = 13
    a = DenseGB300(n, "c128", fast_c128=True)
    b = DenseGB300(n, "c128")
    circ = C.random_circuit(n, 200, 81)
    a.apply(circ)
    b.apply(circ)
    assert a.distance(b) < 1e-12
    L = 2
    params = C.hea_params(n, L, 82)
    pidx = C.hea_param_index(n, L)
    a.apply(C.random_circuit(n, 50, 83))  # leave a float-float state behind
    e_a, g_a = a.adjoint_gradient(C.hea(n, L, params), pidx, len(params), C.tfim_ring(n))
    e_b, g_b = b.adjoint_gradient(C.hea(n, L, params), pidx, len(params), C.tfim_ring(n))
    assert abs(e_a - e_b) < 1e-11
    assert np.max(np.abs(g_a - g_b)) < 1e-10
    # the adjoint leaves |0...0>
    assert abs(a.state()[0] - 1.0) < 1e-15


def test_state_fidelity_across_precisions():
    """kbwg_state_fidelity against numpy on the host copies, for every pair
    of arithmetics (complex64, binary64 complex128, float-float complex128)."""
    n = 15
    circ = C.random_circuit(n, 250, 91, max_controls=2)
    other = C.random_circuit(n, 40, 92)
    sims = {"c64": DenseGB300(n, "c64"), "c128": DenseGB300(n, "c128"),
            "ff": DenseGB300(n, "c128", fast_c128=True)}
    for s in sims.values():
        s.apply(circ)
    sims["c128"].apply(other)  # a different state for the off-diagonal pairs
    host = {k: s.state().astype(np.complex128) for k, s in sims.items()}
    for ka, a in sims.items():
        for kb, b in sims.items():
            x, y = host[ka], host[kb]
            want = abs(np.vdot(x, y)) ** 2 / (np.vdot(x, x).real * np.vdot(y, y).real)
            got = a.fidelity(b)
            assert abs(got - want) < 1e-12, (ka, kb, got, want)
    assert 1 - sims["c64"].fidelity(sims["ff"]) < 1e-10
    assert 1 - sims["ff"].fidelity(sims["ff"]) < 1e-14
    with pytest.raises(KbwgError):
        sims["c64"].fidelity(DenseGB300(n - 1, "c64"))


@pytest.mark.parametrize("prec,fast", [("c64", False), ("c128", True), ("c128", False)])
def test_graph_replay_same_structure_new_angles(prec, fast):
    """Repeated flushes of one gate structure replay a CUDA graph with freshly
    uploaded constants: every repetition (other angles, from |0>) must match
    the oracle and a handle that never uses graphs."""
    import kbw_gb300._native as N
    n = 16
    a = DenseGB300(n, prec, fast_c128=fast)
    b = DenseGB300(n, prec, fast_c128=fast, graphs=False)
    tol = 1e-12 if prec == "c128" else 1e-5
    for rep in range(4):
        # same structure every repetition (brickwork seed fixed), new angles
        circ = C.hea(n, 3, C.hea_params(n, 3, 100 + rep)) + [(k, t, c, 0.1 * rep + 0.3 * i)
                                                            for i, (k, t, c, _) in enumerate(C.brickwork(n, 2, 200))]
        a.clear()
        b.clear()
        l0 = N.launch_count()
        a.apply(circ)
        a.flush()
        assert N.launch_count() - l0 == a.last_flush_stats()[1]
        b.apply(circ)
        ref = oracle.OracleDense(n, prec)
        ref.apply(circ)
        assert rel_err(a.state(), ref.state()) < tol
        assert rel_err(a.state(), b.state()) < tol


@pytest.mark.parametrize("prec,fast", [("c64", False), ("c128", False), ("c128", True)])
def test_folded_diagonal_chains(prec, fast):
    """Runs of diagonal gates (Z, S, T, P, RZ) on a qubit separated only by
    gates that touch it as a control or diagonally are folded into one gate
    on the host; results match the oracle, which applies every gate."""
    n = 15
    rng = np.random.default_rng(301)
    circ = []
    for _ in range(400):
        q = int(rng.integers(0, n))
        r = rng.random()
        if r < 0.45:  # diagonal one-qubit
            kind = [C.Z, C.P, C.RZ][int(rng.integers(0, 3))]
            circ.append((kind, q, (), float(rng.uniform(0, 2 * math.pi))))
        elif r < 0.75:  # CNOT with q as control: keeps q's diagonal run open
            t = int((q + 1 + rng.integers(0, n - 1)) % n)
            circ.append((C.X, t, (q,), 0.0))
        elif r < 0.85:  # controlled phase: diagonal on both qubits
            c = int((q + 1 + rng.integers(0, n - 1)) % n)
            circ.append((C.P, q, (c,), float(rng.uniform(0, 2 * math.pi))))
        else:  # non-diagonal on q: closes the run
            kind = [C.H, C.RX, C.RY, C.Y][int(rng.integers(0, 4))]
            circ.append((kind, q, (), float(rng.uniform(0, 2 * math.pi))))
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    for fold in (True, False):  # KBWG_FLAG_NO_FOLD applies every gate as given
        sim = DenseGB300(n, prec, fast_c128=fast, fold=fold)
        sim.apply(circ)
        assert rel_err(sim.state(), ref.state()) < (1e-12 if prec == "c128" else 1e-5)
        sim.close()


def test_own_generator_is_stdrng_of_kbw_seed(monkeypatch):
    """Without caller draws a handle draws from StdRng::seed_from_u64(KBW_SEED)
    (the reference QubitManager's generator): the outcomes equal those with
    the same stream passed explicitly; sampling continues the stream."""
    from kbw_gb300 import _native as N
    monkeypatch.setenv("KBW_SEED", "20260704")
    n = 10
    circ = C.random_circuit(n, 120, 31, max_controls=1)
    qs = list(range(n))
    a = DenseGB300(n, "c128")
    a.apply(circ)
    own = [a.measure(qs) for _ in range(1)] + [a.sample(qs, 64)]
    b = DenseGB300(n, "c128")
    b.apply(circ)
    d = N.draws(20260704, n + 64)
    given = [b.measure(qs, d[:n])] + [b.sample(qs, 64, d[n:])]
    assert own[0] == given[0]
    assert np.array_equal(own[1][0], given[1][0]) and np.array_equal(own[1][1], given[1][1])
    a.close()
    b.close()


@pytest.mark.parametrize("n,prec,fast", [(33, "c128", True), (33, "c128", False), (34, "c64", False),
                                         (34, "c128", True), (35, "c64", False)])
def test_registers_above_32_qubits(n, prec, fast):
    """Beyond Dense's 32 qubits (DenseGPU and the Block backends have no cap):
    128 and 256 GiB of amplitudes (256 GiB: the largest power of two that
    fits in one GB300's HBM), swept with 64-bit state indices.  A
    random circuit with controls on the top qubits keeps the norm, its
    inverse returns |0...0>, and a Bell pair between the top and the bottom
    qubit reads out exactly (dump, p1, measurement with injected draws)."""
    import gc
    gc.collect()  # earlier tests' handles (up to 64 GiB) must be gone
    circ = C.random_circuit(n, 90, 91, max_controls=2)
    circ += [(C.H, n - 1, (), 0.0), (C.RY, n - 2, (n - 1,), 0.7), (C.X, 0, (n - 1, n - 2), 0.0)]
    inv = [(k, t, c, -a if k in C.PARAMETRIC else a) for (k, t, c, a) in reversed(circ)]
    sim = DenseGB300(n, prec, fast_c128=fast)
    tol = 1e-12 if prec == "c128" else 2e-5
    sim.apply(circ)
    assert abs(sim.exp_value([(1.0, [])]) - 1.0) < tol
    sim.apply(inv)
    top = n - 1
    assert sim.measure_p1(top) < tol and sim.measure_p1(n - 2) < tol and sim.measure_p1(0) < tol
    sim.clear()
    sim.hadamard(top)
    sim.pauli_x(0, [top])
    st, re, im = sim.dump([top, 0])
    assert st.tolist() == [0, 3]
    assert np.allclose(re, [2 ** -0.5] * 2, atol=tol) and np.allclose(im, 0.0, atol=tol)
    assert abs(sim.measure_p1(top) - 0.5) < tol
    assert sim.measure([top, 0], [0.75, 0.1]) in (0, 3)
    sim.close()
    del sim
    gc.collect()
