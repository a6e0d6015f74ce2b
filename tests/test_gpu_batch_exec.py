"""Whole-circuit batch entries (kbwg_batch_exp_value / _sample / _gradient),
the engine's side of the reference's BatchExecution
(src/quantum_execution.rs:367-427): a fresh register per call, the whole
circuit, then the read-out.  Checked against the oracle (expectation values
within the parity tolerance, sampled histograms identical for the same
draws) and against the handle-based entries; registers are pooled between
calls, so a second call must give the same answer as the first."""
import numpy as np
import pytest

import oracle
from kbw_gb300 import (DenseGB300, KbwgError, batch_exp_value, batch_gradient, batch_release,
                       batch_sample)
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 2e-5}


def hamiltonians(n):
    mixed = [(1.0, [(C.PAULI_Z, 0), (C.PAULI_Z, 1)]), (0.3, [(C.PAULI_X, 2), (C.PAULI_Y, n - 1)]),
             (-0.7, [(C.PAULI_Y, 3)])]
    return [C.tfim_ring(n), mixed, []]


@pytest.mark.parametrize("prec,fast", [("c128", False), ("c128", True), ("c64", False)])
def test_batch_exp_value_matches_oracle(prec, fast):
    n = 14
    circ = C.random_circuit(n, 250, 17, max_controls=2)
    hs = hamiltonians(n)
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    want = np.array([ref.exp_value(h) for h in hs])
    got = batch_exp_value(n, circ, hs, prec=prec, fast_c128=fast)
    assert got.shape == (3,) and got[2] == 0.0
    assert np.max(np.abs(got - want)) < TOL[prec] * max(1.0, np.max(np.abs(want)))
    # the second call runs on the pooled register: same answer
    again = batch_exp_value(n, circ, hs, prec=prec, fast_c128=fast)
    assert np.array_equal(again, got)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_batch_sample_matches_oracle(prec):
    n = 13
    circ = C.random_circuit(n, 200, 23, max_controls=2)
    qubits = [0, 3, 5, 8, 12]
    shots = 1024
    draws = C.uniform_draws(shots, 5)
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    ws, wc = ref.sample(qubits, shots, draws)
    for _ in range(2):
        gs, gc = batch_sample(n, circ, qubits, shots, draws, prec=prec)
        assert np.array_equal(gs, ws) and np.array_equal(gc, wc)


def test_batch_sample_fresh_generator_per_call(monkeypatch):
    # BatchExecution::sample builds a fresh QubitManager, whose generator is
    # seeded from KBW_SEED: with the variable set, every call draws the same
    monkeypatch.setenv("KBW_SEED", "1234")
    n = 12
    circ = C.random_circuit(n, 100, 2, max_controls=1)
    a = batch_sample(n, circ, list(range(n)), 500)
    b = batch_sample(n, circ, list(range(n)), 500)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert int(a[1].sum()) == 500


@pytest.mark.parametrize("prec,fast", [("c128", False), ("c64", False)])
def test_batch_gradient_equals_handle_adjoint(prec, fast):
    n, L = 12, 3
    params = C.hea_params(n, L, 8)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    sim = DenseGB300(n, prec, fast_c128=fast)
    e0, g0 = sim.adjoint_gradient(circ, pidx, len(params), ham)
    sim.close()
    e1, g1 = batch_gradient(n, circ, pidx, len(params), ham, prec=prec, fast_c128=fast)
    assert e1 == e0 and np.array_equal(g1, g0)
    o = oracle.OracleDense(n, "c128")
    o.apply(circ)
    assert abs(e1 - o.exp_value(ham)) < (1e-11 if prec == "c128" else 1e-5)


def test_batch_errors_and_release():
    circ = C.random_circuit(12, 50, 1)
    with pytest.raises(KbwgError) as ei:
        batch_exp_value(41, [], [C.tfim_ring(4)])
    assert ei.value.code == N.EQUBITS
    with pytest.raises(KbwgError) as ei:
        batch_sample(12, circ, [], 10, C.uniform_draws(10, 1))
    assert ei.value.code == N.EINVAL
    with pytest.raises(KbwgError) as ei:
        batch_exp_value(12, [(C.X, 12, (), 0.0)], [C.tfim_ring(12)])
    assert ei.value.code == N.EINVAL
    first = batch_exp_value(12, circ, [C.tfim_ring(12)])
    batch_release()
    assert np.array_equal(batch_exp_value(12, circ, [C.tfim_ring(12)]), first)
    batch_release()


def test_batch_empty_circuit_and_no_hamiltonians():
    # no gates: <H> of |0...0>; no Hamiltonians: nothing to return
    n = 12
    got = batch_exp_value(n, [], [[(1.0, [(C.PAULI_Z, 3)])], [(2.0, [(C.PAULI_X, 0)])]])
    assert got.tolist() == [1.0, 0.0]
    assert batch_exp_value(n, C.random_circuit(n, 20, 3), []).shape == (0,)
    st, ct = batch_sample(n, [], [0, 5], 16, C.uniform_draws(16, 2))
    assert st.tolist() == [0] and ct.tolist() == [16]
    batch_release()
