"""Many circuits with their own gates and Pauli Hamiltonians in one launch
(kbwg_batch_circuits_exp_value) against the oracle (restated kbw
Dense<f64>): every circuit's <H> within 1e-10 (complex128) / 5e-5
(complex64) of the oracle's."""
import numpy as np
import pytest

import oracle
from kbw_gb300 import batch_circuits_exp_value, KbwgError
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C

pytestmark = pytest.mark.gpu


def random_hamiltonian(n, rng):
    ham = []
    for _ in range(int(rng.integers(1, 9))):
        k = int(rng.integers(0, min(3, n) + 1))
        qs = rng.choice(n, size=k, replace=False)
        ham.append((float(rng.uniform(-1.5, 1.5)), [(int(rng.integers(1, 4)), int(q)) for q in qs]))
    if rng.random() < 0.3 and n >= 2:
        ham += C.tfim_ring(n)
    return ham


def make_batch(count, seed, nmin=4, nmax=20):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        g = C.random_circuit(n, int(rng.integers(n, 6 * n + 1)), 1000 + i, max_controls=min(2, n - 1))
        out.append((n, g, random_hamiltonian(n, rng)))
    return out


@pytest.fixture(scope="module")
def batch512():
    circs = make_batch(512, 7)
    want = []
    for n, g, h in circs:
        o = oracle.OracleDense(n, "c128")
        o.apply(g)
        want.append(o.pauli_expect(h))
    return circs, np.array(want)


@pytest.mark.parametrize("prec,fast,tol", [("c128", True, 1e-10), ("c128", False, 1e-10), ("c64", False, 5e-5)])
def test_512_mixed_circuits_one_launch(batch512, prec, fast, tol):
    circs, want = batch512
    l0 = N.launch_count()
    got = batch_circuits_exp_value(circs, prec=prec, fast_c128=fast)
    assert N.launch_count() - l0 == 1  # one launch for all circuits
    err = np.abs(got - want)
    assert err.max() < tol, (err.max(), int(err.argmax()), circs[int(err.argmax())][0])


def test_batch_matches_the_hea_entry():
    # the hardware-efficient ansatz and ring TFIM through the general entry
    hea = C.hea_batch(64, seed=3, min_qubits=4, max_qubits=16)
    from kbw_gb300 import batch_hea_tfim
    e_hea = batch_hea_tfim(hea, prec="c128", fast_c128=False)
    circs = [(n, C.hea(n, L, p), C.tfim_ring(n)) for n, L, p in hea]
    got = batch_circuits_exp_value(circs, prec="c128")
    assert np.max(np.abs(got - e_hea)) < 1e-10


def test_batch_edge_cases():
    # empty circuits, empty Hamiltonians, one qubit, identity strings
    circs = [(1, [], [(0.5, [])]), (3, [(C.H, 0, (), 0.0)], []), (2, [(C.X, 1, (0,), 0.0)], [(1.0, [(C.PAULI_Z, 1)])]),
             (13, [(C.H, 12, (), 0.0)], [(2.0, [(C.PAULI_X, 12)])])]
    got = batch_circuits_exp_value(circs, prec="c128")
    assert np.allclose(got, [0.5, 0.0, 1.0, 2.0], atol=1e-12)
    assert len(batch_circuits_exp_value([], prec="c64")) == 0
    with pytest.raises(KbwgError) as e:
        batch_circuits_exp_value([(25, [], [])])
    assert e.value.code == N.EQUBITS
    with pytest.raises(KbwgError) as e:
        batch_circuits_exp_value([(3, [(C.X, 3, (), 0.0)], [])])
    assert e.value.code == N.EINVAL
    with pytest.raises(KbwgError) as e:
        batch_circuits_exp_value([(3, [], [(1.0, [(C.PAULI_Z, 1), (C.PAULI_X, 1)])])])
    assert e.value.code == N.EINVAL
