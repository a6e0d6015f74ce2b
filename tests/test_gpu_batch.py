"""Batched hardware-efficient-ansatz circuits (kbwg_batch_hea_tfim): every
energy against the complex128 oracle.  Covers single-tile circuits (n <= 13)
and tiled ones (n up to 20), every layer count, and the work queue with more
circuits than CTAs."""
import numpy as np
import pytest

import oracle
from kbw_gb300 import batch_hea_tfim
from kbw_gb300 import circuits as C

pytestmark = pytest.mark.gpu


def oracle_energy(n, L, params, zz=1.0, x=0.5):
    o = oracle.OracleDense(n, "c128")
    o.apply(C.hea(n, L, params))
    return o.exp_value(C.tfim_ring(n, zz, x))


@pytest.mark.parametrize("prec,fast,tol", [("c64", False, 2e-5), ("c128", False, 1e-11), ("c128", True, 1e-11)])
def test_small_and_tiled_circuits(prec, fast, tol):
    rng = np.random.default_rng(1)
    sizes = [(2, 3), (3, 1), (5, 2), (8, 4), (9, 2), (12, 8), (13, 3), (14, 2), (16, 3), (18, 2)]
    circs = [(n, L, rng.uniform(-np.pi, np.pi, size=2 * n * L)) for n, L in sizes]
    got = batch_hea_tfim(circs, prec=prec, fast_c128=fast)
    want = np.array([oracle_energy(n, L, p) for n, L, p in circs])
    assert np.max(np.abs(got - want)) < tol * 20, np.abs(got - want)


def test_many_circuits_work_queue():
    circs = C.hea_batch(600, seed=3, min_qubits=8, max_qubits=14, min_layers=2, max_layers=8)
    got = batch_hea_tfim(circs, prec="c64")
    idx = np.random.default_rng(0).choice(len(circs), size=40, replace=False)
    for i in idx:
        n, L, p = circs[i]
        assert abs(got[i] - oracle_energy(n, L, p)) < 2e-5 * n


def test_twenty_qubits_and_coefficients():
    circs = C.hea_batch(6, seed=5, min_qubits=20, max_qubits=20, min_layers=2, max_layers=3)
    got = batch_hea_tfim(circs, zz=-0.7, x=1.3, prec="c64")
    for (n, L, p), e in zip(circs, got):
        assert abs(e - oracle_energy(n, L, p, -0.7, 1.3)) < 5e-5 * n
