"""GPU tests of the sweep settings and their autotuner.

Every compiled tile size and a range of fusion depths must give the oracle's
state within the parity tolerance (complex128 1e-12 relative, complex64
1e-5), since they change only how gates are grouped into sweeps.  The tuner
must leave the handle's state exactly as it found it (it times candidates on
the handle's own state and restores a copy), pick one of the candidates,
reuse its result for a circuit of the same structure, and step aside for the
KBWG_TILE_QUBITS / KBWG_FUSION_DEPTH environment overrides.
"""
import numpy as np
import pytest

import oracle
from kbw_gb300 import DenseGB300, KbwgError
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C
from conftest import rel_err

pytestmark = pytest.mark.gpu

ARITHS = [("c64", False), ("c128", False), ("c128", True)]
TOL = {"c128": 1e-12, "c64": 1e-5}


def arith_id(a):
    return a[0] + ("-ff" if a[1] else "")


@pytest.mark.parametrize("arith", ARITHS, ids=arith_id)
def test_every_tile_size_and_depth_matches_oracle(arith):
    prec, ff = arith
    n = 15
    circ = C.random_circuit(n, 300, 31, max_controls=2)
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    want = ref.state()
    sim = DenseGB300(n, prec, fast_c128=ff)
    opts = sim.tile_options()
    assert len(opts) >= 2 and all(k <= n for k in opts)
    for k in opts:
        passes = {}
        for depth in (256, 64, 16, 1):
            sim.clear()
            sim.set_tuning(k, depth)
            t = sim.tuning()
            assert (t["tile_qubits"], t["fusion_depth"], t["source"]) == (k, depth, "set")
            sim.apply(circ)
            got = sim.state()
            err = rel_err(got, want)
            assert err < TOL[prec], "tile %d depth %d: relative error %.3g" % (k, depth, err)
            passes[depth] = sim.last_flush_stats()[1]
        # depth 1 is one sweep per gate
        assert passes[1] > passes[16] and passes[1] > passes[256]
    sim.close()


def test_small_registers_default_to_the_largest_tile_that_fits():
    # a 12-qubit register is below the complex64 default tile (13 qubits):
    # it runs on 12-qubit tiles; float-float keeps its 11-qubit default
    n = 12
    for prec, ff, k in (("c64", False, 12), ("c128", True, 11)):
        sim = DenseGB300(n, prec, fast_c128=ff)
        assert sim.tile_options()[0] == k and sim.tuning()["tile_qubits"] == k
        circ = C.random_circuit(n, 150, 6, max_controls=2)
        ref = oracle.OracleDense(n, prec)
        ref.apply(circ)
        sim.apply(circ)
        assert rel_err(sim.state(), ref.state()) < TOL[prec]
        sim.close()
    # complex64 11 qubits: 11 fits, 12 and 13 do not
    sim = DenseGB300(11, "c64")
    assert sim.tile_options() == [11] and sim.tuning()["tile_qubits"] == 11
    sim.close()


def test_tile_size_below_default_runs_fused_on_small_registers():
    n = 12
    circ = C.random_circuit(n, 200, 5, max_controls=2)
    ref = oracle.OracleDense(n, "c64")
    ref.apply(circ)
    sim = DenseGB300(n, "c64")
    assert sim.tile_options() == [12, 11]
    for k in (12, 11):
        sim.clear()
        sim.set_tuning(k, 0)
        sim.apply(circ)
        assert rel_err(sim.state(), ref.state()) < TOL["c64"]
        gates, passes = sim.last_flush_stats()
        assert passes < gates
    sim.close()


def test_set_tuning_rejects_unknown_settings():
    sim = DenseGB300(14, "c128", fast_c128=True)
    assert sim.tile_options() == [11, 12]
    for k, d in ((13, 0), (9, 0), (0, 257)):
        with pytest.raises(KbwgError) as ei:
            sim.set_tuning(k, d)
        assert ei.value.code == N.EINVAL
    sim.set_tuning(0, 0)
    assert sim.tuning()["source"] == "default"
    sim.close()


@pytest.mark.parametrize("arith", ARITHS, ids=arith_id)
def test_autotune_keeps_state_and_caches(arith):
    prec, ff = arith
    n = 16
    prep = C.random_circuit(n, 120, 7, max_controls=1)
    circ = C.brickwork(n, 6, 3)
    # twin handle: same preparation, no tuning
    twin = DenseGB300(n, prec, fast_c128=ff)
    twin.apply(prep)
    sim = DenseGB300(n, prec, fast_c128=ff)
    sim.apply(prep)  # queued: the tuner flushes it first, with the default settings
    t = sim.autotune(circ, reps=2)
    opts = sim.tile_options()
    assert t["source"] == "timed"
    assert t["candidates"] == 3 * len(opts)
    assert t["tile_qubits"] in opts and t["fusion_depth"] in (256, 64, 16)
    assert 0 < t["ms_per_run"] <= t["default_ms_per_run"]
    assert sim.tuning() == t
    # the state is the prepared one, bit for bit
    assert np.array_equal(sim.state(), twin.state())
    # the tuned settings give the oracle's result
    ref = oracle.OracleDense(n, prec)
    ref.apply(prep)
    ref.apply(circ)
    sim.apply(circ)
    assert rel_err(sim.state(), ref.state()) < TOL[prec]
    # same structure, other angles: the cached result, nothing timed
    other = [(k, q, c, a + 0.25) for (k, q, c, a) in circ]
    t2 = twin.autotune(other)
    assert t2["source"] == "cached" and t2["candidates"] == 0
    assert (t2["tile_qubits"], t2["fusion_depth"]) == (t["tile_qubits"], t["fusion_depth"])
    sim.close()
    twin.close()


def test_environment_overrides(monkeypatch):
    monkeypatch.setenv("KBWG_TILE_QUBITS", "12")
    monkeypatch.setenv("KBWG_FUSION_DEPTH", "32")
    n = 14
    sim = DenseGB300(n, "c64")
    t = sim.tuning()
    assert (t["tile_qubits"], t["fusion_depth"], t["source"]) == (12, 32, "env")
    circ = C.random_circuit(n, 150, 9, max_controls=2)
    t2 = sim.autotune(circ)  # the override stands: nothing timed
    assert (t2["tile_qubits"], t2["fusion_depth"], t2["source"], t2["candidates"]) == (12, 32, "env", 0)
    sim.apply(circ)
    ref = oracle.OracleDense(n, "c64")
    ref.apply(circ)
    assert rel_err(sim.state(), ref.state()) < TOL["c64"]
    sim.close()
    monkeypatch.setenv("KBWG_TILE_QUBITS", "9")
    with pytest.raises(KbwgError) as ei:
        DenseGB300(n, "c64")
    assert ei.value.code == N.EINVAL


def test_autotune_on_registers_below_every_tile():
    # 8 qubits: no compiled tile fits, the handle runs one kernel per gate;
    # the tuner has nothing to choose and says so without timing
    n = 8
    circ = C.random_circuit(n, 60, 12, max_controls=1)
    sim = DenseGB300(n, "c64")
    assert sim.tile_options() == []
    t = sim.autotune(circ)
    assert t["tile_qubits"] == 0 and t["candidates"] == 0 and t["source"] == "default"
    sim.apply(circ)
    ref = oracle.OracleDense(n, "c64")
    ref.apply(circ)
    assert rel_err(sim.state(), ref.state()) < TOL["c64"]
    with pytest.raises(KbwgError) as ei:
        sim.set_tuning(11, 0)
    assert ei.value.code == N.EINVAL
    sim.close()
