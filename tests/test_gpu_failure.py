"""Failure detection on the GPU without a fault: the bounded wait every tile
kernel uses for its TMA copies is run on a barrier that nothing completes
(kbwg_wait_probe).  Its polls must run out, the kernel must set the error
flag and return, the call must report KBWG_ETIMEOUT through the same host
check the gate kernels use, and the handle must stay usable with its state
untouched.  Nothing here traps, faults or hangs the GPU: the wait is bounded
and no copy is in flight."""
import pytest

import oracle
from kbw_gb300 import DenseGB300, KbwgError
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 1e-5}


@pytest.mark.parametrize("prec,fast", [("c128", True), ("c64", False)])
def test_wait_timeout_is_reported_and_the_handle_survives(prec, fast):
    n = 14
    first = C.random_circuit(n, 120, 3, max_controls=2)
    second = C.random_circuit(n, 80, 4, max_controls=1)
    sim = DenseGB300(n, prec, fast_c128=fast)
    sim.apply(first)  # queued: the probe flushes it before it runs
    for _ in range(2):  # the flag is cleared after each report
        with pytest.raises(KbwgError) as ei:
            sim.wait_probe(512)
        assert ei.value.code == N.ETIMEOUT
    ref = oracle.OracleDense(n, prec)
    ref.apply(first)
    assert rel_err(sim.state(), ref.state()) < TOL[prec]
    sim.apply(second)
    sim.flush()  # no stale error
    ref.apply(second)
    assert rel_err(sim.state(), ref.state()) < TOL[prec]
    sim.close()


def test_wait_probe_rejects_bad_limits():
    sim = DenseGB300(12, "c64")
    for spins in (0, (1 << 22) + 1):
        with pytest.raises(KbwgError) as ei:
            sim.wait_probe(spins)
        assert ei.value.code == N.EINVAL
    sim.close()
