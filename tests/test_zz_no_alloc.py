"""The allocation-free entry point kbwg_masked_norm_noalloc.

It exists for callers that cannot allocate device memory -- work recorded
into a CUDA graph, plugins whose host runtime owns every device allocation,
real-time loops -- and runs the measure_p1 reduction with its scratch in a
fixed device array of the library.  This test calls it through the C ABI on
a state the engine prepared, with an output buffer the caller owns, and
checks it against the existing entry point kbwg_measure_p1 on two calls in a
row (the second call sees the scratch the first one left behind).

This file is collected last so that a failure here cannot hide the others.
"""
import ctypes

import numpy as np
import pytest

from kbw_gb300 import DenseGB300
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 2e-6}


def _noalloc(lib, ptr, n, prec_code, mask, value, out_ptr, stream):
    return lib.kbwg_masked_norm_noalloc(ctypes.c_void_p(ptr), n, prec_code, mask, value,
                                        ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream))


@pytest.mark.parametrize("prec,fast", [("c128", False), ("c64", False), ("c128", True)])
def test_noalloc_matches_measure_p1_twice(prec, fast):
    # fast: a complex128 handle that keeps its state in float-float form
    # between sweeps; reading its device pointer turns it back to binary64
    torch = pytest.importorskip("torch")
    lib = N.load()
    n = 18
    sim = DenseGB300(n, prec, fast_c128=fast)
    sim.apply(C.random_circuit(n, 300, 23, max_controls=2))
    nq, prec_code, ptr, _ = sim.device_info()  # flushes the gate queue
    stream = sim.stream_handle()
    out = torch.zeros(8, dtype=torch.float64, device="cuda")  # caller-owned output
    targets = (0, 5, 11, 17)
    for call in range(2):
        for k, t in enumerate(targets):
            want = sim.measure_p1(t)
            rc = _noalloc(lib, ptr, nq, prec_code, 1 << t, 1 << t, out.data_ptr() + 8 * k, stream)
            assert rc == N.OK, lib.kbwg_last_error()
        torch.cuda.synchronize()
        got = out[: len(targets)].cpu().numpy()
        want = np.array([sim.measure_p1(t) for t in targets])
        assert np.all(np.abs(got - want) <= TOL[prec]), (call, got, want)
        out.zero_()
    # a multi-qubit condition against the host sum of the same amplitudes
    amps = sim.state().astype(np.complex128)
    idx = np.arange(amps.size)
    mask, value = (1 << 3) | (1 << 9), (1 << 9)
    rc = _noalloc(lib, ptr, nq, prec_code, mask, value, out.data_ptr(), stream)
    assert rc == N.OK
    torch.cuda.synchronize()
    ref = float(np.sum(np.abs(amps[(idx & mask) == value]) ** 2))
    assert abs(out[0].item() - ref) <= TOL[prec]


def test_noalloc_rejects_out_of_range():
    torch = pytest.importorskip("torch")
    lib = N.load()
    sim = DenseGB300(4, "c64")
    _, prec_code, ptr, _ = sim.device_info()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert _noalloc(lib, ptr, 33, prec_code, 1, 1, out.data_ptr(), 0) == N.EQUBITS
    assert _noalloc(lib, ptr, 4, prec_code, 1, 2, out.data_ptr(), 0) == N.EINVAL
    assert _noalloc(lib, ptr, 4, prec_code, 1 << 5, 0, out.data_ptr(), 0) == N.EINVAL
    assert _noalloc(lib, 0, 4, prec_code, 1, 1, out.data_ptr(), 0) == N.EINVAL
    # host memory for the state or the output is refused, not handed to the kernel
    host = np.zeros(64, dtype=np.complex64)
    hout = np.zeros(1, dtype=np.float64)
    assert _noalloc(lib, host.ctypes.data, 4, prec_code, 1, 1, out.data_ptr(), 0) == N.EINVAL
    assert _noalloc(lib, ptr, 4, prec_code, 1, 1, hout.ctypes.data, 0) == N.EINVAL
    assert _noalloc(lib, ptr, 4, prec_code, 1, 1, out.data_ptr(), 0) == N.OK
