"""Run-time specialised sweep kernels (NVRTC) against the interpreted sweep.

A specialised kernel applies a sweep's gates as straight-line code with the
structure compiled in, calling the same arithmetic in the same order as the
interpreted k_sweep, so the two give the same amplitudes bit for bit in every
arithmetic and tile geometry.  Both are also held to the oracle (restated
kbw Dense<F>) at the parity tolerances.
"""
import numpy as np
import pytest

import oracle
from kbw_gb300 import DenseGB300
from kbw_gb300 import _native as N
from kbw_gb300 import circuits as C
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 1e-5}

# (precision, float-float complex128, order-preserving planner, tile size (0: default))
CONFIGS = [
    ("c128", True, False, 0), ("c128", True, False, 12),
    ("c128", False, False, 0), ("c128", False, False, 11),
    ("c64", False, False, 0), ("c64", False, False, 12), ("c64", False, False, 11),
    ("c128", False, True, 0), ("c64", False, True, 0),
]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def run(n, circ, prec, fast, exact, tile, jit):
    sim = DenseGB300(n, prec, fast_c128=fast, exact_order=exact, jit=jit)
    if tile:
        sim.set_tuning(tile, 0)
    sim.apply(circ)
    sim.flush()
    _, passes = sim.last_flush_stats()
    spec = sim.jit_info()["last_specialised"]
    return sim, passes, spec


@pytest.mark.parametrize("prec,fast,exact,tile", CONFIGS)
@pytest.mark.parametrize("n", [17, 22])
def test_specialised_equals_interpreted(prec, fast, exact, tile, n):
    # up to three controls: on lane, register and warp bits and outside the
    # tile; at 22 qubits every CTA walks several tiles
    circ = C.random_circuit(n, 500, 7 + tile, max_controls=3)
    a, pa, sa = run(n, circ, prec, fast, exact, tile, N.JIT_OFF)
    b, pb, sb = run(n, circ, prec, fast, exact, tile, N.JIT_ALWAYS)
    assert sa == 0
    assert pa == pb and sb == pb, (pa, pb, sb, N.jit_last_error())
    sa_state, sb_state = a.state(), b.state()
    assert np.array_equal(bits(sa_state), bits(sb_state))
    ref = oracle.OracleDense(n, prec)
    ref.apply(circ)
    assert rel_err(sb_state, ref.state()) < TOL[prec]
    info = N.jit_info()
    assert info["available"] == 1 and info["failed"] == 0, N.jit_last_error()


@pytest.mark.parametrize("prec,fast", [("c128", True), ("c64", False), ("c128", False)])
def test_specialised_brickwork(prec, fast):
    n = 22
    circ = C.brickwork(n, 8, 3)
    a, _, _ = run(n, circ, prec, fast, False, 0, N.JIT_OFF)
    b, passes, spec = run(n, circ, prec, fast, False, 0, N.JIT_ALWAYS)
    assert spec == passes > 0
    assert np.array_equal(bits(a.state()), bits(b.state()))
    # <Z_i> and a measurement read the specialised state like any other
    ham = [[(1.0, [(C.PAULI_Z, q)])] for q in range(n)]
    assert [a.exp_value(h) for h in ham] == [b.exp_value(h) for h in ham]
    draws = C.uniform_draws(n, 5)
    assert a.measure(list(range(n)), draws) == b.measure(list(range(n)), draws)


def test_consecutive_hadamards_on_register_bits():
    # two H gates in a row: the second gate's sums take the first gate's
    # products; each product must be rounded on its own in straight-line code
    n = 16
    rng = np.random.default_rng(1)
    init = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    init = (init / np.linalg.norm(init)).astype(np.complex64)
    circ = [(C.H, 9, (), 0.0), (C.H, 10, (), 0.0), (C.H, 3, (), 0.0), (C.H, 11, (), 0.0)]
    out = []
    for jit in (N.JIT_OFF, N.JIT_ALWAYS):
        s = DenseGB300(n, "c64", jit=jit, fold=False)
        s.set_state(init)
        s.apply(circ)
        out.append(s.state())
    ref = oracle.OracleDense(n, "c64")
    ref.set_state(init)
    ref.apply(circ)
    want = ref.state().astype(np.complex64)
    assert np.array_equal(bits(out[0]), bits(want))
    assert np.array_equal(bits(out[1]), bits(want))


def test_auto_mode_background_compile_and_replay():
    n = 20  # the default threshold of the auto mode
    circ1 = C.brickwork(n, 4, 11)
    # the same structure with other rotation angles
    rng = np.random.default_rng(5)
    circ2 = [(k, t, c, float(rng.uniform(0, 2 * np.pi)) if k >= C.RX else a) for (k, t, c, a) in circ1]
    auto = DenseGB300(n, "c128", fast_c128=True, jit=N.JIT_AUTO)
    off = DenseGB300(n, "c128", fast_c128=True, jit=N.JIT_OFF)
    seen = []
    for i, circ in enumerate((circ1, circ2, circ1, circ2, circ1)):
        if i == 2:
            auto.jit_wait()  # the second flush started the compilation
        for sim in (auto, off):
            sim.apply(circ)
            sim.flush()
        _, passes = auto.last_flush_stats()
        seen.append((auto.jit_info()["last_specialised"], passes))
        assert np.array_equal(bits(auto.state()), bits(off.state()))
    # first sight: interpreted; second: interpreted while its kernels compile
    # (the graph is built); after the wait the graph is rebuilt with the
    # specialised kernels and later flushes replay it
    assert seen[0][0] == 0 and seen[1][0] == 0
    for spec, passes in seen[2:]:
        assert spec == passes > 0
    assert auto.jit_info()["mode"] == N.JIT_AUTO
    assert N.jit_info()["failed"] == 0, N.jit_last_error()


def test_auto_mode_skips_small_registers():
    n = 14  # below the default threshold of 20 qubits
    circ = C.random_circuit(n, 200, 3, max_controls=2)
    sim = DenseGB300(n, "c64", jit=N.JIT_AUTO)
    for _ in range(3):
        sim.apply(circ)
        sim.flush()
        assert sim.jit_info()["last_specialised"] == 0


@pytest.mark.parametrize("prec,fast", [("c64", False), ("c128", True), ("c128", False)])
def test_specialised_adjoint_equals_interpreted(prec, fast):
    # a hardware-efficient ansatz plus controlled rotations and phases (the
    # gradient's control projector on lane, register and outer bits), two
    # checkpoint segments
    n, L = 16, 3
    params = C.hea_params(n, L, 4)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    extra = C.random_circuit(n, 80, 12, max_controls=2, kinds=[C.RX, C.RY, C.RZ, C.P, C.H, C.X])
    k = len(params)
    for g in extra:
        circ.append(g)
        if g[0] in C.PARAMETRIC:
            pidx.append(k)
            k += 1
        else:
            pidx.append(-1)
    ham = C.tfim_ring(n)
    res = []
    for jit in (N.JIT_OFF, N.JIT_ALWAYS):
        sim = DenseGB300(n, prec, fast_c128=fast, jit=jit)
        res.append(sim.adjoint_gradient(circ, pidx, k, ham, max_checkpoints=1))
        sim.close()
    assert res[0][0] == res[1][0]
    assert np.array_equal(res[0][1], res[1][1])
    assert N.jit_info()["failed"] == 0, N.jit_last_error()


def test_exit_while_compiling_in_background():
    # the second flush starts a background compilation; the process exits
    # at once, with NVRTC still compiling: the exit must be clean (the
    # binding stops background compilation before the library teardown)
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from kbw_gb300 import DenseGB300, _native as N, circuits as C\n"
            "s = DenseGB300(21, 'c128', fast_c128=True, jit=N.JIT_AUTO)\n"
            "c = C.brickwork(21, 6, 2)\n"
            "for _ in range(2):\n"
            "    s.apply(c)\n"
            "    s.flush()\n"
            "print('done')\n" % root)
    for _ in range(3):
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
        assert "done" in r.stdout
