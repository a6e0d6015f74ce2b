"""Adjoint gradients (kbwg_adjoint_gradient) against the parameter-shift
rule evaluated on the CPU oracle (restated Dense<f64>), against central
finite differences, and against the GPU parameter-shift entry.  Tolerances
follow the targets: <= 1e-10 (complex128), <= 1e-5 (complex64)."""
import math

import numpy as np
import pytest

import oracle
from kbw_gb300 import DenseGB300, KbwgError
from kbw_gb300 import circuits as C

pytestmark = pytest.mark.gpu


def oracle_energy(n, circ, ham):
    o = oracle.OracleDense(n, "c128")
    o.apply(circ)
    return o.exp_value(ham)


def oracle_param_shift(n, circ, param_index, n_params, ham):
    g = np.zeros(n_params)
    for i, p in enumerate(param_index):
        if p < 0:
            continue
        kind, t, c, a = circ[i]
        plus = list(circ)
        minus = list(circ)
        plus[i] = (kind, t, c, a + math.pi / 2)
        minus[i] = (kind, t, c, a - math.pi / 2)
        g[p] += 0.5 * (oracle_energy(n, plus, ham) - oracle_energy(n, minus, ham))
    return g


@pytest.mark.parametrize("prec,fast,tol", [("c128", False, 1e-10), ("c128", True, 1e-10), ("c64", False, 1e-5)])
def test_adjoint_hea_vs_oracle_param_shift(prec, fast, tol):
    n, L = 12, 2
    params = C.hea_params(n, L, 3)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    sim = DenseGB300(n, prec, fast_c128=fast)
    e, g = sim.adjoint_gradient(circ, pidx, len(params), ham)
    want = oracle_param_shift(n, circ, pidx, len(params), ham)
    assert abs(e - oracle_energy(n, circ, ham)) < (1e-11 if prec == "c128" else 1e-5)
    assert np.max(np.abs(g - want)) < tol, np.max(np.abs(g - want))


def test_adjoint_checkpoints_do_not_change_result():
    n, L = 13, 4
    params = C.hea_params(n, L, 5)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    sim = DenseGB300(n, "c128")
    e0, g0 = sim.adjoint_gradient(circ, pidx, len(params), ham, max_checkpoints=0)
    e1, g1 = sim.adjoint_gradient(circ, pidx, len(params), ham, max_checkpoints=7)
    assert abs(e0 - e1) < 1e-13 and np.max(np.abs(g0 - g1)) < 1e-12


@pytest.mark.parametrize("prec,fast", [("c64", False), ("c128", True)])
def test_adjoint_repeated_calls_reuse_scratch(prec, fast):
    # the handle keeps lambda, the checkpoints and the reverse programs
    # between calls: repeated, shorter, longer and differently checkpointed
    # calls give exactly the results of a fresh handle
    n = 14
    ham = C.tfim_ring(n)
    sim = DenseGB300(n, prec, fast_c128=fast)
    for L, seed, ck in ((3, 1, 16), (1, 2, 16), (5, 3, 2), (3, 1, 16), (2, 4, 0), (3, 1, 16)):
        params = C.hea_params(n, L, seed)
        circ, pidx = C.hea(n, L, params), C.hea_param_index(n, L)
        e, g = sim.adjoint_gradient(circ, pidx, len(params), ham, max_checkpoints=ck)
        fresh = DenseGB300(n, prec, fast_c128=fast)
        e2, g2 = fresh.adjoint_gradient(circ, pidx, len(params), ham, max_checkpoints=ck)
        fresh.close()
        assert e == e2 and np.array_equal(g, g2), (L, seed, ck)
    sim.close()


@pytest.mark.parametrize("fusion,wide", [(True, False), (True, True), (False, False)])
def test_adjoint_float_float_forms_vs_binary64(fusion, wide):
    # float-float complex128: with fused sweeps the whole gradient stays in
    # the float-float form (checkpoints, lambda, reverse sweeps); with one
    # kernel per gate the forward pass is binary64 and the reverse sweeps
    # split it on load.  Both agree with the binary64 adjoint within 1e-12,
    # with lambda in tiled passes or (a wide string) by flip-mask groups.
    n, L = 13, 3
    params = C.hea_params(n, L, 8)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    extra = C.random_circuit(n, 40, 21, max_controls=1, kinds=[C.RX, C.RY, C.RZ, C.P, C.H, C.Y])
    k = len(params)
    for g in extra:
        circ.append(g)
        pidx.append(k if g[0] in C.PARAMETRIC else -1)
        k += 1 if g[0] in C.PARAMETRIC else 0
    ham = C.tfim_ring(n) + [(1.5, [(C.PAULI_Y, 2), (C.PAULI_Y, 7)]), (-0.25, [(C.PAULI_Y, 4)]),
                            (0.5, [(C.PAULI_X, 0), (C.PAULI_Z, 12)])]
    if wide:  # a string flipping more qubits than a tile holds: lambda by flip-mask groups
        ham.append((0.3, [(C.PAULI_X, q) for q in range(n)]))
    ref = DenseGB300(n, "c128")
    e0, g0 = ref.adjoint_gradient(circ, pidx, k, ham, max_checkpoints=3)
    sim = DenseGB300(n, "c128", fast_c128=True, fusion=fusion)
    e1, g1 = sim.adjoint_gradient(circ, pidx, k, ham, max_checkpoints=3)
    assert abs(e1 - e0) < 1e-12
    assert np.max(np.abs(g1 - g0)) < 1e-12, np.max(np.abs(g1 - g0))


def test_adjoint_controlled_phase_shared_params_vs_finite_differences():
    """Controlled rotations, phase gates and a parameter used by two gates:
    compared with central differences (h = 1e-6) of the oracle energy."""
    n = 12
    rng = np.random.default_rng(9)
    th = rng.uniform(-math.pi, math.pi, size=5)

    def build(t):
        c = [(C.H, q, (), 0.0) for q in range(n)]
        c += [(C.RX, 3, (), t[0]), (C.RY, 7, (2,), t[1]), (C.P, 5, (), t[2]), (C.RZ, 11, (0, 4), t[3]),
              (C.X, 6, (5,), 0.0), (C.RY, 1, (), t[4]), (C.P, 9, (8,), t[2]), (C.RX, 10, (), t[0])]
        c += [(C.Z, (q + 1) % n, (q,), 0.0) for q in range(n)]
        c += [(C.RY, q, (), 0.3 * q) for q in range(n)]
        return c

    pidx = [-1] * n + [0, 1, 2, 3, -1, 4, 2, 0] + [-1] * (2 * n)
    ham = C.tfim_ring(n) + [(0.4, [(C.PAULI_Y, 2), (C.PAULI_X, 9)])]
    sim = DenseGB300(n, "c128")
    e, g = sim.adjoint_gradient(build(th), pidx, 5, ham)
    h = 1e-6
    fd = np.zeros(5)
    for p in range(5):
        tp, tm = th.copy(), th.copy()
        tp[p] += h
        tm[p] -= h
        fd[p] = (oracle_energy(n, build(tp), ham) - oracle_energy(n, build(tm), ham)) / (2 * h)
    assert abs(e - oracle_energy(n, build(th), ham)) < 1e-11
    assert np.max(np.abs(g - fd)) < 1e-8, (g, fd)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_adjoint_vs_gpu_param_shift(prec):
    n, L = 16, 3
    params = C.hea_params(n, L, 7)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    sim = DenseGB300(n, prec)
    e_a, g_a = sim.adjoint_gradient(circ, pidx, len(params), ham)
    e_p, g_p = sim.param_shift_gradient(circ, pidx, len(params), ham)
    tol = 1e-10 if prec == "c128" else 1e-5
    assert abs(e_a - e_p) < tol and np.max(np.abs(g_a - g_p)) < tol


def test_param_shift_rejects_controlled_rotations():
    sim = DenseGB300(12, "c128")
    circ = [(C.RY, 1, (0,), 0.3)]
    with pytest.raises(KbwgError):
        sim.param_shift_gradient(circ, [0], 1, C.tfim_ring(12))


def test_torch_autograd_bridge():
    torch = pytest.importorskip("torch")
    from kbw_gb300.autograd import adjoint_energy
    n, L = 12, 2
    ham = C.tfim_ring(n)
    sim = DenseGB300(n, "c128")
    pidx = C.hea_param_index(n, L)
    params = torch.tensor(C.hea_params(n, L, 11), dtype=torch.float64, requires_grad=True)
    e = adjoint_energy(params, sim, lambda p: (C.hea(n, L, p), pidx), ham)
    e.backward()
    want = oracle_param_shift(n, C.hea(n, L, params.detach().numpy()), pidx, params.numel(), ham)
    assert np.max(np.abs(params.grad.numpy() - want)) < 1e-10


def test_adjoint_24q_slice_vs_oracle_param_shift_and_fd():
    """The gradient configuration's register size (24 qubits; two of its ten
    layers): adjoint gradients in all three arithmetics at parameters of both
    layers and both rotation kinds, against parameter shift on the oracle
    (energies from its amplitudes) and central differences with h = 1e-6 on
    the engine's order-preserving binary64 path (the Dense<f64> arithmetic)."""
    n, L = 24, 2
    params = C.hea_params(n, L, 5)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    picks = [0, 7, 29, 47, 50, 71, 88, 95]  # layer 0/1 x RY/RZ
    gate_of = {p: i for i, p in enumerate(pidx) if p >= 0}
    o = oracle.OracleDense(n, "c128")
    done, ps = 0, []
    for k in picks:
        g = gate_of[k]
        o.apply(circ[done:g])
        done = g
        base = o.state()
        kind, t, c, a = circ[g]
        ev = []
        for d in (math.pi / 2, -math.pi / 2):
            o.set_state(base)
            o.apply([(kind, t, c, a + d)] + circ[g + 1:])
            ev.append(o.pauli_expect(ham))
        ps.append(0.5 * (ev[0] - ev[1]))
        o.set_state(base)
    ps = np.array(ps)
    h = 1e-6
    ex = DenseGB300(n, "c128", exact_order=True)
    fd = []
    for k in picks:
        ev = []
        for d in (h, -h):
            p2 = params.copy()
            p2[k] += d
            ex.clear()
            ex.apply(C.hea(n, L, p2))
            ev.append(ex.exp_value(ham))
        fd.append((ev[0] - ev[1]) / (2 * h))
    fd = np.array(fd)
    # the finite differences themselves carry ~1e-10 of rounding (eps / h)
    assert np.max(np.abs(ps - fd)) < 1e-8
    for prec, fast, tol, tol_fd in (("c128", True, 1e-10, 1e-8), ("c128", False, 1e-10, 1e-8),
                                    ("c64", False, 1e-5, 1e-5)):
        sim = DenseGB300(n, prec, fast_c128=fast)
        _, grad = sim.adjoint_gradient(circ, pidx, len(params), ham)
        sim.close()
        gs = grad[picks]
        assert np.max(np.abs(gs - ps)) < tol, (prec, fast, np.max(np.abs(gs - ps)))
        assert np.max(np.abs(gs - fd)) < tol_fd, (prec, fast, np.max(np.abs(gs - fd)))


def test_adjoint_above_32_qubits_vs_finite_differences():
    # 33 qubits in complex64 (64 GiB per state: the state, lambda and one
    # checkpoint): gates on qubit 32 as targets (parameterised and diagonal),
    # as controls, and diagonal gates whose target lies outside every tile.
    # The energy must equal exp_value after the circuit, and the gradient of
    # the parameters on those gates central differences of exp_value (the
    # forward sweeps and reductions, independent of the reverse sweeps).
    import gc
    gc.collect()
    n, L = 33, 2
    params = C.hea_params(n, L, 11)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    k = len(params)
    extra = [(C.P, 32, (), 0.7), (C.RY, 5, (32,), -0.4), (C.RZ, 32, (3,), 1.1), (C.RX, 32, (), 0.3),
             (C.H, 32, (), 0.0), (C.RZ, 32, (), -0.9), (C.RY, 31, (), 0.5), (C.X, 0, (32,), 0.0)]
    checked = []
    for g in extra:
        circ.append(g)
        if g[0] in C.PARAMETRIC:
            pidx.append(k)
            checked.append((len(circ) - 1, k))
            k += 1
        else:
            pidx.append(-1)
    ham = C.tfim_ring(n) + [(0.6, [(C.PAULI_X, 32), (C.PAULI_Z, 0)]), (-0.3, [(C.PAULI_Z, 32)])]
    sim = DenseGB300(n, "c64")
    e, g = sim.adjoint_gradient(circ, pidx, k, ham, max_checkpoints=1)

    def energy(c):
        sim.clear()
        sim.apply(c)
        return sim.exp_value(ham)

    assert abs(e - energy(circ)) < 5e-5
    h = 5e-3
    for gi, p in checked[:4] + [(i, pidx[i]) for i in (0, 31, 32, 65) if pidx[i] >= 0][:3]:
        kind, t, c, a = circ[gi]
        plus, minus = list(circ), list(circ)
        plus[gi] = (kind, t, c, a + h)
        minus[gi] = (kind, t, c, a - h)
        fd = (energy(plus) - energy(minus)) / (2 * h)
        assert abs(g[p] - fd) < 2e-3, (gi, g[p], fd)
    sim.close()
    del sim
    gc.collect()
