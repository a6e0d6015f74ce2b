"""Benchmark of the dense state-vector hot path on GB300.

Workload (one step): the seeded 30-qubit random brickwork circuit, 20 layers
(600 one-qubit gates from {H,X,Y,Z,S,T,RX,RY,RZ} + 290 CNOTs), applied to the
resident complex128 state (16 GiB, far larger than the 129 MB L2, so no L2
flush is needed between steps).  The same circuit in complex64 is reported
as a secondary line item.

value: gate-equivalent GB/s = gates x (2 x 16 B x 2^30) / step time, i.e. the
bytes a one-gate-per-sweep engine (the reference Dense) would move.
roofline: the fused sweep kernel's algorithmic bytes per launch (one full
read + write of the state) over its CUDA-event-timed launch duration, against
the measured HBM copy bandwidth.
e2e: the same metric through the C ABI with host buffers: per step the state
is cleared, every gate is submitted by its own trait call, then <Z_i> for all
qubits and one full-register measurement (host draws) are read back.
Before the warm-up the engine's autotuner times the compiled tile sizes and
fusion depths on the circuit and keeps the fastest (config.tuning;
--no-tune keeps the defaults).  The fused sweeps apply ~50 gates each in
float-float arithmetic and are bound by FP32-pipe issue, not HBM, so the
roofline fraction of a fused launch is low while the step is fast; the
single_gate_sweep line shows the HBM roof of a one-gate sweep.

--impl reference: the reference's CPU Dense path as the restated Dense<f64>
(oracle/, OpenMP on every host core) on the same circuit: the timed steps
apply the whole 890-gate circuit once between them (--ref-gates G: G gates
per step instead), same metric and unit.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "30q gate GB/s vs HBM peak; adjoint vs param-shift grads/s at <=1e-5 err"


def load_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_port_rate(n, prec, gates, budget_s, threads=None):
    """Time the restated Dense<F> (oracle, OpenMP) on the first gates of the
    workload until `budget_s` of CPU work; returns (gate-eq GB/s, info)."""
    import oracle
    if threads:
        oracle.set_num_threads(threads)
    o = None
    for nn in (n, n - 1, n - 2):
        try:
            o = oracle.OracleDense(nn, prec)
            n_used = nn
            break
        except ValueError:
            continue
    if o is None:
        return None, {"sample": "host allocation failed"}
    B = 16 if prec == "c128" else 8
    done, t0 = 0, time.perf_counter()
    while done < len(gates):
        kind, t, c, a = gates[done]
        if t >= n_used or any(q >= n_used for q in c):
            done += 1
            continue
        o.gate(kind, t, c, a)
        done += 1
        if time.perf_counter() - t0 > budget_s and done >= 2:
            break
    dt = time.perf_counter() - t0
    rate = done * 2 * B * (1 << n_used) / dt / 1e9
    return rate, {"gates": done, "qubits": n_used, "seconds": round(dt, 3), "threads": oracle.num_threads()}


def run_reference(args, world, rank):
    """The reference's CPU Dense path, as the oracle port (the Rust crate
    cannot be built here), with every host thread, on the 30-qubit brickwork.
    By default the timed steps apply the whole circuit once between them
    (step s: the s-th of `steps` contiguous chunks, so every layer and the
    CNOT mix are in the rate); each warm-up step applies 4 gates.
    --ref-gates G instead applies G consecutive gates per step."""
    if rank != 0:
        return
    from kbw_gb300 import circuits as C
    import oracle
    n, prec = args.qubits, args.prec
    circ = C.brickwork(n, args.layers, 0)
    o = oracle.OracleDense(n, prec)
    B = 16 if prec == "c128" else 8
    pos = 0

    def apply(count):
        nonlocal pos
        for _ in range(count):
            kind, t, c, a = circ[pos % len(circ)]
            o.gate(kind, t, c, a)
            pos += 1

    for _ in range(args.warmup):
        apply(args.ref_gates or 4)
    if args.ref_gates:
        chunks = [args.ref_gates] * args.steps
    else:
        pos = 0
        chunks = [(s + 1) * len(circ) // args.steps - s * len(circ) // args.steps for s in range(args.steps)]
    t0 = time.perf_counter()
    for cnt in chunks:
        apply(cnt)
    dt = time.perf_counter() - t0
    total = sum(chunks)
    per_step = total / args.steps
    value = total * 2 * B * (1 << n) / dt / 1e9
    sample = ("%d gates per step of the %dq brickwork" % (args.ref_gates, n) if args.ref_gates else
              "the whole %dq brickwork (%d gates) once across the timed steps" % (n, total))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == "c128" else "f32", "data": "synthetic",
        "config": {"workload": "brickwork-%dq-%dlayers-%s" % (n, args.layers, prec), "qubits": n,
                   "layers": args.layers, "gates": len(circ), "precision": prec},
        "gates_per_step": round(per_step, 2),
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": oracle.num_threads(), "kind": "port",
                         "sample": sample + ", restated Dense<f64> (OpenMP)"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_steps(sim, circ, steps, warmup, torch):
    """CUDA-event time of `steps` circuit applications on the engine's stream."""
    for _ in range(warmup):
        sim.apply(circ)
        sim.flush()
    if warmup:
        # the warm-up started compiling the specialised sweep kernels: take them in
        sim.jit_wait()
        sim.apply(circ)
        sim.flush()
    ext = torch.cuda.ExternalStream(sim.stream_handle())
    sim.profile(True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        sim.apply(circ)
        sim.flush()
    e1.record(ext)
    torch.cuda.synchronize()
    nl, kms, kbytes = sim.profile_read()
    sim.profile(False)
    return e0.elapsed_time(e1) / steps, nl, kms, kbytes


def single_gate_sweep(sim, torch, peak, C, reps=5):
    """CUDA-event time of sweeps that each apply one RZ (the lightest full
    read + write of the state through the tile kernel)."""
    g = [(C.RZ, 3, (), 0.3)]
    sim.apply(g)
    sim.flush()
    sim.profile(True)
    torch.cuda.synchronize()
    for _ in range(reps):
        sim.apply(g)
        sim.flush()
    torch.cuda.synchronize()
    nl, kms, kbytes = sim.profile_read()
    sim.profile(False)
    ach = kbytes / (kms * 1e-3) / 1e9
    return {"achieved": round(ach, 1), "frac": round(ach / peak, 4), "unit": "GB/s",
            "avg_launch_ms": round(kms / max(nl, 1), 4), "launches": nl}


def run_adjoint_bench(args, torch, DenseGB300, C, grads):
    """Gradient half of the metric: 24 qubits, 10 layers of RY, RZ on every
    qubit + CZ ring (480 parameters), ring TFIM.  grads/s of the adjoint
    kernel vs the parameter-shift rule on the same GPU, plus the max
    gradient error of each precision against the binary64 adjoint."""
    n, L = args.adj_qubits, args.adj_layers
    params = C.hea_params(n, L, 0)
    circ = C.hea(n, L, params)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    npar = len(params)
    out = {"config": "hea-%dq-%dlayers-%dparams-tfim-ring" % (n, L, npar)}
    ref_g = None
    # binary64 first: its gradient is the reference for the error columns
    for label, prec, fast in (("c128_binary64", "c128", False), ("c64", "c64", False), ("c128_ff", "c128", True)):
        sim = DenseGB300(n, prec, fast_c128=fast)
        # warm-up: the second call starts compiling the forward segments'
        # specialised kernels; wait, then once more to take them in
        sim.adjoint_gradient(circ, pidx, npar, ham)
        sim.adjoint_gradient(circ, pidx, npar, ham)
        sim.jit_wait()
        sim.adjoint_gradient(circ, pidx, npar, ham)
        torch.cuda.synchronize()
        reps = 1 if label == "c128_binary64" else args.adj_reps
        t0 = time.perf_counter()
        for _ in range(reps):
            e, g = sim.adjoint_gradient(circ, pidx, npar, ham)
        torch.cuda.synchronize()
        ta = (time.perf_counter() - t0) / reps
        item = {"energy": e, "adjoint_s": round(ta, 5), "adjoint_grads_per_s": round(npar / ta, 1)}
        if ref_g is None:
            ref_g = g
        else:
            item["max_grad_err_vs_binary64_adjoint"] = float(np.max(np.abs(g - ref_g)))
        if label == "c64" or (label == "c128_ff" and args.adj_ps_c128):
            # the shifted circuits share the circuit's structure: compile its
            # specialised kernels before timing, as for the adjoint
            for _ in range(2):
                sim.apply(circ)
                sim.flush()
            sim.jit_wait()
            sim.clear()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e_ps, g_ps = sim.param_shift_gradient(circ, pidx, npar, ham)
            torch.cuda.synchronize()
            tp = time.perf_counter() - t0
            item.update({"param_shift_s": round(tp, 4), "param_shift_grads_per_s": round(npar / tp, 2),
                         "speedup_adjoint_vs_param_shift": round(tp / ta, 1),
                         "max_grad_err_vs_param_shift": float(np.max(np.abs(g - g_ps)))})
        out[label] = item
        grads[label] = g
        sim.close()
    return out


def run_adjoint_large(args, torch, DenseGB300, C):
    """Large adjoint gradient: 32 qubits in complex64 (32 GiB per state; the
    state, lambda and one checkpoint), 6 layers of RY, RZ + CZ ring (384
    parameters), ring TFIM.  Its error is stated on a 28-qubit replica of the
    same structure: complex64 against the complex128 (float-float) adjoint."""
    n, L = args.adj_large_qubits, 6
    params = C.hea_params(n, L, 0)
    circ, pidx, ham = C.hea(n, L, params), C.hea_param_index(n, L), C.tfim_ring(n)
    sim = DenseGB300(n, "c64")
    # untimed warm-up, as for the 24-qubit line: the second call of each
    # sweep structure starts its background compilation, jit_wait lets it
    # finish, and the timed call runs the specialised kernels
    for _ in range(2):
        sim.adjoint_gradient(circ, pidx, len(params), ham, max_checkpoints=1)
    sim.jit_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e, g = sim.adjoint_gradient(circ, pidx, len(params), ham, max_checkpoints=1)
    torch.cuda.synchronize()
    ta = time.perf_counter() - t0
    specialised = sim.jit_info()["last_specialised"] > 0
    sim.close()
    del sim
    nr = min(28, n)
    pr = C.hea_params(nr, L, 0)
    cr, ir, hr = C.hea(nr, L, pr), C.hea_param_index(nr, L), C.tfim_ring(nr)
    res = {}
    for label, prec, fast in (("c64", "c64", False), ("c128_ff", "c128", True)):
        r = DenseGB300(nr, prec, fast_c128=fast)
        res[label] = r.adjoint_gradient(cr, ir, len(pr), hr)
        r.close()
    return {"config": "hea-%dq-%dlayers-%dparams-tfim-ring c64" % (n, L, len(params)), "energy": e,
            "adjoint_s": round(ta, 3), "adjoint_grads_per_s": round(len(params) / ta, 1),
            "specialised_kernels": specialised,
            "state_gib": (8 << n) >> 30, "buffers": "state + lambda + 1 checkpoint",
            "replica": {"qubits": nr, "max_grad_err_c64_vs_c128": float(np.max(np.abs(res["c64"][1] -
                                                                                        res["c128_ff"][1]))),
                        "abs_dE_c64_vs_c128": abs(res["c64"][0] - res["c128_ff"][0])}}


def run_grover_bench(args, torch, DenseGB300, C):
    """The reference's CPU-runnable case: plain Grover search, 12 qubits,
    complex128, 50 iterations (2,962 gates), marked index seeded in
    [0, 4096); output the probability vector (dump of all qubits) and 1024
    samples from injected draws.  Latency-bound: wall time per run through the
    C ABI against the restated Dense<f64> on the host, and the success
    probability against its closed form."""
    import oracle
    n, it, seeds = 12, 50, 10
    sim = DenseGB300(n, "c128", fast_c128=True)
    qs = list(range(n))[::-1]  # dump packs qubits[0] as the most significant bit: natural index order

    # the workload (gate lists, draws) is generated before any timing; a run
    # is the calls a host makes: clear, the gate list, dump, sample
    marks = [C.grover_marked(sd) for sd in range(seeds)]
    circs = [C.grover(n, m, it) for m in marks]
    draws = [C.uniform_draws(1024, sd) for sd in range(seeds)]

    def run(target, seed):
        target.clear()
        target.apply(circs[seed])
        st, re, im = target.dump(qs)
        hist = target.sample(qs, 1024, draws[seed])
        p = float(np.sum((re * re + im * im)[st == marks[seed]]))
        return p, hist

    # tile size and fusion depth for this register, tuned once on one of the
    # circuits (the setting stays with the handle for the others)
    tuning = rounded(sim.autotune(circs[0], reps=2))
    run(sim, 0)
    run(sim, 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = [run(sim, sd) for sd in range(seeds)]
    torch.cuda.synchronize()
    t_gpu = (time.perf_counter() - t0) / seeds
    o = oracle.OracleDense(n, "c128")
    t0 = time.perf_counter()
    ref = [run(o, sd) for sd in range(2)]
    t_cpu = (time.perf_counter() - t0) / 2
    same = all(np.array_equal(res[i][1][0], ref[i][1][0]) and np.array_equal(res[i][1][1], ref[i][1][1])
               for i in range(2))
    sim.close()
    return {"config": "grover-12q-50it-c128 (probabilities + 1024 samples)", "ms_per_run": round(t_gpu * 1e3, 3),
            "cpu_port_ms_per_run": round(t_cpu * 1e3, 3), "cpu_threads": oracle.num_threads(),
            "success_probability": res[0][0], "closed_form": C.grover_success_probability(n, it),
            "samples_identical_to_oracle": bool(same), "tuning": tuning}


def run_gate_classes(args):
    """Per gate class: CUDA-event time of the sweeps that apply 32 gates of
    one class (first row: a single RZ, the memory-pass floor of a sweep);
    us_per_gate = sweep time / gates, once with the interpreted sweep kernel
    and once with the sweep's run-time-specialised kernel.  Runs of diagonal
    gates are not folded here, so each of the 32 gates is applied."""
    from kbw_gb300 import DenseGB300
    from kbw_gb300 import _native as N
    from kbw_gb300 import circuits as C
    n, prec = args.qubits, args.prec
    sim = DenseGB300(n, prec, fast_c128=(prec == "c128" and args.arith == "ff"), fold=False)
    cases = [("one RZ (memory pass)", [(C.RZ, 3, (), 0.3)]),
             ("32 RY on a register qubit", [(C.RY, 8, (), 0.1 * i) for i in range(32)]),
             ("32 RX on a register qubit", [(C.RX, 8, (), 0.1 * i) for i in range(32)]),
             ("32 H on qubits 6..9", [(C.H, 6 + i % 4, (), 0.0) for i in range(32)]),
             ("32 RZ on a register qubit", [(C.RZ, 8, (), 0.1 * i) for i in range(32)]),
             ("32 P on a register qubit", [(C.P, 8, (), 0.1 * i) for i in range(32)]),
             ("32 Z on a register qubit", [(C.Z, 8, (), 0.0)] * 32),
             ("32 X on a lane qubit", [(C.X, 2, (), 0.0)] * 32),
             ("32 RY on a lane qubit", [(C.RY, 2, (), 0.1 * i) for i in range(32)]),
             ("32 CNOT 7->8 (register control)", [(C.X, 8, (7,), 0.0)] * 32),
             ("brickwork 13 qubits, 3 layers", C.brickwork(13, 3, 0))]
    out = []
    for name, circ in cases:
        row = {"case": name, "gates": len(circ)}
        for mode, jit in (("interpreted", N.JIT_OFF), ("specialised", N.JIT_ALWAYS)):
            sim.set_jit(jit)
            sim.apply(circ)
            sim.flush()
            sim.jit_wait()
            sim.profile(True)
            for _ in range(3):
                sim.apply(circ)
                sim.flush()
            nl, ms, b = sim.profile_read()
            sim.profile(False)
            row["sweeps"] = nl // 3
            row[mode] = {"ms_per_rep": round(ms / 3, 4), "us_per_gate": round(1000 * ms / 3 / len(circ), 3),
                         "specialised_sweeps": sim.jit_info()["last_specialised"]}
        out.append(row)
    sim.close()
    return out


def run_batch_bench(args, torch, C):
    """Batched forward: 4096 hardware-efficient-ansatz circuits (n ~ U{8..20},
    L ~ U{2..8}) in one persistent launch; circuits/s and the max |dE| of the
    complex64 energies against the complex128 oracle on a sample."""
    import oracle
    from kbw_gb300 import batch_hea_tfim
    circs = C.hea_batch(args.batch_circuits, seed=0)
    batch_hea_tfim(circs[:64], prec="c64")  # warm-up
    times = []
    for _ in range(args.batch_reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = batch_hea_tfim(circs, prec="c64")
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t = min(times)
    rng = np.random.default_rng(1)
    small = [i for i, c in enumerate(circs) if c[0] <= 14]
    sample = list(rng.choice(small, size=min(24, len(small)), replace=False))
    sample += [i for i, c in enumerate(circs) if c[0] >= 19][:2]
    err = 0.0
    ref = {}
    for i in sample:
        n, L, p = circs[i]
        o = oracle.OracleDense(n, "c128")
        o.apply(C.hea(n, L, p))
        ref[i] = o.exp_value(C.tfim_ring(n))
        err = max(err, abs(e[i] - ref[i]))
    # the same workload through the general single-launch entry (each circuit
    # its own gate list and Pauli-string Hamiltonian), complex64
    from kbw_gb300.dense import batch_circuits_prepare, batch_circuits_run
    # (the C arrays are built once, as a C or Rust caller holds them; the
    # timed call plans every circuit on the host, copies and launches)
    packed = batch_circuits_prepare([(n, C.hea(n, L, p), C.tfim_ring(n)) for n, L, p in circs])
    batch_circuits_run(batch_circuits_prepare([(n, C.hea(n, L, p), C.tfim_ring(n)) for n, L, p in circs[:64]]),
                       prec="c64")  # warm-up
    gtimes = []
    for _ in range(args.batch_reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eg = batch_circuits_run(packed, prec="c64")
        torch.cuda.synchronize()
        gtimes.append(time.perf_counter() - t0)
    tg = min(gtimes)
    gerr = max(abs(eg[i] - ref[i]) for i in sample)
    general_line = {"seconds": round(tg, 5), "circuits_per_s": round(len(circs) / tg, 1),
                    "max_abs_dE_vs_c128_oracle": gerr,
                    "entry": "kbwg_batch_circuits_exp_value (gates and Hamiltonian per circuit as C arrays; "
                             "the time includes planning every circuit on the host and host<->device copies)"}
    return {"general": general_line,
            "circuits": len(circs), "seconds": round(t, 5), "circuits_per_s": round(len(circs) / t, 1),
            "max_abs_dE_vs_c128_oracle": err, "checked": len(sample), "precision": "c64",
            "config": "hea-batch n~U{8..20} L~U{2..8} ring-TFIM, one persistent launch (incl. host<->device copies)"}


# ---- parity against the oracle at the benchmark's own sizes ----------------------------
# The oracle (oracle/, a C restatement of kbw Dense<f64>) is the checker here,
# run on the host beside the GPU work and never timed: the 30-qubit brickwork
# state, its <Z_q> and one full measurement with injected draws, and
# parameter-shift gradients of the 24-qubit ansatz at a spread of parameters.
PARITY_PARAMS = 24


def run_wide_register(args, torch, DenseGB300, C, peak):
    """Past Dense's 32 qubits: the brickwork on 33 qubits in complex128
    float-float (128 GiB of amplitudes, 64-bit state indices), CUDA-event
    time per step and per sweep against the HBM roofline."""
    n, layers = 33, args.layers
    circ = C.brickwork(n, layers, 0)
    sim = DenseGB300(n, "c128", fast_c128=True)
    ms, nl, kms, kb = time_steps(sim, circ, 2, 2, torch)
    passes = sim.last_flush_stats()[1]
    sim.close()
    ach = kb / (kms * 1e-3) / 1e9
    return {"config": "brickwork-%dq-%dlayers-c128 (float-float)" % (n, layers), "gates": len(circ),
            "state_gib": (16 << n) >> 30, "ms_per_step": round(ms, 2), "sweeps_per_step": passes,
            "value": round(len(circ) * 2 * 16 * (1 << n) / (ms * 1e-3) / 1e9, 1), "unit": "GB/s",
            "roofline": {"achieved": round(ach, 1), "frac": round(ach / peak, 4),
                         "avg_launch_ms": round(kms / max(nl, 1), 3)}}


def parity_param_picks(n, layers, count=PARITY_PARAMS):
    """`count` parameters of the hardware-efficient ansatz spread over every
    layer, alternating RY and RZ, on varying qubits."""
    picks = set()
    for j in range(count):
        layer = (j * layers) // count
        picks.add(layer * 2 * n + (j % 2) * n + (7 * j) % n)
    return sorted(picks)


class OracleParity(threading.Thread):
    def __init__(self, args, C, circ30, n30):
        super().__init__(daemon=True)
        self.args, self.C, self.circ30, self.n30 = args, C, circ30, n30
        self.result = {}
        self.error = None

    def run(self):
        try:
            import oracle
            oracle.set_num_threads(max(1, (os.cpu_count() or 4) - 2))  # two cores stay with the GPU host work
            C = self.C
            t0 = time.perf_counter()
            # 24-qubit gradient: oracle parameter shift at the picked parameters
            n, L = self.args.adj_qubits, self.args.adj_layers
            params = C.hea_params(n, L, 0)
            circ = C.hea(n, L, params)
            pidx = C.hea_param_index(n, L)
            ham = C.tfim_ring(n)
            gate_of = {p: i for i, p in enumerate(pidx) if p >= 0}
            picks = parity_param_picks(n, L)
            o = oracle.OracleDense(n, "c128")
            done = 0  # o holds circ[:done]
            ps = []
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
                ps.append((ev[0] - ev[1]) / 2)
                o.set_state(base)
            del o
            self.result["grad"] = {"picks": picks, "param_shift": ps, "seconds": time.perf_counter() - t0}
            # 30-qubit brickwork from |0>
            t0 = time.perf_counter()
            n = self.n30
            o = oracle.OracleDense(n, "c128")
            o.apply(self.circ30)
            self.result["z"] = o.z_all()
            self.result["state"] = o.state()
            draws = C.uniform_draws(n, 7)
            self.result["bits"] = o.measure(list(range(n)), draws)
            self.result["draws"] = draws
            self.result["seconds30"] = time.perf_counter() - t0
            del o
        except Exception as e:  # reported in the bench line
            self.error = repr(e)


def parity_report(chk, args, torch, DenseGB300, C, circ30, n30, grads):
    """GPU side of the parity checks, after the timed work: the oracle's
    30-qubit state is uploaded to a handle and compared on the device."""
    if chk is None:
        return None
    chk.join()
    import oracle
    oracle.set_num_threads(os.cpu_count() or 1)
    if chk.error:
        return {"error": chk.error}
    r = chk.result
    out = {"checker": "oracle (restated Dense<f64>, OpenMP, %d threads)" % max(1, (os.cpu_count() or 4) - 2)}
    # ---- 30-qubit brickwork ----
    ref = DenseGB300(n30, "c128")
    ref.set_state(r.pop("state"))
    ff = DenseGB300(n30, "c128", fast_c128=True)
    ff.apply(circ30)
    s64 = DenseGB300(n30, "c64")
    s64.apply(circ30)
    zs = [[(1.0, [(C.PAULI_Z, q)])] for q in range(n30)]
    z_ff = np.array([ff.exp_value(h) for h in zs])
    z_64 = np.array([s64.exp_value(h) for h in zs])
    bits_ff = ff.measure(list(range(n30)), r["draws"])
    bits_64 = s64.measure(list(range(n30)), r["draws"])
    ff.close()
    s64.close()
    ff = DenseGB300(n30, "c128", fast_c128=True)
    ff.apply(circ30)
    rel = ff.distance(ref)
    ff.close()
    s64 = DenseGB300(n30, "c64")
    s64.apply(circ30)
    infid = 1.0 - s64.fidelity(ref)
    s64.close()
    ref.close()
    out["brickwork_30q"] = {
        "float_float_relative_l2": rel, "c64_infidelity": infid,
        "max_abs_dZ_float_float": float(np.max(np.abs(z_ff - r["z"]))),
        "max_abs_dZ_c64": float(np.max(np.abs(z_64 - r["z"]))),
        "measurement_equal_float_float": bits_ff == r["bits"], "measurement_equal_c64": bits_64 == r["bits"],
        "oracle_seconds": round(r["seconds30"], 1),
        "bar": "relative L2 <= 1e-12 (complex128); outcomes equal for the same draws"}
    # ---- 24-qubit gradient ----
    g = r["grad"]
    picks = g["picks"]
    ps = np.array(g["param_shift"])
    n, L = args.adj_qubits, args.adj_layers
    params = C.hea_params(n, L, 0)
    pidx = C.hea_param_index(n, L)
    ham = C.tfim_ring(n)
    # central differences, h = 1e-6, on the engine's order-preserving binary64
    # path (the restated Dense<f64> arithmetic, bit for bit)
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
    ex.close()
    fd = np.array(fd)
    item = {"params_checked": len(picks), "layers_covered": len({k // (2 * n) for k in picks}),
            "oracle_param_shift_seconds": round(g["seconds"], 1),
            "fd_h": h, "max_abs_ps_minus_fd": float(np.max(np.abs(ps - fd)))}
    for label, gv in grads.items():
        gs = np.asarray(gv)[picks]
        item[label] = {"max_abs_err_vs_oracle_param_shift": float(np.max(np.abs(gs - ps))),
                       "max_abs_err_vs_central_fd": float(np.max(np.abs(gs - fd)))}
    item["bar"] = ("vs oracle parameter shift <= 1e-10 (complex128), <= 1e-5 (complex64); central differences "
                   "carry their own ~1e-10 error (eps/h), shown as max_abs_ps_minus_fd")
    out["adjoint_24q"] = item
    return out



def rounded(d, digits=3):
    return {k: round(v, digits) if isinstance(v, float) else v for k, v in d.items()}


def run_ours(args, world, rank, local):
    import torch
    import kbw_gb300
    from kbw_gb300 import DenseGB300
    from kbw_gb300 import circuits as C
    from kbw_gb300 import _native as N

    kbw_gb300.load()
    torch.cuda.set_device(local)
    N.select_device(local)
    n, prec = args.qubits, args.prec
    fast = prec == "c128" and args.arith == "ff"
    B = 16 if prec == "c128" else 8
    circ = C.brickwork(n, args.layers, 0)
    G = len(circ)
    step_bytes = G * 2 * B * (1 << n)
    peak, peak_kind = load_peaks()

    # CPU baseline first, on an idle host; then the oracle checker starts
    # beside the GPU work (it never overlaps a CPU timing)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, info = cpu_port_rate(n, prec, circ, args.cpu_seconds)
        if rate is not None:
            cpu = {"value": round(rate, 3), "unit": "GB/s", "cores": info.get("threads"), "kind": "port",
                   "sample": "first %d gates of the %dq brickwork on the restated Dense<%s> (OpenMP), %.1f s"
                             % (info["gates"], info["qubits"], "f64" if prec == "c128" else "f32", info["seconds"])}
    checker = None
    adj_grads = {}
    if rank == 0 and world == 1 and args.parity and prec == "c128" and fast:
        checker = OracleParity(args, C, circ, n)
        checker.start()

    sim = DenseGB300(n, prec, fast_c128=fast)
    ext = torch.cuda.ExternalStream(sim.stream_handle())
    # tile size and fusion depth picked by the engine's autotuner on this
    # circuit (before the warm-up; the handle's state is left unchanged)
    tuning = rounded(sim.autotune(circ, reps=1) if args.tune else sim.tuning())

    def step():
        sim.apply(circ)
        sim.flush()

    for _ in range(args.warmup):
        step()
    # specialised sweep kernels compiled in the background during warm-up
    # (the tuner already waited for those of the chosen settings)
    sim.jit_wait()
    step()
    _, passes = sim.last_flush_stats()
    specialised = sim.jit_info()["last_specialised"]
    sim.profile(True)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    barrier(world)
    l0 = N.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(args.steps):
        step()
    e1.record(ext)
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    launches = N.launch_count() - l0
    clk = clocks.stop()
    nl, kms, kbytes = sim.profile_read()
    sim.profile(False)
    ms = max_over_ranks(world, ms)
    ms_step = ms / args.steps
    value = world * step_bytes / (ms_step * 1e-3) / 1e9

    achieved = kbytes / (kms * 1e-3) / 1e9 if kms > 0 else None
    # DRAM bytes per launch: ncu dram__bytes_read.sum + dram__bytes_write.sum of
    # one k_sweep<FF2> launch on the 25-qubit brickwork (1017.4 MB), scaled to
    # 2^n amplitudes (traffic grows with the state; one read + write each)
    traffic = args.traffic
    if traffic is None and fast:
        traffic = round(1017.4e6 * (1 << n) / (1 << 25))
    pol = {"c64": "FastP", "c128": "FF2" if fast else "Fast<double>"}[prec]
    kname = ("kbwg_jit_sweep (%s, one specialised kernel per sweep)" % pol if specialised == passes
             else "k_sweep<%s>" % pol)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None, "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                "traffic": traffic, "kernel": kname, "launches": nl,
                "avg_launch_ms": round(kms / max(nl, 1), 4), "peak_source": peak_kind + " hbm_gbs (burst copy)"}

    # one gate per sweep: the bandwidth of plain gate application, the bar a
    # one-gate-per-pass engine is held to (fusion then packs ~25 gates a sweep)
    single = single_gate_sweep(sim, torch, peak, C)

    # ---- e2e through the C ABI, host buffers ----
    zs = [(1.0, [(C.PAULI_Z, q)]) for q in range(n)]
    calls = {C.X: sim.pauli_x, C.Y: sim.pauli_y, C.Z: sim.pauli_z, C.H: sim.hadamard,
             C.P: sim.phase, C.RX: sim.rx, C.RY: sim.ry, C.RZ: sim.rz}

    def e2e_step(seed):
        sim.clear()
        for kind, t, c, a in circ:
            if kind in C.PARAMETRIC:
                calls[kind](a, t, c)
            else:
                calls[kind](t, c)
        ez = sim.exp_value(zs)
        bits = sim.measure(list(range(n)), C.uniform_draws(n, seed))
        return ez, bits

    e2e_step(0)
    torch.cuda.synchronize()
    h0, d0 = N.transfer_bytes()
    t0 = time.perf_counter()
    for s in range(args.e2e_steps):
        e2e_step(s + 1)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, (time.perf_counter() - t0) / args.e2e_steps)
    h1, d1 = N.transfer_bytes()
    e2e = {"value": round(world * step_bytes / e2e_s / 1e9, 1), "unit": "GB/s",
           "h2d_bytes_per_step": (h1 - h0) // args.e2e_steps, "d2h_bytes_per_step": (d1 - d0) // args.e2e_steps,
           "ms_per_step": round(e2e_s * 1e3, 2),
           "calls": "clear + %d gate calls + exp_value(%d Z_i) + measure(%d qubits)" % (G, n, n)}

    secondary = {}
    if args.secondary and prec == "c128":
        # parity of the headline arithmetic at full size: one circuit from |0>
        # in float-float and in binary64, compared on the device
        exact = DenseGB300(n, "c128")
        exact.apply(circ)
        exact.flush()
        if fast:
            sim.clear()
            sim.apply(circ)
            sim.flush()
            secondary["parity_vs_binary64"] = {"relative_l2": sim.distance(exact),
                                               "circuit": "one application from |0>"}
        sim.close()
        del sim
        # complex64 error statement: state infidelity of one application of
        # the circuit against the binary64 complex128 one, on the device
        s64 = DenseGB300(n, "c64")
        s64.apply(circ)
        infid64 = 1.0 - s64.fidelity(exact)
        ms_x, nlx, kmsx, kbx = time_steps(exact, circ, min(args.steps, 3), 1, torch)
        achx = kbx / (kmsx * 1e-3) / 1e9
        secondary["c128_binary64"] = {"value": round(step_bytes / (ms_x * 1e-3) / 1e9, 1), "unit": "GB/s",
                                      "ms_per_step": round(ms_x, 2), "dtype": "f64",
                                      "steps": min(args.steps, 3), "warmup": 2,
                                      "roofline": {"achieved": round(achx, 1), "frac": round(achx / peak, 4),
                                                   "avg_launch_ms": round(kmsx / max(nlx, 1), 3)},
                                      "note": "IEEE binary64 gate arithmetic: FP64-issue bound on GB300"}
        exact.close()
        s64.clear()
        tuning64 = rounded(s64.autotune(circ, reps=1) if args.tune else s64.tuning())
        ms64, nl64, kms64, kb64 = time_steps(s64, circ, args.steps, 2, torch)
        ach64 = kb64 / (kms64 * 1e-3) / 1e9
        sweeps64 = s64.last_flush_stats()[1]
        single64 = single_gate_sweep(s64, torch, peak, C)
        secondary["c64"] = {"value": round(G * 2 * 8 * (1 << n) / (ms64 * 1e-3) / 1e9, 1), "unit": "GB/s",
                            "ms_per_step": round(ms64, 3), "sweeps_per_step": sweeps64,
                            "dtype": "f32",
                            "roofline": {"achieved": round(ach64, 1), "frac": round(ach64 / peak, 4),
                                         "avg_launch_ms": round(kms64 / max(nl64, 1), 4)},
                            "single_gate_sweep": single64, "tuning": tuning64,
                            "state_infidelity_vs_c128": infid64}
        s64.close()
    else:
        sim.close()

    if args.adjoint:
        secondary["adjoint"] = run_adjoint_bench(args, torch, DenseGB300, C, adj_grads)
    if args.adjoint_large:
        secondary["adjoint_large"] = run_adjoint_large(args, torch, DenseGB300, C)
    if args.wide and rank == 0:
        secondary["register_33q"] = run_wide_register(args, torch, DenseGB300, C, peak)
    # (joined before the batch and Grover items, which run the oracle on the host)
    if checker is not None:
        secondary["parity_vs_oracle"] = parity_report(checker, args, torch, DenseGB300, C, circ, n, adj_grads)
    if args.batch:
        secondary["batch"] = run_batch_bench(args, torch, C)
    if args.grover:
        secondary["grover"] = run_grover_bench(args, torch, DenseGB300, C)


    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32x2 (float-float; binary64 at the API)" if fast else ("f64" if prec == "c128" else "f32"),
            "data": "synthetic: seeded random brickwork circuit (numpy default_rng(0))",
            "config": {"workload": "brickwork-%dq-%dlayers-%s" % (n, args.layers, prec), "qubits": n,
                       "layers": args.layers, "gates": G, "precision": prec,
                       "arithmetic": "float-float" if fast else "native", "sweeps_per_step": passes,
                       "l2": "state %d GiB > 129 MB L2; no flush needed" % ((B << n) >> 30),
                       "parallelism": "replicas" if world > 1 else "single", "tuning": tuning},
            "sweep_gbs": round(world * passes * 2 * B * (1 << n) / (ms_step * 1e-3) / 1e9, 1),
            "gpu_launches": launches,
            "roofline": roofline, "single_gate_sweep": single, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        }
        line.update(secondary)
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--prec", choices=["c64", "c128"], default="c128")
    ap.add_argument("--arith", choices=["ff", "exact"], default="ff",
                    help="complex128 gate arithmetic: float-float (default) or IEEE binary64")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-wide", dest="wide", action="store_false",
                    help="skip the 33-qubit (128 GiB) register line")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the oracle parity checks at the benchmark sizes (30q state, 24q gradients)")
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="keep the default tile size and fusion depth instead of autotuning them")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-gates", type=int, default=0,
                    help="reference arm: gates per step (0: the whole circuit across the timed steps)")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false")
    ap.add_argument("--no-batch", dest="batch", action="store_false")
    ap.add_argument("--no-adjoint-large", dest="adjoint_large", action="store_false")
    ap.add_argument("--no-grover", dest="grover", action="store_false")
    ap.add_argument("--gate-classes", action="store_true",
                    help="instead of the benchmark: per gate class sweep times on --qubits/--prec/--arith")
    ap.add_argument("--adj-large-qubits", type=int, default=32)
    ap.add_argument("--batch-circuits", type=int, default=4096)
    ap.add_argument("--batch-reps", type=int, default=3)
    ap.add_argument("--adj-qubits", type=int, default=24)
    ap.add_argument("--adj-layers", type=int, default=10)
    ap.add_argument("--adj-reps", type=int, default=3)
    ap.add_argument("--no-adj-ps-c128", dest="adj_ps_c128", action="store_false",
                    help="skip the float-float complex128 parameter-shift timing")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu DRAM bytes (read + write) per sweep launch; default: the 25-qubit capture "
                         "of k_sweep<FF2> (1017.4 MB) scaled by the amplitude count")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.gate_classes:
        import kbw_gb300
        kbw_gb300.load()
        for row in run_gate_classes(args):
            print(json.dumps(row), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
