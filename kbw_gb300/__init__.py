"""GB300 dense state-vector engine: a drop-in backend for the Ket Bitwise
Simulator's dense path (kbw ``Dense``/``DenseV2``), as CUDA kernels for
sm_103a behind the C ABI of include/kbwg.h.

``DenseGB300`` mirrors the reference's ``QuantumExecution`` trait; the
workload generators live in ``kbw_gb300.circuits``.
"""
from .dense import (DenseGB300, batch_circuits_exp_value, batch_exp_value, batch_gradient, batch_hea_tfim, batch_release,  # noqa: F401
                    batch_sample, plan)
from ._native import KbwgError, build_info, launch_count, load  # noqa: F401
