"""torch.autograd bridge for the adjoint gradient (thin test shim).

``adjoint_energy(params, sim, build, hamiltonian)`` returns E(params) as a
0-dim tensor whose backward uses the gradient computed by the engine's
reverse-mode adjoint kernel in the same call.  ``build(params_numpy)`` must
return ``(circuit, param_index)``.
"""
import numpy as np
import torch


class AdjointEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, sim, build, hamiltonian, max_checkpoints):
        circuit, param_index = build(params.detach().cpu().numpy().astype(np.float64))
        energy, grad = sim.adjoint_gradient(circuit, param_index, params.numel(), hamiltonian, max_checkpoints)
        ctx.save_for_backward(torch.as_tensor(grad, dtype=params.dtype))
        return params.new_tensor(energy)

    @staticmethod
    def backward(ctx, grad_output):
        (grad,) = ctx.saved_tensors
        return grad_output * grad.to(grad_output.device), None, None, None, None


def adjoint_energy(params, sim, build, hamiltonian, max_checkpoints=16):
    return AdjointEnergy.apply(params, sim, build, hamiltonian, max_checkpoints)
