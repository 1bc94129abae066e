"""Adjoint-method gradients behind a torch.autograd.Function.

    import torch, adjoint, workloads
    circ = adjoint.AdjointCircuit(20, workloads.hea_ansatz(20, 10), nparams=400,
                                  observable=llgpu.ring_zz_terms(20), max_batch=64)
    theta = torch.rand(64, 400, dtype=torch.float64, device="cuda", requires_grad=True)
    energy = circ(theta)            # [64] expectation values, complex128 state vectors on the GPU
    energy.sum().backward()         # theta.grad from one forward + one reverse sweep

The forward call runs the GPU forward sweep and, when the parameters require gradients, the
reverse (adjoint) sweep in the same native call, so the states never leave HBM; backward()
scales the stored gradients by the incoming gradient.  Parameters and results stay on the
device (the engine reads and writes the tensors' memory directly).
"""
from __future__ import annotations

import numpy as np

import llgpu


class _CircuitEnergy:
    """Builds the autograd.Function lazily so importing this module does not import torch."""

    _fn = None

    @classmethod
    def get(cls):
        if cls._fn is None:
            import torch

            class CircuitEnergy(torch.autograd.Function):
                @staticmethod
                def forward(ctx, theta, circuit, checkpoint_every):
                    if theta.dtype != torch.float64 or not theta.is_cuda:
                        raise TypeError("theta must be a float64 CUDA tensor")
                    theta_c = theta.detach().contiguous()
                    batch = theta_c.shape[0]
                    energies = torch.empty(batch, dtype=torch.float64, device=theta.device)
                    need = theta.requires_grad
                    grads = torch.empty_like(theta_c) if need else None
                    # order the engine's stream after torch's producers of theta
                    torch.cuda.current_stream().synchronize()
                    circuit.handle.run_device(theta_c.data_ptr(), batch, energies.data_ptr(),
                                              grads.data_ptr() if need else None, checkpoint_every)
                    if need:
                        ctx.save_for_backward(grads)
                    return energies

                @staticmethod
                def backward(ctx, grad_energy):
                    (grads,) = ctx.saved_tensors
                    return grad_energy[:, None] * grads, None, None

            cls._fn = CircuitEnergy
        return cls._fn


class AdjointCircuit:
    """A parametrised circuit whose energies are differentiable torch functions of theta."""

    def __init__(self, n: int, ops: np.ndarray, nparams: int, observable, max_batch: int = 64,
                 precision: str = "complex128", checkpoint_every: int = 0):
        self.handle = llgpu.Adjoint(n, ops, nparams, observable, max_batch, precision)
        self.checkpoint_every = checkpoint_every

    def __call__(self, theta):
        return _CircuitEnergy.get().apply(theta, self, self.checkpoint_every)

    def param_shift(self, theta: np.ndarray):
        """Energies and gradients by the parameter-shift rule (the reference's method), on the GPU."""
        return self.handle.param_shift(theta)
