"""torch.autograd bindings of the device adjoints.

ADFLoss:   0.5 * ||P_Omega(x) - y||^2 of a TT x at sampled positions
           (the loss whose projected gradient ADF follows, src/xerus/algorithms/adf.cpp:359-396)
ALSEnergy: <x, A x> - 2 <x, b> for a symmetric TT operator A
           (the functional ALS_SPD minimises, src/xerus/algorithms/als.cpp:265-278)

Both take the cores of x as torch tensors (float64, any device) and return a
scalar; backward returns the gradient for every core, computed on the GPU by
libxtt (xtt_adf_gradient / xtt_als_energy_gradient) in the forward pass.
"""
import numpy as np
import torch

from . import ADFVariant, SinglePointMeasurementSet, TTOperator, TTTensor, als_energy_gradient


def _tt(cores, ctx):
    hc = [c.detach().to("cpu", torch.float64).numpy() for c in cores]
    return TTTensor.from_cores(hc, ctx=ctx)


class ADFLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, values, *cores):
        x = _tt(cores, None)
        m = SinglePointMeasurementSet(np.asarray(positions.cpu(), dtype=np.int64),
                                      np.asarray(values.detach().cpu(), dtype=np.float64))
        loss, grads = ADFVariant.gradient(x, m)
        ctx.grads = [torch.from_numpy(g).to(c.device) for g, c in zip(grads, cores)]
        return torch.tensor(loss, dtype=torch.float64, device=cores[0].device)

    @staticmethod
    def backward(ctx, grad_out):
        return (None, None, *[grad_out * g for g in ctx.grads])


class ALSEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, b, *cores):
        """A: TTOperator, b: TTTensor (device objects); cores: the cores of x."""
        x = _tt(cores, A.ctx)
        J, grads = als_energy_gradient(A, x, b)
        ctx.grads = [torch.from_numpy(g).to(c.device) for g, c in zip(grads, cores)]
        return torch.tensor(J, dtype=torch.float64, device=cores[0].device)

    @staticmethod
    def backward(ctx, grad_out):
        return (None, None, *[grad_out * g for g in ctx.grads])


def adf_loss(positions, values, cores):
    return ADFLoss.apply(positions, values, *cores)


def als_energy(A: TTOperator, b: TTTensor, cores):
    return ALSEnergy.apply(A, b, *cores)
