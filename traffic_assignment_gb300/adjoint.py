"""dVHT/dcapacity through a fixed number of Frank-Wolfe iterations.

``vht(capacity, net, dem, iters)`` is differentiable with PyTorch: the
forward pass solves the network on the GPU with FP32 path costs and the exact
(differentiable) line search, recording a tape of FW directions, step sizes
and checkpointed flows; the backward pass runs the hand-written adjoint
kernels of ``csrc/adjoint.cu`` (FP64 accumulation) over that tape.  The
all-or-nothing loads are held fixed, so the result is the gradient of the
piecewise-smooth map on which they stay constant.

``screen_upgrades`` uses the gradient for a first-order estimate of the VHT
change of candidate capacity upgrades before any full re-solve.
"""

from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .solver import Solver
from .synth import Demand, Network

__all__ = ["vht_and_grad", "VHTFunction", "vht", "screen_upgrades"]


def vht_and_grad(net: Network, dem: Demand, capacity: Optional[np.ndarray] = None,
                 iters: int = 50, precision: str = "fp32", solver: Optional[Solver] = None):
    """(VHT after `iters` FW iterations, dVHT/dcapacity [M]) at `capacity`."""
    own = solver is None
    s = solver or Solver(net, dem, precision=precision, record_tape=True, tape_capacity=iters,
                         line_search="exact")
    try:
        if capacity is not None:
            s.set_capacity(np.asarray(capacity, np.float64))
        s.solve(max_iters=iters)
        return s.adjoint_vht()
    finally:
        if own:
            s.close()


try:
    import torch

    class VHTFunction(torch.autograd.Function):
        """VHT(capacity) with the adjoint as its backward."""

        @staticmethod
        def forward(ctx, capacity, net, dem, iters, precision):
            cap = capacity.detach().to("cpu", torch.float64).numpy()
            v, g = vht_and_grad(net, dem, cap, iters, precision)
            ctx.save_for_backward(torch.as_tensor(g, dtype=torch.float64))
            ctx.cap_dtype, ctx.cap_device = capacity.dtype, capacity.device
            return torch.tensor(v, dtype=torch.float64, device=capacity.device)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            gc = (grad_out.to("cpu", torch.float64) * g).to(ctx.cap_device, ctx.cap_dtype)
            return gc, None, None, None, None

    def vht(capacity, net: Network, dem: Demand, iters: int = 50, precision: str = "fp32"):
        """Differentiable VHT of the network at `capacity` (a torch tensor)."""
        return VHTFunction.apply(capacity, net, dem, iters, precision)

except ImportError:  # pragma: no cover - torch is optional for the C ABI
    VHTFunction = None

    def vht(*a, **k):
        raise RuntimeError("torch is required for the autograd wrapper")


def screen_upgrades(net: Network, dem: Demand, candidates: Sequence[Sequence[int]],
                    gains: Sequence[Sequence[float]], iters: int = 50,
                    precision: str = "fp32"):
    """First-order VHT change of each candidate upgrade: sum_k grad_k * dcap_k,
    where candidate i raises the capacity of links candidates[i] by the
    fractions gains[i].  Returns (estimates, base VHT, gradient); the most
    negative estimates are the upgrades worth a full re-solve."""
    v, g = vht_and_grad(net, dem, None, iters, precision)
    est = []
    for links, gain in zip(candidates, gains):
        links = np.asarray(links, np.int64)
        dcap = net.capacity[links] * np.asarray(gain, np.float64)
        est.append(float(np.dot(g[links], dcap)))
    return np.asarray(est), v, g
