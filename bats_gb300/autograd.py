"""torch.autograd bindings of the BATS kernels.

lif_fc(pre_times, weights, ...) returns the post-synaptic spike times (B, N, K) of a fully-connected LIF
layer as a differentiable function of the pre-synaptic spike times and of the weights; its backward
runs the exact multi-spike backward kernels (reset errors, factors, weight gradient summed over the
batch, pre-spike errors). Spike counts are piecewise constant and carry no gradient; slots without a
spike (+inf) receive none. This is the layer math of bats/Layers/LIFLayer.py:63-110 behind
torch.autograd, so that losses written with torch ops on spike times can be differentiated exactly.
"""
from __future__ import annotations

import numpy as np
import torch

from . import kernels as K


class _LIFFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pre_times, weights, tau_s, theta, delta_theta, max_n_spike, max_simulation):
        pre = pre_times.detach().contiguous().float()
        w = weights.detach().contiguous().float()
        tau32, c, dtt = K.lif_constants(tau_s, theta, delta_theta)
        ev = K.sort_events(pre, np.float32(tau_s), tau32)
        wt = K.transpose_weights(w)
        n, a, x, t, z = K.lif_forward_fc(ev, wt, w.shape[0], int(max_n_spike), tau_s, theta, delta_theta,
                                         max_simulation)
        ctx.save_for_backward(pre, a, x, t, z)
        ctx.ev, ctx.wt = ev, wt
        ctx.consts = (float(np.float32(tau_s)), float(tau32), float(c), float(dtt))
        ctx.n_pre = pre.shape[1]
        ctx.mark_non_differentiable(n)
        return t, n

    @staticmethod
    def backward(ctx, grad_t, grad_n):
        pre, a, x, t, z = ctx.saved_tensors
        tau_s, tau, c, dtt = ctx.consts
        if grad_t is None:
            return None, None, None, None, None, None, None
        errors = torch.where(torch.isinf(t), torch.zeros_like(grad_t), grad_t).contiguous().float().clone()
        tabs = K.backward_prep(t, a, x, z, errors, c, tau, dtt)
        grad_w = None
        if ctx.needs_input_grad[1]:
            grad_w = K.weights_gradient(ctx.ev, t, tabs, ctx.n_pre, per_sample=False, reduce="sum")
        grad_pre = None
        if ctx.needs_input_grad[0]:
            grad_pre = K.pre_errors(ctx.ev, ctx.wt, t, tabs, tau_s, tau)
        return grad_pre, grad_w, None, None, None, None, None


def lif_fc(pre_times: torch.Tensor, weights: torch.Tensor, tau_s: float, theta: float, delta_theta: float,
           max_n_spike: int = 32, max_simulation: float = float("inf")):
    """(spike_times (B, N, K), n_spikes (B, N)) of a fully-connected LIF layer; differentiable in
    pre_times and weights."""
    return _LIFFunction.apply(pre_times, weights, tau_s, theta, delta_theta, max_n_spike, max_simulation)
