"""Central finite differences of a spike-time loss through the float64 oracle network (test infrastructure).

The loss is L(W) = sum over finite output spike times t of r * t, r a fixed array of the output's shape.
A perturbation of weight (i, j) of layer l changes only post neuron i of layer l, so the oracle reuses
the unperturbed outputs of layers < l, recomputes neuron i of layer l alone (bats_ref64.lif_forward on
that weight row: the neurons of a layer do not interact) and then the layers above it in full.
Perturbations that change any spike count (threshold grazing) are reported as such, their loss is not
differentiable there. The work is spread over a `spawn` process pool (safe after CUDA has started in
the parent).

Only the tests call this module; it is test infrastructure, not part of the product path.
"""
from __future__ import annotations

import multiprocessing as mp
import os
from typing import List, Sequence, Tuple

import numpy as np

from . import bats_ref64 as R


def network_forward(pre_times, weights, params, start: int = 0, layer_inputs=None):
    """Forward of layers start.. of an FC network in float64. params: list of (tau_s, theta, delta_theta,
    max_n_spike, max_simulation) per layer. Returns the list of per-layer oracle outputs (n, a, x, t, z)
    for layers >= start."""
    x = pre_times if layer_inputs is None else layer_inputs
    outs = []
    for w, p in zip(weights[start:], params[start:]):
        o = R.lif_forward(x, np.asarray(w, dtype=np.float64), *p)
        outs.append(o)
        x = o[3]
    return outs


def loss_of(out_times, r) -> float:
    f = np.isfinite(out_times)
    return float((np.where(f, out_times, 0.0) * r).sum())


_CTX = {}


def _init(pre_times, weights, params, base_outs, r):
    _CTX.update(pre=pre_times, weights=weights, params=params, base=base_outs, r=r)


def _perturbed(layer: int, i: int, j: int, delta: float) -> Tuple[float, bool]:
    c = _CTX
    weights, params, base = c["weights"], c["params"], c["base"]
    row = np.asarray(weights[layer][i:i + 1], dtype=np.float64).copy()
    row[0, j] += delta
    layer_in = c["pre"] if layer == 0 else base[layer - 1][3]
    one = R.lif_forward(layer_in, row, *params[layer])
    same = bool(np.array_equal(one[0][:, 0], base[layer][0][:, i]))
    t_layer = base[layer][3].copy()
    t_layer[:, i, :] = one[3][:, 0, :]
    outs = network_forward(None, weights, params, start=layer + 1, layer_inputs=t_layer)
    for o, b in zip(outs, base[layer + 1:]):
        same = same and bool(np.array_equal(o[0], b[0]))
    out_t = outs[-1][3] if outs else t_layer
    return loss_of(out_t, c["r"]), same


def _central(args):
    layer, i, j, eps = args
    lp, sp = _perturbed(layer, i, j, eps)
    lm, sm = _perturbed(layer, i, j, -eps)
    return (lp - lm) / (2.0 * eps), sp and sm


def network_gradients(pre_times, weights, params, r):
    """dL/dW of every layer by the oracle's exact backward (reset errors, factors, weight gradient, pre-spike
    errors; the chain of bats/Layers/LIFLayer.py:93-110), summed over the batch, for the loss above."""
    ws = [np.asarray(w, dtype=np.float64) for w in weights]
    outs = network_forward(np.asarray(pre_times, dtype=np.float64), ws, params)
    ins = [np.asarray(pre_times, dtype=np.float64)] + [o[3] for o in outs[:-1]]
    err = np.where(np.isfinite(outs[-1][3]), np.asarray(r, dtype=np.float64), 0.0)
    grads = [None] * len(ws)
    for li in range(len(ws) - 1, -1, -1):
        tau_s, theta, delta_theta = params[li][:3]
        tau = 2.0 * tau_s
        _, a, x, t, z = outs[li]
        R.propagate_recurrent_errors(x, z, err, delta_theta / tau)
        f1, f2 = R.compute_factors(t, a, theta / tau, x, z, tau)
        es, ee = R.compute_pre_exps(ins[li], tau_s, tau)
        grads[li] = R.compute_weights_gradient(f1, f2, t, (ins[li], es, ee), err).sum(0)
        if li > 0:
            err = R.propagate_errors_to_pre_spikes(f1, f2, t, (ins[li], es, ee), ws[li], err, tau_s, tau)
    return grads


def gradient_sensitivity(pre_times, weights, params, r, rho: float = 1e-6):
    """Conditioning of the gradient, for comparing an FP32 evaluation with float64 derivatives: per layer,
    |g(theta (1 + rho)) - g(theta (1 - rho))| / 2 with every layer's threshold moved together, i.e. how far
    the exact gradient moves when the neuron states change at the relative level rho. Entries that depend
    on near-tangential threshold crossings move by orders of magnitude more than rho."""
    def moved(sign):
        p = [(ts, th * (1 + sign * rho), dth, k, ms) for (ts, th, dth, k, ms) in params]
        return network_gradients(pre_times, weights, p, r)
    gp, gm = moved(1.0), moved(-1.0)
    return [np.abs(a - b) / 2 for a, b in zip(gp, gm)]


def _sample_sensitivity(args):
    q, rho = args
    c = _CTX
    pre = c["pre"][q:q + 1]
    r = c["r"][q:q + 1]
    g = network_gradients(pre, c["weights"], c["params"], r)
    s = gradient_sensitivity(pre, c["weights"], c["params"], r, rho)
    return [float(a.max() / max(np.abs(b).max(), 1e-30)) for a, b in zip(s, g)]


def per_sample_sensitivity(pre_times, weights, params, r, rho: float = 1e-6, processes: int | None = None):
    """For each sample alone: per layer, max over weights of gradient_sensitivity / max |gradient|
    (how strongly the sample's gradient amplifies a relative change rho of the neuron states)."""
    pre = np.asarray(pre_times, dtype=np.float64)
    ws = [np.asarray(w, dtype=np.float64) for w in weights]
    r = np.asarray(r, dtype=np.float64)
    jobs = [(q, rho) for q in range(pre.shape[0])]
    processes = processes or min(16, os.cpu_count() or 1)
    if processes > 1:
        with mp.get_context("spawn").Pool(processes, initializer=_init, initargs=(pre, ws, params, None, r)) as pool:
            return np.array(pool.map(_sample_sensitivity, jobs, chunksize=1))
    _init(pre, ws, params, None, r)
    return np.array([_sample_sensitivity(a) for a in jobs])


def central_differences(pre_times, weights, params, r, picks: Sequence[Tuple[int, int, int]], eps: float = 1e-4,
                        processes: int | None = None) -> Tuple[np.ndarray, np.ndarray]:
    """dL/dw for each (layer, i, j) in picks by central differences of step eps in float64.
    Returns (fd values, mask of perturbations that left every spike count unchanged)."""
    pre = np.asarray(pre_times, dtype=np.float64)
    ws = [np.asarray(w, dtype=np.float64) for w in weights]
    base = network_forward(pre, ws, params)
    r = np.asarray(r, dtype=np.float64)
    jobs = [(int(l), int(i), int(j), float(eps)) for (l, i, j) in picks]
    processes = processes or min(16, os.cpu_count() or 1)
    if processes > 1:
        with mp.get_context("spawn").Pool(processes, initializer=_init, initargs=(pre, ws, params, base, r)) as pool:
            res = pool.map(_central, jobs, chunksize=1)
    else:
        _init(pre, ws, params, base, r)
        res = [_central(a) for a in jobs]
    return np.array([v for v, _ in res]), np.array([s for _, s in res])
