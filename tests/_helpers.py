"""Shared input generators and comparison helpers of the parity tests."""
from __future__ import annotations

import numpy as np

from oracle import bats_ref64 as R


def mnist_like_input(batch, n_in=784, p=0.19, t_max=0.01, seed=0):
    """Each input neuron fires once with probability p at U(0, t_max), else stays silent (inf, count 0):
    the synthetic stand-in of the reference's MNIST encoding (experiments/mnist/Dataset.py:66-71)."""
    rng = np.random.default_rng(seed)
    fire = rng.random((batch, n_in)) < p
    t = np.where(fire, rng.uniform(0, t_max, (batch, n_in)), np.inf).astype(np.float32)
    return t[:, :, None], fire.astype(np.int32)


def multi_spike_input(batch, n_in, k, t_max, seed=0, p_silent=0.2):
    """Per neuron 0..k sorted spikes at U(0, t_max)."""
    rng = np.random.default_rng(seed)
    t = np.full((batch, n_in, k), np.inf, dtype=np.float32)
    n = rng.integers(0, k + 1, (batch, n_in))
    n[rng.random((batch, n_in)) < p_silent] = 0
    for s in range(batch):
        for j in range(n_in):
            t[s, j, :n[s, j]] = np.sort(rng.uniform(0, t_max, n[s, j]))
    return t, n.astype(np.int32)


def grazing_mask(pre_t, W, tau_s, theta, delta_theta, K, max_sim, rel=1e-5, conv=None):
    """Neurons whose float64 spike count changes when theta moves by +-rel: their membrane maximum lies
    within rel of the threshold, where an FP32 evaluation may legitimately flip the count.
    Returns (n_low_theta, n_high_theta)."""
    f = R.lif_forward if conv is None else (lambda t, w, *a: R.conv_forward(t, w, conv, *a))
    n_lo = f(pre_t.astype(np.float64), W, tau_s, theta * (1 - rel), delta_theta, K, max_sim)[0]
    n_hi = f(pre_t.astype(np.float64), W, tau_s, theta * (1 + rel), delta_theta, K, max_sim)[0]
    return np.minimum(n_lo, n_hi), np.maximum(n_lo, n_hi)


def conditioned_reference(pre_t, W, tau_s, theta, delta_theta, K, max_sim, conv=None):
    """float64 forward + (count bounds, time sensitivity) for an FP32-vs-FP64 comparison."""
    Wd = W if conv is None else R.conv_dense_weights(W, conv)
    pre = pre_t.astype(np.float64)
    o64 = R.lif_forward(pre, np.asarray(Wd, dtype=np.float64), tau_s, theta, delta_theta, K, max_sim)
    lo, hi, sens = R.threshold_sensitivity(pre, np.asarray(Wd, dtype=np.float64), tau_s, theta, delta_theta, K,
                                           max_sim)
    return o64, (lo, hi), sens


def count_mismatches(n_gpu, n_ref, bounds=None):
    """(# differing counts, # not explained by grazing)."""
    diff = n_gpu != n_ref
    if bounds is None:
        return int(diff.sum()), int(diff.sum())
    lo, hi = bounds
    unexplained = diff & ~((n_gpu >= lo) & (n_gpu <= hi))
    return int(diff.sum()), int(unexplained.sum())


def leading_mask(n, K):
    return np.arange(K)[None, None, :] < n[:, :, None]


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def assert_sum_close(got, ref, abs_scale, rtol=1e-5, what=""):
    """|got - ref| <= rtol |ref| + rtol * abs_scale elementwise, where abs_scale is the sum of the magnitudes
    of the terms that make up ref (a sum of signed terms may cancel far below its terms). Returns
    (entries, entries that need the abs_scale term, worst error / tolerance)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.asarray(abs_scale, dtype=np.float64)
    tol = rtol * np.abs(ref) + rtol * scale + 1e-30
    err = np.abs(got - ref)
    worst = float(np.max(err / tol)) if err.size else 0.0
    assert worst <= 1.0, f"{what}: worst error / tolerance = {worst:.3f}"
    return int(err.size), int((err > rtol * np.abs(ref)).sum()), worst


def ref_layer_backward(layer, errors, want_pre=True):
    """The reference's LIFLayer.backward (bats/Layers/LIFLayer.py:93-110) on its compiled kernels, for a
    refkern.RefLIF layer after its forward, with `errors` (B, N, K) (changed in place by the reset-error
    step, as the reference does). Returns the batch-summed weight gradient and its term-magnitude sum
    (the same kernel on |errors|, |f1|, -|f2|), and the pre-spike errors and their term-magnitude sum
    (|W|, |errors|, |f1|, |f2|, -tau). The gradients are float64 numpy arrays, the pre errors CUDA tensors
    (B, N_pre, K_pre), so that they can feed the layer below (None without want_pre)."""
    from oracle import refkern
    n, a, x, t, z = layer.out
    refkern.propagate_recurrent_errors(x, z, errors, layer.dtt)
    f1, f2 = refkern.compute_factors(t, a, layer.c, x, z, layer.tau)
    g = refkern.compute_weights_gradient(f1, f2, t, layer.pre_t, layer.es, layer.ee, errors)
    g_sum = g.double().sum(0).cpu().numpy()
    del g
    ga = refkern.compute_weights_gradient(f1.abs(), -f2.abs(), t, layer.pre_t, layer.es, layer.ee, errors.abs())
    g_abs = ga.double().sum(0).cpu().numpy()
    del ga
    pre = pre_abs = None
    if want_pre:
        pre = refkern.propagate_errors_to_pre_spikes(f1, f2, t, layer.pre_t, layer.es, layer.ee, layer.w, errors,
                                                     layer.tau_s, layer.tau)
        pre_abs = refkern.propagate_errors_to_pre_spikes(f1.abs(), f2.abs(), t, layer.pre_t, layer.es, layer.ee,
                                                         layer.w.abs(), errors.abs(), layer.tau_s,
                                                         -np.float32(layer.tau))
    return g_sum, g_abs, pre, pre_abs


def ref_conv_layer_backward(layer, errors, want_pre=True):
    """ConvLIFLayer.backward (bats/Layers/ConvLIFLayer.py:109-134) on the reference's compiled kernels for a
    refkern.RefConvLIF layer after its forward, as ref_layer_backward: the batch-summed filter gradient
    (C_out, fx, fy, C_in) and its term-magnitude sum as float64 numpy arrays, the pre-spike errors and their
    term-magnitude sum as CUDA tensors (None without want_pre)."""
    from oracle import refkern
    n, a, x, t, z = layer.out
    refkern.propagate_recurrent_errors(x, z, errors, layer.dtt)
    f1, f2 = refkern.compute_factors(t, a, layer.c, x, z, layer.tau)
    geo = (layer.pre_shape, layer.post_shape, layer.filter_shape)
    g = refkern.compute_weights_gradient_conv(f1, f2, t, layer.pre_t, layer.es, layer.ee, *geo, errors)
    g_sum = g.double().sum(0).cpu().numpy()
    del g
    ga = refkern.compute_weights_gradient_conv(f1.abs(), -f2.abs(), t, layer.pre_t, layer.es, layer.ee, *geo,
                                               errors.abs())
    g_abs = ga.double().sum(0).cpu().numpy()
    del ga
    pre = pre_abs = None
    if want_pre:
        pre = refkern.propagate_errors_to_pre_spikes_conv(f1, f2, t, layer.pre_t, layer.es, layer.ee, layer.w, errors,
                                                          layer.tau_s, layer.tau, *geo)
        pre_abs = refkern.propagate_errors_to_pre_spikes_conv(f1.abs(), f2.abs(), t, layer.pre_t, layer.es, layer.ee,
                                                              layer.w.abs(), errors.abs(), layer.tau_s,
                                                              -np.float32(layer.tau), *geo)
    return g_sum, g_abs, pre, pre_abs


def uneven_input(batch, n_in=1024, seed=11, median=200, lo=20, hi=4000, t_max=0.1):
    """Samples of very uneven length: per-sample input spike count clip(round(lognormal(ln median, 1)), lo, hi),
    channels uniform over n_in, times U(0, t_max). Returns spike trains (B, n_in, K_in) (K_in the largest
    per-channel count, +inf padding), counts (B, n_in) and the per-sample event counts."""
    rng = np.random.default_rng(seed)
    counts = np.clip(np.round(rng.lognormal(np.log(median), 1.0, batch)), lo, hi).astype(np.int64)
    chans = [rng.integers(0, n_in, c) for c in counts]
    times = [np.sort(rng.uniform(0, t_max, c)).astype(np.float32) for c in counts]
    k_in = max(int(np.bincount(ch, minlength=n_in).max()) for ch in chans)
    t = np.full((batch, n_in, k_in), np.inf, dtype=np.float32)
    for q, (ch, tm) in enumerate(zip(chans, times)):
        order = np.argsort(ch, kind="stable")
        ch_s, tm_s = ch[order], tm[order]
        first = np.searchsorted(ch_s, ch_s, side="left")
        t[q, ch_s, np.arange(len(ch_s)) - first] = tm_s
    return t, np.isfinite(t).sum(2).astype(np.int32), counts
