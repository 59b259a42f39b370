"""Float64 NumPy oracle of the BATS hot path: event-based LIF forward and exact multi-spike backward.

TEST INFRASTRUCTURE ONLY. This module is the reference against which the tests check the CUDA kernels of
bats_gb300, and the CPU baseline of bench.py; nothing in the product imports it. It restates the reference's
algorithm (Florian-BACHO/bats, CuPy + CUDA) in plain NumPy float64, one function per reference
kernel, each citing the file:line it follows. Parity is pinned by running the reference's own
unit tests against these functions (tests/golden/make_golden.py, which imports the reference test
modules with a NumPy stand-in for CuPy) and by an independent fixed-step integrator of the neuron
ODE (`simulate_fixed_step`), which replaces the reference's brian2 ground truth.

Neuron model (tests/CudaKernels/Inference/compute_spike_times_tests.py:15-25 of the reference):
    du/dt = -u/tau + v,  dv/dt = -v/tau_s,  input spike of weight w: v += w,
    threshold u >= theta, reset u -= delta_theta, tau = 2 tau_s (bats/Layers/LIFLayer.py:17).
"""
from __future__ import annotations

import numpy as np

INF = np.inf


# --------------------------------------------------------------------------------------------
# Inference
# --------------------------------------------------------------------------------------------

def compute_pre_exps(times, tau_s, tau):
    """exp(t/tau_s), exp(t/tau) (bats/CudaKernels/CuFiles/Inference/compute_pre_exps.cu:18-21)."""
    t = np.asarray(times, dtype=np.float64)
    with np.errstate(over="ignore"):
        return np.exp(t / tau_s), np.exp(t / tau)


def sort_events(times):
    """Time-sorted valid pre-spikes of each sample.

    bats/CudaKernels/Wrappers/Inference/get_sorted_spikes_indices.py:7-17 sorts the flattened
    (N*K) slots of each sample; slots with +inf time are never reached by the forward scan
    (compute_spike_times.cu:120-121), so only slots with time < +inf are kept here. Ties keep slot
    order (stable sort). Returns a list over samples of (t, neuron, slot) arrays.
    """
    times = np.asarray(times, dtype=np.float64)
    B, N, K = times.shape
    out = []
    for s in range(B):
        flat = times[s].reshape(-1)
        slots = np.nonzero(flat < INF)[0]
        order = np.argsort(flat[slots], kind="stable")
        slots = slots[order]
        out.append((flat[slots], slots // K, slots))
    return out


def _solve_crossings(a, b, c, dtt, tau, last, nxt, max_sim, n, K, outs, active):
    """Vectorised compute_spikes (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:34-84).

    For the neurons in `active`, repeatedly solve c z^2 - b z + a = 0 for its smaller root
    z = 2a / (b + sqrt(b^2 - 4ac)), t = tau ln z, accept it if last < t <= min(nxt, max_sim),
    record (a, x, t, z), apply the reset b -= dtt z (line 78) and stop at K spikes (line 80).
    Returns the mask of neurons whose buffer became full.
    """
    a_o, x_o, t_o, z_o = outs
    full = np.zeros_like(active)
    last = np.array(last, dtype=np.float64, copy=True)
    act = active.copy()
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        while act.any():
            disc = b * b - 4.0 * a * c
            ok = act & (disc >= 0)
            x = np.sqrt(np.where(ok, disc, 0.0))
            den = x + b
            ok &= den != 0
            z = np.where(ok, 2.0 * a / np.where(den == 0, 1.0, den), -1.0)
            ok &= ~(z < 0)
            t = tau * np.log(np.where(ok, z, 1.0))
            t = np.where(ok & (z == 0), -INF, t)
            ok &= ~((t <= last) | (t > max_sim) | (t > nxt))
            if not ok.any():
                break
            idx = np.nonzero(ok)[0]
            slot = n[idx]
            a_o[idx, slot] = a[idx]
            x_o[idx, slot] = x[idx]
            t_o[idx, slot] = t[idx]
            z_o[idx, slot] = z[idx]
            last[idx] = t[idx]
            b[idx] -= dtt * z[idx]
            n[idx] += 1
            f = n[idx] >= K
            full[idx[f]] = True
            act = ok & ~full
    return full


def lif_forward(pre_times, weights, tau_s, theta, delta_theta, max_n_spike, max_simulation=INF):
    """Fully-connected LIF forward (bats/Layers/LIFLayer.py:63-91 ->
    compute_spike_times.cu:86-138): per sample, scan the time-sorted input events, accumulate
    a += w exp(t/tau_s), b += w exp(t/tau) (lines 124-125) and search crossings in
    (t_i, t_{i+1}] after every event.

    pre_times (B, N_pre, K_pre); weights (N_post, N_pre). Returns n (B, N_post) int32 and
    a, x, t, z (B, N_post, K) float64 with t, z = +inf and a, x = +inf after the spikes.
    """
    W = np.asarray(weights, dtype=np.float64)
    tau = 2.0 * tau_s
    c = theta / tau
    dtt = delta_theta / tau
    B = pre_times.shape[0]
    N = W.shape[0]
    K = int(max_n_spike)
    n = np.zeros((B, N), dtype=np.int32)
    a_o = np.full((B, N, K), INF)
    x_o = np.full((B, N, K), INF)
    t_o = np.full((B, N, K), INF)
    z_o = np.full((B, N, K), INF)
    for s, (et, ej, _) in enumerate(sort_events(pre_times)):
        es, ee = np.exp(et / tau_s), np.exp(et / tau)
        a = np.zeros(N)
        b = np.zeros(N)
        ns = n[s]
        alive = np.ones(N, dtype=bool)
        outs = (a_o[s], x_o[s], t_o[s], z_o[s])
        E = et.shape[0]
        for m in range(E):
            w = W[:, ej[m]]
            a += w * es[m]
            b += w * ee[m]
            nxt = et[m + 1] if m + 1 < E else INF
            full = _solve_crossings(a, b, c, dtt, tau, np.full(N, et[m]), nxt, max_simulation, ns, K, outs, alive)
            alive &= ~full
            if not alive.any():
                break
    return n, a_o, x_o, t_o, z_o


def convert_to_spike_per_neuron(indices, times, n_neurons):
    """Event list (B, S) of (neuron index, time), index -1 ending a sample, into per-neuron trains
    (B, N, K) + counts (B, N), K the largest per-neuron count of the batch
    (bats/CudaKernels/CuFiles/Inference/convert_to_spike_per_neuron.cu:9-25 and the cp.unique loop of
    Wrappers/Inference/convert_to_spike_per_neuron.py:11-18). Spikes keep their order of appearance."""
    indices = np.asarray(indices)
    times = np.asarray(times, dtype=np.float64)
    B, S = indices.shape
    counts = np.zeros((B, n_neurons), dtype=np.int32)
    for s in range(B):
        for q in range(S):
            j = indices[s, q]
            if j < 0:
                break
            counts[s, j] += 1
    K = int(counts.max()) if counts.size else 0
    out = np.full((B, n_neurons, K), INF)
    fill = np.zeros((B, n_neurons), dtype=np.int64)
    for s in range(B):
        for q in range(S):
            j = indices[s, q]
            if j < 0:
                break
            out[s, j, fill[s, j]] = times[s, q]
            fill[s, j] += 1
    return out, counts


def conv_dense_weights(filters, pre_shape):
    """Dense (N_post, N_pre) matrix of a valid stride-1 convolution with filters (C_out, fx, fy, C_in):
    the weight get_spike_weight returns for each (post, pre) pair, 0 outside the receptive field
    (bats/CudaKernels/CuFiles/Inference/compute_spike_times_conv.cu:93-115)."""
    Wf = np.asarray(filters, dtype=np.float64)
    C_out, fx, fy, C = Wf.shape
    X, Y, Cp = pre_shape
    assert Cp == C
    Xo, Yo = X - fx + 1, Y - fy + 1
    D = np.zeros((Xo, Yo, C_out, X, Y, C))
    for dx in range(fx):
        for dy in range(fy):
            for xo in range(Xo):
                for yo in range(Yo):
                    D[xo, yo, :, xo + dx, yo + dy, :] = Wf[:, dx, dy, :]
    return D.reshape(Xo * Yo * C_out, X * Y * C)


def conv_forward(pre_times, filters, pre_shape, tau_s, theta, delta_theta, max_n_spike, max_simulation=INF):
    """ConvLIFLayer forward (bats/Layers/ConvLIFLayer.py:77-107, compute_spike_times_conv.cu:117-174):
    the same event scan as the FC layer with the receptive-field weight of each event (0 outside),
    which is the FC forward with the dense equivalent weight matrix."""
    return lif_forward(pre_times, conv_dense_weights(filters, pre_shape), tau_s, theta, delta_theta,
                       max_n_spike, max_simulation)


def aggregate_spikes_conv(n_spikes, times, pre_shape):
    """2x2 pooling (bats/CudaKernels/CuFiles/Inference/aggregate_spikes_conv.cu:6-43 plus the argsort
    of Wrappers/Inference/aggregate_spikes_conv.py:24-26): children (0,0),(0,1),(1,0),(1,1) concatenated,
    stably sorted by time; indices are batch-global flat slots."""
    times = np.asarray(times, dtype=np.float64)
    B, N, K = times.shape
    X, Y, C = pre_shape
    Xo, Yo = X // 2, Y // 2
    t5 = times.reshape(B, X, Y, C, K)
    n4 = np.asarray(n_spikes).reshape(B, X, Y, C)
    idx5 = np.arange(B * N * K).reshape(B, X, Y, C, K)
    parts_t, parts_i, cnt = [], [], 0
    for dx in (0, 1):
        for dy in (0, 1):
            sl = (slice(None), slice(dx, 2 * Xo, 2), slice(dy, 2 * Yo, 2))
            parts_t.append(t5[sl])
            parts_i.append(idx5[sl])
            cnt = cnt + n4[sl]
    cat_t = np.concatenate(parts_t, axis=-1).reshape(B, Xo * Yo * C, 4 * K)
    cat_i = np.concatenate(parts_i, axis=-1).reshape(B, Xo * Yo * C, 4 * K)
    order = np.argsort(cat_t, axis=2, kind="stable")
    return (cnt.reshape(B, Xo * Yo * C).astype(np.int32), np.take_along_axis(cat_t, order, 2),
            np.take_along_axis(cat_i, order, 2))


def pool_backward(errors, indices, pre_count):
    """PoolingLayer.backward (bats/Layers/PoolingLayer.py:55-66): pre_errors[indices] = errors."""
    out = np.zeros(pre_count)
    out[np.asarray(indices).reshape(-1)] = np.asarray(errors, dtype=np.float64).reshape(-1)
    return out


# --------------------------------------------------------------------------------------------
# Backpropagation
# --------------------------------------------------------------------------------------------

def propagate_recurrent_errors(x, exp_tau, errors, delta_theta_tau):
    """In-place reset-error scan (bats/CudaKernels/CuFiles/Backpropagation/propagate_recurrent_errors.cu:17-22):
    for k from last to first, skipping slots with inf exp_tau: err_k += C z_k; C += err_k dtt / x_k."""
    x = np.asarray(x, dtype=np.float64)
    z = np.asarray(exp_tau, dtype=np.float64)
    K = errors.shape[-1]
    cum = np.zeros(errors.shape[:-1])
    with np.errstate(invalid="ignore", divide="ignore"):
        for k in range(K - 1, -1, -1):
            valid = ~np.isinf(z[..., k])
            ek = np.where(valid, errors[..., k] + cum * np.where(valid, z[..., k], 0.0), errors[..., k])
            errors[..., k] = ek
            cum = np.where(valid, cum + ek * delta_theta_tau / np.where(valid, x[..., k], 1.0), cum)
    return errors


def compute_factors(spike_times, a, c, x, exp_tau, tau):
    """f1 = tau/a (1 + z c / x), f2 = tau/x, 0 where there is no spike
    (bats/CudaKernels/CuFiles/Backpropagation/compute_factors.cu:20-30)."""
    t = np.asarray(spike_times, dtype=np.float64)
    spike = ~np.isinf(t)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        f1 = np.where(spike, tau / a * (1.0 + exp_tau * c / x), 0.0)
        f2 = np.where(spike, tau / x, 0.0)
    return f1, f2


def _leading_valid(post_times):
    """Number of leading finite post spikes (the loops of compute_weights_gradient.cu:36-38 and
    propagate_errors_to_pre_spikes.cu:43-46 stop at the first inf)."""
    inf = np.isinf(post_times)
    K = post_times.shape[-1]
    first = np.where(inf.any(-1), inf.argmax(-1), K)
    return first


def _suffix_after(post_t, nvalid, coef, times):
    """S[m, i] = sum over k < nvalid_i with post_t[i, k] > times[m] of coef[i, k]."""
    K = post_t.shape[-1]
    valid = np.arange(K)[None, :] < nvalid[:, None]
    cf = np.where(valid, coef, 0.0)
    mask = post_t[None, :, :] > times[:, None, None]
    return np.einsum("mik,ik->mi", mask, cf)


def compute_weights_gradient(f1, f2, post_times, pre_times, errors):
    """Per-sample weight gradient (bats/CudaKernels/CuFiles/Backpropagation/compute_weights_gradient.cu:33-45):
    grad[s, i, j] = sum_k err_k (f1_k sum_{tau<t_k} exp(tau/tau_s) - f2_k sum_{tau<t_k} exp(tau/tau)),
    over pre spikes of j strictly before post spike k. Uses exp of the pre times from the caller:
    pre_times is a tuple (times, exp_tau_s, exp_tau) of (B, N_pre, K_pre) arrays."""
    pt, pes, pe = (np.asarray(v, dtype=np.float64) for v in pre_times)
    f1 = np.asarray(f1, dtype=np.float64)
    f2 = np.asarray(f2, dtype=np.float64)
    err = np.asarray(errors, dtype=np.float64)
    post_times = np.asarray(post_times, dtype=np.float64)
    B, N_post, K_post = f1.shape
    N_pre = pt.shape[1]
    out = np.zeros((B, N_post, N_pre))
    for s in range(B):
        nv = _leading_valid(post_times[s])
        flat_t = pt[s].reshape(-1)
        valid = ~np.isinf(flat_t)
        ev_t = flat_t[valid]
        ev_j = np.nonzero(valid)[0] // pt.shape[2]
        ev_es = pes[s].reshape(-1)[valid]
        ev_e = pe[s].reshape(-1)[valid]
        SA = _suffix_after(post_times[s], nv, err[s] * f1[s], ev_t)
        SB = _suffix_after(post_times[s], nv, err[s] * f2[s], ev_t)
        U = ev_es[:, None] * SA - ev_e[:, None] * SB
        gT = np.zeros((N_pre, N_post))
        np.add.at(gT, ev_j, U)
        out[s] = gT.T
    return out


def propagate_errors_to_pre_spikes(f1, f2, post_times, pre_times, weights, errors, tau_s, tau):
    """dL/d(pre spike) (bats/CudaKernels/CuFiles/Backpropagation/propagate_errors_to_pre_spikes.cu:41-53 +
    the sum over post neurons in Wrappers/Backpropagation/propagate_errors_to_pre_spikes.py:26):
    sum_i w_ij (sum_{t_k > tau} err_k f1_k exp(tau/tau_s)/tau_s - sum_{t_k > tau} err_k f2_k exp(tau/tau)/tau).
    pre_times is (times, exp_tau_s, exp_tau); weights (N_post, N_pre). Returns (B, N_pre, K_pre)."""
    pt, pes, pe = (np.asarray(v, dtype=np.float64) for v in pre_times)
    W = np.asarray(weights, dtype=np.float64)
    f1 = np.asarray(f1, dtype=np.float64)
    f2 = np.asarray(f2, dtype=np.float64)
    err = np.asarray(errors, dtype=np.float64)
    post_times = np.asarray(post_times, dtype=np.float64)
    B, N_pre, K_pre = pt.shape
    out = np.zeros((B, N_pre * K_pre))
    for s in range(B):
        nv = _leading_valid(post_times[s])
        flat_t = pt[s].reshape(-1)
        slots = np.nonzero(~np.isinf(flat_t))[0]
        ev_t = flat_t[slots]
        ev_j = slots // K_pre
        SA = _suffix_after(post_times[s], nv, err[s] * f1[s], ev_t)
        SB = _suffix_after(post_times[s], nv, err[s] * f2[s], ev_t)
        Wj = W[:, ev_j].T  # (E, N_post)
        es = pes[s].reshape(-1)[slots]
        ee = pe[s].reshape(-1)[slots]
        out[s, slots] = np.einsum("mi,mi->m", Wj, SA) * es / tau_s - np.einsum("mi,mi->m", Wj, SB) * ee / tau
    return out.reshape(B, N_pre, K_pre)


def conv_weights_gradient(f1, f2, post_times, pre_times, errors, filters_shape, pre_shape):
    """Per-sample filter gradient (B, C_out, fx, fy, C_in)
    (bats/CudaKernels/CuFiles/Backpropagation/compute_weights_gradient_conv.cu:31-59): the dense FC
    gradient restricted to the receptive-field pairs and folded onto the filter taps."""
    C_out, fx, fy, C = filters_shape
    X, Y, _ = pre_shape
    Xo, Yo = X - fx + 1, Y - fy + 1
    g = compute_weights_gradient(f1, f2, post_times, pre_times, errors)  # (B, N_post, N_pre)
    B = g.shape[0]
    g6 = g.reshape(B, Xo, Yo, C_out, X, Y, C)
    out = np.zeros((B, C_out, fx, fy, C))
    xo = np.arange(Xo)[:, None]
    yo = np.arange(Yo)[None, :]
    for dx in range(fx):
        for dy in range(fy):
            blk = g6[:, xo, yo, :, xo + dx, yo + dy, :]  # (Xo, Yo, B, C_out, C) after fancy indexing
            out[:, :, dx, dy, :] = blk.sum(axis=(0, 1))
    return out


def conv_pre_errors(f1, f2, post_times, pre_times, filters, errors, tau_s, tau, pre_shape):
    """Conv error propagation (bats/CudaKernels/CuFiles/Backpropagation/propagate_errors_to_pre_spikes_conv.cu:40-88)
    = the FC propagation with the dense equivalent weights."""
    return propagate_errors_to_pre_spikes(f1, f2, post_times, pre_times, conv_dense_weights(filters, pre_shape),
                                          errors, tau_s, tau)


# --------------------------------------------------------------------------------------------
# Losses and optimizer
# --------------------------------------------------------------------------------------------

def spike_count_loss(counts, targets, K):
    """loss = 1/2 sum (target - count)^2, errors = (target - count) repeated over K
    (bats/Losses/SpikeCountLoss.py:9-15, 31-38)."""
    d = np.asarray(targets, dtype=np.float64) - np.asarray(counts, dtype=np.float64)
    return 0.5 * np.sum(d * d, axis=1), np.repeat(d[:, :, None], K, axis=2)


def class_targets(labels, n, target_true, target_false):
    """SpikeCountClassLoss targets (bats/Losses/SpikeCountClassLoss.py:15-18)."""
    labels = np.asarray(labels)
    t = np.full((labels.size, n), float(target_false))
    t[np.arange(labels.size), labels] = float(target_true)
    return t


def ttfs_softmax_cross_entropy(spikes, labels, tau):
    """bats/Losses/TTFSSoftmaxCrossEntropy.py:41-56: softmax of exp(-t_first/tau); errors only in slot 0,
    divided by tau, nan_to_num."""
    spikes = np.asarray(spikes, dtype=np.float64)
    labels = np.asarray(labels)
    B = spikes.shape[0]
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        ex = np.exp(-spikes[..., 0] / tau)
        sums = ex.sum(axis=1)
        loss = -np.log(ex[np.arange(B), labels] / sums)
        ns = -ex / sums[:, None]
        ns[np.arange(B), labels] += 1
        ns /= tau
    err = np.zeros_like(spikes)
    err[..., 0] = np.nan_to_num(ns)
    return loss, err


def spike_time_loss(spikes, targets):
    """bats/Losses/SpikeTimeLoss.py:38-47 (compute_loss_and_errors): inf -> 1.0 in a copy of the spikes
    and in the targets (in place); loss on slot 0; errors = spikes - targets (uncopied spikes)."""
    spikes = np.asarray(spikes, dtype=np.float64)
    targets[np.isinf(targets)] = 1.0
    sc = np.where(np.isinf(spikes), 1.0, spikes)
    d = targets[..., 0] - sc[..., 0]
    return 0.5 * np.sum(d * d, axis=1), spikes - targets


class Adam:
    """bats/Optimizers/AdamOptimizer.py:22-55: returns deltas -lr m_hat / (sqrt(v_hat) + eps), with the
    bias corrections 1 - beta^t evaluated from the float32 betas."""

    def __init__(self, learning_rate, beta_1=0.9, beta_2=0.999, epsilon=1e-8):
        self.lr = float(np.float32(learning_rate))
        self.b1 = float(np.float32(beta_1))
        self.b2 = float(np.float32(beta_2))
        self.eps = float(np.float32(epsilon))
        self.m = None
        self.v = None
        self.t = 0

    def step(self, grads):
        self.t += 1
        if self.m is None:
            self.m = [None if g is None else np.zeros(np.shape(g)) for g in grads]
            self.v = [None if g is None else np.zeros(np.shape(g)) for g in grads]
        out = []
        c1 = 1.0 - self.b1 ** self.t
        c2 = 1.0 - self.b2 ** self.t
        for q, g in enumerate(grads):
            if g is None:
                out.append(None)
                continue
            g = np.asarray(g, dtype=np.float64)
            self.m[q] = self.b1 * self.m[q] + (1.0 - self.b1) * g
            self.v[q] = self.b2 * self.v[q] + (1.0 - self.b2) * g * g
            out.append(-(self.lr * (self.m[q] / c1) / (np.sqrt(self.v[q] / c2) + self.eps)))
        return out


class NAdam:
    """bats/Optimizers/NAdamOptimizer.py:23-58: deltas -(lr / (sqrt(v_hat) + eps)) *
    (beta_1 m_hat + (1 - beta_1) g / (1 - beta_1^t))."""

    def __init__(self, learning_rate, beta_1=0.9, beta_2=0.999, epsilon=1e-8):
        self.lr = float(np.float32(learning_rate))
        self.b1 = float(np.float32(beta_1))
        self.b2 = float(np.float32(beta_2))
        self.eps = float(np.float32(epsilon))
        self.m = None
        self.v = None
        self.t = 0

    def step(self, grads):
        self.t += 1
        if self.m is None:
            self.m = [None if g is None else np.zeros(np.shape(g)) for g in grads]
            self.v = [None if g is None else np.zeros(np.shape(g)) for g in grads]
        c1 = 1.0 - self.b1 ** self.t
        c2 = 1.0 - self.b2 ** self.t
        out = []
        for q, g in enumerate(grads):
            if g is None:
                out.append(None)
                continue
            g = np.asarray(g, dtype=np.float64)
            self.m[q] = self.b1 * self.m[q] + (1.0 - self.b1) * g
            self.v[q] = self.b2 * self.v[q] + (1.0 - self.b2) * g * g
            m_hat, v_hat = self.m[q] / c1, self.v[q] / c2
            out.append(-(self.lr / (np.sqrt(v_hat) + self.eps)) * (self.b1 * m_hat + (1.0 - self.b1) * g / c1))
        return out


def weights_synaptic_scaling(weights, silent_ratios, n_spikes, gradient, scaling_threshold, factor):
    """apply_weights_synaptic_scaling.cu:2-25 on a per-sample gradient (B, N_post, N_pre), returned new."""
    g = np.array(gradient, dtype=np.float64)
    apply = (np.asarray(silent_ratios)[:, None] >= scaling_threshold) & (np.asarray(n_spikes) <= 0)
    g -= np.where(apply[:, :, None], factor * np.abs(np.asarray(weights, dtype=np.float64))[None], 0.0)
    return g


def label_weights_synaptic_scaling(weights, labels, n_spikes, gradient, factor):
    """apply_label_weights_synaptic_scaling.cu:2-20 (the label's spike count read from n_spikes[label], the
    first sample's row, as the kernel indexes it)."""
    g = np.array(gradient, dtype=np.float64)
    W = np.abs(np.asarray(weights, dtype=np.float64))
    flat = np.asarray(n_spikes).reshape(-1)
    for s, lab in enumerate(np.asarray(labels).astype(np.int64)):
        if 0 <= lab < W.shape[0] and flat[lab] <= 0:
            g[s, lab] -= factor * W[lab]
    return g


def threshold_sensitivity(pre_times, weights, tau_s, theta, delta_theta, max_n_spike, max_simulation=INF,
                          rel_count=1e-5, rel_time=1e-6):
    """Conditioning of the forward pass, for comparing an FP32 evaluation with this float64 one.

    Returns (n_lo, n_hi, t_sens): the spike-count range over thresholds theta*(1 -+ rel_count) (a count
    outside [n_lo, n_hi] is a real disagreement; inside it, the membrane maximum lies within rel_count of
    the threshold) and, per spike slot, |t(theta*(1+rel_time)) - t(theta*(1-rel_time))| / 2, the spike
    time's sensitivity to a relative perturbation of the neuron state of size rel_time (inf where the
    count changes within that range)."""
    args = (pre_times, weights, tau_s)
    n1 = lif_forward(*args, theta * (1 - rel_count), delta_theta, max_n_spike, max_simulation)[0]
    n2 = lif_forward(*args, theta * (1 + rel_count), delta_theta, max_n_spike, max_simulation)[0]
    m1 = lif_forward(*args, theta * (1 - rel_time), delta_theta, max_n_spike, max_simulation)
    m2 = lif_forward(*args, theta * (1 + rel_time), delta_theta, max_n_spike, max_simulation)
    same = (m1[0] == m2[0])[:, :, None]
    with np.errstate(invalid="ignore"):
        sens = np.where(same, np.abs(m2[3] - m1[3]) / 2, INF)
    sens = np.where(np.isnan(sens), 0.0, sens)
    return np.minimum(n1, n2), np.maximum(n1, n2), sens


# --------------------------------------------------------------------------------------------
# Independent check of the closed-form forward
# --------------------------------------------------------------------------------------------

def simulate_fixed_step(pre_times, weights, tau_s, theta, delta_theta, t_end, dt=1e-6):
    """Fixed-step integration of the neuron ODE for one sample, exact over each step
    (the brian2 'exact' method of the reference's ground-truth tests,
    tests/CudaKernels/Inference/compute_spike_times_tests.py:10-28): an input arriving in a step is
    applied at the end of that step (v += w), u is then tested against theta and reset by
    delta_theta. Returns a list of spike-time arrays per post neuron. Spike times carry an error of
    up to dt (plus the input quantisation), like the brian2 reference."""
    W = np.asarray(weights, dtype=np.float64)
    tau = 2.0 * tau_s
    N = W.shape[0]
    et, ej, _ = sort_events(np.asarray(pre_times, dtype=np.float64)[None])[0]
    steps = int(np.ceil(t_end / dt))
    ev_step = np.ceil(et / dt - 1e-9).astype(np.int64)
    du = np.exp(-dt / tau)
    dv = np.exp(-dt / tau_s)
    kappa = tau * tau_s / (tau - tau_s) * (np.exp(-dt / tau) - np.exp(-dt / tau_s))
    u = np.zeros(N)
    v = np.zeros(N)
    spikes = [[] for _ in range(N)]
    m = 0
    for st in range(steps + 1):
        while m < et.size and ev_step[m] <= st:
            v += W[:, ej[m]]
            m += 1
        over = u >= theta
        while over.any():
            for i in np.nonzero(over)[0]:
                spikes[i].append(st * dt)
            u[over] -= delta_theta
            over = u >= theta
        u, v = u * du + v * kappa, v * dv
    return [np.array(x) for x in spikes]
