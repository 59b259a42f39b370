"""Launcher for the reference's own CUDA kernels ("refkern"), for parity checks and GPU timing.

TEST INFRASTRUCTURE ONLY: used by the GPU parity tests and by bench.py to time the reference's
kernels next to ours; never imported by the product. The device code is the reference's
bats/CudaKernels/CuFiles/**/*.cu compiled unmodified into oracle/_ref/*.fatbin by
oracle/build_ref.sh; this file loads it through the CUDA driver API and replays the reference's
Python wrappers and layer methods step by step, with the same grid and block shapes
(one thread per sample, block = (B, 1, 1)). CuPy's library calls become torch calls:
  cp.argpartition(x, arange(S))[:, :S]  -> torch.sort(stable) truncated to S
      (get_sorted_spikes_indices.py:15-16; equal times only reorder FP32 sums, since no spike can
       fall in the empty window between tied events)
  cp.take_along_axis -> torch.gather, cp.sum/cp.mean -> torch.sum/torch.mean, cp.put -> index assignment.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_cuda = None
_modules = {}


def available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "compute_spike_times.fatbin"))


def _driver():
    global _cuda
    if _cuda is None:
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        _cuda = ctypes.CDLL("libcuda.so.1")
    return _cuda


def _function(file: str, name: str):
    key = (file, name, torch.cuda.current_device())
    if key in _modules:
        return _modules[key]
    cu = _driver()
    mod = ctypes.c_void_p()
    path = os.path.join(REF_DIR, file + ".fatbin").encode()
    r = cu.cuModuleLoad(ctypes.byref(mod), path)
    if r != 0:
        raise RuntimeError(f"cuModuleLoad({path!r}) failed with {r}")
    fn = ctypes.c_void_p()
    r = cu.cuModuleGetFunction(ctypes.byref(fn), mod, name.encode())
    if r != 0:
        raise RuntimeError(f"cuModuleGetFunction({name}) failed with {r}")
    _modules[key] = fn
    return fn


def _arg(v):
    if torch.is_tensor(v):
        return ctypes.c_void_p(v.data_ptr())
    if isinstance(v, (np.float32, float)):
        return ctypes.c_float(float(v))
    if isinstance(v, (int, np.integer)):
        return ctypes.c_int(int(v))
    raise TypeError(type(v))


def launch(file: str, name: str, grid, block, args):
    fn = _function(file, name)
    vals = [_arg(a) for a in args]
    params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
    g = tuple(grid) + (1,) * (3 - len(grid))
    b = tuple(block) + (1,) * (3 - len(block))
    if min(g) == 0 or min(b) == 0:
        return
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    r = _driver().cuLaunchKernel(fn, g[0], g[1], g[2], b[0], b[1], b[2], 0, stream, params, None)
    if r != 0:
        raise RuntimeError(f"cuLaunchKernel({name}) failed with {r}")


def f32(x):
    return np.float32(x)


# ---- wrappers (bats/CudaKernels/Wrappers/**) -------------------------------------------------------------------

def compute_pre_exps(spike_times, tau_s, tau):
    B, N, K = spike_times.shape
    es = torch.empty_like(spike_times)
    ee = torch.empty_like(spike_times)
    launch("compute_pre_exps", "compute_pre_exps_kernel", (K, N, 2), (B,), (spike_times, es, ee, f32(tau_s), f32(tau)))
    return es, ee


def get_sorted_spikes_indices(spike_times_per_neuron, n_spike_per_neuron):
    B, N, K = spike_times_per_neuron.shape
    reshaped = spike_times_per_neuron.reshape(B, N * K)
    S = int(n_spike_per_neuron.sum(1).max().item()) if B > 0 else 0
    order = torch.sort(reshaped, dim=1, stable=True).indices[:, :S]
    return (B, N * K), order, reshaped


def get_spike_weights(weights, spike_indices):
    B, S = spike_indices.shape
    n_post, n_pre = weights.shape
    out = torch.empty((B, n_post, S), dtype=torch.float32, device=weights.device)
    launch("get_spike_weights", "get_spike_weights_kernel", (S, n_post, 1), (B,), (weights, spike_indices, out, n_pre))
    return out


def compute_spike_times(spike_times, exp_tau_s, exp_tau, spike_weights, c, delta_theta_tau, tau, max_simulation,
                        max_n_post_spikes):
    B, n_post, S = spike_weights.shape
    K = int(max_n_post_spikes)
    dev = spike_times.device
    n = torch.zeros((B, n_post), dtype=torch.int32, device=dev)
    a = torch.full((B, n_post, K), float("nan"), device=dev)
    x = torch.full((B, n_post, K), float("nan"), device=dev)
    t = torch.full((B, n_post, K), float("inf"), device=dev)
    z = torch.full((B, n_post, K), float("inf"), device=dev)
    launch("compute_spike_times", "compute_spike_times_kernel", (n_post, 1, 1), (B,),
           (spike_times, exp_tau_s, exp_tau, spike_weights, f32(c), f32(delta_theta_tau), f32(tau),
            f32(max_simulation), S, K, n, a, x, t, z))
    return n, a, x, t, z


def compute_spike_times_conv(spike_indices, spike_times, exp_tau_s, exp_tau, weights, c, delta_theta_tau, tau,
                             max_simulation, max_n_post_spikes, pre_shape, post_shape, filters_shape):
    B, S = spike_times.shape
    Xo, Yo, Co = (int(v) for v in post_shape)
    n_post = Xo * Yo * Co
    K = int(max_n_post_spikes)
    dev = spike_times.device
    n = torch.zeros((B, n_post), dtype=torch.int32, device=dev)
    a = torch.full((B, n_post, K), float("nan"), device=dev)
    x = torch.full((B, n_post, K), float("nan"), device=dev)
    t = torch.full((B, n_post, K), float("inf"), device=dev)
    z = torch.full((B, n_post, K), float("inf"), device=dev)
    shp = lambda v: torch.tensor(np.asarray(v, dtype=np.int32), device=dev)
    launch("compute_spike_times_conv", "compute_spike_times_conv_kernel", (Xo, Yo, Co), (B,),
           (spike_indices, spike_times, exp_tau_s, exp_tau, weights, shp(pre_shape), shp(post_shape),
            shp(filters_shape), n_post, f32(c), f32(delta_theta_tau), f32(tau), f32(max_simulation), S, K,
            n, a, x, t, z))
    return n, a, x, t, z


def aggregate_spikes_conv(n_spikes, spike_times, pre_shape, post_shape):
    B, N, K = spike_times.shape
    Xo, Yo, Co = (int(v) for v in post_shape)
    n_post = Xo * Yo * Co
    dev = spike_times.device
    on = torch.zeros((B, n_post), dtype=torch.int32, device=dev)
    ot = torch.empty((B, n_post, 4 * K), dtype=torch.float32, device=dev)
    oi = torch.empty((B, n_post, 4 * K), dtype=torch.int32, device=dev)
    launch("aggregate_spikes_conv", "aggregate_spikes_conv_kernel", (Xo, Yo, Co), (B,),
           (n_spikes, spike_times, torch.tensor(np.asarray(pre_shape, dtype=np.int32), device=dev), K, on, ot, oi))
    order = torch.sort(ot, dim=2, stable=True).indices
    return on, torch.gather(ot, 2, order), torch.gather(oi, 2, order)


def propagate_recurrent_errors(x, exp_tau, errors, delta_theta_tau):
    B, N, K = errors.shape
    launch("propagate_recurrent_errors", "propagate_recurrent_errors_kernel", (N, 1, 1), (B,),
           (x, exp_tau, errors, f32(delta_theta_tau), K))


def compute_factors(spike_times, a, c, x, exp_tau, tau):
    B, N, K = a.shape
    f1 = torch.empty_like(a)
    f2 = torch.empty_like(a)
    launch("compute_factors", "compute_factors_kernel", (K, N, 2), (B,), (spike_times, a, f32(c), x, exp_tau, f32(tau),
                                                                           f1, f2))
    return f1, f2


def compute_weights_gradient(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, errors):
    B, n_post, k_post = f1.shape
    _, n_pre, k_pre = pre_exp_tau_s.shape
    g = torch.zeros((B, n_post, n_pre), dtype=torch.float32, device=f1.device)
    launch("compute_weights_gradient", "compute_weights_gradient_kernel", (n_post, n_pre), (B,),
           (f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, errors, g, k_post, k_pre))
    return g


def sample_chunks(batch, per_sample, limit=2 ** 31 - 1):
    """(start, stop) sample ranges for the error-propagation kernels, whose element index into their
    (B, N_pre, K_pre, N_post) temporary, (sample * N_pre * K_pre + ...) * N_post, is formed in 32-bit integers
    (propagate_errors_to_pre_spikes.cu:23-31 signed, propagate_errors_to_pre_spikes_conv.cu:55-63 unsigned):
    batches whose temporary has 2^31 elements or more are launched in chunks of samples below that size
    (samples are independent, so each sample's result is that of one launch). The reference's own wrappers
    launch the whole batch at once; for such batches that index would wrap."""
    step = max(1, limit // max(1, per_sample))
    return [(c0, min(batch, c0 + step)) for c0 in range(0, batch, step)]


def propagate_errors_to_pre_spikes(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, weights, errors, tau_s,
                                   tau):
    B, n_post, k_post = f1.shape
    _, n_pre, k_pre = pre_exp_tau_s.shape
    out = torch.empty((B, n_pre, k_pre), dtype=torch.float32, device=f1.device)
    for c0, c1 in sample_chunks(B, n_pre * k_pre * n_post):
        sl = slice(c0, c1)
        tmp = torch.zeros((c1 - c0, n_pre, k_pre, n_post), dtype=torch.float32, device=f1.device)
        launch("propagate_errors_to_pre_spikes", "propagate_errors_to_pre_spikes_kernel", (n_pre, k_pre, n_post),
               (c1 - c0,), (f1[sl], f2[sl], post_times[sl], pre_times[sl], pre_exp_tau_s[sl], pre_exp_tau[sl],
                            weights, errors[sl], tmp, k_post, f32(tau_s), f32(tau)))
        out[sl] = tmp.sum(dim=3)
        del tmp
    return out


def compute_weights_gradient_conv(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, pre_shape, post_shape,
                                  filter_shape, errors):
    B, n_post, k_post = f1.shape
    _, n_pre, k_pre = pre_exp_tau_s.shape
    C_out, fx, fy, C = (int(v) for v in filter_shape)
    dev = f1.device
    g = torch.zeros((B, C_out, fx, fy, C), dtype=torch.float32, device=dev)
    shp = lambda v: torch.tensor(np.asarray(v, dtype=np.int32), device=dev)
    launch("compute_weights_gradient_conv", "compute_weights_gradient_conv_kernel", (fx, fy, C), (B,),
           (f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, errors, shp(pre_shape), shp(post_shape),
            shp(filter_shape), g, n_post, n_pre, k_post, k_pre))
    return g


def propagate_errors_to_pre_spikes_conv(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, weights, errors,
                                        tau_s, tau, pre_shape, post_shape, filter_shape):
    B, n_post, k_post = f1.shape
    _, n_pre, k_pre = pre_exp_tau_s.shape
    C_out, fx, fy, C = (int(v) for v in filter_shape)
    nf = C_out * fx * fy
    dev = f1.device
    shp = lambda v: torch.tensor(np.asarray(v, dtype=np.int32), device=dev)
    out = torch.empty((B, n_pre, k_pre), dtype=torch.float32, device=dev)
    for c0, c1 in sample_chunks(B, n_pre * k_pre * nf):
        sl = slice(c0, c1)
        tmp = torch.zeros((c1 - c0, n_pre, k_pre, nf), dtype=torch.float32, device=dev)
        launch("propagate_errors_to_pre_spikes_conv", "propagate_errors_to_pre_spikes_conv_kernel",
               (n_pre, k_pre, nf), (c1 - c0,),
               (f1[sl], f2[sl], post_times[sl], pre_times[sl], pre_exp_tau_s[sl], pre_exp_tau[sl], weights,
                errors[sl], shp(post_shape), shp(pre_shape), shp(filter_shape), tmp, n_post, k_post, f32(tau_s),
                f32(tau)))
        out[sl] = tmp.sum(dim=3)
        del tmp
    return out


# ---- layers (bats/Layers/LIFLayer.py:63-110, ConvLIFLayer.py:77-134, PoolingLayer.py:49-66) --------------------

def _constants(tau_s, theta, delta_theta):
    tau = np.float32(2 * float(tau_s))
    return np.float32(tau_s), tau, np.float32(float(theta) / float(tau)), np.float32(float(delta_theta) / float(tau))


class RefLIF:
    """LIFLayer.forward/backward with the reference kernels (block = B <= 1024)."""

    def __init__(self, weights, tau_s, theta, delta_theta, max_n_spike):
        self.w = weights.contiguous()
        self.tau_s, self.tau, self.c, self.dtt = _constants(tau_s, theta, delta_theta)
        self.K = int(max_n_spike)

    def forward(self, pre_t, pre_n, max_simulation=np.inf):
        self.pre_t = pre_t
        self.es, self.ee = compute_pre_exps(pre_t, self.tau_s, self.tau)
        new_shape, idx, reshaped = get_sorted_spikes_indices(pre_t, pre_n)
        B = pre_t.shape[0]
        n_post = self.w.shape[0]
        if idx.numel() == 0:
            shape = (B, n_post, self.K)
            dev = pre_t.device
            self.out = (torch.zeros((B, n_post), dtype=torch.int32, device=dev),
                        *(torch.full(shape, float("inf"), device=dev) for _ in range(4)))
            return self.out
        sidx = (idx // pre_t.shape[2]).to(torch.int32).contiguous()
        st = torch.gather(reshaped, 1, idx).contiguous()
        ses = torch.gather(self.es.reshape(new_shape), 1, idx).contiguous()
        see = torch.gather(self.ee.reshape(new_shape), 1, idx).contiguous()
        sw = get_spike_weights(self.w, sidx)
        self.out = compute_spike_times(st, ses, see, sw, self.c, self.dtt, self.tau, max_simulation, self.K)
        return self.out

    def backward(self, errors, want_pre=True):
        n, a, x, t, z = self.out
        propagate_recurrent_errors(x, z, errors, self.dtt)
        f1, f2 = compute_factors(t, a, self.c, x, z, self.tau)
        g = compute_weights_gradient(f1, f2, t, self.pre_t, self.es, self.ee, errors)
        pre = propagate_errors_to_pre_spikes(f1, f2, t, self.pre_t, self.es, self.ee, self.w, errors, self.tau_s,
                                             self.tau) if want_pre else None
        return g, pre


class RefConvLIF:
    """ConvLIFLayer.forward/backward with the reference kernels."""

    def __init__(self, filters, pre_shape, tau_s, theta, delta_theta, max_n_spike):
        self.w = filters.contiguous()
        C_out, fx, fy, C = self.w.shape
        self.pre_shape = np.asarray(pre_shape, dtype=np.int32)
        self.post_shape = np.array([pre_shape[0] - fx + 1, pre_shape[1] - fy + 1, C_out], dtype=np.int32)
        self.filter_shape = np.array([C_out, fx, fy, C], dtype=np.int32)
        self.tau_s, self.tau, self.c, self.dtt = _constants(tau_s, theta, delta_theta)
        self.K = int(max_n_spike)

    def forward(self, pre_t, pre_n, max_simulation=np.inf):
        self.pre_t = pre_t
        self.es, self.ee = compute_pre_exps(pre_t, self.tau_s, self.tau)
        new_shape, idx, reshaped = get_sorted_spikes_indices(pre_t, pre_n)
        B = pre_t.shape[0]
        n_post = int(np.prod(self.post_shape))
        if idx.numel() == 0:
            dev = pre_t.device
            self.out = (torch.zeros((B, n_post), dtype=torch.int32, device=dev),
                        *(torch.full((B, n_post, self.K), float("inf"), device=dev) for _ in range(4)))
            return self.out
        sidx = (idx // pre_t.shape[2]).to(torch.int32).contiguous()
        st = torch.gather(reshaped, 1, idx).contiguous()
        ses = torch.gather(self.es.reshape(new_shape), 1, idx).contiguous()
        see = torch.gather(self.ee.reshape(new_shape), 1, idx).contiguous()
        self.out = compute_spike_times_conv(sidx, st, ses, see, self.w, self.c, self.dtt, self.tau, max_simulation,
                                            self.K, self.pre_shape, self.post_shape, self.filter_shape)
        return self.out

    def backward(self, errors, want_pre=True):
        n, a, x, t, z = self.out
        propagate_recurrent_errors(x, z, errors, self.dtt)
        f1, f2 = compute_factors(t, a, self.c, x, z, self.tau)
        g = compute_weights_gradient_conv(f1, f2, t, self.pre_t, self.es, self.ee, self.pre_shape, self.post_shape,
                                          self.filter_shape, errors)
        pre = propagate_errors_to_pre_spikes_conv(f1, f2, t, self.pre_t, self.es, self.ee, self.w, errors, self.tau_s,
                                                  self.tau, self.pre_shape, self.post_shape,
                                                  self.filter_shape) if want_pre else None
        return g, pre


def pool_forward(n_spikes, times, pre_shape):
    X, Y, C = (int(v) for v in pre_shape)
    return aggregate_spikes_conv(n_spikes, times, pre_shape, (X // 2, Y // 2, C))


def pool_backward(errors, indices, pre_bnk):
    out = torch.empty(int(np.prod(pre_bnk)), dtype=torch.float32, device=errors.device)
    out[indices.reshape(-1).long()] = errors.reshape(-1)
    return out.reshape(pre_bnk)
