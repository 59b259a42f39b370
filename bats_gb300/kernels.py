"""Python wrappers of the C ABI, one per reference kernel wrapper (bats/CudaKernels/Wrappers/).

Every function takes and returns CUDA torch tensors, allocates its outputs with torch, and launches
on the current torch stream. Names and argument meanings follow the reference wrappers; the
functions that take over several reference steps at once (sort_events, lif_forward_fc,
backward_prep) say which.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from ._lib import call, ptr, stream_ptr
from .workspace import workspace

F32 = torch.float32
I32 = torch.int32


def _c(t, dtype=F32):
    """Contiguous CUDA tensor of `dtype`."""
    if not torch.is_tensor(t):
        t = torch.as_tensor(np.asarray(t), dtype=dtype, device="cuda")
    if t.dtype != dtype:
        t = t.to(dtype)
    if not t.is_cuda:
        t = t.cuda()
    return t.contiguous()


def _out(out, shape, dtype=F32):
    """A caller-supplied output: the kernels write through its raw pointer in row-major order, so it must be a
    contiguous CUDA tensor of exactly `shape` and `dtype` (any other layout would be filled wrongly)."""
    if (not torch.is_tensor(out) or not out.is_cuda or out.dtype != dtype or not out.is_contiguous()
            or tuple(out.shape) != tuple(shape)):
        raise ValueError(f"out must be a contiguous CUDA {dtype} tensor of shape {tuple(shape)}")
    return out


def lif_constants(tau_s, theta, delta_theta):
    """(tau, theta/tau, delta_theta/tau) as float32, the way LIFLayer.__init__ forms them
    (bats/Layers/LIFLayer.py:16-19): tau = float32(2 tau_s), the quotients taken in double and rounded."""
    tau32 = np.float32(2 * float(tau_s))
    return tau32, np.float32(float(theta) / float(tau32)), np.float32(float(delta_theta) / float(tau32))


def padded_ld(n: int) -> int:
    """Leading dimension of transposed weights: rows padded to 32 floats (128 bytes)."""
    return max(32, (n + 31) // 32 * 32)


def transpose_weights(weights, out=None):
    """wt (N_pre, ld) = weights (N_post, N_pre)^T, ld = padded_ld(N_post)."""
    w = _c(weights)
    n_post, n_pre = w.shape
    ld = padded_ld(n_post)
    if out is None:
        out = torch.zeros((n_pre, ld), dtype=F32, device=w.device)
    else:
        out = _out(out, (n_pre, ld))
    call("bats_transpose", ptr(w), n_post, n_pre, ptr(out), ld, stream_ptr())
    return out


BUCKET_WIDTH = 32  # pre neurons per bucket of the weight-gradient kernel


@dataclass
class Events:
    """Time-sorted pre-synaptic spikes of a batch: events (B, cap, 4) 16-byte records, the source slot
    of each event (B, cap), and the number of events per sample (B); for the backward pass also the
    same events grouped in buckets of BUCKET_WIDTH pre neurons (time order kept inside a bucket) with
    the bucket offsets (B, n_buckets + 1)."""
    events: torch.Tensor
    slots: torch.Tensor
    counts: torch.Tensor
    n_neurons: int
    k: int
    bucketed: torch.Tensor | None = None
    bucket_offsets: torch.Tensor | None = None
    bucket_width: int = BUCKET_WIDTH

    @property
    def cap(self) -> int:
        return self.n_neurons * self.k

    @property
    def batch(self) -> int:
        return self.events.shape[0]


def alloc_events(batch: int, n_neurons: int, k: int, device="cuda", bucketed: bool = True,
                 bucket_width: int = BUCKET_WIDTH) -> Events:
    cap = n_neurons * k
    ev = Events(torch.empty((batch, cap, 4), dtype=F32, device=device),
                torch.empty((batch, cap), dtype=I32, device=device),
                torch.empty((batch,), dtype=I32, device=device), n_neurons, k, bucket_width=int(bucket_width))
    n_buckets = (n_neurons + bucket_width - 1) // bucket_width
    if bucketed and n_buckets <= 255:
        ev.bucketed = torch.empty((batch, cap, 4), dtype=F32, device=device)
        ev.bucket_offsets = torch.empty((batch, n_buckets + 1), dtype=I32, device=device)
    return ev


def sample_order(ev_count) -> torch.Tensor:
    """The samples longest first by their event counts ev_count (B,) int32 (bats_sample_order), as an int32
    permutation of 0 .. B-1 on ev_count's device."""
    c = _c(ev_count, I32)
    order = torch.empty(c.shape[0], dtype=I32, device=c.device)
    call("bats_sample_order", ptr(c), c.shape[0], ptr(order), stream_ptr())
    return order


def order_pays(batch: int, device) -> bool:
    """Whether a longest-first sample order can shorten a one-CTA-per-sample launch of the counted sort:
    only when the batch is wider than its resident CTAs (two per SM)."""
    if not torch.cuda.is_available():
        return batch > 2 * 152
    return batch > 2 * torch.cuda.get_device_properties(device).multi_processor_count


def sort_events(spike_times, tau_s: float, tau: float, exp_tau_s=None, exp_tau=None, out: Events | None = None,
                bucketed: bool = True, bucket_width: int = BUCKET_WIDTH, pre_counts=None, sample_order=None):
    """Per-sample time sort of all valid pre-spikes (replaces get_sorted_spikes_indices, the
    take_along_axis gathers and compute_pre_exps; bats/Layers/LIFLayer.py:66-84). With `bucketed`, also
    the bucketed copy used by the weight gradient. `pre_counts` (B, N) int32, the spike counts of a LIF
    layer's output (slots past each count are +inf), lets the sort read only the slots below the counts;
    with it, `sample_order` (B,) int32, a permutation of the samples (sample_order above), sets the order in
    which the sort's CTAs take them (the results do not depend on it)."""
    t = _c(spike_times)
    B, N, K = t.shape
    if out is None:
        out = alloc_events(B, N, K, t.device, bucketed=bucketed, bucket_width=bucket_width)
    ws_bytes = call_size("bats_sort_events_workspace_bytes", B, N, K)
    ws = workspace(ws_bytes, t.device) if ws_bytes else None
    es = _c(exp_tau_s) if exp_tau_s is not None else None
    ee = _c(exp_tau) if exp_tau is not None else None
    if pre_counts is not None:
        pc = _c(pre_counts, I32)
        assert tuple(pc.shape) == (B, N), "pre_counts must be (B, N)"
        if sample_order is not None:
            so = _c(sample_order, I32)
            assert tuple(so.shape) == (B,), "sample_order must be (B,)"
            call("bats_sort_events_counted_ordered", ptr(t), ptr(pc), B, N, K, float(tau_s), float(tau), ptr(es),
                 ptr(ee), ptr(out.events), ptr(out.slots), ptr(out.counts), ptr(out.bucketed),
                 ptr(out.bucket_offsets), out.bucket_width, ptr(so), ptr(ws), ws_bytes, stream_ptr())
            return out
        call("bats_sort_events_counted", ptr(t), ptr(pc), B, N, K, float(tau_s), float(tau), ptr(es), ptr(ee),
             ptr(out.events), ptr(out.slots), ptr(out.counts), ptr(out.bucketed), ptr(out.bucket_offsets),
             out.bucket_width, ptr(ws), ws_bytes, stream_ptr())
        return out
    assert sample_order is None, "sample_order needs pre_counts"
    call("bats_sort_events", ptr(t), B, N, K, float(tau_s), float(tau), ptr(es), ptr(ee), ptr(out.events),
         ptr(out.slots), ptr(out.counts), ptr(out.bucketed), ptr(out.bucket_offsets), out.bucket_width, ptr(ws),
         ws_bytes, stream_ptr())
    return out


def copy_on_stream(dst: torch.Tensor, src: torch.Tensor, stream: int) -> None:
    """dst <- src (same shape, contiguous: one device-to-device copy) enqueued on the raw CUDA stream
    `stream`, the stream argument of a train step's launches."""
    assert dst.shape == src.shape and dst.dtype == src.dtype and dst.is_contiguous() and src.is_contiguous()
    call("bats_copy_device", ptr(dst), ptr(src), dst.numel() * dst.element_size(), stream)


def call_size(name, *args) -> int:
    from ._lib import load
    return int(getattr(load(), name)(*args))


def compute_pre_exps(spike_times, tau_s, tau):
    """exp(t/tau_s), exp(t/tau) (bats/CudaKernels/Wrappers/Inference/compute_pre_exps.py:10-18)."""
    t = _c(spike_times)
    es = torch.empty_like(t)
    ee = torch.empty_like(t)
    call("bats_compute_pre_exps", ptr(t), t.numel(), float(tau_s), float(tau), ptr(es), ptr(ee), stream_ptr())
    return es, ee


def get_sorted_spikes_indices(spike_times_per_neuron, n_spike_per_neuron):
    """Compatibility form of the reference's sort (Wrappers/Inference/get_sorted_spikes_indices.py:7-17):
    returns (new_shape, sorted_indices (B, S) int64, spike_times_reshaped) with S the largest spike count
    of the batch (one host read) and sorted_indices pointing at inf slots past a sample's spikes."""
    t = _c(spike_times_per_neuron)
    B, N, K = t.shape
    ev = sort_events(t, 1.0, 1.0, bucketed=False)
    S = int(ev.counts.max().item()) if B > 0 else 0
    reshaped = t.reshape(B, N * K)
    idx = ev.slots[:, :S].to(torch.int64)
    # Fill the tail of short samples with their (inf) unused slots, in slot order.
    pos = torch.arange(S, device=t.device)[None, :]
    short = pos >= ev.counts[:, None].to(torch.int64)
    if short.any():
        for s in torch.nonzero(short.any(1)).flatten().tolist():
            n = int(ev.counts[s])
            spare = torch.nonzero(~(reshaped[s] < float("inf"))).flatten()[: S - n]
            idx[s, n:] = spare
    return (B, N * K), idx, reshaped


FWD_AUTO, FWD_TILE, FWD_LANES, FWD_TILE64 = 0, 1, 2, 3
FWD_NO_PAD = 0x100  # OR-ed into the algo: no +inf past the spike counts (outputs read only below them)
FWD_STAGE = 0x200  # OR-ed into a tile or queue algo: one no-crossing test per neuron and stage first (quiet layers)
# Python-side choices that route to bats_lif_forward_fc_queue (one persistent launch over a work queue of
# (sample, tile) items, longest samples first), with the tile width of FWD_TILE or FWD_TILE64.
FWD_QUEUE, FWD_QUEUE64 = 4, 5


def is_queue_algo(algo: int) -> bool:
    return (algo & ~(FWD_NO_PAD | FWD_STAGE)) in (FWD_QUEUE, FWD_QUEUE64)


def queue_workspace_bytes(batch: int) -> int:
    return call_size("bats_lif_forward_fc_queue_workspace_bytes", int(batch))


def forward_fc_call(events: Events, weights_t, n_post: int, k_post: int, c, dtt, tau32, max_simulation, outs,
                    algo: int, stream: int, workspace=None, workspace_bytes: int = 0):
    """One FC forward launch through the C ABI: bats_lif_forward_fc_queue for FWD_QUEUE / FWD_QUEUE64 (with the
    given workspace), bats_lif_forward_fc_algo otherwise."""
    n, a, x, t, z = outs
    common = (ptr(events.events), ptr(events.counts), events.cap, ptr(weights_t), weights_t.shape[1], events.batch,
              n_post, k_post, float(c), float(dtt), float(tau32), float(np.float32(max_simulation)), ptr(n), ptr(a),
              ptr(x), ptr(t), ptr(z))
    if is_queue_algo(algo):
        tile = FWD_TILE64 if (algo & ~(FWD_NO_PAD | FWD_STAGE)) == FWD_QUEUE64 else FWD_TILE
        call("bats_lif_forward_fc_queue", *common, tile | (algo & (FWD_NO_PAD | FWD_STAGE)), workspace,
             int(workspace_bytes), stream)
    else:
        call("bats_lif_forward_fc_algo", *common, int(algo), stream)


def lif_forward_fc(events: Events, weights_t, n_post: int, k_post: int, tau_s: float, theta: float,
                   delta_theta: float, max_simulation: float = float("inf"), outs=None, algo: int = FWD_AUTO):
    """FC LIF forward (replaces get_spike_weights + compute_spike_times,
    bats/CudaKernels/Wrappers/Inference/compute_spike_times.py:11-32). Returns n, a, x, times, post_exp_tau.
    algo: FWD_TILE (CTA per neuron tile and sample), FWD_LANES (warp per neuron and sample, 32 events in
    parallel), FWD_QUEUE / FWD_QUEUE64 (persistent CTAs over a longest-first work queue) or FWD_AUTO, the tile
    and queue kinds optionally with FWD_STAGE (one no-crossing test per stage first); all give identical
    results."""
    B = events.batch
    tau32, c, dtt = lif_constants(tau_s, theta, delta_theta)
    dev = events.events.device
    if outs is None:
        outs = (torch.empty((B, n_post), dtype=I32, device=dev),
                *(torch.empty((B, n_post, k_post), dtype=F32, device=dev) for _ in range(4)))
    ws = None
    if is_queue_algo(algo):
        ws = torch.empty(queue_workspace_bytes(B), dtype=torch.uint8, device=dev)
    forward_fc_call(events, weights_t, n_post, k_post, c, dtt, tau32, max_simulation, outs, algo, stream_ptr(),
                    ptr(ws), 0 if ws is None else ws.numel())
    return tuple(outs)


def conv_forward(events: Events, filters, pre_shape, k_post: int, tau_s: float, theta: float, delta_theta: float,
                 max_simulation: float = float("inf"), outs=None):
    """Conv LIF forward (replaces compute_spike_times_conv, Wrappers/Inference/compute_spike_times_conv.py:11-35)."""
    W = _c(filters)
    C_out, fx, fy, C = W.shape
    X, Y, Cp = (int(v) for v in pre_shape)
    assert Cp == C, "filter input channels must match the previous layer"
    Xo, Yo = X - fx + 1, Y - fy + 1
    B = events.batch
    n_post = Xo * Yo * C_out
    tau32, c, dtt = lif_constants(tau_s, theta, delta_theta)
    dev = events.events.device
    if outs is None:
        outs = (torch.empty((B, n_post), dtype=I32, device=dev),
                *(torch.empty((B, n_post, k_post), dtype=F32, device=dev) for _ in range(4)))
    n, a, x, t, z = outs
    call("bats_conv_forward", ptr(events.events), ptr(events.counts), events.cap, ptr(W), B, X, Y, C, fx, fy, C_out,
         k_post, float(c), float(dtt), float(tau32), float(np.float32(max_simulation)), ptr(n), ptr(a), ptr(x),
         ptr(t), ptr(z), stream_ptr())
    return n, a, x, t, z


def convert_to_spike_per_neuron(indices, times, n_neurons: int, k_cap: int | None = None, overflow=None):
    """Event list (B, S) of (neuron index, time), index < 0 ending a sample, into per-neuron spike trains
    (B, N, K) + counts (B, N) (Wrappers/Inference/convert_to_spike_per_neuron.py:20-33). With k_cap None,
    K is the batch's largest per-neuron count, as in the reference (one host read); otherwise K = k_cap and
    spikes beyond it are dropped (counted in `overflow`, an int32 CUDA tensor of one element)."""
    idx = _c(indices, I32)
    tm = _c(times)
    B, S = idx.shape
    dev = idx.device
    if k_cap is None:
        scratch = torch.empty((B, int(n_neurons)), dtype=I32, device=dev)
        mx = torch.empty((B,), dtype=I32, device=dev)
        call("bats_events_max_per_neuron", ptr(idx), B, S, int(n_neurons), ptr(scratch), ptr(mx), stream_ptr())
        k_cap = max(1, int(mx.max().item())) if B > 0 else 1
    out_t = torch.empty((B, int(n_neurons), int(k_cap)), dtype=F32, device=dev)
    out_n = torch.empty((B, int(n_neurons)), dtype=I32, device=dev)
    call("bats_events_to_trains", ptr(idx), ptr(tm), B, S, int(n_neurons), int(k_cap), ptr(out_t), ptr(out_n),
         ptr(overflow), stream_ptr())
    return out_t, out_n


def intensity_to_spike_times(pixels, time_window: float = 100e-3, max_value: float = 255.0):
    """8-bit intensities (B, N) -> single-spike trains (B, N, 1) and counts (B, N)
    (experiments/mnist/Dataset.py:66-71: t = time_window * (1 - x / max_value), no spike where x == 0)."""
    px = _c(pixels, torch.uint8)
    B, N = px.shape
    times = torch.empty((B, N, 1), dtype=F32, device=px.device)
    counts = torch.empty((B, N), dtype=I32, device=px.device)
    call("bats_intensity_to_spike_times", ptr(px), B, N, float(time_window), float(max_value), ptr(times),
         ptr(counts), stream_ptr())
    return times, counts


def aggregate_spikes_conv(n_spikes, spike_times, pre_shape):
    """2x2 pooling (replaces aggregate_spikes_conv + argsort, Wrappers/Inference/aggregate_spikes_conv.py:10-28).
    Returns (n_spikes (B, N_out), times (B, N_out, 4K), indices (B, N_out, 4K) int32)."""
    n = _c(n_spikes, I32)
    t = _c(spike_times)
    B, N, K = t.shape
    X, Y, C = (int(v) for v in pre_shape)
    n_out = (X // 2) * (Y // 2) * C
    on = torch.empty((B, n_out), dtype=I32, device=t.device)
    ot = torch.empty((B, n_out, 4 * K), dtype=F32, device=t.device)
    oi = torch.empty((B, n_out, 4 * K), dtype=I32, device=t.device)
    call("bats_pool_forward", ptr(n), ptr(t), B, X, Y, C, K, ptr(on), ptr(ot), ptr(oi), stream_ptr())
    return on, ot, oi


def pool_backward(errors, indices, pre_shape_bnk):
    """pre_errors[indices] = errors (bats/Layers/PoolingLayer.py:55-66)."""
    e = _c(errors)
    idx = _c(indices, I32)
    out = torch.empty(pre_shape_bnk, dtype=F32, device=e.device)
    call("bats_pool_backward", ptr(e), ptr(idx), e.numel(), ptr(out), out.numel(), stream_ptr())
    return out


@dataclass
class BackwardTables:
    f1: torch.Tensor
    f2: torch.Tensor
    tables: torch.Tensor  # (B, N, K+1, 2)
    nvalid: torch.Tensor  # (B, N)
    heads: torch.Tensor | None = None  # cursor heads (bats_cursor_heads_bytes), written by the counted prep


def alloc_cursor_heads(batch: int, n_post: int, device="cuda") -> torch.Tensor:
    """Buffer for the cursor heads of bats_backward_prep_counted / bats_weights_gradient (uint8, 16-byte
    aligned as torch allocations are)."""
    return torch.empty(max(1, call_size("bats_cursor_heads_bytes", batch, n_post)), dtype=torch.uint8, device=device)


def backward_prep(post_times, a, x, post_exp_tau, errors, c: float, tau: float, delta_theta_tau: float,
                  recurrent: bool = True, out: BackwardTables | None = None, want_factors: bool = False,
                  n_spikes=None) -> BackwardTables:
    """Reset errors in place + factors + suffix tables (replaces propagate_recurrent_errors and
    compute_factors, Wrappers/Backpropagation/propagate_recurrent_errors.py:9-16, compute_factors.py:11-22).
    For the forward kernels' outputs (the layer path); f1/f2 are only materialised if want_factors. With the
    forward's spike counts `n_spikes` (B, N) only the slots below them are read."""
    B, N, K = post_times.shape
    dev = post_times.device
    need_f = want_factors or K > 32 or not recurrent
    counted = recurrent and n_spikes is not None and not need_f
    if out is None:
        out = BackwardTables(torch.empty((B, N, K), dtype=F32, device=dev) if need_f else None,
                             torch.empty((B, N, K), dtype=F32, device=dev) if need_f else None,
                             torch.empty((B, N, K + 1, 2), dtype=F32, device=dev),
                             torch.empty((B, N), dtype=I32, device=dev),
                             alloc_cursor_heads(B, N, dev) if counted else None)
    if not counted:
        out.heads = None  # only the counted prep writes the cursor heads
    if counted:
        call("bats_backward_prep_counted", ptr(post_times), ptr(_c(n_spikes, I32)), ptr(a), ptr(x),
             ptr(post_exp_tau), ptr(errors), B, N, K, float(c), float(tau), float(delta_theta_tau),
             ptr(out.tables), ptr(out.nvalid), ptr(out.heads), stream_ptr())
    elif recurrent:
        call("bats_backward_prep_layer", ptr(post_times), ptr(a), ptr(x), ptr(post_exp_tau), ptr(errors), B, N, K,
             float(c), float(tau), float(delta_theta_tau), ptr(out.f1), ptr(out.f2), ptr(out.tables),
             ptr(out.nvalid), stream_ptr())
    else:
        call("bats_backward_prep", ptr(post_times), ptr(a), ptr(x), ptr(post_exp_tau), ptr(errors), B, N, K,
             float(c), float(tau), float(delta_theta_tau), 0, 1, ptr(out.f1), ptr(out.f2), ptr(out.tables),
             ptr(out.nvalid), stream_ptr())
    return out


def tables_from_factors(post_times, f1, f2, errors) -> BackwardTables:
    """Suffix tables from given factors and errors (no recurrent step)."""
    t, f1, f2, e = _c(post_times), _c(f1), _c(f2), _c(errors)
    B, N, K = t.shape
    out = BackwardTables(f1, f2, torch.empty((B, N, K + 1, 2), dtype=F32, device=t.device),
                         torch.empty((B, N), dtype=I32, device=t.device))
    call("bats_backward_prep", ptr(t), None, None, None, ptr(e), B, N, K, 0.0, 1.0, 0.0, 0, 0, ptr(f1), ptr(f2),
         ptr(out.tables), ptr(out.nvalid), stream_ptr())
    return out


def propagate_recurrent_errors(x, exp_tau, errors, delta_theta_tau):
    """In place on `errors` (Wrappers/Backpropagation/propagate_recurrent_errors.py:9-16)."""
    x, z = _c(x), _c(exp_tau)
    B, N, K = errors.shape
    call("bats_backward_prep", ptr(z), None, ptr(x), ptr(z), ptr(errors), B, N, K, 0.0, 1.0, float(delta_theta_tau),
         1, 0, None, None, None, None, stream_ptr())


def compute_factors(spike_times, a, c, x, exp_tau, tau):
    """f1, f2 (Wrappers/Backpropagation/compute_factors.py:11-22)."""
    t, a, x, z = _c(spike_times), _c(a), _c(x), _c(exp_tau)
    B, N, K = t.shape
    f1 = torch.empty_like(t)
    f2 = torch.empty_like(t)
    dummy = torch.empty((1,), dtype=F32, device=t.device)
    call("bats_backward_prep", ptr(t), ptr(a), ptr(x), ptr(z), ptr(dummy), B, N, K, float(c), float(tau), 0.0, 0, 1,
         ptr(f1), ptr(f2), None, None, stream_ptr())
    return f1, f2


def weights_gradient(events: Events, post_times, tabs: BackwardTables, n_pre: int, per_sample: bool = True,
                     group: int | None = None, out=None, reduce: str = "mean"):
    """Per-sample gradient (B, N_post, N_pre) like compute_weights_gradient
    (Wrappers/Backpropagation/compute_weights_gradient.py:10-24), or its batch mean / sum (N_post, N_pre)."""
    B, n_post, k_post = post_times.shape
    dev = post_times.device
    if per_sample:
        g = 1
        shape = (B, n_post, n_pre)
    else:
        g = max(2, int(group or default_group(B, n_post, n_pre)))  # group >= 2 selects the batch-reduced path
        shape = (n_post, n_pre)
    if out is None:
        out = torch.empty(shape, dtype=F32, device=dev)
    else:
        out = _out(out, shape)
    ws_bytes = call_size("bats_weights_gradient_workspace_bytes", B, n_post, n_pre, g)
    ws = workspace(ws_bytes, dev) if ws_bytes else None
    # The bucketed copy serves this kernel only when it is grouped by BUCKET_WIDTH pre neurons.
    by_bucket = events.bucketed is not None and events.bucket_width == BUCKET_WIDTH
    call("bats_weights_gradient", ptr(events.events), ptr(events.counts), ptr(events.bucketed if by_bucket else None),
         ptr(events.bucket_offsets if by_bucket else None), events.cap, ptr(post_times), ptr(tabs.tables),
         ptr(tabs.nvalid), ptr(tabs.heads), B, n_post,
         k_post, n_pre, g, int(reduce == "mean"), ptr(out), ptr(ws), ws_bytes, stream_ptr())
    return out


def grad_tile(n_post: int) -> int:
    return 32 if n_post <= 32 else 64


def default_group(batch: int, n_post: int, n_pre: int, target_ctas: int = 2432) -> int:
    """Samples per group of the batch-reduced weight gradient: enough groups for ~16 two-warp CTAs per SM of
    a 152-SM GB300, but at most 32 partial gradients (narrow layers, N_post <= 32, whose partials are small
    and whose kernel runs one warp per bucket and group: up to 4 warps per SM, any number of partials)."""
    if n_post <= 32:
        buckets = (n_pre + BUCKET_WIDTH - 1) // BUCKET_WIDTH
        groups = max(1, min(batch, -(-4 * 152 // buckets)))
        return max(1, -(-batch // groups))
    tiles = (n_post + grad_tile(n_post) - 1) // grad_tile(n_post)
    buckets = (n_pre + BUCKET_WIDTH - 1) // BUCKET_WIDTH
    groups = max(1, min(batch, -(-target_ctas // (tiles * buckets)), 32))
    return max(1, -(-batch // groups))


def pre_errors(events: Events, weights_t, post_times, tabs: BackwardTables, tau_s: float, tau: float, out=None):
    """Errors of the pre-spikes (B, N_pre, K_pre) (replaces propagate_errors_to_pre_spikes,
    Wrappers/Backpropagation/propagate_errors_to_pre_spikes.py:11-27)."""
    B, n_post, k_post = post_times.shape
    dev = post_times.device
    if out is None:
        out = torch.empty((B, events.n_neurons, events.k), dtype=F32, device=dev)
    else:
        out = _out(out, (B, events.n_neurons, events.k))
    ws_bytes = call_size("bats_pre_errors_workspace_bytes", B, events.cap, n_post)
    ws = workspace(ws_bytes, dev) if ws_bytes else None
    call("bats_pre_errors", ptr(events.events), ptr(events.slots), ptr(events.counts), events.cap, ptr(weights_t),
         weights_t.shape[1], ptr(post_times), ptr(tabs.tables), ptr(tabs.nvalid), B, n_post, k_post,
         events.n_neurons, events.k, float(tau_s), float(tau), ptr(out), ptr(ws), ws_bytes, stream_ptr())
    return out


def conv_backward(events: Events, filters, pre_shape, post_times, tabs: BackwardTables, tau_s: float, tau: float,
                  want_pre_errors: bool = True):
    """Per-sample filter gradient (B, C_out, fx, fy, C) and pre errors (replaces compute_weights_gradient_conv
    and propagate_errors_to_pre_spikes_conv, Wrappers/Backpropagation/*_conv.py)."""
    W = _c(filters)
    C_out, fx, fy, C = W.shape
    X, Y, _ = (int(v) for v in pre_shape)
    B, n_post, k_post = post_times.shape
    dev = post_times.device
    grad = torch.empty((B, C_out, fx, fy, C), dtype=F32, device=dev)
    pre = torch.empty((B, events.n_neurons, events.k), dtype=F32, device=dev) if want_pre_errors else None
    if (events.bucketed is not None and events.bucket_width == C and X * Y <= 255 and C_out * fx * fy <= 1024
            and C_out * fx * fy * C * 4 + 4 * C <= 160 * 1024):
        # Events grouped by input position: one post neuron per tap and group.
        call("bats_conv_backward_grouped", ptr(events.bucketed), ptr(events.bucket_offsets), events.cap, ptr(W), B,
             X, Y, C, fx, fy, C_out, events.k, ptr(post_times), ptr(tabs.tables), ptr(tabs.nvalid), k_post,
             float(tau_s), float(tau), ptr(grad), ptr(pre), stream_ptr())
        return grad, pre
    call("bats_conv_backward", ptr(events.events), ptr(events.slots), ptr(events.counts), events.cap, ptr(W), B, X, Y,
         C, fx, fy, C_out, events.k, ptr(post_times), ptr(tabs.tables), ptr(tabs.nvalid), k_post, float(tau_s),
         float(tau), ptr(grad), ptr(pre), stream_ptr())
    return grad, pre


# ---- Reference-signature kernel wrappers (used by the kernel-level parity tests) ---------------------------------

def compute_weights_gradient(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, errors):
    """Same arguments and result as the reference wrapper
    (Wrappers/Backpropagation/compute_weights_gradient.py:10-24): per-sample (B, N_post, N_pre)."""
    pt = _c(pre_times)
    B, N_pre, K_pre = pt.shape
    ev = sort_events(pt, 1.0, 1.0, pre_exp_tau_s, pre_exp_tau)
    post = _c(post_times)
    tabs = tables_from_factors(post, f1, f2, errors)
    return weights_gradient(ev, post, tabs, N_pre, per_sample=True)


def propagate_errors_to_pre_spikes(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, weights, errors,
                                   tau_s, tau):
    """Same arguments and result as the reference wrapper
    (Wrappers/Backpropagation/propagate_errors_to_pre_spikes.py:11-27): (B, N_pre, K_pre)."""
    pt = _c(pre_times)
    ev = sort_events(pt, 1.0, 1.0, pre_exp_tau_s, pre_exp_tau)
    post = _c(post_times)
    tabs = tables_from_factors(post, f1, f2, errors)
    return pre_errors(ev, transpose_weights(weights), post, tabs, float(tau_s), float(tau))


def compute_weights_gradient_conv(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, pre_shape, post_shape,
                                  filter_shape, errors):
    """Same arguments and result as the reference wrapper (Wrappers/Backpropagation/compute_weights_gradient_conv.py:11-32)."""
    pt = _c(pre_times)
    ev = sort_events(pt, 1.0, 1.0, pre_exp_tau_s, pre_exp_tau)
    post = _c(post_times)
    tabs = tables_from_factors(post, f1, f2, errors)
    C_out, fx, fy, C = (int(v) for v in filter_shape)
    dummy_w = torch.zeros((C_out, fx, fy, C), dtype=F32, device=post.device)
    g, _ = conv_backward(ev, dummy_w, pre_shape, post, tabs, 1.0, 1.0, want_pre_errors=False)
    return g


def propagate_errors_to_pre_spikes_conv(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, filters, errors,
                                        tau_s, tau, pre_shape):
    """Conv error propagation with filters (C_out, fx, fy, C_in)
    (Wrappers/Backpropagation/propagate_errors_to_pre_spikes_conv.py:11-32)."""
    pt = _c(pre_times)
    ev = sort_events(pt, 1.0, 1.0, pre_exp_tau_s, pre_exp_tau)
    post = _c(post_times)
    tabs = tables_from_factors(post, f1, f2, errors)
    _, pre = conv_backward(ev, filters, pre_shape, post, tabs, float(tau_s), float(tau), want_pre_errors=True)
    return pre


# ---- Losses / optimizer -------------------------------------------------------------------------------------------

def spike_count_loss(n_spike_per_neuron, targets=None, labels=None, target_true=0.0, target_false=0.0, k=1,
                     want_loss=True, want_errors=True):
    counts = n_spike_per_neuron
    if not torch.is_tensor(counts) or not counts.is_cuda:
        counts = _c(counts)
    is_float = counts.dtype != I32
    if is_float:
        counts = _c(counts, F32)
    else:
        counts = counts.contiguous()
    B, N = counts.shape
    tg = _c(targets) if targets is not None else None
    lb = _c(labels, I32) if labels is not None else None
    loss = torch.empty((B,), dtype=F32, device=counts.device) if want_loss else None
    err = torch.empty((B, N, k), dtype=F32, device=counts.device) if want_errors else None
    call("bats_spike_count_loss", ptr(counts), int(is_float), ptr(tg), ptr(lb), float(target_true),
         float(target_false), B, N, k, ptr(loss), ptr(err), stream_ptr())
    return loss, err


def ttfs_softmax_cross_entropy(spikes, labels, tau: float, want_loss=True, want_errors=True):
    sp = _c(spikes)
    lb = _c(labels, I32)
    B, N, K = sp.shape
    loss = torch.empty((B,), dtype=F32, device=sp.device) if want_loss else None
    err = torch.empty((B, N, K), dtype=F32, device=sp.device) if want_errors else None
    call("bats_ttfs_softmax_cross_entropy", ptr(sp), ptr(lb), B, N, K, float(tau), ptr(loss), ptr(err), stream_ptr())
    return loss, err


def spike_time_loss(spikes, targets, mode: int):
    sp = _c(spikes)
    B, N, K = sp.shape
    loss = torch.empty((B,), dtype=F32, device=sp.device) if mode != 1 else None
    err = torch.empty((B, N, K), dtype=F32, device=sp.device) if mode != 0 else None
    call("bats_spike_time_loss", ptr(sp), ptr(targets), B, N, K, mode, ptr(loss), ptr(err), stream_ptr())
    return loss, err


def adam_step(grad, m, v, beta_1, beta_2, epsilon, lr, bias1, bias2, delta=None, weights=None, weights_t=None):
    n_post, n_pre, ld = 0, 0, 0
    if weights_t is not None:
        n_post, n_pre = weights.shape
        ld = weights_t.shape[1]
    call("bats_adam_step", ptr(grad), ptr(m), ptr(v), grad.numel(), float(beta_1), float(beta_2), float(epsilon),
         float(lr), float(bias1), float(bias2), ptr(delta), ptr(weights), ptr(weights_t), n_post, n_pre, ld,
         stream_ptr())


def nadam_step(grad, m, v, beta_1, beta_2, epsilon, lr, bias1, bias2, delta):
    """NAdam on one tensor (bats/Optimizers/NAdamOptimizer.py:35-58); m, v in place, delta written."""
    call("bats_nadam_step", ptr(grad), ptr(m), ptr(v), grad.numel(), float(beta_1), float(beta_2), float(epsilon),
         float(lr), float(bias1), float(bias2), ptr(delta), stream_ptr())


def apply_weights_synaptic_scaling(weights, silent_ratios, n_spikes, gradient, scaling_threshold: float,
                                   factor: float):
    """In place on the per-sample gradient (B, N_post, N_pre)
    (CuFiles/Regularization/apply_weights_synaptic_scaling.cu)."""
    B, n_post, n_pre = gradient.shape
    call("bats_weights_synaptic_scaling", ptr(_c(weights)), ptr(_c(silent_ratios)), ptr(_c(n_spikes, I32)),
         ptr(gradient), B, n_post, n_pre, float(scaling_threshold), float(factor), stream_ptr())
    return gradient


def apply_label_weights_synaptic_scaling(weights, labels, n_spikes, gradient, factor: float):
    """In place on the per-sample gradient (B, N_post, N_pre)
    (CuFiles/Regularization/apply_label_weights_synaptic_scaling.cu)."""
    B, n_post, n_pre = gradient.shape
    call("bats_label_weights_synaptic_scaling", ptr(_c(weights)), ptr(_c(labels)), ptr(_c(n_spikes, I32)),
         ptr(gradient), B, n_post, n_pre, float(factor), stream_ptr())
    return gradient


def add_deltas(weights, delta, weights_t=None):
    n_pre = weights.shape[-1]
    ld = weights_t.shape[1] if weights_t is not None else 0
    call("bats_add_deltas", ptr(weights), ptr(_c(delta)), weights.numel(), ptr(weights_t), n_pre, ld, stream_ptr())
