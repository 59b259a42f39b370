"""Continuous-batching inference server for fully-connected BATS networks.

Requests are spike-event lists of different lengths (neuron index, time). They are admitted into device
"lanes": each lane owns a CUDA stream and device-resident buffers for up to `max_batch` requests (event
lists, spike trains, per-layer sorted events and outputs) plus pinned host staging, and the network's
transposed weights are uploaded once. Whenever a lane is free and requests are waiting, the pending
requests (up to max_batch, oldest first) are packed into one flat event list and launched on that lane
with a single native call (bats_serve_fc_batch): host -> device copy, event-list -> spike-train
conversion, and per layer the event sort and the LIF forward, then the output spike counts and times
are copied back. Several lanes are in flight at once, so requests that arrive while
others are on the GPU start as soon as a lane frees up and their work overlaps on the device. The number
of lanes is max_lanes or as many as the free HBM reported by the driver (cudaMemGetInfo, times
hbm_fraction) holds, all allocated up front so that serving never allocates; admission refuses requests
when free HBM (re-read at most every 5 ms) falls below a floor or the queue is full. Many lanes of small
batches (16 x 16 by default) keep the per-batch latency short while the lanes together fill the GPU. The forward
kernel variant of every layer is chosen per batch-size bucket by autotune(). A request's result does not
depend on which other requests share its batch (the kernels treat samples independently), which
tests/test_gpu_serving.py checks bit for bit.
"""
from __future__ import annotations

import collections
import contextlib
import ctypes
import gc
import time
from dataclasses import dataclass, field
from typing import Deque, Dict, List, Optional, Sequence

import numpy as np
import torch

from . import kernels as K
from ._lib import BatsFcLayer, call, ptr
from .autotune import Autotuner, get_tuner


@contextlib.contextmanager
def no_gc_pauses():
    """Automatic garbage collection off while serving (restored afterwards): a generation-2 collection
    over the tens of thousands of request and result objects of a busy loop stops the host for about
    30 ms, which shows up directly in the latency tail. The serving objects hold no reference cycles."""
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()


@dataclass
class LayerSpec:
    n_neurons: int
    tau_s: float
    theta: float
    delta_theta: float
    max_n_spike: int


@dataclass
class Request:
    rid: int
    indices: np.ndarray  # (n,) int32 neuron index per event, in order of appearance
    times: np.ndarray    # (n,) float32
    t_arrival: float = 0.0


@dataclass
class Result:
    rid: int
    counts: np.ndarray        # (N_out,) int32 output spike counts
    spike_times: np.ndarray   # (N_out, K_out) float32, +inf padded
    t_arrival: float
    t_done: float

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival


class _Lane:
    def __init__(self, server: "InferenceServer", device):
        s = server
        B, E = s.max_batch, s.max_events
        f32, i32 = torch.float32, torch.int32
        self.stream = torch.cuda.Stream(device=device)
        # Flat event list of a batch (up to B * E events) + offsets, pinned on the host and on the device.
        self.h_idx = torch.empty((B * E,), dtype=i32, pin_memory=True)
        self.h_t = torch.empty((B * E,), dtype=f32, pin_memory=True)
        self.h_off = torch.empty((B + 1,), dtype=i32, pin_memory=True)
        self.d_idx = torch.empty((B * E,), dtype=i32, device=device)
        self.d_t = torch.empty((B * E,), dtype=f32, device=device)
        self.d_off = torch.empty((B + 1,), dtype=i32, device=device)
        self.trains = torch.empty((B, s.n_inputs, s.k_in), dtype=f32, device=device)
        self.train_counts = torch.empty((B, s.n_inputs), dtype=i32, device=device)
        self.overflow = torch.zeros((1,), dtype=i32, device=device)
        self.ev, self.out = [], []
        n_prev, k_prev = s.n_inputs, s.k_in
        for spec in s.specs:
            self.ev.append(K.alloc_events(B, n_prev, k_prev, device, bucketed=False))
            self.out.append((torch.empty((B, spec.n_neurons), dtype=i32, device=device),
                             *(torch.empty((B, spec.n_neurons, spec.max_n_spike), dtype=f32, device=device)
                               for _ in range(4))))
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        self.ws = torch.empty(max(256, s.sort_ws), dtype=torch.uint8, device=device)
        self.h_counts = torch.empty(self.out[-1][0].shape, dtype=i32, pin_memory=True)
        self.h_times = torch.empty(self.out[-1][3].shape, dtype=f32, pin_memory=True)
        self.h_overflow = torch.zeros((1,), dtype=i32, pin_memory=True)
        self.done = torch.cuda.Event()
        self.batch: List[Request] = []
        # numpy views of the pinned buffers (no per-request torch calls on the host path)
        self.np_idx = self.h_idx.numpy()
        self.np_t = self.h_t.numpy()
        self.np_off = self.h_off.numpy()
        self.np_counts = self.h_counts.numpy()
        self.np_times = self.h_times.numpy()
        self.np_overflow = self.h_overflow.numpy()
        # The layer descriptors of bats_serve_fc_batch, pointing at this lane's buffers.
        self.layers = (BatsFcLayer * len(s.specs))()
        n_prev, k_prev = s.n_inputs, s.k_in
        for li, spec in enumerate(s.specs):
            tau32, c, dtt = s.consts[li]
            n, a, x, t, z = self.out[li]
            self.layers[li] = BatsFcLayer(n_prev, k_prev, spec.n_neurons, spec.max_n_spike, ptr(s.wt[li]),
                                          s.wt[li].shape[1], float(np.float32(spec.tau_s)), float(tau32), float(c),
                                          float(dtt), float(np.float32(s.max_sim)), K.FWD_AUTO,
                                          ptr(self.ev[li].events), ptr(self.ev[li].slots), ptr(self.ev[li].counts),
                                          ptr(n), ptr(a), ptr(x), ptr(t), ptr(z))
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike

    def busy(self) -> bool:
        return bool(self.batch) and not self.done.query()

    @staticmethod
    def bytes_needed(server: "InferenceServer") -> int:
        s = server
        B, E = s.max_batch, s.max_events
        total = B * E * 8 + (B + 1) * 4 + B * s.n_inputs * (s.k_in * 4 + 4)
        n_prev, k_prev = s.n_inputs, s.k_in
        for spec in s.specs:
            total += B * n_prev * k_prev * 20 + B * 4
            total += B * spec.n_neurons * (4 + 16 * spec.max_n_spike)
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        return total + s.sort_ws


class InferenceServer:
    def __init__(self, weights: Sequence, specs: Sequence[LayerSpec], n_inputs: int, max_events: int,
                 k_in: int = 32, max_batch: int = 16, max_lanes: int = 16, hbm_fraction: float = 0.5,
                 max_simulation: float = float("inf"), max_pending: int = 1 << 16, device="cuda"):
        self.dev = torch.device(device)
        self.specs = list(specs)
        self.n_inputs, self.max_events, self.k_in = int(n_inputs), int(max_events), int(k_in)
        self.max_batch = int(max_batch)
        self.max_sim = float(max_simulation)
        self.hbm_fraction = float(hbm_fraction)
        # Network state resident on the device: transposed weights for the forward kernels.
        self.wt = [K.transpose_weights(torch.as_tensor(w, dtype=torch.float32, device=self.dev))
                   for w in weights]
        self.consts = [K.lif_constants(sp.tau_s, sp.theta, sp.delta_theta) for sp in self.specs]
        self.sort_ws = 0
        n_prev, k_prev = self.n_inputs, self.k_in
        for spec in self.specs:
            self.sort_ws = max(self.sort_ws, K.call_size("bats_sort_events_workspace_bytes", self.max_batch,
                                                         n_prev, k_prev))
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        self.lane_bytes = _Lane.bytes_needed(self)
        self.max_lanes = int(max_lanes)
        self.max_pending = int(max_pending)
        self._free_hbm, self._free_t = 0, -1.0
        # Lanes are the batch slots: as many as max_lanes, or as free HBM (times hbm_fraction) allows, all
        # allocated here so that no allocation happens while serving.
        n_lanes = int(min(self.max_lanes, (self._free_hbm_now(force=True) * self.hbm_fraction) // self.lane_bytes))
        if n_lanes < 1:
            raise RuntimeError(f"not enough free HBM for one lane ({self.lane_bytes} bytes)")
        self.lanes = [_Lane(self, self.dev) for _ in range(n_lanes)]
        self.pending: Deque[Request] = collections.deque()
        self.results: Dict[int, Result] = {}
        self.rejected: List[int] = []
        self.batches_launched = 0
        self.algo_table: Dict[int, List[int]] = {}

    # -- admission --------------------------------------------------------------------------------------
    HBM_FLOOR = 64 * 1024 * 1024  # free HBM kept for the rest of the process

    def _free_hbm_now(self, force: bool = False) -> int:
        """Free device memory from the driver, re-read at most every 5 ms."""
        now = time.perf_counter()
        if force or now - self._free_t > 0.005:
            self._free_hbm, _ = torch.cuda.mem_get_info(self.dev)
            self._free_t = now
        return self._free_hbm

    def submit(self, req: Request, now: Optional[float] = None) -> bool:
        """Queue a request; refused (False) if it exceeds the lane capacity, the queue is full, or free HBM
        is below the floor."""
        req.t_arrival = time.perf_counter() if now is None else now
        if (len(req.indices) > self.max_events or len(req.indices) != len(req.times)
                or len(self.pending) >= self.max_pending or self._free_hbm_now() < self.HBM_FLOOR):
            self.rejected.append(req.rid)
            return False
        self.pending.append(req)
        return True

    # -- device work ------------------------------------------------------------------------------------
    def _launch(self, lane: _Lane, batch: List[Request]) -> None:
        """Pack the batch as one flat event list + offsets into the lane's pinned buffers and enqueue the whole
        batch (copies, conversion, every layer, copies back) with one call of bats_serve_fc_batch."""
        B = len(batch)
        lens = np.fromiter((len(r.indices) for r in batch), dtype=np.int64, count=B)
        off = lane.np_off[:B + 1]
        off[0] = 0
        np.cumsum(lens, out=off[1:])
        total = int(off[B])
        if total:
            np.concatenate([r.indices for r in batch], out=lane.np_idx[:total], casting="unsafe")
            np.concatenate([r.times for r in batch], out=lane.np_t[:total], casting="unsafe")
        for li, algo in enumerate(self._algos_for(B)):
            lane.layers[li].algo = int(algo)
        lane.batch = batch
        with torch.cuda.stream(lane.stream):
            call("bats_serve_fc_batch", lane.h_idx.data_ptr(), lane.h_t.data_ptr(), lane.h_off.data_ptr(), B, total,
                 ptr(lane.d_idx), ptr(lane.d_t), ptr(lane.d_off), self.n_inputs, self.k_in, ptr(lane.trains),
                 ptr(lane.train_counts), ptr(lane.overflow), ctypes.addressof(lane.layers), len(self.specs),
                 ptr(lane.ws), lane.ws.numel(), lane.h_counts.data_ptr(), lane.h_times.data_ptr(),
                 lane.h_overflow.data_ptr(), lane.stream.cuda_stream)
            lane.done.record(lane.stream)
        self.batches_launched += 1

    def _layers(self, lane: _Lane, B: int, algos: Sequence[int], s: int, only: Optional[int] = None) -> None:
        """Per layer: event sort of the previous layer's spike trains, then the LIF forward with the given
        kernel variant. With `only`, just that layer's forward (used by the autotuner)."""
        pre, pre_n = lane.trains, None
        for li, spec in enumerate(self.specs):
            ev = lane.ev[li]
            tau32, c, dtt = self.consts[li]
            if only is None and pre_n is None:
                call("bats_sort_events", ptr(pre), B, ev.n_neurons, ev.k, float(np.float32(spec.tau_s)),
                     float(tau32), None, None, ptr(ev.events), ptr(ev.slots), ptr(ev.counts), None, None, 0,
                     ptr(lane.ws), lane.ws.numel(), s)
            elif only is None:
                call("bats_sort_events_counted", ptr(pre), ptr(pre_n), B, ev.n_neurons, ev.k,
                     float(np.float32(spec.tau_s)), float(tau32), None, None, ptr(ev.events), ptr(ev.slots),
                     ptr(ev.counts), None, None, 0, ptr(lane.ws), lane.ws.numel(), s)
            n, a, x, t, z = lane.out[li]
            if only is None or only == li:
                call("bats_lif_forward_fc_algo", ptr(ev.events), ptr(ev.counts), ev.cap, ptr(self.wt[li]),
                     self.wt[li].shape[1], B, spec.n_neurons, spec.max_n_spike, float(c), float(dtt), float(tau32),
                     float(np.float32(self.max_sim)), ptr(n), ptr(a), ptr(x), ptr(t), ptr(z),
                     int(algos[li]) | (K.FWD_NO_PAD if li + 1 < len(self.specs) else 0), s)
            pre, pre_n = t, n

    @staticmethod
    def _bucket(B: int) -> int:
        return 1 << max(0, int(B - 1).bit_length())

    def _algos_for(self, B: int) -> List[int]:
        return self.algo_table.get(self._bucket(B), [K.FWD_AUTO] * len(self.specs))

    def autotune(self, requests: Sequence[Request], tuner: Optional[Autotuner] = None) -> Dict[int, List[str]]:
        """Per batch-size bucket (powers of two up to max_batch) and layer, the faster forward kernel variant,
        timed on batches drawn from `requests` (cycled) on the first lane."""
        tuner = tuner or get_tuner()
        lane = self.lanes[0]
        s = lane.stream.cuda_stream
        out = {}
        b = 1
        while b <= self.max_batch:
            batch = [requests[q % len(requests)] for q in range(b)]
            self._launch(lane, batch)
            lane.done.synchronize()
            self._collect(lane)
            names = []
            algos = list(self._algos_for(b))
            with torch.cuda.stream(lane.stream):
                for li, spec in enumerate(self.specs):
                    ev_mean = max(1, int(lane.ev[li].counts[:b].float().mean().item()))
                    shape = (b, lane.ev[li].n_neurons, lane.ev[li].k, spec.n_neurons, spec.max_n_spike,
                             int(np.log2(ev_mean)))

                    def run(algo, li=li):
                        trial = list(algos)
                        trial[li] = algo
                        self._layers(lane, b, trial, s, only=li)

                    cands = {"tile": K.FWD_TILE, "lanes": K.FWD_LANES, "tile_stage": K.FWD_TILE | K.FWD_STAGE}
                    if spec.n_neurons > 64:
                        cands["tile64"] = K.FWD_TILE64
                    best = tuner.pick("fc_forward", shape, {k: (lambda a=a: run(a)) for k, a in cands.items()})
                    algos[li] = cands[best]
                    names.append(best)
            torch.cuda.synchronize()
            self.algo_table[b] = algos
            out[b] = names
            b *= 2
        return out

    def _collect(self, lane: _Lane) -> List[Result]:
        now = time.perf_counter()
        if int(lane.np_overflow[0]) != 0:
            raise RuntimeError("a request has more spikes on one input neuron than the server's k_in")
        B = len(lane.batch)
        counts = lane.np_counts[:B].copy()  # one copy per batch; results are views into it
        times = lane.np_times[:B].copy()
        out = []
        for q, r in enumerate(lane.batch):
            res = Result(r.rid, counts[q], times[q], r.t_arrival, now)
            self.results[r.rid] = res
            out.append(res)
        lane.batch = []
        return out

    def pump(self) -> List[Result]:
        """Collect finished lanes and launch pending requests on free lanes. Non-blocking."""
        done = []
        for lane in self.lanes:
            if lane.batch and lane.done.query():
                done.extend(self._collect(lane))
        for lane in self.lanes:
            if not self.pending:
                break
            if lane.batch:
                continue
            self._launch(lane, [self.pending.popleft() for _ in range(min(self.max_batch, len(self.pending)))])
        return done

    def drain(self) -> List[Result]:
        out = []
        with no_gc_pauses():
            while self.pending or any(l.batch for l in self.lanes):
                out.extend(self.pump())
        return out

    def infer(self, requests: Sequence[Request]) -> List[Result]:
        """Convenience: submit all, run to completion, return results in request order."""
        for r in requests:
            self.submit(r)
        self.drain()
        return [self.results[r.rid] for r in requests]


def make_network(sizes: Sequence[int] = (700, 512, 512, 20), max_n_spike: int = 30, tau_s: float = 0.13,
                 theta_hidden: float = 1.0, theta_out: float = 1.3, mean: float = 1.5, seed: int = 0):
    """Synthetic serving network: FP32 weights N(mean, 1) / sqrt(fan_in) per layer (the positive mean makes
    requests of a few hundred events and more drive the network to the output layer), thresholds
    theta_hidden / theta_out with delta_theta = theta. Returns (weights [(N_out, N_in)], specs)."""
    rng = np.random.default_rng(seed)
    ws = [((rng.normal(0.0, 1.0, (o, i)) + mean) / np.sqrt(i)).astype(np.float32)
          for i, o in zip(sizes[:-1], sizes[1:])]
    specs = [LayerSpec(o, tau_s, theta_hidden, theta_hidden, max_n_spike) for o in sizes[1:-1]]
    specs.append(LayerSpec(sizes[-1], tau_s, theta_out, theta_out, max_n_spike))
    return ws, specs


def make_requests(n: int, n_channels: int = 700, lo: int = 50, hi: int = 5000, t_max: float = 0.2, seed: int = 0,
                  rid0: int = 0) -> List[Request]:
    """Synthetic serving workload: each request is an event stream over n_channels input neurons with
    exp(U(ln lo, ln hi)) events (log-uniform count), channels uniform, times U(0, t_max), in time order."""
    rng = np.random.default_rng(seed)
    reqs = []
    for q in range(n):
        m = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        t = np.sort(rng.uniform(0, t_max, m)).astype(np.float32)
        c = rng.integers(0, n_channels, m).astype(np.int32)
        reqs.append(Request(rid0 + q, c, t))
    return reqs


def run_poisson(server: InferenceServer, requests: Sequence[Request], rate: float, seed: int = 0) -> List[Result]:
    """Submits `requests` with Poisson arrivals at `rate` per second (in real time) while pumping the server;
    returns all results (latency = completion - arrival)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, len(requests))
    t0 = time.perf_counter()
    arrivals = t0 + np.cumsum(gaps)
    q = 0
    results = []
    with no_gc_pauses():
        while q < len(requests) or server.pending or any(l.batch for l in server.lanes):
            now = time.perf_counter()
            while q < len(requests) and arrivals[q] <= now:
                server.submit(requests[q], now=arrivals[q])
                q += 1
            results.extend(server.pump())
    return results


def latency_stats(results: Sequence[Result]) -> dict:
    lat = np.array([r.latency for r in results]) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "n": int(lat.size)}
