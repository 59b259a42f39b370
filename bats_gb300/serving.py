"""Continuous-batching inference server for fully-connected BATS networks.

Requests are spike-event lists of different lengths (neuron index, time). They are admitted into device
"lanes": each lane owns a CUDA stream and device-resident buffers for up to `max_batch` requests (event
lists, spike trains, per-layer sorted events and outputs) plus pinned host staging, and the network's
transposed weights are uploaded once. Whenever a lane is free and requests are waiting, the pending
requests (up to max_batch, oldest first) are packed and launched on that lane: host -> device copy,
event-list -> spike-train conversion, and per layer the event sort and the LIF forward, then the output
spike counts and times are copied back. Several lanes are in flight at once, so requests that arrive while
others are on the GPU start as soon as a lane frees up and their work overlaps on the device. The lane
pool starts with one lane and grows, while every lane is busy and requests wait, up to max_lanes, each new
lane only if the free HBM reported by the driver (cudaMemGetInfo) leaves room for it; admission refuses
requests when free HBM (re-read at most every 5 ms) falls below a floor or the queue is full. The forward
kernel variant of every layer is chosen per batch-size bucket by autotune(). A request's result does not
depend on which other requests share its batch (the kernels treat samples independently), which
tests/test_gpu_serving.py checks bit for bit.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field
from typing import Deque, Dict, List, Optional, Sequence

import numpy as np
import torch

from . import kernels as K
from ._lib import call, ptr
from .autotune import Autotuner, get_tuner


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
        self.h_idx = torch.empty((B, E), dtype=i32, pin_memory=True)
        self.h_t = torch.empty((B, E), dtype=f32, pin_memory=True)
        self.d_idx = torch.empty((B, E), dtype=i32, device=device)
        self.d_t = torch.empty((B, E), dtype=f32, device=device)
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
        self.h_overflow = torch.empty((1,), dtype=i32, pin_memory=True)
        self.done = torch.cuda.Event()
        self.batch: List[Request] = []
        # numpy views of the pinned buffers (no per-request torch calls on the host path)
        self.np_idx = self.h_idx.numpy().reshape(-1)
        self.np_t = self.h_t.numpy().reshape(-1)
        self.np_counts = self.h_counts.numpy()
        self.np_times = self.h_times.numpy()
        self.np_overflow = self.h_overflow.numpy()

    def busy(self) -> bool:
        return bool(self.batch) and not self.done.query()

    @staticmethod
    def bytes_needed(server: "InferenceServer") -> int:
        s = server
        B, E = s.max_batch, s.max_events
        total = B * E * 8 + B * s.n_inputs * (s.k_in * 4 + 4)
        n_prev, k_prev = s.n_inputs, s.k_in
        for spec in s.specs:
            total += B * n_prev * k_prev * 20 + B * 4
            total += B * spec.n_neurons * (4 + 16 * spec.max_n_spike)
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        return total + s.sort_ws


class InferenceServer:
    def __init__(self, weights: Sequence, specs: Sequence[LayerSpec], n_inputs: int, max_events: int,
                 k_in: int = 32, max_batch: int = 64, max_lanes: int = 4, hbm_fraction: float = 0.5,
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
        if self._free_hbm_now(force=True) * self.hbm_fraction < self.lane_bytes:
            raise RuntimeError(f"not enough free HBM for one lane ({self.lane_bytes} bytes)")
        self.lanes = [_Lane(self, self.dev)]
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

    def _grow(self) -> Optional[_Lane]:
        """A new lane when every lane is busy, requests wait and free HBM allows it."""
        if len(self.lanes) >= self.max_lanes:
            return None
        if self._free_hbm_now(force=True) * self.hbm_fraction < self.lane_bytes + self.HBM_FLOOR:
            return None
        lane = _Lane(self, self.dev)
        self.lanes.append(lane)
        return lane

    # -- device work ------------------------------------------------------------------------------------
    def _launch(self, lane: _Lane, batch: List[Request]) -> None:
        B = len(batch)
        L = max(1, max(len(r.indices) for r in batch))
        # Pack the batch contiguously as (B, L); a sample ends at its first negative index.
        hi = lane.np_idx[:B * L].reshape(B, L)
        ht = lane.np_t[:B * L].reshape(B, L)
        for q, r in enumerate(batch):
            n = len(r.indices)
            hi[q, :n] = r.indices
            ht[q, :n] = r.times
            if n < L:
                hi[q, n] = -1
        lane.batch = batch
        with torch.cuda.stream(lane.stream):
            s = lane.stream.cuda_stream
            d_idx = lane.d_idx.view(-1)[:B * L]
            d_t = lane.d_t.view(-1)[:B * L]
            d_idx.copy_(lane.h_idx.view(-1)[:B * L], non_blocking=True)
            d_t.copy_(lane.h_t.view(-1)[:B * L], non_blocking=True)
            lane.overflow.zero_()
            call("bats_events_to_trains", ptr(d_idx), ptr(d_t), B, L, self.n_inputs, self.k_in,
                 ptr(lane.trains), ptr(lane.train_counts), ptr(lane.overflow), s)
            self._layers(lane, B, self._algos_for(B), s)
            lane.h_counts[:B].copy_(lane.out[-1][0][:B], non_blocking=True)
            lane.h_times[:B].copy_(lane.out[-1][3][:B], non_blocking=True)
            lane.h_overflow.copy_(lane.overflow, non_blocking=True)
            lane.done.record(lane.stream)
        self.batches_launched += 1

    def _layers(self, lane: _Lane, B: int, algos: Sequence[int], s: int, only: Optional[int] = None) -> None:
        """Per layer: event sort of the previous layer's spike trains, then the LIF forward with the given
        kernel variant. With `only`, just that layer's forward (used by the autotuner)."""
        pre = lane.trains
        for li, spec in enumerate(self.specs):
            ev = lane.ev[li]
            tau32, c, dtt = self.consts[li]
            if only is None:
                call("bats_sort_events", ptr(pre), B, ev.n_neurons, ev.k, float(np.float32(spec.tau_s)),
                     float(tau32), None, None, ptr(ev.events), ptr(ev.slots), ptr(ev.counts), None, None, 0,
                     ptr(lane.ws), lane.ws.numel(), s)
            n, a, x, t, z = lane.out[li]
            if only is None or only == li:
                call("bats_lif_forward_fc_algo", ptr(ev.events), ptr(ev.counts), ev.cap, ptr(self.wt[li]),
                     self.wt[li].shape[1], B, spec.n_neurons, spec.max_n_spike, float(c), float(dtt), float(tau32),
                     float(np.float32(self.max_sim)), ptr(n), ptr(a), ptr(x), ptr(t), ptr(z), int(algos[li]), s)
            pre = t

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

                    best = tuner.pick("fc_forward", shape, {"tile": lambda: run(K.FWD_TILE),
                                                             "lanes": lambda: run(K.FWD_LANES)})
                    algos[li] = K.FWD_TILE if best == "tile" else K.FWD_LANES
                    names.append(best)
            torch.cuda.synchronize()
            self.algo_table[b] = algos
            out[b] = names
            b *= 2
        return out

    def _collect(self, lane: _Lane) -> List[Result]:
        now = time.perf_counter()
        out = []
        if int(lane.np_overflow[0]) != 0:
            raise RuntimeError("a request has more spikes on one input neuron than the server's k_in")
        for q, r in enumerate(lane.batch):
            res = Result(r.rid, lane.np_counts[q].copy(), lane.np_times[q].copy(), r.t_arrival, now)
            self.results[r.rid] = res
            out.append(res)
        lane.batch = []
        return out

    def pump(self) -> List[Result]:
        """Collect finished lanes and launch pending requests on free lanes (growing the lane pool while
        free HBM allows). Non-blocking."""
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
        while self.pending:
            lane = self._grow()
            if lane is None:
                break
            self._launch(lane, [self.pending.popleft() for _ in range(min(self.max_batch, len(self.pending)))])
        return done

    def drain(self) -> List[Result]:
        out = []
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
