"""Benchmark of the BATS train step on GB300: samples/s of forward + spike-count loss + exact backward
+ Adam on the 784-800-800-10 network, batch 256 (synthetic MNIST-like spike input).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is the device-resident batched train step (bats_gb300.train.FCTrainStep,
replayed as a CUDA graph when capture works) in the reference's MNIST training regime (weights U(-1, 1),
hidden threshold 0.2, output 1.3), where every layer spikes (`spikes_per_layer` beside it); `literal`
repeats every measurement with the configuration's literal constants (weights N(0, 1/sqrt(fan_in)),
thresholds 1.0 hidden / 1.3 output), where the hidden layers stay silent. `e2e` is the same step through
the public API with host inputs (pinned host -> device copy and the loss read back inside the timed
region). `plain_api` is the layer-by-layer drop-in API (Network / LIFLayer / AdamOptimizer with
per-sample gradients and the caller's batch mean); `refkern` runs the reference's own CUDA kernels on
the same GPU; `cpu_baseline` is the float64 oracle on the host cores. `--impl reference` times the
reference path on the host cores on the same workload and configuration (the reference has no CPU
implementation of its own, so this is the oracle port of it).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "samples/s fwd+exact-bwd and serve p99 ms vs plain kernels, 1 GB300, tol 1e-5"
B = 256
SIZES = [784, 800, 800, 10]
TAU_S = 0.13
K_SPIKE = 30
MAX_SIM = 0.2
TARGET_TRUE, TARGET_FALSE = 15.0, 3.0
LR = 3e-3


def make_inputs(batch, seed):
    rng = np.random.default_rng(seed)
    fire = rng.random((batch, SIZES[0])) < 0.19
    t = np.where(fire, rng.uniform(0, 0.01, (batch, SIZES[0])), np.inf).astype(np.float32)[:, :, None]
    labels = rng.integers(0, SIZES[-1], batch).astype(np.int32)
    return t, fire.astype(np.int32), labels


def make_weights(variant, seed=0):
    rng = np.random.default_rng(seed)
    ws = []
    for n_pre, n_post in zip(SIZES[:-1], SIZES[1:]):
        if variant == "literal":
            ws.append(rng.normal(0, 1 / np.sqrt(n_pre), (n_post, n_pre)).astype(np.float32))
        else:
            ws.append(rng.uniform(-1, 1, (n_post, n_pre)).astype(np.float32))
    return ws


def thresholds(variant):
    hidden = 1.0 if variant == "literal" else 0.2
    return [hidden] * (len(SIZES) - 2) + [1.3]


HEADLINE = "active"
VARIANT_DESC = {"active": "active: W~U(-1,1), theta 0.2 hidden / 1.3 out (the reference's MNIST training regime)",
                "literal": "literal: W~N(0,1/sqrt(fan_in)), theta 1.0 hidden / 1.3 out"}


def headline_config(world):
    """The workload both arms of the comparison measure (the same dict in both JSON lines)."""
    return {"workload": "784-800-800-10 BATS train step (forward, spike-count loss, exact backward, Adam), "
                        "synthetic MNIST-shaped input (784 inputs, p 0.19 at U(0, 0.01) s), max_n_spike 30",
            "global_batch": B * world, "variant": VARIANT_DESC[HEADLINE], "parallelism": f"replicas x{world}",
            "l2": "GPU arm: flushed between timed steps (512 MB write)"}


# ---------------------------------------------------------------------------------------------------------------------
# CPU baseline (float64 oracle), run in spawned worker processes

def _oracle_train_samples(args):
    """Forward + loss + exact backward of a few samples with the float64 oracle (no GPU)."""
    times, labels, weights, ths = args
    sys.path.insert(0, ROOT)
    from oracle import bats_ref64 as R
    tau = 2 * TAU_S
    outs = []
    pre = times.astype(np.float64)
    layer_in = [pre]
    for w, th in zip(weights, ths):
        o = R.lif_forward(layer_in[-1], w.astype(np.float64), TAU_S, th, th, K_SPIKE, MAX_SIM)
        outs.append(o)
        layer_in.append(o[3])
    n_out = outs[-1][0]
    targets = R.class_targets(labels, weights[-1].shape[0], TARGET_TRUE, TARGET_FALSE)
    _, err = R.spike_count_loss(n_out, targets, K_SPIKE)
    grads = []
    for li in range(len(weights) - 1, -1, -1):
        n, a, x, t, z = outs[li]
        th = ths[li]
        R.propagate_recurrent_errors(x, z, err, th / tau)
        f1, f2 = R.compute_factors(t, a, th / tau, x, z, tau)
        pin = layer_in[li]
        es, ee = R.compute_pre_exps(pin, TAU_S, tau)
        grads.append(R.compute_weights_gradient(f1, f2, t, (pin, es, ee), err).sum(0))
        if li > 0:
            err = R.propagate_errors_to_pre_spikes(f1, f2, t, (pin, es, ee), weights[li], err, TAU_S, tau)
    return times.shape[0]


def cpu_baseline(variant, budget_s=12.0, cores=None):
    cores = cores or os.cpu_count() or 1
    times, _, labels = make_inputs(4 * cores, seed=1)
    ws = make_weights(variant)
    ths = thresholds(variant)
    ctx = mp.get_context("spawn")
    chunks = [(times[i:i + 1], labels[i:i + 1], ws, ths) for i in range(times.shape[0])]
    with ctx.Pool(cores) as pool:
        pool.map(_oracle_train_samples, chunks[:cores])  # warm the workers up
        t0 = time.perf_counter()
        done = 0
        while True:
            done += sum(pool.map(_oracle_train_samples, chunks))
            el = time.perf_counter() - t0
            if el >= budget_s or done >= 64 * cores:
                break
    return {"value": done / el, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": f"{done} samples of the {variant} 784-800-800-10 train step (forward, loss, exact backward; "
                      f"float64 NumPy oracle, one process per core), {el:.1f} s"}


def batching_cpu_baseline(budget_s=12.0, cores=None, stride=32):
    """The float64 oracle on the uneven-batch workload (batching_inputs, 1024-1024-20): one sample per
    `stride` of the 4096 taken at evenly spaced ranks of the event count (the same spread of lengths), one
    sample per task, as many processes as host cores, in whole passes over that set until the budget is
    spent; samples/s."""
    cores = cores or os.cpu_count() or 1
    t, labels, counts = batching_inputs()
    ws, ths = batching_weights()
    idx = np.sort(np.argsort(counts, kind="stable")[stride // 2::stride])
    chunks = [(t[i:i + 1], labels[i:i + 1], ws, ths) for i in idx]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_oracle_train_samples, chunks[:cores])
        t0 = time.perf_counter()
        done = 0
        while True:
            done += sum(pool.map(_oracle_train_samples, chunks))
            el = time.perf_counter() - t0
            if el >= budget_s or done >= 8 * len(chunks):
                break
    return {"value": done / el, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": f"{done} samples ({len(chunks)} of the 4096-sample uneven batch at evenly spaced event-count "
                      f"ranks, mean {float(counts[idx].mean()):.0f} input events vs {float(counts.mean()):.0f} "
                      f"for all 4096) of the 1024-1024-20 train step (forward, loss, exact backward; float64 NumPy "
                      f"oracle, one process per core), {el:.1f} s"}


# ---------------------------------------------------------------------------------------------------------------------
# GPU helpers

class ClockSampler:
    """nvidia-smi SM clock / throttle sampling (every 50 ms) during the timed region, which starts after the
    sampler's first sample; that sample is left out of the summary unless it is the only one. The samples go to
    clocks_<pid>.csv in BATS_GB300_CLOCKS_DIR (default: the system's temporary directory)."""

    def __init__(self, index=0):
        import tempfile
        self.index = index
        self.proc = None
        self.path = os.path.join(os.environ.get("BATS_GB300_CLOCKS_DIR") or tempfile.gettempdir(),
                                 f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return self
        # nvidia-smi takes a while to start: wait (at most 5 s) for its first sample, so that the timed region
        # that follows is sampled from its start.
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            self.f.flush()
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)
        self.skip = 1 if os.path.getsize(self.path) > 0 else 0  # that first sample predates the timed region
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.count(",") >= 8]
        rows = rows[getattr(self, "skip", 0):] or rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip().lower() == "active"})
        loaded = [v for v in sm if v > 0.5 * mx] or sm
        return {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].strip() not in ("", "[N/A]"))}


def flush_l2(buf):
    buf.add_(1.0)  # 512 MB read-modify-write: evicts the 129 MB L2 between timed steps


def time_steps(fn, steps, warmup, flush_buf, kernel_timer=None, dist=None):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        flush_l2(flush_buf)
        starts[i].record()
        fn()
        ends[i].record()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    wall = time.perf_counter() - t0
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    return ms, wall


def reduce_max(value, dist):
    """The largest of the ranks' values (the slowest replica's time); the value itself with one process. The
    reduction runs on a CUDA tensor under NCCL and on a CPU tensor under gloo."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_train_step(variant, graph=True):
    import torch
    from bats_gb300.train import FCLayerSpec, FCTrainStep
    ths = thresholds(variant)
    specs = [FCLayerSpec(n, TAU_S, th, th, K_SPIKE) for n, th in zip(SIZES[1:], ths)]
    ws = [torch.tensor(w) for w in make_weights(variant)]
    ts = FCTrainStep(B, SIZES[0], 1, specs, ws, TARGET_TRUE, TARGET_FALSE, learning_rate=LR, max_simulation=MAX_SIM)
    t, _, labels = make_inputs(B, seed=0)
    ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    return ts


def kernel_breakdown(ts, reps=5):
    """Device time of each launch of a step (CUDA events around every launch): the median over `reps` eager
    steps, so that one slow launch does not pick the dominant kernel."""
    import torch
    acc = {}
    for _ in range(reps):
        rec = ts.profile_step()
        torch.cuda.synchronize()
        for k, (s, e) in rec.items():
            acc.setdefault(k, []).append(s.elapsed_time(e))
    return {k: float(np.median(v)) for k, v in acc.items()}


def spike_counts(ts):
    return [int(o[0].sum().item()) for o in ts.out]


def algorithmic_bytes(ts, name):
    """SpMM-convention bytes of one launch (one FP32 weight read per event x post-neuron synapse). The forward
    writes the spike counts (4 bytes per neuron), a, x, t and post_exp_tau of every spike it emits (16 bytes
    per spike) and, only when the layer's trains are padded, +inf into t and post_exp_tau of every slot past
    the count (8 bytes per empty slot); it reads 8 bytes (time and index) per input event."""
    li = int(name[1]) - 1
    kind = name.split(".")[1]
    ev = ts.ev[li]
    S = int(ev.counts.sum().item())
    spec = ts.specs[li]
    N = spec.n_neurons
    if kind == "forward":
        n_spk = int(ts.out[li][0].sum().item())
        pad = ts._pad_flag(li) == 0
        pad_bytes = 8 * (ts.B * N * spec.max_n_spike - n_spk) if pad else 0
        return 8 * S + 4 * S * N + 4 * ts.B * N + 16 * n_spk + pad_bytes
    if kind in ("grad", "grad_adam", "pre_err"):
        n_spk = int(ts.out[li][0].sum().item())
        # + the batch-mean gradient write (grad), or the Adam update that consumes it in place: read W, m, v,
        # write W, its transposed copy, m, v and the gradient (grad_adam)
        extra = {"grad": 4, "grad_adam": 32, "pre_err": 0}[kind] * N * ev.n_neurons
        return 4 * S * N + 16 * n_spk + extra
    if kind == "sort":
        return ts.B * ev.cap * 4 + 20 * S
    return None


def run_ours(args, dist, rank, world):
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    import bats_gb300
    bats_gb300.load_library()
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    flush = torch.zeros(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
    result = {}
    variants = (HEADLINE, "literal") if args.workload == "all" else (
        (args.workload,) if args.workload in ("literal", "active") else ())
    for variant in variants:
        ts = build_train_step(variant)
        tuned = ts.autotune()
        graphed = ts.try_capture()
        fn = ts.replay if graphed else ts.step
        with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
            ms, wall = time_steps(fn, args.steps, args.warmup, flush, dist=dist)
        clocks = clk.summary()
        ms = reduce_max(ms, dist)
        sps = world * B * args.steps / (ms / 1e3)
        kb = kernel_breakdown(ts)
        top = max(kb, key=kb.get)
        # Live timing of the dominant kernel over timed steps.
        top_ms = ts.time_launch(top, args.steps, flush)
        abytes = algorithmic_bytes(ts, top)
        achieved = abytes / (top_ms / 1e3) / 1e9 if abytes else None
        e2e = None
        # End to end through the host-batch training API: every step copies its inputs from host memory
        # and reads its losses back (the copies overlap the previous step's compute).
        t_host, _, l_host = make_inputs(B, seed=0)
        ts.train_host([(t_host, l_host)] * args.warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ts.train_host([(t_host, l_host)] * args.steps)
        e2e_s = time.perf_counter() - t0
        e2e = {"value": world * B * args.steps / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": ts.h2d_bytes,
               "d2h_bytes_per_step": ts.d2h_bytes, "api": "FCTrainStep.train_host"}
        traffic, traffic_src, tinfo = None, None, {}
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            tinfo = json.load(open(tpath)).get(variant, {})
            if tinfo.get("kernel") == top:
                traffic, traffic_src = tinfo.get("bytes"), tinfo.get("source")
            else:
                tinfo = {}
        roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if achieved else None, "traffic": traffic,
                "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": abytes, "launch_ms": top_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"}
        if traffic:
            # What the DRAM actually moved per launch (ncu capture) over the live launch time: the weights stay
            # in L2, so this is far below the SpMM-convention fraction.
            roof["dram_frac"] = traffic / (top_ms / 1e3) / 1e9 / hbm_peak
        if tinfo.get("warp_instructions") and tinfo.get("warp_events"):
            roof["warp_instructions_per_warp_event"] = tinfo["warp_instructions"] / tinfo["warp_events"]
        result[variant] = {
            "value": sps, "ms_per_step": ms / args.steps, "graph": graphed, "autotuned": tuned, "clocks": clocks,
            "e2e": e2e,
            "spikes_per_layer": spike_counts(ts), "kernels_ms": {k: round(v, 4) for k, v in kb.items()},
            "roofline": roof,
            "gpu_launches": ts.launches_per_step * args.steps,
        }
        del ts
        torch.cuda.empty_cache()
    # Plain (layer-by-layer) drop-in API and the reference kernels, both configurations (few steps).
    if args.workload == "all":
        for variant in (HEADLINE, "literal"):
            result[variant]["plain_api"] = plain_api_rate(variant, max(2, args.steps // 4), flush)
            result[variant]["autograd"] = autograd_rate(variant, max(2, args.steps // 4), flush)
            result[variant]["refkern"] = refkern_rate(variant, 2, flush)
    return result


def profile_one_step(workload):
    """One eager train step (literal, active, batching or conv workload) inside an NVTX range "step", with a
    nested range per launch (L1.sort, L1.forward, ...), after set-up, autotuning and 3 warm-up steps, for
    targeted ncu captures:
    ncu --nvtx --nvtx-include "step/" (the step's launch list) or --nvtx-include "step/L2.forward/"."""
    import torch
    if workload == "conv":
        step, layers, (t, n, labels) = conv_network()
        del step, layers
        torch.cuda.empty_cache()
        ts = conv_train_step(t, labels)
    elif workload == "batching":
        from bats_gb300.train import FCLayerSpec, FCTrainStep
        t, labels, _ = batching_inputs()
        ws_np, ths = batching_weights()
        ws = [torch.tensor(w) for w in ws_np]
        specs = [FCLayerSpec(1024, TAU_S, ths[0], ths[0], K_SPIKE), FCLayerSpec(20, TAU_S, ths[1], ths[1], K_SPIKE)]
        ts = FCTrainStep(t.shape[0], 1024, t.shape[2], specs, ws, TARGET_TRUE, TARGET_FALSE, learning_rate=LR,
                         max_simulation=MAX_SIM)
        ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    else:
        ts = build_train_step(workload)
    if hasattr(ts, "autotune"):
        ts.autotune()
    for _ in range(3):
        ts.step()
    flush = torch.zeros(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
    flush_l2(flush)
    torch.cuda.synchronize()
    from bats_gb300._lib import stream_ptr
    s = stream_ptr()
    torch.cuda.nvtx.range_push("step")
    for name, fn in ts.launches:
        torch.cuda.nvtx.range_push(name)
        fn(s)
        torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    print(json.dumps({"profiled_step": workload, "launches": [n for n, _ in ts.launches]}))


def profile_kernels():
    """Every kernel of the library on the workloads' own shapes: each entry-point call runs once as a warm-up,
    then once more inside a named NVTX range under "census", for one ncu pass over all of them
    (ncu --nvtx --nvtx-include "census/" ...). The calls: the active 784-800-800-10 train step (batch 256,
    forward variants tile / work queue / lanes on layers 1 / 2 / 3), the same step through the drop-in layer
    API (per-sample gradients, Adam deltas), the conv train step (batch 128), and one call of each other
    entry point: pre-exponentials, the intensity encoder, event-list conversion of a 16-request serving
    batch, the TTFS and spike-time losses, untiled Adam, NAdam, both synaptic-scaling regularizers,
    transpose, add_deltas, the generic backward prep (reset errors, factors), the longest-first sample order
    and the counted sort that takes it, the conv backward for filters
    too large for shared memory, the allocation-free gradient, and one 16-request batch of the serving loop
    (700-512-512-20 network, one foreign call: conversion, then per layer the sort and the forward)."""
    import ctypes

    import torch
    from bats_gb300 import _lib
    from bats_gb300 import kernels as K
    from bats_gb300._lib import stream_ptr
    torch.cuda.set_device(0)
    rng = np.random.default_rng(21)
    dev = "cuda"
    calls = []

    ts = build_train_step("active")
    ts.fwd_algo = [K.FWD_TILE, K.FWD_QUEUE, K.FWD_LANES]
    for name, fn in ts.launches:
        calls.append((f"step.{name}", lambda fn=fn: fn(stream_ptr())))
    calls.append(("api_step", plain_api_step("active")))
    conv_step, _, _ = conv_network()
    calls.append(("conv_step", conv_step))

    tau = 2 * TAU_S
    tau32, c, dtt = K.lif_constants(TAU_S, 0.2, 0.2)
    calls.append(("pre_exps", lambda: K.compute_pre_exps(ts.in_times, TAU_S, tau)))
    px = torch.tensor(rng.integers(0, 256, (B, SIZES[0])).astype(np.uint8), device=dev)
    calls.append(("intensity_to_spike_times", lambda: K.intensity_to_spike_times(px)))
    n_ev = np.exp(rng.uniform(np.log(50), np.log(5000), 16)).astype(np.int64)
    idx = np.full((16, int(n_ev.max())), -1, np.int32)
    tms = np.zeros(idx.shape, np.float32)
    for q, m in enumerate(n_ev):
        idx[q, :m] = rng.integers(0, 700, m)
        tms[q, :m] = np.sort(rng.uniform(0, 0.2, m))
    idx_d, tms_d = torch.tensor(idx, device=dev), torch.tensor(tms, device=dev)
    calls.append(("events_to_trains", lambda: K.convert_to_spike_per_neuron(idx_d, tms_d, 700)))
    out_t = ts.out[-1][3]
    targets = torch.full(out_t.shape, float("inf"), device=dev)
    calls.append(("ttfs_softmax_cross_entropy", lambda: K.ttfs_softmax_cross_entropy(out_t, ts.labels, tau)))
    calls.append(("spike_time_loss", lambda: K.spike_time_loss(out_t, targets, 2)))
    g = ts.grad[0]
    m1, v1, m2, v2 = (torch.zeros_like(g) for _ in range(4))
    d1, d2 = torch.empty_like(g), torch.empty_like(g)
    calls.append(("adam_step", lambda: K.adam_step(g, m1, v1, 0.9, 0.999, 1e-8, LR, 0.9, 0.999, delta=d1)))
    calls.append(("nadam_step", lambda: K.nadam_step(g, m2, v2, 0.9, 0.999, 1e-8, LR, 0.9, 0.999, d2)))
    gps = torch.zeros((64, SIZES[1], SIZES[0]), device=dev)
    ratios = torch.tensor(rng.uniform(0, 1, 64).astype(np.float32), device=dev)
    labels_f = torch.tensor(rng.integers(0, SIZES[1], 64).astype(np.float32), device=dev)
    calls.append(("weights_synaptic_scaling", lambda: K.apply_weights_synaptic_scaling(
        ts.W[0], ratios, ts.out[0][0][:64].contiguous(), gps, 0.5, 0.1)))
    calls.append(("label_weights_synaptic_scaling", lambda: K.apply_label_weights_synaptic_scaling(
        ts.W[0], labels_f, ts.out[0][0][:64].contiguous(), gps, 0.1)))
    calls.append(("transpose", lambda: K.transpose_weights(ts.W[0])))
    w_copy = ts.W[0].clone()
    calls.append(("add_deltas", lambda: K.add_deltas(w_copy, d1)))
    errs = torch.tensor(rng.uniform(-1, 1, (B, SIZES[1], K_SPIKE)).astype(np.float32), device=dev)
    t1, a1, x1, z1 = (o.clone() for o in ts.out[0][1:])  # the padded first hidden layer after a step
    calls.append(("propagate_recurrent_errors", lambda: K.propagate_recurrent_errors(x1, z1, errs, dtt)))
    calls.append(("compute_factors", lambda: K.compute_factors(t1, a1, c, x1, z1, tau32)))
    # The longest-first sample order and the ordered counted sort (the step uses them on wider batches).
    so = K.sample_order(ts.ev[0].counts)
    n1, h1 = ts.out[0][0].clone(), ts.out[0][3].clone()  # the first hidden layer's spike counts and times
    calls.append(("sample_order", lambda: K.sample_order(ts.ev[0].counts)))
    calls.append(("sort_events_counted_ordered", lambda: K.sort_events(h1, TAU_S, tau, pre_counts=n1,
                                                                         sample_order=so)))
    # A conv layer whose per-sample filter gradient (128 x 5 x 5 x 15 floats) exceeds shared memory.
    ct = np.full((32, 12 * 12 * 15, 4), np.inf, np.float32)
    nf = rng.integers(0, 5, ct.shape[:2])
    for q in range(4):
        ct[:, :, q] = np.where(q < nf, rng.uniform(0.01 * q, 0.01 * (q + 1), ct.shape[:2]), np.inf)
    cev = K.sort_events(torch.tensor(ct, device=dev), np.float32(TAU_S), np.float32(tau), bucketed=False)
    cw = torch.tensor(rng.uniform(0, 0.2, (128, 5, 5, 15)).astype(np.float32), device=dev)
    co = K.conv_forward(cev, cw, (12, 12, 15), 10, TAU_S, 0.3, 0.3, MAX_SIM)
    ctc, ccc, cdc = K.lif_constants(TAU_S, 0.3, 0.3)
    cerr = torch.tensor(rng.uniform(-1, 1, co[3].shape).astype(np.float32), device=dev)
    ctabs = K.backward_prep(co[3], co[1], co[2], co[4], cerr, ccc, ctc, cdc)
    calls.append(("conv_backward_large_filters", lambda: K.conv_backward(cev, cw, (12, 12, 15), co[3], ctabs, TAU_S,
                                                                          tau)))
    na_out = torch.empty((SIZES[1], SIZES[0]), device=dev)
    lib = _lib.load()

    def noalloc():
        ev, tb = ts.ev[0], ts.tabs[0]
        st = lib.bats_weights_gradient_mean_noalloc(
            ev.events.data_ptr(), ev.counts.data_ptr(), ev.cap, ts.out[0][3].data_ptr(), tb.tables.data_ptr(),
            tb.nvalid.data_ptr(), B, SIZES[1], K_SPIKE, SIZES[0], 32, na_out.data_ptr(),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st != 0:
            raise RuntimeError(lib.bats_last_error().decode())
    calls.append(("weights_gradient_mean_noalloc", noalloc))
    from bats_gb300.serving import InferenceServer, make_network, make_requests
    sws, sspecs = make_network()
    server = InferenceServer(sws, sspecs, 700, 5000, k_in=32, max_batch=16, max_lanes=1)
    sreqs = make_requests(16, seed=7)
    calls.append(("serve_batch_16", lambda: server.infer(sreqs)))

    for _, fn in calls:  # warm-up: module load, first-call set-up
        fn()
    torch.cuda.synchronize()
    flush = torch.zeros(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    flush_l2(flush)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("census")
    for name, fn in calls:
        torch.cuda.nvtx.range_push(name)
        fn()
        torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    _lib.check_device_status()
    print(json.dumps({"profiled": "census", "calls": [n for n, _ in calls]}))


def plain_api_step(variant):
    """One train step of the 784-800-800-10 network through the drop-in layer API (per-sample gradients, the
    caller's batch mean, AdamOptimizer deltas applied by the network), as a no-argument function."""
    import torch
    from bats_gb300 import Network, SpikeCountClassLoss
    from bats_gb300.Layers import InputLayer, LIFLayer
    from bats_gb300.Optimizers import AdamOptimizer
    ws = make_weights(variant)
    ths = thresholds(variant)
    net = Network()
    prev = InputLayer(n_neurons=SIZES[0], name="in")
    net.add_layer(prev, input=True)
    for i, (w, th) in enumerate(zip(ws, ths)):
        layer = LIFLayer(prev, n_neurons=w.shape[0], tau_s=TAU_S, theta=th, delta_theta=th,
                         weight_initializer=lambda a, b, w=w: torch.tensor(w, device="cuda"), max_n_spike=K_SPIKE,
                         name=f"l{i}")
        net.add_layer(layer)
        prev = layer
    loss_fn = SpikeCountClassLoss(TARGET_TRUE, TARGET_FALSE)
    opt = AdamOptimizer(learning_rate=LR)
    t, n, labels = make_inputs(B, 0)
    labels_d = torch.tensor(labels, device="cuda")

    def step():
        net.reset()
        net.forward(t, n, max_simulation=MAX_SIM, training=True)
        sp, nsp = net.output_spike_trains
        loss, err = loss_fn.compute_loss_and_errors(sp, nsp, labels_d)
        g = net.backward(err)
        d = opt.step([None if x is None else x.mean(0) for x in g])
        net.apply_deltas(d)

    return step


def plain_api_rate(variant, steps, flush):
    step = plain_api_step(variant)
    ms, _ = time_steps(step, steps, 1, flush)
    return {"value": B * steps / (ms / 1e3), "unit": "samples/s", "steps": steps,
            "what": "Network/LIFLayer/SpikeCountClassLoss/AdamOptimizer drop-in API, per-sample gradients"}


def autograd_rate(variant, steps, flush):
    """The differentiation pattern: 784-800-800-10 as three bats_gb300.autograd.lif_fc layers (batch 256), a
    loss written with torch ops on the output spike times (their sum over the slots that hold a spike), and
    torch.autograd.grad of it with respect to every layer's weights (the exact backward kernels behind the
    autograd Function, the weight gradient summed over the batch)."""
    import torch
    from bats_gb300.autograd import lif_fc
    ws = [torch.tensor(w, device="cuda", requires_grad=True) for w in make_weights(variant)]
    ths = thresholds(variant)
    t, _, _ = make_inputs(B, 0)
    x0 = torch.tensor(t, device="cuda")

    def step():
        x = x0
        for w, th in zip(ws, ths):
            x, _ = lif_fc(x, w, TAU_S, th, th, K_SPIKE, MAX_SIM)
        loss = torch.where(torch.isfinite(x), x, torch.zeros_like(x)).sum()
        torch.autograd.grad(loss, ws, allow_unused=True)

    ms, _ = time_steps(step, steps, 2, flush)
    return {"value": B * steps / (ms / 1e3), "unit": "samples/s", "ms_per_step": ms / steps, "steps": steps,
            "what": "forward + torch.autograd.grad through bats_gb300.autograd.lif_fc (weights' gradients)"}


def refkern_rate(variant, steps, flush):
    import torch
    from oracle import refkern
    if not refkern.available():
        return {"unavailable": "reference kernels not built (oracle/_ref)"}
    ws = [torch.tensor(w, device="cuda") for w in make_weights(variant)]
    ths = thresholds(variant)
    layers = [refkern.RefLIF(w, TAU_S, th, th, K_SPIKE) for w, th in zip(ws, ths)]
    t, n, labels = make_inputs(B, 0)
    td, nd = torch.tensor(t, device="cuda"), torch.tensor(n, device="cuda")
    m = [torch.zeros_like(w) for w in ws]
    v = [torch.zeros_like(w) for w in ws]
    state = {"t": 0}
    tt = torch.full((B, SIZES[-1]), TARGET_FALSE, device="cuda")
    tt[torch.arange(B), torch.tensor(labels, device="cuda").long()] = TARGET_TRUE

    def step():
        x, c = td, nd
        for L in layers:
            o = L.forward(x, c, np.float32(MAX_SIM))
            x, c = o[3], o[0]
        err = (tt - c.float())[:, :, None].repeat(1, 1, K_SPIKE).contiguous()
        grads = []
        for i in range(len(layers) - 1, -1, -1):
            g, err = layers[i].backward(err, want_pre=i > 0)
            grads.insert(0, g.mean(0))
        state["t"] += 1
        for i, g in enumerate(grads):
            m[i].mul_(0.9).add_(0.1 * g)
            v[i].mul_(0.999).add_(0.001 * g * g)
            mh = m[i] / (1 - 0.9 ** state["t"])
            vh = v[i] / (1 - 0.999 ** state["t"])
            layers[i].w.add_(-(LR * mh / (vh.sqrt() + 1e-8)))

    ms, _ = time_steps(step, steps, 1, flush)
    return {"value": B * steps / (ms / 1e3), "unit": "samples/s", "steps": steps,
            "what": "reference CUDA kernels (unmodified, oracle/_ref) with the reference wrappers' launch shapes"}


def batching_inputs(batch=4096, n_in=1024, seed=11, median=200, lo=20, hi=4000, t_max=0.1):
    """Per-sample input spike count clip(round(lognormal(ln median, 1)), lo, hi), channels uniform over
    n_in, times U(0, t_max): spike trains (B, n_in, K_in) with K_in the largest per-channel count, and
    labels."""
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
        slot = np.arange(len(ch_s)) - first
        t[q, ch_s, slot] = tm_s
    labels = rng.integers(0, 20, batch).astype(np.int32)
    return t, labels, counts


def batching_weights():
    """Weights U(-1, 1) of the 1024-1024-20 network (seeded) and its thresholds 0.2 hidden / 1.3 output."""
    rng = np.random.default_rng(12)
    sizes = [1024, 1024, 20]
    ws = [rng.uniform(-1, 1, (o, i)).astype(np.float32) for i, o in zip(sizes[:-1], sizes[1:])]
    return ws, [0.2, 1.3]


def batching_plain_rate(t, labels, flush, steps=2):
    """The uneven batch through the drop-in layer API (Network / LIFLayer / SpikeCountClassLoss /
    AdamOptimizer, per-sample gradients and the caller's batch mean), one launch chain per layer and no
    graph: the plain per-layer path the batched step is compared with."""
    import torch
    from bats_gb300 import Network, SpikeCountClassLoss
    from bats_gb300.Layers import InputLayer, LIFLayer
    from bats_gb300.Optimizers import AdamOptimizer
    ws, ths = batching_weights()
    net = Network()
    prev = InputLayer(n_neurons=1024, name="in")
    net.add_layer(prev, input=True)
    for i, (w, th) in enumerate(zip(ws, ths)):
        layer = LIFLayer(prev, n_neurons=w.shape[0], tau_s=TAU_S, theta=th, delta_theta=th,
                         weight_initializer=lambda a, b, w=w: torch.tensor(w, device="cuda"), max_n_spike=K_SPIKE,
                         name=f"l{i}")
        net.add_layer(layer)
        prev = layer
    loss_fn = SpikeCountClassLoss(TARGET_TRUE, TARGET_FALSE)
    opt = AdamOptimizer(learning_rate=LR)
    td = torch.tensor(t, device="cuda")
    nd = torch.isfinite(td).sum(2).to(torch.int32)
    labels_d = torch.tensor(labels, device="cuda")

    def step():
        net.reset()
        net.forward(td, nd, max_simulation=MAX_SIM, training=True)
        sp, nsp = net.output_spike_trains
        loss, err = loss_fn.compute_loss_and_errors(sp, nsp, labels_d)
        g = net.backward(err)
        net.apply_deltas(opt.step([None if x is None else x.mean(0) for x in g]))

    ms, _ = time_steps(step, steps, 1, flush)
    del net
    torch.cuda.empty_cache()
    return {"value": t.shape[0] * steps / (ms / 1e3), "unit": "samples/s", "ms_per_step": ms / steps,
            "steps": steps, "what": "Network/LIFLayer/SpikeCountClassLoss/AdamOptimizer drop-in API, per-sample "
                                    "gradients (4096 x 1024 x 1024 for the first layer), no graph"}


def batching_bench(steps: int = 5, warmup: int = 3):
    """Uneven batches: 4096 samples over 1024 input channels with lognormal spike counts (median 200,
    20-4000), times U(0, 0.1) s, network 1024-1024-20, max_n_spike 30, in the reference's MNIST regime
    (weights U(-1, 1), hidden threshold 0.2, output 1.3); the whole train step (forward, spike-count
    loss, exact backward, Adam) autotuned and replayed as one CUDA graph."""
    import torch
    from bats_gb300.train import FCLayerSpec, FCTrainStep
    t, labels, counts = batching_inputs()
    ws_np, ths = batching_weights()
    ws = [torch.tensor(w) for w in ws_np]
    specs = [FCLayerSpec(1024, TAU_S, ths[0], ths[0], K_SPIKE), FCLayerSpec(20, TAU_S, ths[1], ths[1], K_SPIKE)]
    ts = FCTrainStep(t.shape[0], 1024, t.shape[2], specs, ws, TARGET_TRUE, TARGET_FALSE, learning_rate=LR,
                     max_simulation=MAX_SIM)
    ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    tuned = ts.autotune()
    graphed = ts.try_capture()
    fn = ts.replay if graphed else ts.step
    flush = torch.zeros(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ms, _ = time_steps(fn, steps, warmup, flush)
    kb = kernel_breakdown(ts)
    out = {"value": t.shape[0] * steps / (ms / 1e3), "unit": "samples/s", "ms_per_step": ms / steps,
           "steps": steps, "batch": int(t.shape[0]), "k_in": int(t.shape[2]), "graph": graphed, "autotuned": tuned,
           "input_events": {"mean": float(counts.mean()), "max": int(counts.max()), "min": int(counts.min())},
           "spikes_per_layer": spike_counts(ts), "kernels_ms": {k: round(v, 4) for k, v in kb.items()},
           "network": "1024-1024-20, K 30, U(-1,1) weights, theta 0.2 hidden / 1.3 output"}
    del ts
    torch.cuda.empty_cache()
    out["plain_api"] = batching_plain_rate(t, labels, flush)
    out["batched_vs_plain"] = out["value"] / out["plain_api"]["value"]
    return out


CONV_THETAS = (0.04, 0.8, 0.6, 0.3)


def conv_weights(seed=3):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1, 1, (15, 5, 5, 1)).astype(np.float32), rng.uniform(-1, 1, (40, 5, 5, 15)).astype(np.float32),
            rng.uniform(-1, 1, (300, 640)).astype(np.float32), rng.uniform(-1, 1, (10, 300)).astype(np.float32)]


def conv_network():
    """The convolutional network of the reference's MNIST conv experiment (experiments/mnist/train_conv.py:
    conv 5x5x15 -> pool -> conv 5x5x40 -> pool -> FC 300 -> 10, thresholds 0.04 / 0.8 / 0.6 / 0.3 with
    delta_theta = theta, tau_s 0.13, weights U(-1, 1)), max_n_spike 10 in every layer, batch 128, on
    synthetic MNIST-shaped single-spike input; full train step (forward, spike-count loss, exact backward,
    Adam) through the drop-in layer API. Returns (step, layers, inputs (t, n, labels))."""
    import torch
    from bats_gb300 import Network, SpikeCountClassLoss
    from bats_gb300.Layers import ConvInputLayer, ConvLIFLayer, LIFLayer, PoolingLayer
    from bats_gb300.Optimizers import AdamOptimizer
    Bc, Kc = 128, 10
    w1, w2, w3, w4 = conv_weights()
    net = Network()
    inp = ConvInputLayer(neurons_shape=np.array([28, 28, 1]), name="in")
    net.add_layer(inp, input=True)
    c1 = ConvLIFLayer(inp, filters_shape=np.array([5, 5, 15]), tau_s=TAU_S, theta=CONV_THETAS[0],
                      delta_theta=CONV_THETAS[0], weight_initializer=lambda *a: torch.tensor(w1, device="cuda"),
                      max_n_spike=Kc, name="conv1")
    net.add_layer(c1)
    p1 = PoolingLayer(c1, name="pool1")
    net.add_layer(p1)
    c2 = ConvLIFLayer(p1, filters_shape=np.array([5, 5, 40]), tau_s=TAU_S, theta=CONV_THETAS[1],
                      delta_theta=CONV_THETAS[1], weight_initializer=lambda *a: torch.tensor(w2, device="cuda"),
                      max_n_spike=Kc, name="conv2")
    net.add_layer(c2)
    p2 = PoolingLayer(c2, name="pool2")
    net.add_layer(p2)
    f1 = LIFLayer(p2, n_neurons=300, tau_s=TAU_S, theta=CONV_THETAS[2], delta_theta=CONV_THETAS[2],
                  weight_initializer=lambda *a: torch.tensor(w3, device="cuda"), max_n_spike=Kc, name="fc")
    net.add_layer(f1)
    out = LIFLayer(f1, n_neurons=10, tau_s=TAU_S, theta=CONV_THETAS[3], delta_theta=CONV_THETAS[3],
                   weight_initializer=lambda *a: torch.tensor(w4, device="cuda"), max_n_spike=Kc, name="out")
    net.add_layer(out)
    loss_fn = SpikeCountClassLoss(TARGET_TRUE, TARGET_FALSE)
    opt = AdamOptimizer(learning_rate=LR)
    t, n, labels = make_inputs(Bc, 5)
    labels_d = torch.tensor(labels, device="cuda")
    layers = [c1, p1, c2, p2, f1, out]

    def step():
        net.reset()
        net.forward(t, n, max_simulation=MAX_SIM, training=True)
        sp, nsp = net.output_spike_trains
        loss, err = loss_fn.compute_loss_and_errors(sp, nsp, labels_d)
        g = net.backward(err)
        net.apply_deltas(opt.step([None if x is None else x.mean(0) for x in g]))

    return step, layers, (t, n, labels)


def conv_train_step(t, labels, group=2):
    """The conv network of conv_network as a bats_gb300.conv_train.ConvTrainStep (batch-reduced filter
    gradients fused with Adam, one CUDA graph), same weights and inputs."""
    import torch
    from bats_gb300.conv_train import ConvLayerSpec, ConvTrainStep, PoolLayerSpec
    from bats_gb300.train import FCLayerSpec
    Kc = 10
    w1, w2, w3, w4 = conv_weights()
    specs = [ConvLayerSpec((5, 5, 15), TAU_S, CONV_THETAS[0], CONV_THETAS[0], Kc), PoolLayerSpec(),
             ConvLayerSpec((5, 5, 40), TAU_S, CONV_THETAS[1], CONV_THETAS[1], Kc), PoolLayerSpec(),
             FCLayerSpec(300, TAU_S, CONV_THETAS[2], CONV_THETAS[2], Kc),
             FCLayerSpec(10, TAU_S, CONV_THETAS[3], CONV_THETAS[3], Kc)]
    ws = [torch.tensor(w1), None, torch.tensor(w2), None, torch.tensor(w3), torch.tensor(w4)]
    ts = ConvTrainStep(t.shape[0], (28, 28, 1), 1, specs, ws, TARGET_TRUE, TARGET_FALSE, learning_rate=LR,
                       max_simulation=MAX_SIM, conv_group=group)
    ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    return ts


def conv_bench(steps: int = 5):
    """The conv network's train step: batch-reduced and graph-captured (ConvTrainStep, `value`), through the
    drop-in layer API (conv_network, `plain_api`), and on the reference's own CUDA kernels (`refkern`)."""
    import torch
    Bc = 128
    step, layers, (t, n, labels) = conv_network()
    flush = torch.zeros(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
    ms_api, _ = time_steps(step, steps, 3, flush)
    spikes = [int(L.spike_trains[1].sum().item()) for L in layers]
    del step, layers
    torch.cuda.empty_cache()
    ts = conv_train_step(t, labels)
    graphed = ts.try_capture()
    ms, _ = time_steps(ts.replay if graphed else ts.step, steps, 3, flush)
    kb = kernel_breakdown(ts)
    res = {"value": Bc * steps / (ms / 1e3), "unit": "samples/s", "ms_per_step": ms / steps, "steps": steps,
           "batch": Bc, "graph": graphed, "spikes_per_layer": spikes,
           "kernels_ms": {k: round(v, 4) for k, v in kb.items()},
           "network": "28x28x1 -> conv 5x5x15 -> pool -> conv 5x5x40 -> pool -> 300 -> 10, K 10",
           "what": "ConvTrainStep: batch-reduced filter gradients fused with Adam, whole step as one CUDA graph",
           "plain_api": {"value": Bc * steps / (ms_api / 1e3), "unit": "samples/s", "ms_per_step": ms_api / steps,
                         "what": "Network/ConvLIFLayer/PoolingLayer/LIFLayer/AdamOptimizer drop-in API, per-sample "
                                 "gradients and the caller's batch mean"}}
    res["batched_vs_plain"] = res["value"] / res["plain_api"]["value"]
    del ts
    torch.cuda.empty_cache()
    res["refkern"] = refkern_conv_rate(t, n, labels, flush)
    return res


def refkern_conv_rate(t, n, labels, flush, steps=1):
    """The conv network's train step on the reference's own CUDA kernels (oracle/refkern.py), same weights
    and inputs."""
    import torch
    from oracle import refkern
    if not refkern.available():
        return {"unavailable": "reference kernels not built (oracle/_ref)"}
    Kc = 10
    ws = [torch.tensor(w, device="cuda") for w in conv_weights()]
    L1 = refkern.RefConvLIF(ws[0], (28, 28, 1), TAU_S, CONV_THETAS[0], CONV_THETAS[0], Kc)
    L2 = refkern.RefConvLIF(ws[1], (12, 12, 15), TAU_S, CONV_THETAS[1], CONV_THETAS[1], Kc)
    L3 = refkern.RefLIF(ws[2], TAU_S, CONV_THETAS[2], CONV_THETAS[2], Kc)
    L4 = refkern.RefLIF(ws[3], TAU_S, CONV_THETAS[3], CONV_THETAS[3], Kc)
    td, nd = torch.tensor(t, device="cuda"), torch.tensor(n, device="cuda")
    Bc = td.shape[0]
    tt = torch.full((Bc, 10), TARGET_FALSE, device="cuda")
    tt[torch.arange(Bc), torch.tensor(labels, device="cuda").long()] = TARGET_TRUE
    params = [L1.w, L2.w, L3.w, L4.w]
    m = [torch.zeros_like(w) for w in params]
    v = [torch.zeros_like(w) for w in params]
    state = {"t": 0}

    def step():
        o1 = L1.forward(td, nd, np.float32(MAX_SIM))
        pn1, pt1, pi1 = refkern.pool_forward(o1[0], o1[3], (24, 24, 15))
        o2 = L2.forward(pt1, pn1, np.float32(MAX_SIM))
        pn2, pt2, pi2 = refkern.pool_forward(o2[0], o2[3], (8, 8, 40))
        o3 = L3.forward(pt2, pn2, np.float32(MAX_SIM))
        o4 = L4.forward(o3[3], o3[0], np.float32(MAX_SIM))
        err = (tt - o4[0].float())[:, :, None].repeat(1, 1, Kc).contiguous()
        g4, e3 = L4.backward(err, want_pre=True)
        g3, ep2 = L3.backward(e3, want_pre=True)
        e2 = refkern.pool_backward(ep2, pi2, o2[3].shape)
        g2, ep1 = L2.backward(e2.contiguous(), want_pre=True)
        e1 = refkern.pool_backward(ep1, pi1, o1[3].shape)
        g1, _ = L1.backward(e1.contiguous(), want_pre=False)
        state["t"] += 1
        for i, g in enumerate((g1, g2, g3, g4)):
            g = g.mean(0)
            m[i].mul_(0.9).add_(0.1 * g)
            v[i].mul_(0.999).add_(0.001 * g * g)
            mh = m[i] / (1 - 0.9 ** state["t"])
            vh = v[i] / (1 - 0.999 ** state["t"])
            params[i].add_(-(LR * mh / (vh.sqrt() + 1e-8)))

    ms, _ = time_steps(step, steps, 1, flush)
    return {"value": Bc * steps / (ms / 1e3), "unit": "samples/s", "steps": steps,
            "what": "reference CUDA kernels (unmodified, oracle/_ref) with the reference wrappers' launch shapes"}


def serving_bench(n_sat: int = 3000, poisson_seconds: float = 2.0, load: float = 0.8):
    """Serving loop on the 700-512-512-20 network (max_n_spike 30): requests of 50-5000 events
    (log-uniform) over 700 channels at times U(0, 0.2) s. Peak throughput = requests completed per second
    when n_sat requests are queued at once; then Poisson arrivals at `load` x peak for about
    poisson_seconds, reporting p50/p99 of arrival -> result-on-host latency."""
    import dataclasses
    import torch
    from bats_gb300.serving import InferenceServer, latency_stats, make_network, make_requests, run_poisson
    ws, specs = make_network()
    server = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=16, max_lanes=16)
    pool = make_requests(1000, seed=7)
    tuned = server.autotune(pool[:64])

    def batch_of(n, rid0):
        return [dataclasses.replace(pool[q % len(pool)], rid=rid0 + q) for q in range(n)]

    server.infer(batch_of(200, 0))  # warm-up: kernels loaded, lanes touched
    torch.cuda.synchronize()
    reqs = batch_of(n_sat, 10_000)
    t0 = time.perf_counter()
    server.infer(reqs)
    sat_s = time.perf_counter() - t0
    peak = n_sat / sat_s
    rate = load * peak
    n_p = int(min(40_000, max(1000, rate * poisson_seconds)))
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        res = run_poisson(server, batch_of(n_p, 100_000), rate, seed=1)
    st = latency_stats(res)
    events = np.array([len(r.indices) for r in pool])
    return {"network": "700-512-512-20, max_n_spike 30, W~(N(1.5,1))/sqrt(fan_in), theta 1.0/1.3",
            "requests": "50-5000 events log-uniform over 700 channels, times U(0, 0.2) s",
            "mean_events_per_request": float(events.mean()),
            "peak_throughput_rps": peak, "load_rps": rate, "load_fraction": load, "n_requests": n_p,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
            "lanes": len(server.lanes), "max_batch": server.max_batch, "rejected": len(server.rejected),
            "forward_variant_per_batch_bucket": tuned,
            "batches": server.batches_launched, "clocks": clk.summary()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--workload", default="all", choices=["all", "literal", "active", "serving", "conv", "batching"],
                    help="all (default): every measurement; otherwise only that one (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline (profiling runs)")
    ap.add_argument("--profile-kernels", action="store_true",
                    help="run every kernel of the library once inside NVTX ranges under \"census\" (for ncu)")
    ap.add_argument("--profile-step", action="store_true",
                    help="with --workload literal|active|batching: set up and autotune the step, then run one "
                         "eager step with an NVTX range named after every launch (for ncu --nvtx-include)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        # The reference's path on the host cores, on the headline's workload and configuration (same config
        # dict as our arm's line); a step is a bounded sample of it.
        cb = cpu_baseline(HEADLINE, budget_s=max(5.0, min(60.0, args.cpu_budget * args.steps / 10)))
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "samples/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * B / cb["value"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": headline_config(args.gpus),
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "samples/s", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.profile_step:
        profile_one_step(args.workload)
        return
    if args.profile_kernels:
        profile_kernels()
        return

    # CPU baselines first (spawned workers, before any GPU context exists in this process).
    cb = cpu_baseline(HEADLINE, budget_s=args.cpu_budget) if rank == 0 and not args.no_cpu else None
    cb_batching = (batching_cpu_baseline(budget_s=args.cpu_budget)
                   if rank == 0 and not args.no_cpu and args.workload in ("all", "batching") else None)

    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl")
        dist = dist_mod
    res = run_ours(args, dist, rank, world)
    serving = serving_bench() if args.workload in ("all", "serving") else None
    conv = conv_bench() if args.workload in ("all", "conv") else None
    batching = batching_bench() if args.workload in ("all", "batching") else None
    if batching is not None:
        batching["cpu_baseline"] = cb_batching
    if rank != 0:
        return
    if args.workload != "all":
        head = res.get(args.workload, {})
        print(json.dumps({"metric": METRIC, "workload": args.workload, "value": head.get("value"),
                          "unit": "samples/s", "steps": args.steps, "warmup": args.warmup, "detail": head,
                          "serving": serving, "conv": conv, "batching": batching}))
        return
    head, lit = res[HEADLINE], res["literal"]
    line = {
        "metric": METRIC, "value": head["value"], "spikes_per_layer": head["spikes_per_layer"], "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(world), "cuda_graph": head["graph"],
        "roofline": head["roofline"], "e2e": head["e2e"], "gpu_launches": head["gpu_launches"],
        "clocks": head["clocks"], "cpu_baseline": cb,
        "plain_api": head.get("plain_api"), "batched_vs_plain": (head["value"] / head["plain_api"]["value"]
                                                                 if head.get("plain_api") else None),
        "autograd": head.get("autograd"), "refkern": head.get("refkern"),
        "autotuned": head["autotuned"], "kernels_ms": head["kernels_ms"],
        "serving": serving, "conv": conv, "batching": batching, "literal": lit,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
