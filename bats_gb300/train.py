"""Batched training step of a fully-connected BATS network with every buffer preallocated.

FCTrainStep runs forward (per-layer event sort + LIF forward), the spike-count classification loss,
the exact backward with batch-mean weight gradients, and Adam updates of the weights and of their
transposed copies, with no host synchronisation and no allocation after construction, so that the
whole step can be captured once as a CUDA graph and replayed (capture()). It computes the same
arithmetic as the layer-by-layer API (Network + LIFLayer + SpikeCountClassLoss + AdamOptimizer +
the caller's batch mean), only without materialising the per-sample gradients. The spike trains of
its hidden layers (self.out) hold valid times only below their spike counts (no +inf padding).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import kernels as K
from ._lib import call, ptr, stream_ptr
from .autotune import Autotuner, get_tuner


@dataclass
class FCLayerSpec:
    n_neurons: int
    tau_s: float
    theta: float
    delta_theta: float
    max_n_spike: int


class FCTrainStep:
    def __init__(self, batch: int, n_inputs: int, k_input: int, layers: Sequence[FCLayerSpec],
                 weights: Sequence[torch.Tensor], target_true: float, target_false: float,
                 learning_rate: float = 3e-3, beta_1: float = 0.9, beta_2: float = 0.999, epsilon: float = 1e-8,
                 max_simulation: float = np.inf, grad_group: int = 0, device="cuda"):
        self.B = int(batch)
        self.dev = torch.device(device)
        self.specs = list(layers)
        self.max_sim = float(max_simulation)
        self.tt, self.tf = np.float32(target_true), np.float32(target_false)
        self.lr, self.b1, self.b2, self.eps = (np.float32(v) for v in (learning_rate, beta_1, beta_2, epsilon))
        self.t = 0
        self.grad_group = int(grad_group)
        B, dev = self.B, self.dev
        f32, i32 = torch.float32, torch.int32
        # Inputs (device-resident).
        self.in_times = torch.full((B, n_inputs, k_input), float("inf"), dtype=f32, device=dev)
        self.labels = torch.zeros((B,), dtype=i32, device=dev)
        # Per-layer state.
        self.W, self.Wt, self.m, self.v, self.ev, self.out, self.tabs, self.grad, self.pre_err = ([] for _ in range(9))
        n_prev, k_prev = n_inputs, k_input
        for spec, w in zip(self.specs, weights):
            w = w.to(device=dev, dtype=f32).contiguous().clone()
            assert w.shape == (spec.n_neurons, n_prev)
            self.W.append(w)
            self.Wt.append(K.transpose_weights(w))
            self.m.append(torch.zeros_like(w))
            self.v.append(torch.zeros_like(w))
            self.ev.append(K.alloc_events(B, n_prev, k_prev, dev))
            N, Kp = spec.n_neurons, spec.max_n_spike
            self.out.append((torch.empty((B, N), dtype=i32, device=dev),
                             *(torch.empty((B, N, Kp), dtype=f32, device=dev) for _ in range(4))))
            need_f = Kp > 32
            self.tabs.append(K.BackwardTables(torch.empty((B, N, Kp), dtype=f32, device=dev) if need_f else None,
                                              torch.empty((B, N, Kp), dtype=f32, device=dev) if need_f else None,
                                              torch.empty((B, N, Kp + 1, 2), dtype=f32, device=dev),
                                              torch.empty((B, N), dtype=i32, device=dev),
                                              K.alloc_cursor_heads(B, N, dev) if not need_f else None))
            self.grad.append(torch.empty((N, n_prev), dtype=f32, device=dev))
            self.pre_err.append(torch.empty((B, n_prev, k_prev), dtype=f32, device=dev))
            n_prev, k_prev = N, Kp
        self.loss = torch.empty((B,), dtype=f32, device=dev)
        self.errors = torch.empty((B, n_prev, k_prev), dtype=f32, device=dev)
        # Samples per gradient group (>= 2 selects the batch-mean path) and scratch for the largest user.
        self.groups = []
        ws = 0
        n_prev, k_prev = n_inputs, k_input
        for spec in self.specs:
            grp = max(2, self.grad_group or K.default_group(B, spec.n_neurons, n_prev))
            self.groups.append(grp)
            ws = max(ws, K.call_size("bats_sort_events_workspace_bytes", B, n_prev, k_prev),
                     K.queue_workspace_bytes(B),
                     K.call_size("bats_weights_gradient_workspace_bytes", B, spec.n_neurons, n_prev, grp),
                     K.call_size("bats_pre_errors_workspace_bytes", B, n_prev * k_prev, spec.n_neurons))
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        # (bats_fc_train_step, native_step, keeps its sample order in front of the same workspaces: B ints in
        # 256-byte lines)
        self.ws = torch.empty(max(ws, 256) + -(-B * 4 // 256) * 256, dtype=torch.uint8, device=dev)
        # Batches wider than the sort's resident CTAs sort each hidden layer's spikes with the samples longest
        # first: a sample's input event count ranks its output spike count closely (the order of the work-queue
        # forward), so the long samples start in the first wave instead of setting the launch's tail.
        self.order = [torch.empty(B, dtype=i32, device=dev) if li > 0 and K.order_pays(B, dev) else None
                      for li in range(len(self.specs))]
        # The gradient + Adam of every layer above the first runs on a second stream, beside the pre-spike
        # errors that read the layer's old transposed weights: it writes the new ones into a staging copy
        # (copied over Wt at the end of the step) and uses its own workspace (as large as the first, so that
        # every gradient group the autotuner may pick fits both).
        self.Wt_next = [wt.clone() if li > 0 else None for li, wt in enumerate(self.Wt)]
        self.ws2 = torch.empty_like(self.ws)
        self.aux = torch.cuda.Stream(device=dev) if torch.cuda.is_available() else None
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.capture_error = None
        # beta_1^t, beta_2^t on the device, advanced by one launch per step (keeps the step capturable).
        self.powers = torch.tensor([1.0, 1.0, 0.0, 0.0], dtype=torch.float64, device=dev)
        # Host staging for end-to-end steps.
        self.h_times = torch.empty(self.in_times.shape, dtype=f32, pin_memory=True)
        self.h_labels = torch.empty((B,), dtype=i32, pin_memory=True)
        self.h_loss = torch.empty((B,), dtype=f32, pin_memory=True)
        self.fwd_algo = [K.FWD_AUTO] * len(self.specs)
        self.launches = self._build_launches()

    def _pad_flag(self, li: int) -> int:
        """Hidden layers skip the +inf padding of their spike trains: everything that reads them (the next
        layer's counted sort, the counted prep, the gradient and pre-error kernels) stays below the spike
        counts. The output layer (read by the loss) and layers with K > 32 (whose prep scans the times)
        keep it."""
        last = li + 1 == len(self.specs)
        return 0 if last or self.specs[li].max_n_spike > 32 else K.FWD_NO_PAD

    # -- the step as a fixed list of launches --------------------------------------------------------
    def _build_launches(self):
        """(name, fn(stream)) for every entry-point call of one step, in order. All pointers are fixed.
        Adam's bias-correction powers are advanced first; each layer's backward is prep, pre-spike errors (which
        read the layer's weights before their update), then the batch-mean gradient fused with the layer's
        Adam update."""
        B = self.B
        ws, wsb = ptr(self.ws), self.ws.numel()
        L = [("adam.powers", lambda s: call("bats_adam_powers_advance", ptr(self.powers), float(self.b1),
                                              float(self.b2), s))]
        pre_times, pre_counts = self.in_times, None
        for li, spec in enumerate(self.specs):
            ev = self.ev[li]
            tau32, c, dtt = K.lif_constants(spec.tau_s, spec.theta, spec.delta_theta)
            tag = f"L{li + 1}"
            if pre_counts is None:  # the network input: every slot is read
                L.append((f"{tag}.sort", lambda s, pt=ptr(pre_times), ev=ev, spec=spec, tau32=tau32: call(
                    "bats_sort_events", pt, B, ev.n_neurons, ev.k, float(np.float32(spec.tau_s)), float(tau32),
                    None, None, ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ptr(ev.bucketed),
                    ptr(ev.bucket_offsets), K.BUCKET_WIDTH, ws, wsb, s)))
            elif self.order[li] is None:  # a LIF layer's output: only the slots below its spike counts
                L.append((f"{tag}.sort", lambda s, pt=ptr(pre_times), pc=ptr(pre_counts), ev=ev, spec=spec,
                          tau32=tau32: call(
                    "bats_sort_events_counted", pt, pc, B, ev.n_neurons, ev.k, float(np.float32(spec.tau_s)),
                    float(tau32), None, None, ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ptr(ev.bucketed),
                    ptr(ev.bucket_offsets), K.BUCKET_WIDTH, ws, wsb, s)))
            else:  # the same with the samples longest first, ranked by the previous layer's input event counts
                L.append((f"{tag}.order", lambda s, c=ptr(self.ev[li - 1].counts), o=ptr(self.order[li]): call(
                    "bats_sample_order", c, B, o, s)))
                L.append((f"{tag}.sort", lambda s, pt=ptr(pre_times), pc=ptr(pre_counts), ev=ev, spec=spec,
                          tau32=tau32, o=ptr(self.order[li]): call(
                    "bats_sort_events_counted_ordered", pt, pc, B, ev.n_neurons, ev.k, float(np.float32(spec.tau_s)),
                    float(tau32), None, None, ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ptr(ev.bucketed),
                    ptr(ev.bucket_offsets), K.BUCKET_WIDTH, o, ws, wsb, s)))
            n, a, x, t, z = self.out[li]
            L.append((f"{tag}.forward", lambda s, ev=ev, li=li, spec=spec, c=c, dtt=dtt, tau32=tau32, o=self.out[li]:
                      K.forward_fc_call(ev, self.Wt[li], spec.n_neurons, spec.max_n_spike, c, dtt, tau32,
                                        self.max_sim, o, self.fwd_algo[li] | self._pad_flag(li), s, ws, wsb)))
            pre_times, pre_counts = t, n
        n_out = self.out[-1][0]
        L.append(("loss", lambda s: call("bats_spike_count_loss", ptr(n_out), 0, None, ptr(self.labels),
                                         float(self.tt), float(self.tf), B, n_out.shape[1],
                                         self.specs[-1].max_n_spike, ptr(self.loss), ptr(self.errors), s)))
        errors = self.errors
        for li in range(len(self.specs) - 1, -1, -1):
            spec = self.specs[li]
            ev = self.ev[li]
            n, a, x, t, z = self.out[li]
            tau32, c, dtt = K.lif_constants(spec.tau_s, spec.theta, spec.delta_theta)
            tb = self.tabs[li]
            tag = f"L{li + 1}"
            if spec.max_n_spike <= 32:  # only the slots below the forward's spike counts are read
                L.append((f"{tag}.prep", lambda s, o=self.out[li], e=errors, spec=spec, c=c, tau32=tau32, dtt=dtt,
                          tb=tb: call("bats_backward_prep_counted", ptr(o[3]), ptr(o[0]), ptr(o[1]), ptr(o[2]),
                                      ptr(o[4]), ptr(e), B, spec.n_neurons, spec.max_n_spike, float(c),
                                      float(tau32), float(dtt), ptr(tb.tables), ptr(tb.nvalid), ptr(tb.heads), s)))
            else:
                L.append((f"{tag}.prep", lambda s, o=self.out[li], e=errors, spec=spec, c=c, tau32=tau32, dtt=dtt,
                          tb=tb: call("bats_backward_prep_layer", ptr(o[3]), ptr(o[1]), ptr(o[2]), ptr(o[4]),
                                      ptr(e), B, spec.n_neurons, spec.max_n_spike, float(c), float(tau32),
                                      float(dtt), ptr(tb.f1), ptr(tb.f2), ptr(tb.tables), ptr(tb.nvalid), s)))
            if li > 0:
                pe = self.pre_err[li]
                L.append((f"{tag}.pre_err", lambda s, ev=ev, t=t, tb=tb, spec=spec, li=li, pe=pe, tau32=tau32: call(
                    "bats_pre_errors", ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ev.cap, ptr(self.Wt[li]),
                    self.Wt[li].shape[1], ptr(t), ptr(tb.tables), ptr(tb.nvalid), B, spec.n_neurons,
                    spec.max_n_spike, ev.n_neurons, ev.k, float(np.float32(spec.tau_s)), float(tau32), ptr(pe), ws,
                    wsb, s)))
                errors = pe
            # Above the first layer: the staging copy of Wt and the second workspace (see __init__).
            wt_out = self.Wt_next[li] if li > 0 else self.Wt[li]
            gws, gwsb = (ptr(self.ws2), self.ws2.numel()) if li > 0 else (ws, wsb)
            L.append((f"{tag}.grad_adam", lambda s, ev=ev, t=t, tb=tb, spec=spec, li=li, wt_out=wt_out, gws=gws,
                      gwsb=gwsb: call(
                "bats_weights_gradient_adam", ptr(ev.events), ptr(ev.counts), ptr(ev.bucketed),
                ptr(ev.bucket_offsets), ev.cap, ptr(t), ptr(tb.tables), ptr(tb.nvalid), ptr(tb.heads), B,
                spec.n_neurons, spec.max_n_spike, ev.n_neurons, self.groups[li], ptr(self.grad[li]), ptr(self.m[li]),
                ptr(self.v[li]), float(self.b1), float(self.b2), float(self.eps), float(self.lr), ptr(self.powers),
                ptr(self.W[li]), ptr(wt_out), self.Wt[li].shape[1], gws, gwsb, s)))
        for li in range(len(self.specs) - 1, 0, -1):
            L.append((f"L{li + 1}.wt_copy", lambda s, li=li: K.copy_on_stream(self.Wt[li], self.Wt_next[li], s)))
        return L

    def _side_launches(self):
        """{gradient launch: the launch it waits for}: each layer's gradient + Adam above the first, which
        needs only its layer's prep (and what came before it)."""
        return {f"L{li + 1}.grad_adam": f"L{li + 1}.prep" for li in range(1, len(self.specs))}

    def _enqueue(self, main, aux=None) -> None:
        """Enqueue one step on the torch stream `main` (and `aux`: see enqueue_launches)."""
        enqueue_launches(self.launches, self._side_launches(), main, aux)

    # -- the same step as one foreign call (bats_fc_train_step) -------------------------------------
    def native_layers(self):
        """The layers as an array of struct BatsFcTrainLayer for bats_fc_train_step, built from this step's
        buffers, forward variants and gradient groups as they are now (call again after autotune)."""
        from ._lib import BatsFcLayer, BatsFcTrainLayer
        arr = (BatsFcTrainLayer * len(self.specs))()
        n_prev, k_prev = self.in_times.shape[1], self.in_times.shape[2]
        for li, spec in enumerate(self.specs):
            ev, tb = self.ev[li], self.tabs[li]
            n, a, x, t, z = self.out[li]
            tau32, c, dtt = K.lif_constants(spec.tau_s, spec.theta, spec.delta_theta)
            algo = self.fwd_algo[li]
            fwd = BatsFcLayer(n_prev, k_prev, spec.n_neurons, spec.max_n_spike, ptr(self.Wt[li]), self.Wt[li].shape[1],
                              float(np.float32(spec.tau_s)), float(tau32), float(c), float(dtt),
                              float(np.float32(self.max_sim)), int(algo), ptr(ev.events), ptr(ev.slots),
                              ptr(ev.counts), ptr(n), ptr(a), ptr(x), ptr(t), ptr(z))
            arr[li] = BatsFcTrainLayer(fwd, ptr(self.W[li]), ptr(self.m[li]), ptr(self.v[li]), ptr(self.grad[li]),
                                       ptr(ev.bucketed), ptr(ev.bucket_offsets), ptr(tb.tables), ptr(tb.nvalid),
                                       ptr(tb.heads), ptr(tb.f1), ptr(tb.f2),
                                       ptr(self.pre_err[li]) if li > 0 else None,
                                       int(self.groups[li]))
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        return arr

    def native_step(self) -> None:
        """One training step as a single call of the C ABI's bats_fc_train_step: the same launches, arguments
        and results as step()."""
        import ctypes
        layers = self.native_layers()
        need = K.call_size("bats_fc_train_step_workspace_bytes", self.B, ctypes.cast(layers, ctypes.c_void_p),
                           len(self.specs))
        assert need <= self.ws.numel(), "workspace smaller than bats_fc_train_step needs"
        call("bats_fc_train_step", ptr(self.in_times), ptr(self.labels), self.B, ctypes.cast(layers, ctypes.c_void_p),
             len(self.specs), float(self.tt), float(self.tf), float(self.b1), float(self.b2), float(self.eps),
             float(self.lr), ptr(self.powers), ptr(self.loss), ptr(self.errors), ptr(self.ws), self.ws.numel(),
             stream_ptr())
        self.t += 1

    def _grad_only(self, li: int, group: int, s) -> None:
        """The batch-mean weight gradient of layer li into self.grad[li] (no weight update), from the tables of
        the last backward pass: what the autotuner times for the gradient group size."""
        spec, ev = self.specs[li], self.ev[li]
        t, tb = self.out[li][3], self.tabs[li]
        call("bats_weights_gradient", ptr(ev.events), ptr(ev.counts), ptr(ev.bucketed), ptr(ev.bucket_offsets),
             ev.cap, ptr(t), ptr(tb.tables), ptr(tb.nvalid), ptr(tb.heads), self.B, spec.n_neurons,
             spec.max_n_spike, ev.n_neurons, group, 1, ptr(self.grad[li]), ptr(self.ws), self.ws.numel(), s)

    @property
    def launches_per_step(self) -> int:
        """Kernels of this library launched by one step with the current variant choices (memsets not
        counted), following the branches of the entry points."""
        return self._count_launches()

    def _kernels_of(self, name: str) -> int:
        tag, _, kind = name.rpartition(".")  # "L2.grad_adam", "adam.powers", "loss"
        if tag[:1] == "L" and tag[1:].isdigit():
            li = int(tag[1:]) - 1
            spec, n_pre = self.specs[li], self.ev[li].n_neurons
        if kind == "forward":  # the work queue adds its order kernel
            return 2 if K.is_queue_algo(self.fwd_algo[li]) else 1
        if kind == "pre_err":  # narrow layers: one event-parallel kernel; else the tile kernel and the scatter
            return 1 if spec.n_neurons <= 32 else 2
        if kind == "wt_copy":  # a device-to-device copy, no kernel
            return 0
        if kind == "grad_adam":  # the gradient, then the fused reduce-Adam, or for few weight tiles and
            groups = -(-self.B // self.groups[li])  # several partials the reduction and the tiled Adam
            tiles = -(-n_pre // 32) * -(-spec.n_neurons // 32)
            return 3 if groups > 1 and tiles < 2 * 152 else 2
        return 1  # sort, order, loss, prep, powers

    def _count_launches(self):
        return sum(self._kernels_of(name) for name, _ in self.launches)

    def step(self) -> None:
        """One training step on the device-resident inputs (in_times, labels), launched eagerly (with the
        gradients above the first layer on the second stream, as in the graph)."""
        self._enqueue(torch.cuda.current_stream(), self.aux)
        self.t += 1

    def autotune(self, tuner: Optional[Autotuner] = None, force: bool = False) -> dict:
        """Pick, per layer, the forward kernel variant and the samples per partial gradient by timing the
        candidates on this step's own buffers (after one forward/backward pass without the optimizer, so
        the weights are unchanged). Call before try_capture. Returns the choices."""
        tuner = tuner or get_tuner()
        s = stream_ptr()
        for name, fn in self.launches:
            # leave the weights and Adam state alone (no update, no staged transposed weights copied in)
            if not name.endswith(("grad_adam", "wt_copy")) and name != "adam.powers":
                fn(s)
        torch.cuda.synchronize()
        B = self.B
        choice = {}
        n_prev = self.in_times.shape[1]
        k_prev = self.in_times.shape[2]
        fwd = {nm: fn for nm, fn in self.launches if nm.endswith(".forward")}
        wsb = self.ws.numel()
        for li, spec in enumerate(self.specs):
            tag = f"L{li + 1}"
            ev_mean = max(1, int(self.ev[li].counts.float().mean().item()))
            bucket = int(np.log2(ev_mean))
            shape = (B, n_prev, k_prev, spec.n_neurons, spec.max_n_spike, bucket)

            def run_fwd(algo, li=li):
                saved = self.fwd_algo[li]
                self.fwd_algo[li] = algo
                fwd[f"{tag}.forward"](s)
                self.fwd_algo[li] = saved

            algos = {"tile": K.FWD_TILE, "lanes": K.FWD_LANES, "queue": K.FWD_QUEUE,
                     "tile_stage": K.FWD_TILE | K.FWD_STAGE, "queue_stage": K.FWD_QUEUE | K.FWD_STAGE}
            if spec.n_neurons > 64:
                algos["tile64"] = K.FWD_TILE64
                algos["queue64"] = K.FWD_QUEUE64
            best = tuner.pick("fc_forward", shape, {k: (lambda a=a: run_fwd(a)) for k, a in algos.items()},
                              force=force)
            self.fwd_algo[li] = algos[best]
            cands = {}
            for parts in ((4, 8, 16, 32, 64, 128) if spec.n_neurons > 32 else (16, 32, 64, 128, 256)):
                g = max(2, -(-B // parts))
                if K.call_size("bats_weights_gradient_workspace_bytes", B, spec.n_neurons, n_prev, g) <= wsb:
                    cands[str(g)] = g
            if len(cands) > 1:
                def run_grad(g, li=li):
                    self._grad_only(li, g, s)

                bg = tuner.pick("fc_grad_group", shape, {k: (lambda g=g: run_grad(g)) for k, g in cands.items()},
                                force=force)
                self.groups[li] = cands[bg]
            choice[tag] = {"forward": best, "grad_group": self.groups[li]}
            fwd_ms = tuner.timings.get(tuner.key("fc_forward", *shape))
            if fwd_ms:  # timed now (not taken from the cache): every candidate's time, for the record
                choice[tag]["forward_ms"] = {k: round(v, 4) for k, v in fwd_ms.items()}
            n_prev, k_prev = spec.n_neurons, spec.max_n_spike
        torch.cuda.synchronize()
        self.tuned = choice
        return choice

    def try_capture(self) -> bool:
        """Record one step as a CUDA graph (after an eager warm-up step); False if capture fails."""
        try:
            self.step()
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                with torch.cuda.graph(g, stream=side):
                    self._enqueue(side, self.aux)
            torch.cuda.current_stream().wait_stream(side)
            torch.cuda.synchronize()
            self.graph = g
            return True
        except Exception as exc:  # pragma: no cover - reported by the caller
            self.graph = None
            self.capture_error = repr(exc)
            return False

    def replay(self) -> None:
        self.graph.replay()
        self.t += 1

    def run(self) -> None:
        if self.graph is not None:
            self.replay()
        else:
            self.step()

    def profile_step(self):
        """One eager step with CUDA events around every launch: {name: (start, end)}."""
        s = stream_ptr()
        rec = {}
        for name, fn in self.launches:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn(s)
            b.record()
            rec[name] = (a, b)
        self.t += 1
        return rec

    def time_launch(self, name, steps, flush=None) -> float:
        """Average device time (ms) of one named launch over `steps` eager steps."""
        s = stream_ptr()
        total = 0.0
        evs = []
        for _ in range(steps):
            if flush is not None:
                flush.add_(1.0)
            for nm, fn in self.launches:
                if nm == name:
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record()
                    fn(s)
                    b.record()
                    evs.append((a, b))
                else:
                    fn(s)
            self.t += 1
        torch.cuda.synchronize()
        for a, b in evs:
            total += a.elapsed_time(b)
        return total / max(1, len(evs))

    def set_inputs(self, times, labels) -> None:
        self.in_times.copy_(torch.as_tensor(times), non_blocking=True)
        self.labels.copy_(torch.as_tensor(labels).to(torch.int32), non_blocking=True)

    def step_host(self, times: np.ndarray, labels: np.ndarray) -> np.ndarray:
        """End-to-end step from host arrays: pinned host -> device copy, step, loss back to the host."""
        self.h_times.numpy()[...] = times
        self.h_labels.numpy()[...] = labels
        self.in_times.copy_(self.h_times, non_blocking=True)
        self.labels.copy_(self.h_labels, non_blocking=True)
        self.run()
        self.h_loss.copy_(self.loss, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return self.h_loss.numpy()

    def train_host(self, batches) -> List[np.ndarray]:
        """Train on an iterable of host batches (times (B, N_in, K_in), labels (B,)), one step per batch;
        returns each step's per-sample losses. Every step copies its inputs host -> device and its losses
        back, as step_host does, but the copies are pipelined: batch i+1 is staged into pinned memory and
        copied on a side stream while step i computes (two pinned and two device slots), and step i's
        losses are read back when its slot is reused. Results are those of step_host called per batch."""
        dev = self.in_times.device
        if not hasattr(self, "_pipe"):
            h_in = [torch.empty(self.in_times.shape, dtype=torch.float32, pin_memory=True) for _ in range(2)]
            h_lab = [torch.empty((self.B,), dtype=torch.int32, pin_memory=True) for _ in range(2)]
            h_loss = [torch.empty((self.B,), dtype=torch.float32, pin_memory=True) for _ in range(2)]
            self._pipe = {
                "h_in": h_in, "h_lab": h_lab, "h_loss": h_loss,
                # numpy views of the pinned slots and the slots' events, made once: each event is re-recorded
                # once per use of its slot, and every wait or synchronize refers to its latest record
                "np_in": [t.numpy() for t in h_in], "np_lab": [t.numpy() for t in h_lab],
                "np_loss": [t.numpy() for t in h_loss],
                "d_in": [torch.empty_like(self.in_times) for _ in range(2)],
                "d_lab": [torch.empty_like(self.labels) for _ in range(2)],
                "staged": [torch.cuda.Event() for _ in range(2)],
                "consumed": [torch.cuda.Event() for _ in range(2)],
                "done": [torch.cuda.Event() for _ in range(2)],
                "copy": torch.cuda.Stream(device=dev),
            }
        P = self._pipe
        comp = torch.cuda.current_stream(dev)
        cs = P["copy"]
        staged, consumed, done = P["staged"], P["consumed"], P["done"]
        used = [False, False]  # the slot has been used (its events recorded) in this call
        losses: List[np.ndarray] = []
        order: List[int] = []
        for i, (times, labels) in enumerate(batches):
            k = i & 1
            if used[k]:
                done[k].synchronize()       # step i-2 finished: its losses are in the pinned slot
                losses.append(P["np_loss"][k].copy())
                staged[k].synchronize()     # its host -> device copies finished: the pinned slot may be refilled
                cs.wait_event(consumed[k])  # and the device slot was copied into the step's inputs
            np.copyto(P["np_in"][k], times)
            np.copyto(P["np_lab"][k], labels, casting="unsafe")
            with torch.cuda.stream(cs):
                P["d_in"][k].copy_(P["h_in"][k], non_blocking=True)
                P["d_lab"][k].copy_(P["h_lab"][k], non_blocking=True)
                staged[k].record(cs)
            comp.wait_event(staged[k])
            self.in_times.copy_(P["d_in"][k], non_blocking=True)
            self.labels.copy_(P["d_lab"][k], non_blocking=True)
            consumed[k].record(comp)
            self.run()
            P["h_loss"][k].copy_(self.loss, non_blocking=True)
            done[k].record(comp)
            used[k] = True
            order.append(k)
        n = len(order)
        for k in order[max(0, n - 2):]:  # the last one or two steps, in step order
            done[k].synchronize()
            losses.append(P["np_loss"][k].copy())
        return losses

    @property
    def h2d_bytes(self) -> int:
        return self.h_times.numel() * 4 + self.h_labels.numel() * 4

    @property
    def d2h_bytes(self) -> int:
        return self.h_loss.numel() * 4


def enqueue_launches(launches, side, main, aux=None) -> None:
    """Enqueue a step's launch list on the torch stream `main`. With `aux`, the launches named in `side`
    ({launch: the launch it waits for}) run on `aux`, each after its dependency has been enqueued on `main`,
    and `main` waits for `aux` before the first `.wt_copy` launch (which copies the staged transposed weights
    that those launches wrote) or at the end. The launches on `aux` read only what their dependency and the
    launches before it wrote, and write nothing that `main` reads before the join, so the results are those
    of the list run in order on one stream."""
    sm = main.cuda_stream
    if aux is None:
        for _, fn in launches:
            fn(sm)
        return
    forks = set(side.values())
    events = {}
    joined = False
    for name, fn in launches:
        if name in side:
            aux.wait_event(events[side[name]])
            fn(aux.cuda_stream)
            continue
        if name.endswith(".wt_copy") and not joined:
            main.wait_stream(aux)
            joined = True
        fn(sm)
        if name in forks:
            e = torch.cuda.Event()
            e.record(main)
            events[name] = e
    if not joined:
        main.wait_stream(aux)
