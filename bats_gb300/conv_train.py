"""Batched training step of a convolutional BATS network with every buffer preallocated.

ConvTrainStep is to the conv network what FCTrainStep is to the fully-connected one: the layers of
bats/Layers/ConvLIFLayer.py, PoolingLayer.py and LIFLayer.py in any order a Network would stack them
(conv and pooling layers on a (X, Y, C) input, then fully-connected layers), with the spike-count
classification loss and Adam, as one fixed list of launches with no host synchronisation and no
allocation after construction, so that the whole step is captured once as a CUDA graph and replayed.
The arithmetic is that of the layer-by-layer API (Network.forward/backward, the caller's batch mean,
AdamOptimizer.step, apply_deltas) except where the batch mean is formed: each conv layer's filter
gradient is accumulated over groups of samples by the backward kernel itself and reduced in group order
(bats_conv_backward_adam, fused with the layer's Adam update), and each fully-connected layer's as in
FCTrainStep (bats_weights_gradient_adam), so no per-sample gradient is written. The reference's
counterpart is the training iteration of experiments/mnist/train_conv.py (Network.forward, the loss,
Network.backward, the batch mean of every gradient, AdamOptimizer.step, apply_deltas).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np
import torch

from . import kernels as K
from ._lib import call, ptr, stream_ptr
from .train import FCLayerSpec, enqueue_launches


@dataclass
class ConvLayerSpec:
    """LIFLayerConv(filters_shape=[fx, fy, C_out], tau_s, theta, delta_theta, max_n_spike)."""
    filters_shape: Tuple[int, int, int]
    tau_s: float
    theta: float
    delta_theta: float
    max_n_spike: int


@dataclass
class PoolLayerSpec:
    """PoolingLayer: 2x2 union of the children's spike trains (K -> 4K)."""


Spec = Union[ConvLayerSpec, PoolLayerSpec, FCLayerSpec]


class ConvTrainStep:
    def __init__(self, batch: int, input_shape: Sequence[int], k_input: int, layers: Sequence[Spec],
                 weights: Sequence[Optional[torch.Tensor]], target_true: float, target_false: float,
                 learning_rate: float = 3e-3, beta_1: float = 0.9, beta_2: float = 0.999, epsilon: float = 1e-8,
                 max_simulation: float = np.inf, conv_group: int = 2, device="cuda"):
        """weights: one tensor per layer, None for pooling layers; conv filters (C_out, fx, fy, C_in), FC weights
        (N_post, N_pre) (as the reference's layers hold them). conv_group: samples per partial filter gradient."""
        self.B = int(batch)
        self.dev = torch.device(device)
        self.specs = list(layers)
        self.max_sim = float(max_simulation)
        self.tt, self.tf = np.float32(target_true), np.float32(target_false)
        self.lr, self.b1, self.b2, self.eps = (np.float32(v) for v in (learning_rate, beta_1, beta_2, epsilon))
        self.t = 0
        B, dev = self.B, self.dev
        f32, i32 = torch.float32, torch.int32
        X, Y, C = (int(v) for v in input_shape)
        self.in_times = torch.full((B, X * Y * C, k_input), float("inf"), dtype=f32, device=dev)
        self.labels = torch.zeros((B,), dtype=i32, device=dev)
        self.L: List[dict] = []
        shape, k_prev, spatial = (X, Y, C), int(k_input), True
        ws = 256
        for li, (spec, w) in enumerate(zip(self.specs, weights)):
            n_prev = int(np.prod(shape)) if spatial else shape
            d = {"spec": spec, "in_shape": shape, "n_pre": n_prev, "k_pre": k_prev}
            if isinstance(spec, PoolLayerSpec):
                assert spatial, "pooling needs a spatial input"
                Xp, Yp, Cp = shape
                out_shape = (Xp // 2, Yp // 2, Cp)
                N = out_shape[0] * out_shape[1] * out_shape[2]
                d.update(kind="pool", out_shape=out_shape, n=N, k=4 * k_prev,
                         out=(torch.empty((B, N), dtype=i32, device=dev),
                              torch.empty((B, N, 4 * k_prev), dtype=f32, device=dev),
                              torch.empty((B, N, 4 * k_prev), dtype=i32, device=dev)))
                shape, k_prev = out_shape, 4 * k_prev
            else:
                w = w.to(device=dev, dtype=f32).contiguous().clone()
                Kp = int(spec.max_n_spike)
                d["tau32"], d["c"], d["dtt"] = K.lif_constants(spec.tau_s, spec.theta, spec.delta_theta)
                if isinstance(spec, ConvLayerSpec):
                    assert spatial, "a conv layer needs a spatial input"
                    fx, fy, C_out = (int(v) for v in spec.filters_shape)
                    Xp, Yp, Cp = shape
                    assert w.shape == (C_out, fx, fy, Cp)
                    out_shape = (Xp - fx + 1, Yp - fy + 1, C_out)
                    N = out_shape[0] * out_shape[1] * C_out
                    by_pos = Xp * Yp <= 255
                    d.update(kind="conv", out_shape=out_shape, n=N, k=Kp, group=max(1, int(conv_group)),
                             ev=K.alloc_events(B, n_prev, k_prev, dev, bucketed=by_pos, bucket_width=Cp))
                    ws = max(ws, K.call_size("bats_conv_backward_adam_workspace_bytes", B, Cp, fx, fy, C_out,
                                             d["group"]))
                    shape = out_shape
                else:
                    N = int(spec.n_neurons)
                    assert w.shape == (N, n_prev)
                    d.update(kind="fc", n=N, k=Kp, ev=K.alloc_events(B, n_prev, k_prev, dev),
                             Wt=K.transpose_weights(w), algo=K.FWD_AUTO,
                             group=max(2, K.default_group(B, N, n_prev)))
                    ws = max(ws, K.call_size("bats_weights_gradient_workspace_bytes", B, N, n_prev, d["group"]),
                             K.call_size("bats_pre_errors_workspace_bytes", B, n_prev * k_prev, N),
                             K.queue_workspace_bytes(B))
                    shape, spatial = N, False
                ws = max(ws, K.call_size("bats_sort_events_workspace_bytes", B, n_prev, k_prev))
                d.update(W=w, m=torch.zeros_like(w), v=torch.zeros_like(w), grad=torch.empty_like(w),
                         out=(torch.empty((B, N), dtype=i32, device=dev),
                              *(torch.empty((B, N, Kp), dtype=f32, device=dev) for _ in range(4))),
                         tables=torch.empty((B, N, Kp + 1, 2), dtype=f32, device=dev),
                         nvalid=torch.empty((B, N), dtype=i32, device=dev),
                         heads=K.alloc_cursor_heads(B, N, dev) if d["kind"] == "fc" else None)
                assert Kp <= 32, "the train step's counted backward prep handles at most 32 spikes per neuron"
                k_prev = Kp
            # Errors of this layer's input spikes (the incoming errors of the layer below); none for the first.
            d["pre_err"] = torch.empty((B, n_prev, d["k_pre"]), dtype=f32, device=dev) if li > 0 else None
            self.L.append(d)
        last = self.L[-1]
        assert last["kind"] == "fc", "the loss reads a fully-connected output layer"
        self.loss = torch.empty((B,), dtype=f32, device=dev)
        self.errors = torch.empty((B, last["n"], last["k"]), dtype=f32, device=dev)
        self.ws = torch.empty(ws, dtype=torch.uint8, device=dev)
        # The gradient + Adam of the fully-connected layers that propagate errors below them runs on a second
        # stream beside the rest of the backward (as in FCTrainStep): it writes the layer's new transposed
        # weights into a staging copy, copied over Wt at the end of the step, and uses its own workspace.
        for li, d in enumerate(self.L):
            if d["kind"] == "fc" and li > 0:
                d["Wt_next"] = d["Wt"].clone()
        self.ws2 = torch.empty_like(self.ws)
        self.aux = torch.cuda.Stream(device=dev) if torch.cuda.is_available() else None
        self.powers = torch.tensor([1.0, 1.0, 0.0, 0.0], dtype=torch.float64, device=dev)
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.capture_error = None
        self.launches = self._build_launches()

    def _pad_flag(self, li: int) -> int:
        """A fully-connected layer followed by another one leaves the slots past its spike counts as they are
        (the next sort, the counted prep, the gradient and the pre errors stay below the counts); the output
        layer and anything read by pooling are padded with +inf."""
        nxt = self.L[li + 1]["kind"] if li + 1 < len(self.L) else None
        return K.FWD_NO_PAD if self.L[li]["kind"] == "fc" and nxt == "fc" else 0

    def _build_launches(self):
        """(name, fn(stream)) for every entry-point call of one step, in order; all pointers fixed."""
        B = self.B
        ws, wsb = ptr(self.ws), self.ws.numel()
        L = [("adam.powers", lambda s: call("bats_adam_powers_advance", ptr(self.powers), float(self.b1),
                                              float(self.b2), s))]
        pre_t, pre_n, pre_padded = self.in_times, None, True
        for li, d in enumerate(self.L):
            tag = f"L{li + 1}"
            if d["kind"] == "pool":
                X, Y, C = d["in_shape"]
                n_o, t_o, i_o = d["out"]
                L.append((f"{tag}.pool", lambda s, pn=ptr(pre_n), pt=ptr(pre_t), X=X, Y=Y, C=C, k=d["k_pre"], o=d["out"]:
                          call("bats_pool_forward", pn, pt, B, X, Y, C, k, ptr(o[0]), ptr(o[1]), ptr(o[2]), s)))
                pre_n, pre_t, pre_padded = n_o, t_o, True
                continue
            ev, spec = d["ev"], d["spec"]
            tau_s = float(np.float32(spec.tau_s))
            bw = ev.bucket_width
            if pre_padded:  # the network input, or a padded output (conv, pooling): every slot is read
                L.append((f"{tag}.sort", lambda s, pt=ptr(pre_t), ev=ev, tau_s=tau_s, d=d, bw=bw: call(
                    "bats_sort_events", pt, B, ev.n_neurons, ev.k, tau_s, float(d["tau32"]), None, None,
                    ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ptr(ev.bucketed), ptr(ev.bucket_offsets), bw, ws,
                    wsb, s)))
            else:  # an unpadded fully-connected output: only the slots below its spike counts
                L.append((f"{tag}.sort", lambda s, pt=ptr(pre_t), pc=ptr(pre_n), ev=ev, tau_s=tau_s, d=d, bw=bw: call(
                    "bats_sort_events_counted", pt, pc, B, ev.n_neurons, ev.k, tau_s, float(d["tau32"]), None, None,
                    ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ptr(ev.bucketed), ptr(ev.bucket_offsets), bw, ws,
                    wsb, s)))
            n, a, x, t, z = d["out"]
            if d["kind"] == "conv":
                X, Y, C = d["in_shape"]
                fx, fy, C_out = (int(v) for v in spec.filters_shape)
                L.append((f"{tag}.forward", lambda s, ev=ev, d=d, X=X, Y=Y, C=C, fx=fx, fy=fy, C_out=C_out: call(
                    "bats_conv_forward", ptr(ev.events), ptr(ev.counts), ev.cap, ptr(d["W"]), B, X, Y, C, fx, fy,
                    C_out, d["k"], float(d["c"]), float(d["dtt"]), float(d["tau32"]), float(np.float32(self.max_sim)),
                    *(ptr(o) for o in d["out"]), s)))
                pre_padded = True
            else:
                L.append((f"{tag}.forward", lambda s, ev=ev, d=d, li=li: K.forward_fc_call(
                    ev, d["Wt"], d["n"], d["k"], d["c"], d["dtt"], d["tau32"], self.max_sim, d["out"],
                    d["algo"] | self._pad_flag(li), s, ws, wsb)))
                pre_padded = self._pad_flag(li) == 0
            pre_t, pre_n = t, n
        out = self.L[-1]
        L.append(("loss", lambda s: call("bats_spike_count_loss", ptr(out["out"][0]), 0, None, ptr(self.labels),
                                         float(self.tt), float(self.tf), B, out["n"], out["k"], ptr(self.loss),
                                         ptr(self.errors), s)))
        errors = self.errors
        for li in range(len(self.L) - 1, -1, -1):
            d = self.L[li]
            tag = f"L{li + 1}"
            pe = d["pre_err"]
            if d["kind"] == "pool":
                n_o, t_o, i_o = d["out"]
                L.append((f"{tag}.pool_back", lambda s, e=errors, i_o=i_o, pe=pe: call(
                    "bats_pool_backward", ptr(e), ptr(i_o), e.numel(), ptr(pe), pe.numel(), s)))
                errors = pe
                continue
            spec = d["spec"]
            tau_s = float(np.float32(spec.tau_s))
            L.append((f"{tag}.prep", lambda s, d=d, e=errors: call(
                "bats_backward_prep_counted", ptr(d["out"][3]), ptr(d["out"][0]), ptr(d["out"][1]), ptr(d["out"][2]),
                ptr(d["out"][4]), ptr(e), B, d["n"], d["k"], float(d["c"]), float(d["tau32"]), float(d["dtt"]),
                ptr(d["tables"]), ptr(d["nvalid"]), ptr(d["heads"]), s)))
            ev = d["ev"]
            if d["kind"] == "conv":
                X, Y, C = d["in_shape"]
                fx, fy, C_out = (int(v) for v in spec.filters_shape)
                L.append((f"{tag}.grad_adam", lambda s, d=d, ev=ev, X=X, Y=Y, C=C, fx=fx, fy=fy, C_out=C_out,
                          tau_s=tau_s, pe=pe: call(
                    "bats_conv_backward_adam", ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ptr(ev.bucketed),
                    ptr(ev.bucket_offsets), ev.cap, ptr(d["W"]), B, X, Y, C, fx, fy, C_out, ev.k, ptr(d["out"][3]),
                    ptr(d["tables"]), ptr(d["nvalid"]), d["k"], tau_s, float(d["tau32"]), ptr(pe), d["group"],
                    ptr(d["grad"]), ptr(d["m"]), ptr(d["v"]), float(self.b1), float(self.b2), float(self.eps),
                    float(self.lr), ptr(self.powers), ws, wsb, s)))
            else:
                if pe is not None:
                    L.append((f"{tag}.pre_err", lambda s, d=d, ev=ev, tau_s=tau_s, pe=pe: call(
                        "bats_pre_errors", ptr(ev.events), ptr(ev.slots), ptr(ev.counts), ev.cap, ptr(d["Wt"]),
                        d["Wt"].shape[1], ptr(d["out"][3]), ptr(d["tables"]), ptr(d["nvalid"]), B, d["n"], d["k"],
                        ev.n_neurons, ev.k, tau_s, float(d["tau32"]), ptr(pe), ws, wsb, s)))
                staged = "Wt_next" in d
                wt_out = d["Wt_next"] if staged else d["Wt"]
                gws, gwsb = (ptr(self.ws2), self.ws2.numel()) if staged else (ws, wsb)
                L.append((f"{tag}.grad_adam", lambda s, d=d, ev=ev, wt_out=wt_out, gws=gws, gwsb=gwsb: call(
                    "bats_weights_gradient_adam", ptr(ev.events), ptr(ev.counts), ptr(ev.bucketed),
                    ptr(ev.bucket_offsets), ev.cap, ptr(d["out"][3]), ptr(d["tables"]), ptr(d["nvalid"]),
                    ptr(d["heads"]), B, d["n"], d["k"], ev.n_neurons, d["group"], ptr(d["grad"]), ptr(d["m"]),
                    ptr(d["v"]), float(self.b1),
                    float(self.b2), float(self.eps), float(self.lr), ptr(self.powers), ptr(d["W"]), ptr(wt_out),
                    d["Wt"].shape[1], gws, gwsb, s)))
            if pe is not None:
                errors = pe
        for li in range(len(self.L) - 1, -1, -1):
            d = self.L[li]
            if "Wt_next" in d:
                L.append((f"L{li + 1}.wt_copy", lambda s, d=d: K.copy_on_stream(d["Wt"], d["Wt_next"], s)))
        return L

    def _side_launches(self):
        """{gradient launch: its layer's prep} for the layers whose transposed weights are staged."""
        return {f"L{li + 1}.grad_adam": f"L{li + 1}.prep" for li, d in enumerate(self.L) if "Wt_next" in d}

    # -- running ----------------------------------------------------------------------------------------
    def step(self) -> None:
        enqueue_launches(self.launches, self._side_launches(), torch.cuda.current_stream(), self.aux)
        self.t += 1

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
                    enqueue_launches(self.launches, self._side_launches(), side, self.aux)
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

    def set_inputs(self, times, labels) -> None:
        self.in_times.copy_(torch.as_tensor(times), non_blocking=True)
        self.labels.copy_(torch.as_tensor(labels).to(torch.int32), non_blocking=True)

    @property
    def weights(self) -> List[Optional[torch.Tensor]]:
        return [d.get("W") for d in self.L]

    def spike_counts(self) -> List[int]:
        return [int(d["out"][0].sum().item()) for d in self.L]
