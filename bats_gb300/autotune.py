"""Autotuner for the kernel variants: picks, per shape and GPU, the variant that runs fastest on the
caller's own buffers, and caches the choice.

Tuned today: the FC forward kernel (tile: CTA per post-neuron tile and sample, producer warp streaming
weight rows; lanes: warp per post neuron and sample, 32 events evaluated at once; queue: persistent CTAs
over a longest-first work queue; the tile and queue kinds with or without the per-stage no-crossing
screen) and the number of
samples per partial gradient of the batch-reduced weight gradient. Every candidate computes identical
results (the forward variants bit for bit, the gradient up to the order of the partial sums), so the
choice only changes speed.

The cache is a JSON file (BATS_GB300_AUTOTUNE, default ~/.cache/bats_gb300/autotune.json) keyed by the
kind of kernel, the shape and the GPU (name and SM count); set BATS_GB300_AUTOTUNE=off to keep it in
memory only.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Callable, Dict, Optional

import torch

_LOCK = threading.Lock()


def _default_path() -> Optional[str]:
    p = os.environ.get("BATS_GB300_AUTOTUNE")
    if p == "off":
        return None
    return p or os.path.join(os.path.expanduser("~"), ".cache", "bats_gb300", "autotune.json")


class Autotuner:
    def __init__(self, path: Optional[str] = "default", reps: int = 3):
        self.path = _default_path() if path == "default" else path
        self.reps = int(reps)
        self.cache: Dict[str, str] = {}
        self.timings: Dict[str, Dict[str, float]] = {}
        if self.path and os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.cache = dict(json.load(f))
            except (OSError, ValueError):
                self.cache = {}

    @staticmethod
    def device_tag(device=None) -> str:
        p = torch.cuda.get_device_properties(device if device is not None else torch.cuda.current_device())
        return f"{p.name}|sm{p.multi_processor_count}"

    def key(self, kind: str, *shape) -> str:
        return "|".join([kind, self.device_tag()] + [str(int(v)) for v in shape])

    def _save(self) -> None:
        if not self.path:
            return
        with _LOCK:
            try:
                os.makedirs(os.path.dirname(self.path), exist_ok=True)
                tmp = f"{self.path}.{os.getpid()}.tmp"
                with open(tmp, "w") as f:
                    json.dump(self.cache, f, indent=0, sort_keys=True)
                os.replace(tmp, self.path)
            except OSError:
                pass

    def pick(self, kind: str, shape, candidates: Dict[str, Callable[[], None]], force: bool = False) -> str:
        """Name of the fastest candidate for (kind, shape); each candidate is a no-argument callable that
        launches its variant on the current stream. Cached results are reused unless force."""
        k = self.key(kind, *shape)
        if not force and self.cache.get(k) in candidates:
            return self.cache[k]
        stream = torch.cuda.current_stream()
        times = {}
        for name, fn in candidates.items():
            fn()  # warm-up (module load, caches)
            # A short spin kernel ahead of the timed launches keeps the GPU busy while the host enqueues
            # them, so that the events time the kernels and not the host's launch calls (short kernels).
            torch.cuda._sleep(1_000_000)
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            start.record(stream)
            for _ in range(self.reps):
                fn()
            end.record(stream)
            end.synchronize()
            times[name] = start.elapsed_time(end) / self.reps
        best = _choose(times, list(candidates))
        self.cache[k] = best
        self.timings[k] = times
        self._save()
        return best


def _choose(times: Dict[str, float], order) -> str:
    """The candidate to keep from measured times (ms): candidates within 3 % (or 2 us) of the fastest count as
    tied, and the first of them in the caller's order (simplest variant first) wins, so that timing noise on
    near-empty work does not pick a heavier variant."""
    fastest = min(times.values())
    return next(n for n in order if times[n] <= max(fastest * 1.03, fastest + 0.002))


_GLOBAL: Optional[Autotuner] = None


def get_tuner() -> Autotuner:
    global _GLOBAL
    if _GLOBAL is None:
        _GLOBAL = Autotuner()
    return _GLOBAL
