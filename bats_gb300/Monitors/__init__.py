"""Training monitors with the reference's interface (bats/Monitors/*.py), accumulating on the device."""
from __future__ import annotations

import time
from typing import Dict, List, Optional

import numpy as np
import torch

from ..AbstractMonitor import AbstractMonitor


def _dev(x, dtype=None):
    t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))
    if torch.cuda.is_available() and not t.is_cuda:
        t = t.cuda()
    return t if dtype is None else t.to(dtype)


class _Counter:
    """A device-side running sum (float64) that is read only on record()."""

    def __init__(self):
        self.value = None

    def add(self, t: torch.Tensor) -> None:
        v = t.to(torch.float64)
        self.value = v if self.value is None else self.value + v

    def take(self) -> float:
        out = 0.0 if self.value is None else float(self.value.item())
        self.value = None
        return out


class AccuracyMonitor(AbstractMonitor):
    """bats/Monitors/AccuracyMonitor.py: percentage of predictions equal to the targets."""

    def __init__(self, **kwargs):
        super().__init__("Accuracy (%)", **kwargs)
        self._hits, self._n = _Counter(), 0

    def add(self, predictions, targets) -> None:
        p, t = _dev(predictions), _dev(targets)
        self._hits.add((p.to(t.dtype) == t).sum())
        self._n += int(t.shape[0])

    def record(self, epoch) -> float:
        acc = self._hits.take() / self._n * 100
        self._n = 0
        super()._record(epoch, acc)
        return acc


class LossMonitor(AbstractMonitor):
    """bats/Monitors/LossMonitor.py: mean of the finite per-sample losses."""

    def __init__(self, **kwargs):
        super().__init__("Loss", **kwargs)
        self._sum, self._cnt = _Counter(), _Counter()

    def add(self, losses) -> None:
        l = _dev(losses)
        ok = torch.isfinite(l)
        self._sum.add(torch.where(ok, l, torch.zeros_like(l)).sum())
        self._cnt.add(ok.sum())

    def record(self, epoch) -> float:
        loss = self._sum.take() / self._cnt.take()
        super()._record(epoch, loss)
        return loss


class SilentLabelsMonitor(AbstractMonitor):
    """bats/Monitors/SilentLabelsMonitor.py: percentage of samples whose label neuron did not spike."""

    def __init__(self, **kwargs):
        super().__init__("Silent labels (%)", **kwargs)
        self._silent, self._n = _Counter(), 0

    def add(self, n_out_spikes, targets) -> None:
        n, t = _dev(n_out_spikes), _dev(targets, torch.int64)
        self._silent.add((torch.gather(n, 1, t[:, None]) == 0).sum())
        self._n += int(t.shape[0])

    def record(self, epoch) -> float:
        ratio = self._silent.take() / self._n * 100
        self._n = 0
        super()._record(epoch, ratio)
        return ratio


class SilentNeuronsMonitor(AbstractMonitor):
    """bats/Monitors/SilentNeuronsMonitor.py: percentage of neurons that never spiked over the recorded
    samples."""

    def __init__(self, layer_name: str, **kwargs):
        super().__init__(layer_name + " silents (%)", **kwargs)
        self._total = None

    def add(self, n_spikes) -> None:
        s = _dev(n_spikes).to(torch.int64).sum(0)
        self._total = s if self._total is None else self._total + s

    def record(self, epoch) -> float:
        ratio = float((self._total == 0).double().mean().item()) * 100
        self._total = None
        super()._record(epoch, ratio)
        return ratio


class SpikeCountMonitor(AbstractMonitor):
    """bats/Monitors/SpikeCountMonitor.py: mean spike count of a layer per sample."""

    def __init__(self, layer_name: str, **kwargs):
        super().__init__(layer_name + " spike counts", **kwargs)
        self._counts, self._n = _Counter(), 0

    def add(self, n_spike_per_neuron) -> None:
        n = _dev(n_spike_per_neuron)
        self._counts.add(n.sum())
        self._n += int(n.shape[0])

    def record(self, epoch) -> float:
        avg = self._counts.take() / self._n
        self._n = 0
        super()._record(epoch, avg)
        return avg


class WeightsNormMonitor(AbstractMonitor):
    """bats/Monitors/WeightsNormMonitor.py: Frobenius norm of a weight tensor."""

    def __init__(self, layer_name: str, **kwargs):
        super().__init__(layer_name + " weights norm", **kwargs)
        self._norm = None

    def add(self, weights) -> None:
        self._norm = torch.linalg.norm(_dev(weights).to(torch.float32))

    def record(self, epoch) -> float:
        v = float(self._norm.item())
        super()._record(epoch, v)
        return v


class TimeMonitor(AbstractMonitor):
    """bats/Monitors/TimeMonitor.py: wall time since start()."""

    def __init__(self, **kwargs):
        super().__init__("Time (s)", **kwargs)
        self._start = 0.0

    def start(self) -> None:
        self._start = time.time()

    def record(self, epoch) -> float:
        v = time.time() - self._start
        super()._record(epoch, v)
        return v


class ValueMonitor(AbstractMonitor):
    """bats/Monitors/ValueMonitor.py: the last value given."""

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self._value = 0.0

    def add(self, value) -> None:
        self._value = value

    def record(self, epoch) -> float:
        v = float(self._value.item()) if isinstance(self._value, torch.Tensor) else float(self._value)
        self._record(epoch, v)
        return v


class MonitorsManager:
    """bats/Monitors/MonitorsManager.py: prints, records and exports a list of monitors."""

    def __init__(self, monitors: Optional[List[AbstractMonitor]] = None, print_prefix: str = ""):
        self._monitors = list(monitors) if monitors else []
        self._print_prefix = print_prefix

    def add(self, monitor: AbstractMonitor) -> None:
        self._monitors.append(monitor)

    def print(self, epoch: float, decimal: int = 1) -> None:
        line = self._print_prefix + f"Epoch {np.around(epoch, decimal)}"
        for q, m in enumerate(self._monitors):
            line += (" | " if q == 0 else ", ") + str(m)
        print(line)

    def record(self, epoch: float) -> Dict:
        return {m: m.record(epoch) for m in self._monitors}

    def export(self) -> None:
        for m in self._monitors:
            m.export()


__all__ = ["AccuracyMonitor", "LossMonitor", "SilentLabelsMonitor", "SilentNeuronsMonitor", "SpikeCountMonitor",
           "WeightsNormMonitor", "TimeMonitor", "ValueMonitor", "MonitorsManager"]
