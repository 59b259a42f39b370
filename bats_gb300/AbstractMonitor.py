"""Base of the training monitors (bats/AbstractMonitor.py:9-48): a named series of (epoch, value) records,
printed as "<name>: <value>" and exported as an .npz file (epochs, values). Monitors here accumulate on
the device (torch tensors, no host synchronisation in add()); record() reads the accumulated value once."""
from __future__ import annotations

from abc import ABC, abstractmethod
from pathlib import Path
from typing import Optional

import numpy as np


class AbstractMonitor(ABC):
    def __init__(self, name: str, export_path: Optional[Path] = None, decimal: int = 2):
        self._name = name
        self._export_path = export_path
        self._decimal = decimal
        self._epochs = []
        self._values = []

    def __str__(self) -> str:
        return self._name + ": " + self._format()

    def _format(self) -> str:
        return str(np.around(self._values[-1], self._decimal))

    def reset(self) -> None:
        self._epochs = []
        self._values = []

    def _record(self, epoch: float, value: float) -> None:
        self._epochs.append(epoch)
        self._values.append(value)

    @abstractmethod
    def record(self, epoch: float) -> float:
        pass

    def export(self) -> None:
        """Writes <export_path>.npz with the epochs and values (the reference also plots them; no plotting
        library is assumed here)."""
        if self._export_path is None:
            return
        np.savez(self._export_path, epochs=np.asarray(self._epochs), values=np.asarray(self._values))
