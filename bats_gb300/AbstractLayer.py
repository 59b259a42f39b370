"""Layer contract (bats/AbstractLayer.py:11-70): spike trains in, spike trains out, per-sample
weight gradients and pre-spike errors back; weights stored as <name>_weights.npy."""
from __future__ import annotations

from abc import ABC, abstractmethod
from pathlib import Path
from typing import Optional, Tuple

import numpy as np
import torch

WEIGHTS_FILE_SUFFIX = "_weights.npy"


class AbstractLayer(ABC):
    def __init__(self, n_neurons: int, name: str = ""):
        self._n_neurons: int = int(n_neurons)
        self._name: str = name

    @property
    def n_neurons(self) -> int:
        return self._n_neurons

    @property
    def name(self) -> str:
        return self._name

    @property
    @abstractmethod
    def trainable(self) -> bool:
        ...

    @property
    @abstractmethod
    def spike_trains(self) -> Tuple[torch.Tensor, torch.Tensor]:
        ...

    @property
    @abstractmethod
    def weights(self) -> Optional[torch.Tensor]:
        ...

    @weights.setter
    @abstractmethod
    def weights(self, weights) -> None:
        ...

    @abstractmethod
    def reset(self) -> None:
        ...

    @abstractmethod
    def forward(self, max_simulation: float, training: bool = False) -> None:
        ...

    @abstractmethod
    def backward(self, errors: torch.Tensor) -> Optional[Tuple[torch.Tensor, torch.Tensor]]:
        ...

    @abstractmethod
    def add_deltas(self, delta_weights: torch.Tensor) -> None:
        ...

    def store(self, dir_path: Path) -> None:
        weights = self.weights
        if weights is not None:
            filename = Path(dir_path) / (self._name + WEIGHTS_FILE_SUFFIX)
            np.save(filename, weights.detach().cpu().numpy())

    def restore(self, dir_path: Path) -> None:
        filename = Path(dir_path) / (self._name + WEIGHTS_FILE_SUFFIX)
        if filename.exists():
            self.weights = np.load(filename)
