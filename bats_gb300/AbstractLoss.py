"""Loss contract (bats/AbstractLoss.py:6-24)."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Tuple

import torch


class AbstractLoss(ABC):
    @abstractmethod
    def predict(self, spikes_per_neuron, n_spike_per_neuron) -> torch.Tensor:
        ...

    @abstractmethod
    def compute_loss(self, spikes_per_neuron, n_spike_per_neuron, labels) -> torch.Tensor:
        ...

    @abstractmethod
    def compute_errors(self, spikes_per_neuron, n_spike_per_neuron, labels) -> torch.Tensor:
        ...

    @abstractmethod
    def compute_loss_and_errors(self, spikes_per_neuron, n_spike_per_neuron,
                                labels) -> Tuple[torch.Tensor, torch.Tensor]:
        ...
