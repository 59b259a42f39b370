"""Squared error of first spike times (bats/Losses/SpikeTimeLoss.py:7-47). Silent neurons count as 1.0;
the targets tensor is modified in place (inf -> 1.0) as in the reference, and compute_loss_and_errors
subtracts the targets from the spikes as given (inf stays inf), like the reference."""
from __future__ import annotations

from typing import Tuple

import torch

from .. import kernels as K
from ..AbstractLoss import AbstractLoss
from ..tensors import to_device


def _targets(targets) -> torch.Tensor:
    t = to_device(targets, torch.float32)
    return t


class SpikeTimeLoss(AbstractLoss):
    def predict(self, spikes_per_neuron, n_spike_per_neuron) -> torch.Tensor:
        return torch.argmin(spikes_per_neuron[..., 0], dim=1)

    def compute_loss(self, spikes_per_neuron, n_spike_per_neuron, targets) -> torch.Tensor:
        loss, _ = K.spike_time_loss(spikes_per_neuron, _targets(targets), mode=0)
        return loss

    def compute_errors(self, spikes_per_neuron, n_spike_per_neuron, targets) -> torch.Tensor:
        _, err = K.spike_time_loss(spikes_per_neuron, _targets(targets), mode=1)
        return err

    def compute_loss_and_errors(self, spikes_per_neuron, n_spike_per_neuron,
                                targets) -> Tuple[torch.Tensor, torch.Tensor]:
        return K.spike_time_loss(spikes_per_neuron, _targets(targets), mode=2)
