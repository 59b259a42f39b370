"""Spike-count loss (bats/Losses/SpikeCountLoss.py:7-38): loss = 1/2 sum (target - count)^2 per sample,
errors = (target - count) repeated over the K spike slots."""
from __future__ import annotations

from typing import Tuple

import torch

from .. import kernels as K
from ..AbstractLoss import AbstractLoss


class SpikeCountLoss(AbstractLoss):
    def predict(self, spikes_per_neuron, n_spike_per_neuron) -> torch.Tensor:
        return torch.argmax(n_spike_per_neuron, dim=1)

    def compute_loss(self, spikes_per_neuron, n_spike_per_neuron, targets) -> torch.Tensor:
        loss, _ = K.spike_count_loss(n_spike_per_neuron, targets=targets, want_errors=False)
        return loss

    def compute_errors(self, spikes_per_neuron, n_spike_per_neuron, targets) -> torch.Tensor:
        _, err = K.spike_count_loss(n_spike_per_neuron, targets=targets, k=spikes_per_neuron.shape[2],
                                    want_loss=False)
        return err

    def compute_loss_and_errors(self, spikes_per_neuron, n_spike_per_neuron,
                                targets) -> Tuple[torch.Tensor, torch.Tensor]:
        return K.spike_count_loss(n_spike_per_neuron, targets=targets, k=spikes_per_neuron.shape[2])
