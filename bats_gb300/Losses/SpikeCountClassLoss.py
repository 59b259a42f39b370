"""Spike-count classification loss (bats/Losses/SpikeCountClassLoss.py:8-33): target_true spikes for the
label neuron, target_false for the others; the targets are formed inside the loss kernel."""
from __future__ import annotations

from typing import Tuple

import numpy as np
import torch

from .. import kernels as K
from .SpikeCountLoss import SpikeCountLoss


class SpikeCountClassLoss(SpikeCountLoss):
    def __init__(self, target_true: float, target_false: float):
        super().__init__()
        self.__target_true = np.float32(target_true)
        self.__target_false = np.float32(target_false)

    def compute_loss(self, spikes_per_neuron, n_spike_per_neuron, labels) -> torch.Tensor:
        loss, _ = K.spike_count_loss(n_spike_per_neuron, labels=labels, target_true=self.__target_true,
                                     target_false=self.__target_false, want_errors=False)
        return loss

    def compute_errors(self, spikes_per_neuron, n_spike_per_neuron, labels) -> torch.Tensor:
        _, err = K.spike_count_loss(n_spike_per_neuron, labels=labels, target_true=self.__target_true,
                                    target_false=self.__target_false, k=spikes_per_neuron.shape[2],
                                    want_loss=False)
        return err

    def compute_loss_and_errors(self, spikes_per_neuron, n_spike_per_neuron,
                                labels) -> Tuple[torch.Tensor, torch.Tensor]:
        return K.spike_count_loss(n_spike_per_neuron, labels=labels, target_true=self.__target_true,
                                  target_false=self.__target_false, k=spikes_per_neuron.shape[2])
