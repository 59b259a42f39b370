"""Time-to-first-spike softmax cross-entropy (bats/Losses/TTFSSoftmaxCrossEntropy.py:7-56): softmax of
exp(-t_first/tau); errors (softmax - onehot... negated, divided by tau) only in slot 0, nan_to_num."""
from __future__ import annotations

from typing import Tuple

import numpy as np
import torch

from .. import kernels as K
from ..AbstractLoss import AbstractLoss


class TTFSSoftmaxCrossEntropy(AbstractLoss):
    def __init__(self, tau: float):
        self.__tau_literal = float(tau)
        self.__tau = np.float32(tau)

    def predict(self, spikes_per_neuron, n_spike_per_neuron) -> torch.Tensor:
        return torch.argmin(spikes_per_neuron, dim=1).flatten()

    def compute_loss(self, spikes_per_neuron, n_spike_per_neuron, labels) -> torch.Tensor:
        loss, _ = K.ttfs_softmax_cross_entropy(spikes_per_neuron, labels, self.__tau_literal, want_errors=False)
        return loss

    def compute_errors(self, spikes_per_neuron, n_spike_per_neuron, labels) -> torch.Tensor:
        _, err = K.ttfs_softmax_cross_entropy(spikes_per_neuron, labels, self.__tau_literal, want_loss=False)
        return err

    def compute_loss_and_errors(self, spikes_per_neuron, n_spike_per_neuron,
                                labels) -> Tuple[torch.Tensor, torch.Tensor]:
        return K.ttfs_softmax_cross_entropy(spikes_per_neuron, labels, self.__tau_literal)
