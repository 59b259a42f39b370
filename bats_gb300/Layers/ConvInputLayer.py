"""Convolutional input layer (bats/Layers/ConvInputLayer.py:9-47)."""
from __future__ import annotations

from typing import Optional, Tuple

import torch

from ..AbstractConvLayer import AbstractConvLayer
from ..tensors import to_device


class ConvInputLayer(AbstractConvLayer):
    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.__times_per_neuron: Optional[torch.Tensor] = None
        self.__n_spike_per_neuron: Optional[torch.Tensor] = None

    @property
    def trainable(self) -> bool:
        return False

    @property
    def spike_trains(self) -> Tuple[torch.Tensor, torch.Tensor]:
        return self.__times_per_neuron, self.__n_spike_per_neuron

    def set_spike_trains(self, times_per_neuron, n_times_per_neuron) -> None:
        self.__times_per_neuron = to_device(times_per_neuron, torch.float32)
        self.__n_spike_per_neuron = to_device(n_times_per_neuron, torch.int32)

    @property
    def weights(self) -> Optional[torch.Tensor]:
        return None

    @weights.setter
    def weights(self, weights) -> None:
        pass

    def reset(self) -> None:
        pass

    def forward(self, max_simulation: float, training: bool = False) -> None:
        pass

    def backward(self, errors, labels=None) -> Optional[Tuple[torch.Tensor, torch.Tensor]]:
        return None

    def add_deltas(self, delta_weights) -> None:
        pass
