"""2x2 spike-union pooling (bats/Layers/PoolingLayer.py:13-69): each output neuron carries the union of
its four children's spike trains (K_out = 4 K_in), sorted by time; backward scatters the errors back."""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import torch

from .. import kernels as K
from ..AbstractConvLayer import AbstractConvLayer


class PoolingLayer(AbstractConvLayer):
    def __init__(self, previous_layer: AbstractConvLayer, **kwargs):
        prev_x, prev_y, prev_c = (int(v) for v in previous_layer.neurons_shape)
        super().__init__(neurons_shape=np.array([prev_x // 2, prev_y // 2, prev_c], dtype=np.int32), **kwargs)
        self.__previous_layer = previous_layer
        self.reset()

    @property
    def trainable(self) -> bool:
        return True

    @property
    def spike_trains(self) -> Tuple[torch.Tensor, torch.Tensor]:
        return self.__spike_times_per_neuron, self.__n_spike_per_neuron

    @property
    def spike_indices(self) -> Optional[torch.Tensor]:
        return self.__spike_indices

    @property
    def previous_layer(self):
        return self.__previous_layer

    @property
    def weights(self) -> Optional[torch.Tensor]:
        return None

    @weights.setter
    def weights(self, weights) -> None:
        pass

    def reset(self) -> None:
        self.__n_spike_per_neuron = None
        self.__spike_times_per_neuron = None
        self.__spike_indices = None

    def forward(self, max_simulation: float, training: bool = False) -> None:
        pre_spike_per_neuron, pre_n_spike_per_neuron = self.__previous_layer.spike_trains
        self.__n_spike_per_neuron, self.__spike_times_per_neuron, self.__spike_indices = \
            K.aggregate_spikes_conv(pre_n_spike_per_neuron, pre_spike_per_neuron, self.__previous_layer.neurons_shape)

    def backward(self, errors) -> Optional[Tuple[torch.Tensor, torch.Tensor]]:
        if self.__previous_layer.trainable:
            batch_size, n_neurons, max_n_spike = errors.shape
            pre_errors = K.pool_backward(errors, self.__spike_indices,
                                         (batch_size, self.__previous_layer.n_neurons, max_n_spike // 4))
        else:
            pre_errors = None
        return None, pre_errors

    def add_deltas(self, delta_weights) -> None:
        pass
