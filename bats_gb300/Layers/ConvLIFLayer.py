"""Convolutional LIF layer (bats/Layers/ConvLIFLayer.py:15-137): valid convolution, stride 1, filters
(C_out, fx, fy, C_in), neurons (x, y, c) with c fastest."""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np
import torch

from .. import kernels as K
from ..AbstractConvLayer import AbstractConvLayer
from ..tensors import to_device


class ConvLIFLayer(AbstractConvLayer):
    def __init__(self, previous_layer: AbstractConvLayer, filters_shape, tau_s: float, theta: float,
                 delta_theta: float, weight_initializer: Callable[[int, int, int, int], torch.Tensor] = None,
                 max_n_spike: int = 32, **kwargs):
        prev_x, prev_y, prev_c = (int(v) for v in previous_layer.neurons_shape)
        filter_x, filter_y, filter_c = (int(v) for v in filters_shape)
        neurons_shape = np.array([prev_x - filter_x + 1, prev_y - filter_y + 1, filter_c], dtype=np.int32)
        super().__init__(neurons_shape=neurons_shape, **kwargs)
        self.__filters_shape = np.array([filter_c, filter_x, filter_y, prev_c], dtype=np.int32)
        self.__previous_layer = previous_layer
        self.__tau_s = np.float32(tau_s)
        self.__tau, self.__c, self.__delta_theta_tau = K.lif_constants(tau_s, theta, delta_theta)
        self.__theta = float(theta)
        self.__delta_theta = float(delta_theta)
        if weight_initializer is None:
            self.__weights = torch.zeros(tuple(int(v) for v in self.__filters_shape), dtype=torch.float32,
                                         device="cuda")
        else:
            self.__weights = to_device(weight_initializer(filter_c, filter_x, filter_y, prev_c), torch.float32)
        self.__max_n_spike = int(max_n_spike)
        self.reset()

    @property
    def trainable(self) -> bool:
        return True

    @property
    def spike_trains(self) -> Tuple[torch.Tensor, torch.Tensor]:
        return self.__spike_times_per_neuron, self.__n_spike_per_neuron

    @property
    def weights(self) -> Optional[torch.Tensor]:
        return self.__weights

    @weights.setter
    def weights(self, weights) -> None:
        self.__weights = to_device(weights, torch.float32).clone()

    @property
    def filters_shape(self) -> np.ndarray:
        return self.__filters_shape

    @property
    def previous_layer(self):
        return self.__previous_layer

    @property
    def tau_s(self) -> float:
        return float(self.__tau_s)

    @property
    def theta(self) -> float:
        return self.__theta

    @property
    def delta_theta(self) -> float:
        return self.__delta_theta

    @property
    def max_n_spike(self) -> int:
        return self.__max_n_spike

    @property
    def solver_state(self):
        return self.__a, self.__x, self.__post_exp_tau

    def reset(self) -> None:
        self.__n_spike_per_neuron = None
        self.__spike_times_per_neuron = None
        self.__a = None
        self.__x = None
        self.__post_exp_tau = None
        self.__events = None

    def forward(self, max_simulation: float, training: bool = False) -> None:
        pre_spike_per_neuron, _ = self.__previous_layer.spike_trains
        # Bucketed copy grouped by input position (bucket width = input channels) for the backward pass,
        # when the input has at most 255 positions.
        X, Y, C = (int(v) for v in self.__previous_layer.neurons_shape)
        self.__events = K.sort_events(pre_spike_per_neuron, self.__tau_s, self.__tau, bucketed=X * Y <= 255,
                                      bucket_width=C)
        (self.__n_spike_per_neuron, self.__a, self.__x, self.__spike_times_per_neuron,
         self.__post_exp_tau) = K.conv_forward(self.__events, self.__weights, self.__previous_layer.neurons_shape,
                                               self.__max_n_spike, self.__tau_s, self.__theta, self.__delta_theta,
                                               max_simulation)

    def backward(self, errors) -> Optional[Tuple[torch.Tensor, torch.Tensor]]:
        """Per-sample filter gradient (B, C_out, fx, fy, C_in) and pre-spike errors (or None)."""
        if not (torch.is_tensor(errors) and errors.is_cuda and errors.dtype == torch.float32
                and errors.is_contiguous()):
            errors = to_device(errors, torch.float32).clone()
        tabs = K.backward_prep(self.__spike_times_per_neuron, self.__a, self.__x, self.__post_exp_tau, errors,
                               self.__c, self.__tau, self.__delta_theta_tau)
        grad, pre_errors = K.conv_backward(self.__events, self.__weights, self.__previous_layer.neurons_shape,
                                           self.__spike_times_per_neuron, tabs, self.__tau_s, self.__tau,
                                           want_pre_errors=self.__previous_layer.trainable)
        return grad, pre_errors

    def add_deltas(self, delta_weights) -> None:
        K.add_deltas(self.__weights, delta_weights)


LIFLayerConv = ConvLIFLayer
