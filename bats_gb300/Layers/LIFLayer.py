"""Fully-connected LIF layer (bats/Layers/LIFLayer.py:11-113) on the sm_103a kernels.

forward: sort the previous layer's spikes per sample, then the event scan with closed-form
crossings; backward: reset errors + factors + suffix tables, per-sample weight gradient and, when
the previous layer is trainable, the pre-spike errors. The weights are (N_post, N_pre); a transposed
copy (N_pre, ld) is refreshed before each forward for the coalesced weight reads.
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np
import torch

from .. import kernels as K
from ..AbstractLayer import AbstractLayer
from ..tensors import to_device


class LIFLayer(AbstractLayer):
    def __init__(self, previous_layer: AbstractLayer, tau_s: float, theta: float, delta_theta: float,
                 weight_initializer: Callable[[int, int], torch.Tensor] = None, max_n_spike: int = 32, **kwargs):
        super().__init__(**kwargs)
        self.__previous_layer = previous_layer
        self.__tau_s = np.float32(tau_s)
        self.__tau, self.__c, self.__delta_theta_tau = K.lif_constants(tau_s, theta, delta_theta)
        self.__theta = float(theta)
        self.__delta_theta = float(delta_theta)
        if weight_initializer is None:
            self.__weights = torch.zeros((self.n_neurons, previous_layer.n_neurons), dtype=torch.float32,
                                         device="cuda")
        else:
            self.__weights = to_device(weight_initializer(self.n_neurons, previous_layer.n_neurons), torch.float32)
        self.__max_n_spike = int(max_n_spike)
        self.reset()

    # -- properties --------------------------------------------------------------------------
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
    def previous_layer(self) -> AbstractLayer:
        return self.__previous_layer

    @property
    def solver_state(self):
        """(a, x, post_exp_tau) of the last forward, (B, N, K)."""
        return self.__a, self.__x, self.__post_exp_tau

    @property
    def events(self) -> Optional[K.Events]:
        return self.__events

    def reset(self) -> None:
        self.__n_spike_per_neuron = None
        self.__spike_times_per_neuron = None
        self.__a = None
        self.__x = None
        self.__post_exp_tau = None
        self.__events = None
        self.__wt = None

    # -- compute -----------------------------------------------------------------------------
    def forward(self, max_simulation: float, training: bool = False) -> None:
        pre_spike_per_neuron, pre_n_spike_per_neuron = self.__previous_layer.spike_trains
        # A LIF layer's trains are +inf past their counts, so the sort reads only the slots below them.
        counted = isinstance(self.__previous_layer, LIFLayer) and pre_n_spike_per_neuron is not None
        self.__events = K.sort_events(pre_spike_per_neuron, self.__tau_s, self.__tau,
                                      pre_counts=pre_n_spike_per_neuron if counted else None)
        self.__wt = K.transpose_weights(self.__weights)
        (self.__n_spike_per_neuron, self.__a, self.__x, self.__spike_times_per_neuron,
         self.__post_exp_tau) = K.lif_forward_fc(self.__events, self.__wt, self.n_neurons, self.__max_n_spike,
                                                 self.__tau_s, self.__theta, self.__delta_theta, max_simulation)

    def backward(self, errors) -> Optional[Tuple[torch.Tensor, torch.Tensor]]:
        """Per-sample weight gradient (B, N_post, N_pre) and pre-spike errors (or None when the previous
        layer is not trainable). `errors` (B, N, K) receives the reset errors in place."""
        if not (torch.is_tensor(errors) and errors.is_cuda and errors.dtype == torch.float32
                and errors.is_contiguous()):
            errors = to_device(errors, torch.float32).clone()
        tabs = K.backward_prep(self.__spike_times_per_neuron, self.__a, self.__x, self.__post_exp_tau, errors,
                               self.__c, self.__tau, self.__delta_theta_tau, n_spikes=self.__n_spike_per_neuron)
        weights_grad = K.weights_gradient(self.__events, self.__spike_times_per_neuron, tabs,
                                          self.__previous_layer.n_neurons, per_sample=True)
        if self.__previous_layer.trainable:
            pre_errors = K.pre_errors(self.__events, self.__wt, self.__spike_times_per_neuron, tabs,
                                      self.__tau_s, self.__tau)
        else:
            pre_errors = None
        return weights_grad, pre_errors

    def add_deltas(self, delta_weights) -> None:
        K.add_deltas(self.__weights, delta_weights)
