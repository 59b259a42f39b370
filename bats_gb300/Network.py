"""Network orchestrator, same contract as bats/Network.py:10-63."""
from __future__ import annotations

from pathlib import Path
from typing import List, Optional, Tuple

import numpy as np
import torch

from .AbstractLayer import AbstractLayer


class Network:
    def __init__(self):
        self.__layers: List[AbstractLayer] = []
        self.__input_layer: Optional[AbstractLayer] = None

    @property
    def layers(self) -> List[AbstractLayer]:
        return self.__layers

    @property
    def input_layer(self) -> Optional[AbstractLayer]:
        return self.__input_layer

    @property
    def output_spike_trains(self) -> Tuple[torch.Tensor, torch.Tensor]:
        return self.__layers[-1].spike_trains

    def add_layer(self, layer: AbstractLayer, input: bool = False) -> None:
        self.__layers.append(layer)
        if input:
            self.__input_layer = layer

    def reset(self):
        for layer in self.__layers:
            layer.reset()

    def forward(self, spikes_per_neuron, n_spikes_per_neuron, max_simulation: float = np.inf,
                training: bool = False) -> None:
        self.__input_layer.set_spike_trains(spikes_per_neuron, n_spikes_per_neuron)
        for layer in self.__layers:
            layer.forward(max_simulation, training)

    def backward(self, output_errors) -> List[Optional[torch.Tensor]]:
        """Per-sample gradients per layer, None for the input layer (bats/Network.py:38-48).
        `output_errors` is modified in place like the reference."""
        errors = output_errors
        gradient = []
        for layer in reversed(self.__layers):
            if not layer.trainable:  # Reached input layer
                gradient.insert(0, None)
                break
            weights_grad, errors = layer.backward(errors)
            gradient.insert(0, weights_grad)
        return gradient

    def apply_deltas(self, deltas) -> None:
        for layer, delta in zip(self.__layers, deltas):
            if delta is None:
                continue
            layer.add_deltas(delta)

    def store(self, dir_path: Path) -> None:
        dir_path = Path(dir_path)
        dir_path.mkdir(parents=True, exist_ok=True)
        for it in self.__layers:
            it.store(dir_path)

    def restore(self, dir_path: Path) -> None:
        for it in self.__layers:
            it.restore(Path(dir_path))
