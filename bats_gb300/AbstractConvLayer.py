"""Convolutional layer contract (bats/AbstractConvLayer.py:11-19): neurons laid out (x, y, c), c fastest."""
from __future__ import annotations

import numpy as np

from .AbstractLayer import AbstractLayer


class AbstractConvLayer(AbstractLayer):
    def __init__(self, neurons_shape, name: str = ""):
        shape = np.asarray(neurons_shape, dtype=np.int32).reshape(3)
        super().__init__(int(shape[0] * shape[1] * shape[2]), name)
        self._neurons_shape = shape

    @property
    def neurons_shape(self) -> np.ndarray:
        return self._neurons_shape
