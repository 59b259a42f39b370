"""Optimizer contract (bats/AbstractOptimizer.py:6-20): step(gradients) -> deltas."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import List

import numpy as np


class AbstractOptimizer(ABC):
    def __init__(self, learning_rate: float):
        self._learning_rate = np.float32(learning_rate)

    @property
    def learning_rate(self) -> np.float32:
        return self._learning_rate

    @learning_rate.setter
    def learning_rate(self, value: float) -> None:
        self._learning_rate = np.float32(value)

    @abstractmethod
    def step(self, gradient: List) -> List:
        ...
