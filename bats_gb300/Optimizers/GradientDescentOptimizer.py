"""Plain gradient descent (bats/Optimizers/GradientDescentOptimizer.py:7-9): deltas = -lr * g."""
from __future__ import annotations

from typing import List

import torch

from ..AbstractOptimizer import AbstractOptimizer
from ..tensors import to_device


class GradientDescentOptimizer(AbstractOptimizer):
    def step(self, gradient: List) -> List:
        return [None if g is None else to_device(g, torch.float32) * (-float(self._learning_rate))
                for g in gradient]
