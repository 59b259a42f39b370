"""NAdam (bats/Optimizers/NAdamOptimizer.py:23-58): step(gradients) returns the deltas
-(lr / (sqrt(v_hat) + eps)) * (beta_1 m_hat + (1 - beta_1) g / (1 - beta_1^t)); m and v are created on the
first step; the bias corrections 1 - beta^t use the float32 betas, evaluated in double."""
from __future__ import annotations

from typing import List, Optional

import numpy as np
import torch

from .. import kernels as K
from ..AbstractOptimizer import AbstractOptimizer
from ..tensors import to_device


class NAdamOptimizer(AbstractOptimizer):
    def __init__(self, beta_1=0.9, beta_2=0.999, epsilon=1e-8, **kwargs):
        super().__init__(**kwargs)
        self.__beta_1 = np.float32(beta_1)
        self.__beta_2 = np.float32(beta_2)
        self.__epsilon = np.float32(epsilon)
        self.__m: Optional[List[Optional[torch.Tensor]]] = None
        self.__v: Optional[List[Optional[torch.Tensor]]] = None
        self.__t = 0

    @property
    def state(self):
        """(t, m list, v list) for checkpointing."""
        return self.__t, self.__m, self.__v

    def load_state(self, t, m, v) -> None:
        self.__t = int(t)
        self.__m = [None if x is None else to_device(x, torch.float32).clone() for x in m]
        self.__v = [None if x is None else to_device(x, torch.float32).clone() for x in v]

    def step(self, gradient: List) -> List:
        self.__t += 1
        grads = [None if g is None else to_device(g, torch.float32) for g in gradient]
        if self.__m is None:
            self.__m = [None if g is None else torch.zeros_like(g) for g in grads]
            self.__v = [None if g is None else torch.zeros_like(g) for g in grads]
        b1 = 1.0 - float(self.__beta_1) ** self.__t
        b2 = 1.0 - float(self.__beta_2) ** self.__t
        deltas = []
        for g, m, v in zip(grads, self.__m, self.__v):
            if g is None:
                deltas.append(None)
                continue
            d = torch.empty_like(g)
            K.nadam_step(g, m, v, self.__beta_1, self.__beta_2, self.__epsilon, self._learning_rate, b1, b2, d)
            deltas.append(d)
        return deltas
