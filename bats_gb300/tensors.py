"""Host/device conversions used by the layers."""
from __future__ import annotations

import numpy as np
import torch


def to_device(x, dtype, device="cuda") -> torch.Tensor:
    """A contiguous CUDA tensor of `dtype`; device tensors of the right type are used as they are."""
    if torch.is_tensor(x):
        if x.is_cuda and x.dtype == dtype and x.is_contiguous():
            return x
        return x.to(device=device, dtype=dtype).contiguous()
    arr = np.ascontiguousarray(np.asarray(x))
    return torch.from_numpy(arr).to(device=device, dtype=dtype, non_blocking=False).contiguous()
