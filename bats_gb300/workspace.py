"""Grow-only scratch buffers shared by the kernel wrappers, one per (device, slot).

All kernels of a step are launched on one stream, so one buffer can serve them in turn; when a
buffer grows, the old tensor is released through torch's stream-ordered caching allocator.
Code that captures a CUDA graph reserves the sizes first (reserve) so that no buffer moves while
the graph is recorded.
"""
from __future__ import annotations

import torch

_buffers: dict = {}


def workspace(nbytes: int, device, slot: int = 0) -> torch.Tensor:
    """A uint8 CUDA tensor of at least nbytes (256-byte aligned, as torch allocations are)."""
    dev = torch.device(device)
    key = (dev.index if dev.index is not None else torch.cuda.current_device(), slot)
    buf = _buffers.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
        _buffers[key] = buf
    return buf


def reserve(nbytes: int, device, slot: int = 0) -> None:
    workspace(nbytes, device, slot)


def release_all() -> None:
    _buffers.clear()
