"""Training checkpoints: the network's weights in the reference's on-disk format (one
`<layer name>_weights.npy` per layer, bats/AbstractLayer.py:61-70, so models move between the reference and
this package), plus the optimizer's state (step count and the m, v moments of Adam or NAdam) in
`optimizer_state.npz`, which the reference does not save."""
from __future__ import annotations

from pathlib import Path

import numpy as np

OPTIMIZER_FILE = "optimizer_state.npz"


def save(dir_path, network, optimizer=None) -> None:
    dir_path = Path(dir_path)
    network.store(dir_path)
    if optimizer is None or not hasattr(optimizer, "state"):
        return
    t, m, v = optimizer.state
    arrays = {"t": np.asarray(t, dtype=np.int64), "n": np.asarray(0 if m is None else len(m), dtype=np.int64)}
    for q, (mq, vq) in enumerate(zip(m or [], v or [])):
        if mq is not None:
            arrays[f"m{q}"] = mq.detach().cpu().numpy()
            arrays[f"v{q}"] = vq.detach().cpu().numpy()
    np.savez(dir_path / OPTIMIZER_FILE, **arrays)


def load(dir_path, network, optimizer=None) -> None:
    dir_path = Path(dir_path)
    network.restore(dir_path)
    f = dir_path / OPTIMIZER_FILE
    if optimizer is None or not f.exists():
        return
    d = np.load(f)
    n = int(d["n"])
    m = [d[f"m{q}"] if f"m{q}" in d else None for q in range(n)]
    v = [d[f"v{q}"] if f"v{q}" in d else None for q in range(n)]
    optimizer.load_state(int(d["t"]), m, v)
