"""Monitors (bats/Monitors/*.py interface) on CUDA tensors from a real forward pass of the drop-in API: the
values equal those computed on the host from the same arrays, and add() never synchronises the device (the
counters stay on the GPU until record(); checked with torch's synchronisation debug mode set to raise)."""
import numpy as np
import pytest
import torch

from bats_gb300.Monitors import (AccuracyMonitor, LossMonitor, SilentLabelsMonitor, SilentNeuronsMonitor,
                                 SpikeCountMonitor, WeightsNormMonitor)
from tests._helpers import mnist_like_input

pytestmark = pytest.mark.gpu


def test_monitors_accumulate_on_the_device(cuda):
    from bats_gb300 import Network, SpikeCountClassLoss
    from bats_gb300.Layers import InputLayer, LIFLayer
    rng = np.random.default_rng(4)
    net = Network()
    inp = InputLayer(n_neurons=784, name="in")
    net.add_layer(inp, input=True)
    w1 = torch.tensor(rng.uniform(-1, 1, (120, 784)).astype(np.float32), device="cuda")
    w2 = torch.tensor(rng.uniform(-1, 1, (10, 120)).astype(np.float32), device="cuda")
    hid = LIFLayer(inp, n_neurons=120, tau_s=0.13, theta=0.2, delta_theta=0.2, weight_initializer=lambda *a: w1,
                   max_n_spike=30, name="hid")
    net.add_layer(hid)
    out = LIFLayer(hid, n_neurons=10, tau_s=0.13, theta=1.3, delta_theta=1.3, weight_initializer=lambda *a: w2,
                   max_n_spike=30, name="out")
    net.add_layer(out)
    loss_fn = SpikeCountClassLoss(15, 3)
    mons = dict(acc=AccuracyMonitor(), loss=LossMonitor(), silent_labels=SilentLabelsMonitor(),
                silent=SilentNeuronsMonitor("hid"), count=SpikeCountMonitor("hid"), wnorm=WeightsNormMonitor("hid"))
    host = {k: [] for k in ("pred", "labels", "loss", "n_out", "n_hid")}
    for batch in range(3):
        t, n = mnist_like_input(32, seed=batch)
        labels = torch.tensor(rng.integers(0, 10, 32), device="cuda")
        net.reset()
        net.forward(t, n, max_simulation=0.2)
        sp, n_out = net.output_spike_trains
        loss = loss_fn.compute_loss(sp, n_out, labels)
        pred = loss_fn.predict(sp, n_out)
        n_hid = hid.spike_trains[1]
        torch.cuda.synchronize()
        torch.cuda.set_sync_debug_mode("error")
        try:
            mons["acc"].add(pred, labels)
            mons["loss"].add(loss)
            mons["silent_labels"].add(n_out, labels)
            mons["silent"].add(n_hid)
            mons["count"].add(n_hid)
        finally:
            torch.cuda.set_sync_debug_mode("default")
        for k, v in (("pred", pred), ("labels", labels), ("loss", loss), ("n_out", n_out), ("n_hid", n_hid)):
            host[k].append(v.cpu().numpy())
    mons["wnorm"].add(w1)
    h = {k: np.concatenate(v) for k, v in host.items()}
    assert int(h["n_hid"].sum()) > 0
    assert np.isclose(mons["acc"].record(1.0), np.mean(h["pred"] == h["labels"]) * 100)
    fin = np.isfinite(h["loss"])
    assert np.isclose(mons["loss"].record(1.0), h["loss"][fin].mean(), rtol=1e-6)
    rows = np.arange(len(h["labels"]))
    assert np.isclose(mons["silent_labels"].record(1.0), np.mean(h["n_out"][rows, h["labels"]] == 0) * 100)
    assert np.isclose(mons["silent"].record(1.0), np.mean(h["n_hid"].sum(0) == 0) * 100)
    assert np.isclose(mons["count"].record(1.0), h["n_hid"].sum() / len(h["n_hid"]))
    assert np.isclose(mons["wnorm"].record(1.0), np.linalg.norm(w1.cpu().numpy().astype(np.float64)), rtol=1e-5)
