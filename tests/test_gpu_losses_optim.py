"""GPU checks of the losses, Adam and the layer API (known answers of the reference tests and the
float64 oracle), including the reference's 200-epoch LIF training known answer."""
import os
from pathlib import Path

import numpy as np
import pytest
import torch

from bats_gb300 import Network, SpikeCountClassLoss, SpikeCountLoss, SpikeTimeLoss, TTFSSoftmaxCrossEntropy
from bats_gb300.Layers import InputLayer, LIFLayer
from bats_gb300.Optimizers import AdamOptimizer, GradientDescentOptimizer
from bats_gb300 import kernels as K
from oracle import bats_ref64 as R
from tests._helpers import mnist_like_input

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def cu(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), device="cuda", dtype=dtype)


def test_spike_count_class_loss(cuda):
    rng = np.random.default_rng(0)
    counts = rng.integers(0, 15, (100, 10))
    labels = rng.integers(0, 10, 100)
    targets = R.class_targets(labels, 10, 10, 2)
    exp_loss, exp_err = R.spike_count_loss(counts, targets, 15)
    loss_fn = SpikeCountClassLoss(target_true=10, target_false=2)
    for dtype in (torch.int32, torch.float32):
        loss, err = loss_fn.compute_loss_and_errors(torch.empty((100, 10, 15), device="cuda"), cu(counts, dtype),
                                                    cu(labels, torch.int32))
        np.testing.assert_allclose(loss.cpu().numpy(), exp_loss, rtol=1e-6)
        np.testing.assert_allclose(err.cpu().numpy(), exp_err, rtol=1e-6)
    np.testing.assert_allclose(loss_fn.compute_loss(None, cu(counts, torch.int32), cu(labels, torch.int32)).cpu(),
                               exp_loss, rtol=1e-6)
    assert torch.equal(loss_fn.predict(None, cu(counts, torch.int32)).cpu(), torch.tensor(counts).argmax(1))
    plain = SpikeCountLoss()
    loss, err = plain.compute_loss_and_errors(torch.empty((100, 10, 3), device="cuda"), cu(counts), cu(targets))
    np.testing.assert_allclose(loss.cpu().numpy(), exp_loss, rtol=1e-6)


def test_ttfs_known_answer(cuda):
    d = np.load(os.path.join(GOLDEN, "kat_ttfs.npz"))
    fn = TTFSSoftmaxCrossEntropy(float(d["tau"]))
    loss, err = fn.compute_loss_and_errors(cu(d["spikes"]), None, cu(d["labels"], torch.int32))
    np.testing.assert_allclose(loss.cpu().numpy(), d["loss"], rtol=1e-5)
    np.testing.assert_allclose(err.cpu().numpy(), d["errors"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(fn.compute_loss(cu(d["spikes"]), None, cu(d["labels"], torch.int32)).cpu().numpy(),
                               d["loss"], rtol=1e-5)


def test_spike_time_loss(cuda):
    rng = np.random.default_rng(3)
    sp = rng.uniform(0, 0.5, (5, 4, 3)).astype(np.float32)
    sp[0, 1, :] = np.inf
    tg = rng.uniform(0, 0.5, (5, 4, 3)).astype(np.float32)
    tg[1, 2, 0] = np.inf
    t_dev = cu(tg)
    loss, err = SpikeTimeLoss().compute_loss_and_errors(cu(sp), None, t_dev)
    tg64 = tg.astype(np.float64)
    el, ee = R.spike_time_loss(sp, tg64)
    np.testing.assert_allclose(loss.cpu().numpy(), el, rtol=1e-5)
    np.testing.assert_allclose(err.cpu().numpy(), ee, rtol=1e-5)
    assert float(t_dev[1, 2, 0]) == 1.0  # targets modified in place like the reference


def test_adam_matches_oracle_over_steps(cuda):
    rng = np.random.default_rng(1)
    g = [None, rng.normal(size=(5, 10)).astype(np.float32), rng.normal(size=(2, 5)).astype(np.float32)]
    ours = AdamOptimizer(learning_rate=0.05)
    ref = R.Adam(0.05)
    for step in range(20):
        d = ours.step([None if x is None else cu(x) for x in g])
        e = ref.step(g)
        for a, b in zip(d, e):
            if b is None:
                assert a is None
                continue
            np.testing.assert_allclose(a.cpu().numpy(), b, rtol=2e-5, atol=1e-9)
        g = [None if x is None else (x * 0.9).astype(np.float32) for x in g]


def test_optimizers_drive_weights_to_zero(cuda):
    """AdamOptimizer.py / GradientDescentOptimizer.py of the reference tests: use the weights as gradients."""
    for opt in (AdamOptimizer(learning_rate=0.05), GradientDescentOptimizer(learning_rate=0.05)):
        torch.manual_seed(0)
        weights = [None, torch.randn(5, 10, device="cuda"), torch.randn(2, 5, device="cuda")]
        for _ in range(1000):
            deltas = opt.step(weights)
            for w, d in zip(weights, deltas):
                if w is not None:
                    w += d
        for w in weights[1:]:
            assert torch.allclose(w, torch.zeros_like(w), atol=1e-5 if isinstance(opt, AdamOptimizer) else 1e-8)


def test_lif_training_known_answer(cuda):
    """LIFLayer_tests.py:91-132: 200 epochs of first-spike-time MSE descent on a 7->5 layer put every first
    spike within 5e-4 of its target."""
    d = np.load(os.path.join(GOLDEN, "kat_lif_training.npz"))
    inp = InputLayer(n_neurons=d["spike_per_neuron"].shape[1])
    layer = LIFLayer(previous_layer=inp, n_neurons=int(d["n_post"]), tau_s=float(d["tau_s"]), theta=float(d["theta"]),
                     delta_theta=float(d["delta_theta"]),
                     weight_initializer=lambda a, b: cu(d["weights0"]), max_n_spike=int(d["max_n_spike"]))
    inp.set_spike_trains(d["spike_per_neuron"], d["n_spike_per_neuron"])
    targets = cu(d["targets"])
    lr = float(d["learning_rate"])
    for _ in range(int(d["n_epoch"])):
        layer.reset()
        layer.forward(float(d["max_simulation"]))
        sp, _ = layer.spike_trains
        err = torch.zeros_like(sp)
        err[:, :, 0] = sp[:, :, 0] - targets
        g, _ = layer.backward(err)
        layer.add_deltas(-lr * g.mean(0))
    sp, _ = layer.spike_trains
    np.testing.assert_allclose(sp[:, :, 0].cpu().numpy(), d["targets"], atol=float(d["atol"]))


def test_store_restore(cuda, tmp_path):
    """LIFLayer_tests.py:134-161."""
    inp = InputLayer(n_neurons=7)
    w = torch.randn(5, 7, device="cuda")
    layer = LIFLayer(previous_layer=inp, n_neurons=5, tau_s=0.01, theta=0.01, delta_theta=0.01,
                     weight_initializer=lambda a, b: w, max_n_spike=8, name="test_layer")
    net = Network()
    net.add_layer(inp, input=True)
    net.add_layer(layer)
    net.store(Path(tmp_path))
    layer2 = LIFLayer(previous_layer=inp, n_neurons=5, tau_s=0.01, theta=0.01, delta_theta=0.01, max_n_spike=8,
                      name="test_layer")
    layer2.restore(Path(tmp_path))
    assert torch.allclose(layer2.weights, w)
    assert os.path.exists(tmp_path / "test_layer_weights.npy")


def test_nadam_matches_oracle_and_converges(cuda):
    from bats_gb300.Optimizers import NAdamOptimizer
    rng = np.random.default_rng(2)
    g = [None, rng.normal(size=(5, 10)).astype(np.float32), rng.normal(size=(2, 5)).astype(np.float32)]
    ours = NAdamOptimizer(learning_rate=0.05)
    ref = R.NAdam(0.05)
    for step in range(20):
        d = ours.step([None if x is None else cu(x) for x in g])
        e = ref.step(g)
        for a, b in zip(d, e):
            if b is None:
                assert a is None
                continue
            np.testing.assert_allclose(a.cpu().numpy(), b, rtol=2e-5, atol=1e-9)
        g = [None if x is None else (x * 0.9).astype(np.float32) for x in g]
    opt = NAdamOptimizer(learning_rate=0.05)
    torch.manual_seed(0)
    w = torch.randn(5, 10, device="cuda")
    for _ in range(1000):
        w += opt.step([w])[0]
    assert torch.allclose(w, torch.zeros_like(w), atol=1e-4)


def test_synaptic_scaling_regularizers(cuda):
    rng = np.random.default_rng(3)
    B, N, M = 6, 7, 9
    W = rng.normal(size=(N, M)).astype(np.float32)
    grad = rng.normal(size=(B, N, M)).astype(np.float32)
    n_sp = rng.integers(0, 2, (B, N)).astype(np.int32)
    ratios = rng.uniform(0, 1, B).astype(np.float32)
    g = cu(grad)
    K.apply_weights_synaptic_scaling(cu(W), cu(ratios), cu(n_sp, torch.int32), g, 0.5, 0.1)
    np.testing.assert_allclose(g.cpu().numpy(), R.weights_synaptic_scaling(W, ratios, n_sp, grad, 0.5, 0.1),
                               rtol=1e-6, atol=1e-7)
    labels = rng.integers(0, N, B).astype(np.float32)
    labels[0] = N + 3  # not a neuron: skipped
    g = cu(grad)
    K.apply_label_weights_synaptic_scaling(cu(W), cu(labels), cu(n_sp, torch.int32), g, 0.2)
    np.testing.assert_allclose(g.cpu().numpy(), R.label_weights_synaptic_scaling(W, labels, n_sp, grad, 0.2),
                               rtol=1e-6, atol=1e-7)


def test_checkpoint_resumes_training_exactly(cuda, tmp_path):
    """Weights (reference format) + Adam state saved after 3 steps; a fresh network and optimizer loaded from
    the checkpoint take the same next 2 steps bit for bit."""
    from bats_gb300 import checkpoint

    def make():
        rng = np.random.default_rng(0)
        net = Network()
        inp = InputLayer(n_neurons=40, name="in")
        net.add_layer(inp, input=True)
        hid = LIFLayer(inp, n_neurons=30, tau_s=0.1, theta=0.2, delta_theta=0.2, max_n_spike=8, name="hid",
                       weight_initializer=lambda a, b: rng.uniform(-1, 1, (a, b)).astype(np.float32))
        net.add_layer(hid)
        out = LIFLayer(hid, n_neurons=5, tau_s=0.1, theta=0.5, delta_theta=0.5, max_n_spike=8, name="out",
                       weight_initializer=lambda a, b: rng.uniform(-1, 1, (a, b)).astype(np.float32))
        net.add_layer(out)
        return net, hid, out

    rng = np.random.default_rng(1)
    t = np.where(rng.random((8, 40, 1)) < 0.5, rng.uniform(0, 0.05, (8, 40, 1)), np.inf).astype(np.float32)
    n = np.isfinite(t[:, :, 0]).astype(np.int32)
    labels = torch.tensor(rng.integers(0, 5, 8), device="cuda")
    loss_fn = SpikeCountClassLoss(5.0, 1.0)

    def step(net, opt):
        net.reset()
        net.forward(t, n, max_simulation=0.2, training=True)
        sp, nsp = net.output_spike_trains
        _, err = loss_fn.compute_loss_and_errors(sp, nsp, labels)
        g = net.backward(err)
        net.apply_deltas(opt.step([None if x is None else x.mean(0) for x in g]))

    net, hid, out = make()
    opt = AdamOptimizer(learning_rate=0.01)
    for _ in range(3):
        step(net, opt)
    checkpoint.save(tmp_path, net, opt)
    assert (tmp_path / "hid_weights.npy").exists() and (tmp_path / "out_weights.npy").exists()
    for _ in range(2):
        step(net, opt)
    net2, hid2, out2 = make()
    opt2 = AdamOptimizer(learning_rate=0.01)
    checkpoint.load(tmp_path, net2, opt2)
    for _ in range(2):
        step(net2, opt2)
    assert torch.equal(hid.weights, hid2.weights) and torch.equal(out.weights, out2.weights)


@pytest.mark.parametrize("group,bucketed,n_post", [(8, True, 120), (8, False, 120), (64, True, 120), (4, True, 400)])
def test_fused_gradient_adam_equals_gradient_then_adam(cuda, group, bucketed, n_post):
    """bats_weights_gradient_adam (group partials summed, divided by the batch and fed to Adam by one tiled
    kernel; for layers of few weight tiles the row-parallel reduction, then the tiled Adam) gives the gradient,
    m, v, weights and transposed weights of bats_weights_gradient followed by bats_adam_step_device bit for
    bit, over two steps: several partials (group 8 of a batch of 32) with the bucketed or the plain event
    list, one partial (group >= batch), and a layer of 400 x 784 weights (325 tiles: the fused kernel)."""
    from bats_gb300._lib import call, ptr, stream_ptr
    B, n_in = 32, 784
    t, _ = mnist_like_input(B, seed=12)
    rng = np.random.default_rng(13)
    W = torch.tensor(rng.uniform(-1, 1, (n_post, n_in)).astype(np.float32), device="cuda")
    ev = K.sort_events(torch.tensor(t, device="cuda"), np.float32(0.13), np.float32(0.26), bucketed=bucketed)
    wt = K.transpose_weights(W)
    n, a, x, ts, z = K.lif_forward_fc(ev, wt, n_post, 20, 0.13, 0.2, 0.2, 0.2)
    assert int(n.sum()) > 0
    err = torch.tensor(rng.uniform(-1, 1, ts.shape).astype(np.float32), device="cuda")
    tau32, c, dtt = K.lif_constants(0.13, 0.2, 0.2)
    tabs = K.backward_prep(ts, a, x, z, err, c, tau32, dtt)
    ws_bytes = max(256, K.call_size("bats_weights_gradient_workspace_bytes", B, n_post, n_in, group))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    state = []
    for fused in (False, True):
        w, wtt = W.clone(), wt.clone()
        m, v = torch.zeros_like(W), torch.zeros_like(W)
        g = torch.zeros_like(W)
        powers = torch.tensor([1.0, 1.0, 0.0, 0.0], dtype=torch.float64, device="cuda")
        for _ in range(2):
            call("bats_adam_powers_advance", ptr(powers), 0.9, 0.999, stream_ptr())
            common = (ptr(ev.events), ptr(ev.counts), ptr(ev.bucketed), ptr(ev.bucket_offsets), ev.cap, ptr(ts),
                      ptr(tabs.tables), ptr(tabs.nvalid), ptr(tabs.heads), B, n_post, 20, n_in, group)
            if fused:
                call("bats_weights_gradient_adam", *common, ptr(g), ptr(m), ptr(v), 0.9, 0.999, 1e-8, 3e-3,
                     ptr(powers), ptr(w), ptr(wtt), wtt.shape[1], ptr(ws), ws_bytes, stream_ptr())
            else:
                call("bats_weights_gradient", *common, 1, ptr(g), ptr(ws), ws_bytes, stream_ptr())
                call("bats_adam_step_device", ptr(g), ptr(m), ptr(v), w.numel(), 0.9, 0.999, 1e-8, 3e-3,
                     ptr(powers), ptr(w), ptr(wtt), n_post, n_in, wtt.shape[1], stream_ptr())
        torch.cuda.synchronize()
        state.append([v_.cpu().numpy() for v_ in (g, m, v, w, wtt)])
    assert np.abs(state[0][0]).max() > 0
    for name, p, q in zip(("grad", "m", "v", "weights", "transposed weights"), *state):
        assert np.array_equal(p.view(np.uint32), q.view(np.uint32)), name
