"""The batched, graph-captured conv train step (bats_gb300.conv_train.ConvTrainStep) against the layer-by-layer
drop-in API on the reference's MNIST conv network (28x28x1 -> conv 5x5x15 -> pool -> conv 5x5x40 -> pool -> 300
-> 10, max_n_spike 10, thresholds 0.04 / 0.8 / 0.6 / 0.3, weights U(-1, 1)), batch 32, Adam lr 3e-3:

* the first step's loss and every layer's spike counts are identical (same forward kernels and loss);
* every layer's batch-mean gradient of the first step agrees within 1e-5 of the layer's largest entry: the
  batch mean is the same sum taken in another order (per-group partials accumulated by the backward kernels
  instead of per-sample gradients and torch.mean);
* the weights after that step agree within 1e-6 of the layer's weight scale wherever the gradient is not tiny
  (|g| > 1e-3 max|g|): Adam's first step moves a weight by lr g / (|g| + eps), which for a gradient that is a
  cancelling sum near zero turns last-bit differences of g into differences of the step itself;
* replaying the captured CUDA graph gives the eager step's weights bit for bit.
"""
import numpy as np
import pytest
import torch

from bats_gb300.conv_train import ConvLayerSpec, ConvTrainStep, PoolLayerSpec
from bats_gb300.train import FCLayerSpec
from tests._helpers import mnist_like_input

pytestmark = pytest.mark.gpu

B, KC, TAU_S, LR, MAX_SIM = 32, 10, 0.13, 3e-3, 0.2
THETAS = (0.04, 0.8, 0.6, 0.3)


def weights(seed=3):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1, 1, (15, 5, 5, 1)).astype(np.float32), rng.uniform(-1, 1, (40, 5, 5, 15)).astype(np.float32),
            rng.uniform(-1, 1, (300, 640)).astype(np.float32), rng.uniform(-1, 1, (10, 300)).astype(np.float32)]


def make_step(ws, t, labels, group=2):
    specs = [ConvLayerSpec((5, 5, 15), TAU_S, THETAS[0], THETAS[0], KC), PoolLayerSpec(),
             ConvLayerSpec((5, 5, 40), TAU_S, THETAS[1], THETAS[1], KC), PoolLayerSpec(),
             FCLayerSpec(300, TAU_S, THETAS[2], THETAS[2], KC), FCLayerSpec(10, TAU_S, THETAS[3], THETAS[3], KC)]
    w = [torch.tensor(ws[0]), None, torch.tensor(ws[1]), None, torch.tensor(ws[2]), torch.tensor(ws[3])]
    ts = ConvTrainStep(t.shape[0], (28, 28, 1), 1, specs, w, 15.0, 3.0, learning_rate=LR, max_simulation=MAX_SIM,
                       conv_group=group)
    ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    return ts


def api_steps(ws, t, n, labels, steps):
    from bats_gb300 import Network, SpikeCountClassLoss
    from bats_gb300.Layers import ConvInputLayer, ConvLIFLayer, LIFLayer, PoolingLayer
    from bats_gb300.Optimizers import AdamOptimizer
    cu = lambda a: torch.tensor(a, device="cuda")
    net = Network()
    inp = ConvInputLayer(neurons_shape=np.array([28, 28, 1]), name="in")
    net.add_layer(inp, input=True)
    c1 = ConvLIFLayer(inp, filters_shape=np.array([5, 5, 15]), tau_s=TAU_S, theta=THETAS[0], delta_theta=THETAS[0],
                      weight_initializer=lambda *a: cu(ws[0]), max_n_spike=KC, name="c1")
    p1 = PoolingLayer(c1, name="p1")
    c2 = ConvLIFLayer(p1, filters_shape=np.array([5, 5, 40]), tau_s=TAU_S, theta=THETAS[1], delta_theta=THETAS[1],
                      weight_initializer=lambda *a: cu(ws[1]), max_n_spike=KC, name="c2")
    p2 = PoolingLayer(c2, name="p2")
    f1 = LIFLayer(p2, n_neurons=300, tau_s=TAU_S, theta=THETAS[2], delta_theta=THETAS[2],
                  weight_initializer=lambda *a: cu(ws[2]), max_n_spike=KC, name="f1")
    f2 = LIFLayer(f1, n_neurons=10, tau_s=TAU_S, theta=THETAS[3], delta_theta=THETAS[3],
                  weight_initializer=lambda *a: cu(ws[3]), max_n_spike=KC, name="f2")
    for L in (c1, p1, c2, p2, f1, f2):
        net.add_layer(L)
    loss_fn = SpikeCountClassLoss(15.0, 3.0)
    opt = AdamOptimizer(learning_rate=LR)
    lab = torch.tensor(labels, device="cuda")
    out = []
    for _ in range(steps):
        net.reset()
        net.forward(t, n, max_simulation=MAX_SIM, training=True)
        sp, nsp = net.output_spike_trains
        loss, err = loss_fn.compute_loss_and_errors(sp, nsp, lab)
        g = net.backward(err)
        net.apply_deltas(opt.step([None if x is None else x.mean(0) for x in g]))
        out.append((loss.clone(), [L.weights.clone() for L in (c1, c2, f1, f2)],
                    [int(L.spike_trains[1].sum()) for L in (c1, c2, f1, f2)],
                    [x.mean(0) for x in g if x is not None]))
    return out


def test_conv_train_step_matches_layer_api(cuda):
    t, n = mnist_like_input(B, seed=7)
    labels = np.random.default_rng(8).integers(0, 10, B).astype(np.int32)
    ws = weights()
    ref = api_steps(ws, t, n, labels, 1)
    ts = make_step(ws, t, labels)
    ts.step()
    torch.cuda.synchronize()
    assert torch.equal(ts.loss, ref[0][0]), "first-step loss differs from the layer API"
    spikes = [c for c, d in zip(ts.spike_counts(), ts.L) if d["kind"] != "pool"]
    assert spikes == ref[0][2] and min(spikes[:3]) > 0, spikes
    grads = [d["grad"] for d in ts.L if d["kind"] != "pool"]
    mine = [w for w in ts.weights if w is not None]
    for li, (g, rg, w, rw) in enumerate(zip(grads, ref[0][3], mine, ref[0][1])):
        scale = float(rg.abs().max())
        assert scale > 0, f"layer {li}: zero gradient"
        assert float((g - rg).abs().max()) <= 1e-5 * scale, f"layer {li}: gradient"
        big = rg.abs() > 1e-3 * scale
        assert float((w - rw)[big].abs().max()) <= 1e-6 * float(rw.abs().max()), f"layer {li}: weights"


@pytest.mark.parametrize("group", [1, 3])
def test_conv_train_step_graph_replay_equals_eager(cuda, group):
    t, _ = mnist_like_input(B, seed=9)
    labels = np.random.default_rng(10).integers(0, 10, B).astype(np.int32)
    ws = weights(seed=4)
    eager, graphed = make_step(ws, t, labels, group), make_step(ws, t, labels, group)
    assert graphed.try_capture(), graphed.capture_error  # one eager step, then the capture
    eager.step()
    for _ in range(2):
        eager.step()
        graphed.replay()
    torch.cuda.synchronize()
    for a, b in zip(eager.weights, graphed.weights):
        if a is not None:
            assert torch.equal(a, b)
    assert torch.equal(eager.loss, graphed.loss)


def test_conv_train_step_second_stream_keeps_results(cuda):
    """The fully-connected layers' gradient + Adam on the second stream (staged transposed weights copied in
    at the end of the step) gives the weights, transposed weights and losses of the launch list run in order
    on one stream, bit for bit, eagerly and under graph capture."""
    t, _ = mnist_like_input(B, seed=5)
    labels = np.random.default_rng(6).integers(0, 10, B).astype(np.int32)
    ws = weights(seed=7)
    one, two, graphed = make_step(ws, t, labels), make_step(ws, t, labels), make_step(ws, t, labels)
    one.aux = None
    assert two.aux is not None and any("Wt_next" in d for d in two.L)
    assert graphed.try_capture(), graphed.capture_error
    one.step()
    two.step()
    for _ in range(2):
        one.step()
        two.step()
        graphed.replay()
    torch.cuda.synchronize()
    for a, b, c in zip(one.weights, two.weights, graphed.weights):
        if a is not None:
            assert torch.equal(a, b) and torch.equal(a, c)
    for da, db in zip(one.L, two.L):
        if "Wt" in da:
            assert torch.equal(da["Wt"], db["Wt"])
    assert torch.equal(one.loss, two.loss) and torch.equal(one.loss, graphed.loss)

