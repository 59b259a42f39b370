"""The batched, graph-captured train step (bats_gb300.train.FCTrainStep) against the layer-by-layer drop-in
API on the same network, inputs and Adam settings: forward, spike-count loss, exact backward with the
batch-mean gradient and Adam.

* The first step's loss is identical (same forward kernels and loss).
* After each of 3 steps the weights agree within 1e-6 of the weight scale: the batch mean is the same sum
  taken in another order (group partials instead of per-sample gradients and torch.mean), so the
  gradients differ in the last bits, and Adam's first steps move every weight by about the learning rate.
* Replaying the captured CUDA graph gives the eager step's result bit for bit, and the autotuned step
  (other kernel variants and gradient groups) agrees with the untuned one within the same tolerance.
"""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from bats_gb300 import Network, SpikeCountClassLoss
from bats_gb300 import kernels as KN
from bats_gb300.Layers import InputLayer, LIFLayer
from bats_gb300.Optimizers import AdamOptimizer
from bats_gb300.autotune import Autotuner
from bats_gb300.train import FCLayerSpec, FCTrainStep
from tests._helpers import mnist_like_input

pytestmark = pytest.mark.gpu

SIZES = [784, 120, 10]
THETAS = [0.2, 1.3]
TAU_S, K, LR, MAX_SIM = 0.13, 20, 3e-3, 0.2


def case(B=32, seed=0):
    t, n = mnist_like_input(B, seed=seed)
    rng = np.random.default_rng(seed + 1)
    ws = [rng.uniform(-1, 1, (o, i)).astype(np.float32) for i, o in zip(SIZES[:-1], SIZES[1:])]
    labels = rng.integers(0, SIZES[-1], B).astype(np.int32)
    return t, n, ws, labels


def make_step(t, ws, labels):
    specs = [FCLayerSpec(o, TAU_S, th, th, K) for o, th in zip(SIZES[1:], THETAS)]
    ts = FCTrainStep(t.shape[0], SIZES[0], 1, specs, [torch.tensor(w) for w in ws], 15.0, 3.0, learning_rate=LR,
                     max_simulation=MAX_SIM)
    ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    return ts


def api_steps(t, n, ws, labels, steps):
    net = Network()
    prev = InputLayer(n_neurons=SIZES[0], name="in")
    net.add_layer(prev, input=True)
    layers = []
    for i, (w, th) in enumerate(zip(ws, THETAS)):
        L = LIFLayer(prev, n_neurons=w.shape[0], tau_s=TAU_S, theta=th, delta_theta=th, max_n_spike=K,
                     weight_initializer=lambda a, b, w=w: torch.tensor(w, device="cuda"), name=f"l{i}")
        net.add_layer(L)
        layers.append(L)
        prev = L
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
        out.append((loss.clone(), [L.weights.clone() for L in layers]))
    return out


def test_train_step_matches_layer_api(cuda):
    t, n, ws, labels = case()
    ref = api_steps(t, n, ws, labels, 3)
    ts = make_step(t, ws, labels)
    for k in range(3):
        ts.step()
        torch.cuda.synchronize()
        if k == 0:
            assert torch.equal(ts.loss, ref[0][0]), "first-step loss differs from the layer API"
        for w, rw in zip(ts.W, ref[k][1]):
            assert float((w - rw).abs().max()) <= 1e-6 * float(rw.abs().max()), f"step {k}"
    assert int(ts.out[0][0].sum()) > 0, "the hidden layer should spike"


def test_graph_replay_equals_eager_and_autotune_keeps_results(cuda):
    t, n, ws, labels = case(seed=3)
    eager = make_step(t, ws, labels)
    graphed = make_step(t, ws, labels)
    assert graphed.try_capture(), graphed.capture_error  # runs one eager step, then captures
    eager.step()
    for _ in range(2):
        eager.step()
        graphed.replay()
    torch.cuda.synchronize()
    for a, b in zip(eager.W, graphed.W):
        assert torch.equal(a, b)
    tuned = make_step(t, ws, labels)
    tuned.autotune(Autotuner(path=None), force=True)
    plain = make_step(t, ws, labels)
    for _ in range(2):
        tuned.step()
        plain.step()
    torch.cuda.synchronize()
    for a, b in zip(tuned.W, plain.W):
        assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())


def test_train_host_pipeline_matches_step_host(cuda):
    """train_host (inputs copied from host memory on a side stream while the previous step computes,
    losses read back per step) gives the losses and weights of step_host called batch by batch, bit for
    bit, over five different batches (graph replay in both)."""
    batches = []
    for q in range(5):
        t, _, _, labels = case(seed=10 + q)
        batches.append((t, labels))
    t0, _, ws, labels0 = case()
    a = make_step(t0, ws, labels0)
    b = make_step(t0, ws, labels0)
    assert a.try_capture() and b.try_capture()
    ref = [a.step_host(t, lab).copy() for t, lab in batches]
    got = b.train_host(batches)
    torch.cuda.synchronize()
    assert len(got) == len(ref)
    for q, (x, y) in enumerate(zip(ref, got)):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), f"loss of step {q}"
    for wa, wb in zip(a.W, b.W):
        assert torch.equal(wa, wb)


def test_work_queue_forward_step_equals_tile_step_under_graph_capture(cuda):
    """Every layer's forward on the persistent work-queue kernel (order kernel + queue kernel, captured in the
    step's CUDA graph and replayed) gives the weights of the tile-kernel step bit for bit over 3 steps, on a
    batch of uneven samples."""
    t, n, ws, labels = case(B=48, seed=5)
    keep = np.random.default_rng(6).random(t.shape[:2]) < np.linspace(0.05, 1.0, 48)[:, None]
    t = np.where(keep[:, :, None], t, np.inf).astype(np.float32)  # 5 % to 100 % of the events per sample
    tile = make_step(t, ws, labels)
    tile.fwd_algo = [KN.FWD_TILE] * len(tile.fwd_algo)
    queue = make_step(t, ws, labels)
    queue.fwd_algo = [KN.FWD_QUEUE] * len(queue.fwd_algo)
    assert queue.launches_per_step == tile.launches_per_step + len(queue.fwd_algo)
    assert queue.try_capture(), queue.capture_error  # one eager step, then the capture
    tile.step()
    for _ in range(2):
        tile.step()
        queue.replay()
    torch.cuda.synchronize()
    assert int(queue.out[0][0].sum()) > 0
    for a, b in zip(tile.W, queue.W):
        assert torch.equal(a, b)


_CHILD_STEP_SCRIPT = """
import sys
import numpy as np
import torch
sys.path.insert(0, {root!r})
from tests.test_gpu_train_step import case, make_step
t, n, ws, labels = case(seed=9)
ts = make_step(t, ws, labels)
assert ts.try_capture(), ts.capture_error
for _ in range(2):
    ts.replay()
torch.cuda.synchronize()
np.savez({out!r}, *[w.cpu().numpy() for w in ts.W])
"""


def test_programmatic_dependent_launch_keeps_results(cuda, tmp_path):
    """With BATS_GB300_PDL=1 every kernel is launched with programmatic stream serialization (its successor's
    CTAs start while it drains and wait in their prologue). The graph-replayed train step gives bit-identical
    weights with it (child process: the setting is read once per process) and in plain stream order."""
    if os.environ.get("BATS_GB300_PDL") == "1":
        pytest.skip("this process already runs with programmatic dependent launch")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = str(tmp_path / "pdl.npz")
    env = dict(os.environ, BATS_GB300_PDL="1")
    subprocess.run([sys.executable, "-c", _CHILD_STEP_SCRIPT.format(root=root, out=out)], env=env, check=True,
                   timeout=600)
    t, n, ws, labels = case(seed=9)
    ts = make_step(t, ws, labels)
    assert ts.try_capture(), ts.capture_error
    for _ in range(2):
        ts.replay()
    torch.cuda.synchronize()
    pdl = np.load(out)
    for q, w in enumerate(ts.W):
        assert np.array_equal(w.cpu().numpy().view(np.uint32), pdl[f"arr_{q}"].view(np.uint32)), f"layer {q}"


@pytest.mark.parametrize("tuned,wide", [(False, False), (True, False), (False, True)])
def test_c_abi_train_step_equals_the_launch_list(cuda, tuned, wide):
    """bats_fc_train_step (the whole train step as one call of the C ABI, for foreign callers) enqueues the same
    entry points with the same arguments as FCTrainStep's launch list: after two steps the weights, their
    transposed copies, Adam's moments, the gradients and the losses are bit-identical; with the autotuner's
    variants (work-queue forward, other gradient groups) too, on a batch wider than two CTAs per SM (the hidden
    layer's sort with the samples longest first), and the call can be captured in a CUDA graph."""
    B = 2 * torch.cuda.get_device_properties(0).multi_processor_count + 16 if wide else 48
    t, n, ws, labels = case(B=B, seed=4)
    a, b = make_step(t, ws, labels), make_step(t, ws, labels)
    assert ("L2.order" in [name for name, _ in a.launches]) == wide
    if tuned:
        choice = a.autotune(Autotuner(path=None), force=True)
        b.fwd_algo, b.groups = list(a.fwd_algo), list(a.groups)
        assert choice
    for _ in range(2):
        a.step()
        b.native_step()
    torch.cuda.synchronize()
    for name in ("W", "Wt", "m", "v", "grad"):
        for x, y in zip(getattr(a, name), getattr(b, name)):
            assert torch.equal(x, y), name
    assert torch.equal(a.loss, b.loss)
    # Captured: one foreign call per step inside the graph.
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            b.native_step()
    torch.cuda.current_stream().wait_stream(side)
    g.replay()
    a.step()
    torch.cuda.synchronize()
    for x, y in zip(a.W, b.W):
        assert torch.equal(x, y)


def test_second_stream_keeps_results(cuda):
    """Each upper layer's gradient + Adam on the second stream gives the weights, transposed weights, Adam
    moments and losses of the launch list run in order on one stream, bit for bit."""
    t, n, ws, labels = case(seed=8)
    one, two = make_step(t, ws, labels), make_step(t, ws, labels)
    one.aux = None
    for _ in range(3):
        one.step()
        two.step()
    torch.cuda.synchronize()
    for name in ("W", "Wt", "m", "v", "grad"):
        for x, y in zip(getattr(one, name), getattr(two, name)):
            assert torch.equal(x, y), name
    assert torch.equal(one.loss, two.loss)



def test_longest_first_sort_keeps_results(cuda):
    """A batch wider than the sort's resident CTAs sorts the hidden layer's spikes with the samples longest
    first (an order launch before the second layer's sort); the weights, moments and losses are those of the
    same step without the order, bit for bit."""
    B = 2 * torch.cuda.get_device_properties(0).multi_processor_count + 16
    t, n, ws, labels = case(B=B, seed=9)
    plain, ordered = make_step(t, ws, labels), make_step(t, ws, labels)
    assert ordered.order[1] is not None and "L2.order" in [name for name, _ in ordered.launches]
    plain.order = [None] * len(plain.order)
    plain.launches = plain._build_launches()
    assert "L2.order" not in [name for name, _ in plain.launches]
    for _ in range(3):
        plain.step()
        ordered.step()
    torch.cuda.synchronize()
    for name in ("W", "Wt", "m", "v", "grad"):
        for x, y in zip(getattr(plain, name), getattr(ordered, name)):
            assert torch.equal(x, y), name
    assert torch.equal(plain.loss, ordered.loss)
