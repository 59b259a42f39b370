"""Parity of the convolutional network at its configuration's own size: 28x28x1 MNIST-shaped single-spike input
(each pixel fires once with probability 0.19 at U(0, 0.01) s) -> LIFLayerConv 5x5x15 -> PoolingLayer 2x2 ->
LIFLayerConv 5x5x40 -> PoolingLayer 2x2 -> LIF FC 300 -> 10, max_n_spike 10 in every LIF layer, batch 128,
the thresholds of the reference's MNIST conv experiment (0.04 / 0.8 / 0.6 / 0.3, delta_theta = theta,
tau_s 0.13, weights U(-1, 1)), max_simulation 0.2, spike-count class loss (targets 15 / 3).

Our side is the drop-in layer API (Network, ConvLIFLayer, PoolingLayer, LIFLayer); the reference side is its
compiled kernels with its wrappers' launch shapes (oracle/refkern.py). Forward: every layer's spike counts
equal and a, x, t, z bit-identical in every valid slot; the pooled trains equal. Backward, layer by layer from
the same incoming errors (the loss errors for the output layer, the reference's own errors of the layer above
otherwise): each layer's batch-summed gradient and its pre-spike errors within
1e-5 |ref| + 1e-5 sum|terms| (sum|terms|: the reference kernels on |errors|, |f1|, -|f2|, |W|, -tau); the
pooling layers' scattered errors equal. The test prints, per layer, how many entries needed the sum|terms|
part. The reference's conv error propagation indexes its (B, N_pre, K_pre, C_out fx fy) temporary in unsigned
32-bit arithmetic, which wraps at this size for the second conv layer (B >= 50), so oracle/refkern.py runs
it in chunks of samples."""
import numpy as np
import pytest
import torch

from oracle import refkern
from tests._helpers import assert_sum_close, mnist_like_input, ref_conv_layer_backward, ref_layer_backward

pytestmark = pytest.mark.gpu

B, KC = 128, 10
TAU_S = np.float32(0.13)
THETAS = (0.04, 0.8, 0.6, 0.3)
MAX_SIM = np.float32(0.2)


def _weights(seed=3):
    rng = np.random.default_rng(seed)
    return [rng.uniform(-1, 1, (15, 5, 5, 1)).astype(np.float32), rng.uniform(-1, 1, (40, 5, 5, 15)).astype(np.float32),
            rng.uniform(-1, 1, (300, 640)).astype(np.float32), rng.uniform(-1, 1, (10, 300)).astype(np.float32)]


def _same_forward(ours, ref, K, what):
    n, t = ours.spike_trains[1], ours.spike_trains[0]
    a, x, z = ours.solver_state
    rn, ra, rx, rt, rz = ref
    assert torch.equal(n, rn), f"{what}: spike counts differ from the reference kernels"
    valid = torch.arange(K, device="cuda")[None, None, :] < rn[:, :, None]
    for name, u, v in (("a", a, ra), ("x", x, rx), ("t", t, rt), ("z", z, rz)):
        assert torch.equal(u[valid], v[valid]), f"{what}: {name} differs from the reference kernels"


def test_conv_network_vs_reference_kernels_batch_128(cuda):
    if not refkern.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    from bats_gb300 import Network
    from bats_gb300.Layers import ConvInputLayer, ConvLIFLayer, LIFLayer, PoolingLayer
    t, n_in = mnist_like_input(B, seed=5)
    rng = np.random.default_rng(6)
    labels = rng.integers(0, 10, B)
    w1, w2, w3, w4 = _weights()
    cu = lambda a: torch.tensor(a, device="cuda")
    net = Network()
    inp = ConvInputLayer(neurons_shape=np.array([28, 28, 1]), name="in")
    net.add_layer(inp, input=True)
    c1 = ConvLIFLayer(inp, filters_shape=np.array([5, 5, 15]), tau_s=TAU_S, theta=THETAS[0], delta_theta=THETAS[0],
                      weight_initializer=lambda *a: cu(w1), max_n_spike=KC, name="conv1")
    net.add_layer(c1)
    p1 = PoolingLayer(c1, name="pool1")
    net.add_layer(p1)
    c2 = ConvLIFLayer(p1, filters_shape=np.array([5, 5, 40]), tau_s=TAU_S, theta=THETAS[1], delta_theta=THETAS[1],
                      weight_initializer=lambda *a: cu(w2), max_n_spike=KC, name="conv2")
    net.add_layer(c2)
    p2 = PoolingLayer(c2, name="pool2")
    net.add_layer(p2)
    f1 = LIFLayer(p2, n_neurons=300, tau_s=TAU_S, theta=THETAS[2], delta_theta=THETAS[2],
                  weight_initializer=lambda *a: cu(w3), max_n_spike=KC, name="fc")
    net.add_layer(f1)
    out = LIFLayer(f1, n_neurons=10, tau_s=TAU_S, theta=THETAS[3], delta_theta=THETAS[3],
                   weight_initializer=lambda *a: cu(w4), max_n_spike=KC, name="out")
    net.add_layer(out)
    net.forward(t, n_in, max_simulation=MAX_SIM, training=True)

    R1 = refkern.RefConvLIF(cu(w1), (28, 28, 1), TAU_S, THETAS[0], THETAS[0], KC)
    R2 = refkern.RefConvLIF(cu(w2), (12, 12, 15), TAU_S, THETAS[1], THETAS[1], KC)
    R3 = refkern.RefLIF(cu(w3), TAU_S, THETAS[2], THETAS[2], KC)
    R4 = refkern.RefLIF(cu(w4), TAU_S, THETAS[3], THETAS[3], KC)
    r1 = R1.forward(cu(t), cu(n_in), MAX_SIM)
    _same_forward(c1, r1, KC, "conv1")
    pn1, pt1, pi1 = refkern.pool_forward(r1[0], r1[3], (24, 24, 15))
    assert torch.equal(p1.spike_trains[1], pn1) and torch.equal(p1.spike_trains[0], pt1), "pool1 differs"
    r2 = R2.forward(pt1, pn1, MAX_SIM)
    _same_forward(c2, r2, KC, "conv2")
    pn2, pt2, pi2 = refkern.pool_forward(r2[0], r2[3], (8, 8, 40))
    assert torch.equal(p2.spike_trains[1], pn2) and torch.equal(p2.spike_trains[0], pt2), "pool2 differs"
    r3 = R3.forward(pt2, pn2, MAX_SIM)
    _same_forward(f1, r3, KC, "fc 300")
    r4 = R4.forward(r3[3], r3[0], MAX_SIM)
    _same_forward(out, r4, KC, "out 10")
    spikes = [int(v.sum()) for v in (r1[0], r2[0], r3[0], r4[0])]
    assert min(spikes[:3]) > 1000, spikes

    tt = torch.full((B, 10), 3.0, device="cuda")
    tt[torch.arange(B), torch.as_tensor(labels, device="cuda").long()] = 15.0
    err = (tt - r4[0].float())[:, :, None].repeat(1, 1, KC).contiguous()
    report = []

    def check_fc(layer, ref_layer, e_in, tag):
        g, pe = layer.backward(e_in.clone())
        g_ref, g_abs, pe_ref, pe_abs = ref_layer_backward(ref_layer, e_in.clone(), want_pre=True)
        st = assert_sum_close(g.double().sum(0).cpu().numpy(), g_ref, g_abs, what=f"{tag} gradient")
        report.append(f"{tag} W: {st[1]}/{st[0]} need sum|terms|, worst {st[2]:.3f}")
        st = assert_sum_close(pe.double().cpu().numpy(), pe_ref.double().cpu().numpy(), pe_abs.double().cpu().numpy(),
                              what=f"{tag} pre errors")
        report.append(f"{tag} pre: {st[1]}/{st[0]}, worst {st[2]:.3f}")
        return pe_ref.contiguous()

    def check_conv(layer, ref_layer, e_in, tag, want_pre):
        g, pe = layer.backward(e_in.clone())
        g_ref, g_abs, pe_ref, pe_abs = ref_conv_layer_backward(ref_layer, e_in.clone(), want_pre=want_pre)
        st = assert_sum_close(g.double().sum(0).cpu().numpy(), g_ref, g_abs, what=f"{tag} gradient")
        report.append(f"{tag} W: {st[1]}/{st[0]} need sum|terms|, worst {st[2]:.3f}")
        if want_pre:
            st = assert_sum_close(pe.double().cpu().numpy(), pe_ref.double().cpu().numpy(),
                                  pe_abs.double().cpu().numpy(), what=f"{tag} pre errors")
            report.append(f"{tag} pre: {st[1]}/{st[0]}, worst {st[2]:.3f}")
            return pe_ref.contiguous()
        return None

    e3 = check_fc(out, R4, err, "out 10")
    e_p2 = check_fc(f1, R3, e3, "fc 300")
    _, e2 = p2.backward(e_p2.clone())
    e2_ref = refkern.pool_backward(e_p2, pi2, r2[3].shape)
    assert torch.equal(e2, e2_ref), "pool2 backward differs"
    e_p1 = check_conv(c2, R2, e2_ref.contiguous(), "conv2", want_pre=True)
    _, e1 = p1.backward(e_p1.clone())
    e1_ref = refkern.pool_backward(e_p1, pi1, r1[3].shape)
    assert torch.equal(e1, e1_ref), "pool1 backward differs"
    check_conv(c1, R1, e1_ref.contiguous(), "conv1", want_pre=False)
    print(f"\n[conv network batch 128, spikes per LIF layer {spikes}] " + "; ".join(report))
