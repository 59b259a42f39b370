"""The differentiation pattern: the LIF layer behind torch.autograd (bats_gb300.autograd.lif_fc) on the
784-800-800-10 network.

* Central finite differences (eps 1e-4) of a smooth loss of the output spike times (sum of r * t over the
  finite output spikes, r fixed Gaussian) on 64 random weights per layer, in the multi-spike regime of
  the network's LIF constants (tau_s 0.13, thresholds 1.0 hidden / 1.3 output, max_n_spike 30) with
  weights N(3.5, 1)/sqrt(fan_in): every hidden neuron spikes, the second hidden layer 6-7 times on
  average. The differences are taken in float64 through the oracle network (oracle/fd.py) on the same
  FP32 weights and inputs, because the FP32 forward's own rounding (about 1e-8 s per spike time,
  summed over thousands of spikes) is of the order of the change a 1e-4 perturbation makes.
  The check is made away from threshold-grazing events: of 8 candidate samples, those whose FP32
  forward differs from the float64 oracle in any spike count of any layer, or whose exact gradient
  moves by more than 1e-4 of its maximum when every threshold moves by 1e-6 relative (a
  near-tangential crossing, where the FP32 forward's rounding of the neuron state is amplified into
  the gradient: the reference's FP32 kernels, which give bit-identical spike times, share it), are set
  aside and the first 2 others are used; perturbations that change any spike count are skipped.
  Tolerance: |g_autograd - g_fd| <= 1e-2 |g_fd| + 1e-3 max|g_fd| + 30 s, s the entry's movement under
  that threshold change (oracle/fd.py gradient_sensitivity); the 1e-2 relative term covers the central
  difference's own truncation error at eps 1e-4.
* The same gradients as the reference's CUDA kernels (oracle/refkern.py), batch 256, in the reference's
  MNIST regime (hidden threshold 0.2, weights U(-1, 1)), layer by layer: each lif_fc layer gets the
  reference's own input spikes and incoming errors (the loss errors for the output layer, the reference's
  pre-spike errors of the layer above otherwise), and torch.autograd.grad's weight gradient and input-time
  gradient must match the reference's batch-summed gradient and pre-spike errors within
  1e-5 |ref| + 1e-5 sum|terms| (sum|terms|: the reference kernels on |errors|, |f1|, -|f2|, |W|, -tau).
* The whole network differentiated in one torch.autograd.grad call, batch 256: the forward is bit-identical
  to the reference's, and every layer's gradient within 1e-4 of the layer's largest entry of the
  reference's chained backward (the incoming errors of the lower layers differ from the reference's by the
  upper layers' rounding, which the chained sums carry along).
"""
import numpy as np
import pytest
import torch

from bats_gb300.autograd import lif_fc
from oracle import fd as FD
from oracle import refkern
from tests._helpers import assert_sum_close, mnist_like_input, ref_layer_backward

pytestmark = pytest.mark.gpu

SIZES = [784, 800, 800, 10]
TAU_S, K = 0.13, 30
THETAS = [0.2, 0.2, 1.3]
MAX_SIM = 0.2
FD_THETAS = [1.0, 1.0, 1.3]


def make_case(batch=256, seed=0):
    t, n = mnist_like_input(batch, seed=seed)
    rng = np.random.default_rng(seed + 1)
    ws = [rng.uniform(-1, 1, (o, i)).astype(np.float32) for i, o in zip(SIZES[:-1], SIZES[1:])]
    return t, n, ws


def forward(t_in, ws, thetas=THETAS):
    x = t_in
    counts = []
    for w, th in zip(ws, thetas):
        x, n = lif_fc(x, w, TAU_S, th, th, K, MAX_SIM)
        counts.append(n)
    return x, counts


def smooth_loss_weights(shape, seed=3):
    return np.random.default_rng(seed).normal(size=shape).astype(np.float32)


def test_finite_differences_on_64_weights_per_layer(cuda):
    t_all, _ = mnist_like_input(8, seed=0)
    rng = np.random.default_rng(1)
    ws_np = [((rng.normal(0, 1, (o, i)) + 3.5) / np.sqrt(i)).astype(np.float32) for i, o in zip(SIZES[:-1], SIZES[1:])]
    params = [(TAU_S, th, th, K, MAX_SIM) for th in FD_THETAS]
    r_all = smooth_loss_weights((8, SIZES[-1], K))
    with torch.no_grad():
        _, counts = forward(torch.tensor(t_all, device="cuda"), [torch.tensor(w, device="cuda") for w in ws_np],
                            FD_THETAS)
    oracle_outs = FD.network_forward(t_all.astype(np.float64), ws_np, params)
    agree = np.ones(len(t_all), dtype=bool)
    for c, o in zip(counts, oracle_outs):
        agree &= (c.cpu().numpy() == o[0]).all(axis=1)
    sens_rel = FD.per_sample_sensitivity(t_all, ws_np, params, r_all)
    usable = agree & (sens_rel.max(axis=1) <= 1e-4)
    sel = np.nonzero(usable)[0][:2]
    assert len(sel) == 2, (agree, sens_rel)
    t = np.ascontiguousarray(t_all[sel])
    r = np.ascontiguousarray(r_all[sel])
    t_in = torch.tensor(t, device="cuda")
    ws = [torch.tensor(w, device="cuda", requires_grad=True) for w in ws_np]
    out, counts = forward(t_in, ws, FD_THETAS)
    rd = torch.tensor(r, device="cuda")
    fin = torch.isfinite(out)
    assert int(fin.sum()) > 10, "the output layer should spike"
    grads = [g.cpu().numpy() for g in torch.autograd.grad(out, ws, grad_outputs=torch.where(fin, rd, torch.zeros_like(rd)))]
    rng = np.random.default_rng(11)
    picks = []
    for li, g in enumerate(grads):
        # Random weights among those whose pre-synaptic neuron spikes before some post spike.
        nz = np.argwhere(np.abs(g) > 0)
        assert len(nz) > 64
        picks += [(li, i, j) for i, j in nz[rng.choice(len(nz), 64, replace=False)]]
    fd, smooth = FD.central_differences(t, ws_np, params, r, picks, eps=1e-4)
    sens = FD.gradient_sensitivity(t, ws_np, params, r)
    layer = np.array([p[0] for p in picks])
    ad = np.array([grads[l][i, j] for l, i, j in picks], dtype=np.float64)
    s = np.array([sens[l][i, j] for l, i, j in picks])
    for li in range(3):
        m = (layer == li) & smooth
        assert m.sum() >= 48, f"layer {li}: too many grazing perturbations ({64 - m.sum()})"
        tol = 1e-2 * np.abs(fd[m]) + 1e-3 * np.abs(fd[m]).max() + 30 * s[m]
        bad = np.abs(ad[m] - fd[m]) > tol
        assert not bad.any(), (li, np.c_[ad[m][bad], fd[m][bad]][:5])


def test_autograd_layers_match_reference_kernels_batch_256(cuda):
    if not refkern.available():
        pytest.skip("reference kernels not built")
    t, n, ws_np = make_case(batch=256, seed=5)
    layers = [refkern.RefLIF(torch.tensor(w, device="cuda"), TAU_S, th, th, K) for w, th in zip(ws_np, THETAS)]
    x, c = torch.tensor(t, device="cuda"), torch.tensor(n, device="cuda")
    inputs = []
    for L in layers:
        inputs.append(x)
        o = L.forward(x, c, np.float32(MAX_SIM))
        x, c = o[3], o[0]
    r = torch.tensor(smooth_loss_weights(x.shape, seed=7), device="cuda")
    e_in = torch.where(torch.isfinite(x), r, torch.zeros_like(r)).contiguous()
    report = []
    for li in (2, 1, 0):
        x_in = inputs[li].clone().requires_grad_(li > 0)
        w = torch.tensor(ws_np[li], device="cuda", requires_grad=True)
        out, cnt = lif_fc(x_in, w, TAU_S, THETAS[li], THETAS[li], K, MAX_SIM)
        assert torch.equal(cnt, layers[li].out[0]), f"layer {li + 1}: spike counts differ from the reference"
        wanted = [w, x_in] if li > 0 else [w]
        grads = torch.autograd.grad(out, wanted, grad_outputs=e_in)
        g_ref, g_abs, pe_ref, pe_abs = ref_layer_backward(layers[li], e_in.clone(), want_pre=li > 0)
        st = assert_sum_close(grads[0].double().cpu().numpy(), g_ref, g_abs, what=f"layer {li + 1} weight gradient")
        report.append(f"L{li + 1} W: {st[1]}/{st[0]} need sum|terms|, worst {st[2]:.3f}")
        if li > 0:
            st = assert_sum_close(grads[1].double().cpu().numpy(), pe_ref.double().cpu().numpy(),
                                  pe_abs.double().cpu().numpy(), what=f"layer {li + 1} input-time gradient")
            report.append(f"L{li + 1} input times: {st[1]}/{st[0]} need sum|terms|, worst {st[2]:.3f}")
            e_in = pe_ref.contiguous()
        torch.cuda.empty_cache()
    print("\n[autograd vs reference kernels, batch 256] " + "; ".join(report))


def test_autograd_network_matches_reference_chain_batch_256(cuda):
    if not refkern.available():
        pytest.skip("reference kernels not built")
    t, n, ws_np = make_case(batch=256, seed=5)
    t_in = torch.tensor(t, device="cuda")
    ws = [torch.tensor(w, device="cuda", requires_grad=True) for w in ws_np]
    out, counts = forward(t_in, ws)
    r = torch.tensor(smooth_loss_weights(out.shape, seed=7), device="cuda")
    fin = torch.isfinite(out)
    err = torch.where(fin, r, torch.zeros_like(r))
    grads = torch.autograd.grad(out, ws, grad_outputs=err)
    # Reference kernels: forward, then the layer backward chain with the same output errors.
    layers = [refkern.RefLIF(torch.tensor(w, device="cuda"), TAU_S, th, th, K) for w, th in zip(ws_np, THETAS)]
    x, c = t_in, torch.tensor(n, device="cuda")
    for L in layers:
        o = L.forward(x, c, np.float32(MAX_SIM))
        x, c = o[3], o[0]
    for ours, L in zip(counts, layers):
        assert torch.equal(ours, L.out[0])
    e = err.clone().contiguous()
    ref_grads = [None] * 3
    for li in (2, 1, 0):
        g, e = layers[li].backward(e, want_pre=li > 0)
        ref_grads[li] = g.sum(0)
    for li in range(3):
        a, b = grads[li].cpu().numpy().astype(np.float64), ref_grads[li].cpu().numpy().astype(np.float64)
        scale = np.abs(b).max()
        assert scale > 0
        assert np.max(np.abs(a - b)) <= 1e-4 * scale, (li, np.max(np.abs(a - b)) / scale)
