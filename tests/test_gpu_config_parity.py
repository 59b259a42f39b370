"""Backward parity at the 784-800-800-10 configuration's own size: batch 256, MNIST-shaped input (784
inputs, each firing once with probability 0.19 at U(0, 0.01) s), tau_s 0.13, max_n_spike 30, max_simulation
0.2, spike-count class loss (targets 15 / 3), in two regimes:
  * literal: weights N(0, 1/sqrt(fan_in)), thresholds 1.0 hidden / 1.3 output (the hidden layers stay silent);
  * active: the reference's MNIST training regime, weights U(-1, 1), hidden threshold 0.2.

Per layer, our kernels and the reference's compiled kernels (oracle/refkern.py) start from the same state:
the forward outputs (asserted bit-identical: equal counts, equal a, x, t, z in every valid slot) and the same
incoming errors (the loss errors for the output layer, the reference's own pre-spike errors of the layer
above for the hidden layers), so each layer's comparison measures that layer's kernels alone. The gradient is
the batch sum of bats_weights_gradient with the train step's own sample grouping; the pre-spike errors come
from bats_pre_errors. Tolerance, as in the other backward tests, 1e-5 relative to the reference value plus
1e-5 of the sum of the magnitudes of its terms (the reference kernels evaluated on |errors|, |f1|, -|f2| and
|W|, -tau): |ours - ref| <= 1e-5 |ref| + 1e-5 sum|terms|. Each test prints, per layer, how many entries
needed the sum|terms| part (their error exceeds 1e-5 |ref| alone, where the sum cancels).

A second test runs the product's train step (bats_gb300.train.FCTrainStep: counted sort, unpadded hidden
layers, counted prep, fused gradient + Adam) for one step and checks that its forward state and its
batch-mean gradients equal those of the kernel-level chain run on our own errors (bit for bit where the
arithmetic is the same, within 1e-6 relative otherwise).
"""
import numpy as np
import pytest
import torch

from bats_gb300 import kernels as K
from oracle import refkern
from tests._helpers import assert_sum_close, mnist_like_input, ref_layer_backward

pytestmark = pytest.mark.gpu

SIZES = [784, 800, 800, 10]
B = 256
TAU_S = np.float32(0.13)
KP = 30
MAX_SIM = np.float32(0.2)
TARGET_TRUE, TARGET_FALSE = 15.0, 3.0


def _case(variant, seed=0):
    t, n_in = mnist_like_input(B, seed=seed)
    rng = np.random.default_rng(seed + 100)
    ws = []
    for n_pre, n_post in zip(SIZES[:-1], SIZES[1:]):
        if variant == "literal":
            ws.append(rng.normal(0, 1 / np.sqrt(n_pre), (n_post, n_pre)).astype(np.float32))
        else:
            ws.append(rng.uniform(-1, 1, (n_post, n_pre)).astype(np.float32))
    hidden = 1.0 if variant == "literal" else 0.2
    thetas = [hidden, hidden, 1.3]
    labels = rng.integers(0, SIZES[-1], B).astype(np.int32)
    return t, n_in, ws, thetas, labels


def _count_errors(n_out, labels):
    tt = torch.full(n_out.shape, TARGET_FALSE, device="cuda")
    tt[torch.arange(n_out.shape[0], device="cuda"), torch.as_tensor(labels, device="cuda").long()] = TARGET_TRUE
    return (tt - n_out.float())[:, :, None].repeat(1, 1, KP).contiguous()


def _assert_same_forward(ours, ref, what):
    n, a, x, t, z = ours
    rn, ra, rx, rt, rz = ref
    assert torch.equal(n, rn), f"{what}: spike counts differ from the reference kernels"
    valid = torch.arange(KP, device="cuda")[None, None, :] < rn[:, :, None]
    for name, u, v in (("a", a, ra), ("x", x, rx), ("t", t, rt), ("z", z, rz)):
        assert torch.equal(u[valid], v[valid]), f"{what}: {name} differs from the reference kernels"


@pytest.mark.parametrize("variant", ["literal", "active"])
def test_layer_backward_vs_reference_kernels_784_800_800_10_batch_256(cuda, variant):
    if not refkern.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    t, n_in, ws, thetas, labels = _case(variant)
    tau32 = np.float32(2 * TAU_S)
    # Forward chain, ours and the reference's, bit-identical layer by layer.
    x_ours, x_ref, c_ref = torch.tensor(t, device="cuda"), torch.tensor(t, device="cuda"), torch.tensor(n_in,
                                                                                                      device="cuda")
    ours, refs, evs, wts = [], [], [], []
    for li, (w, th) in enumerate(zip(ws, thetas)):
        ev = K.sort_events(x_ours, TAU_S, tau32)
        wt = K.transpose_weights(torch.tensor(w, device="cuda"))
        o = K.lif_forward_fc(ev, wt, w.shape[0], KP, TAU_S, th, th, MAX_SIM)
        L = refkern.RefLIF(torch.tensor(w, device="cuda"), TAU_S, th, th, KP)
        r = L.forward(x_ref, c_ref, MAX_SIM)
        _assert_same_forward(o, r, f"{variant} layer {li + 1}")
        ours.append(o)
        refs.append(L)
        evs.append(ev)
        wts.append(wt)
        x_ours, x_ref, c_ref = o[3], r[3], r[0]
    spikes = [int(o[0].sum()) for o in ours]
    if variant == "active":
        assert min(spikes) > 1000, spikes
    # Backward, layer by layer from the same incoming errors.
    err_in = _count_errors(refs[-1].out[0], labels)
    report = []
    for li in (2, 1, 0):
        n, a, x, ts, z = ours[li]
        th = thetas[li]
        _, c, dtt = K.lif_constants(TAU_S, th, th)
        mine = err_in.clone()
        tabs = K.backward_prep(ts, a, x, z, mine, c, tau32, dtt)
        group = max(2, K.default_group(B, SIZES[li + 1], SIZES[li]))
        g = K.weights_gradient(evs[li], ts, tabs, SIZES[li], per_sample=False, group=group,
                               reduce="sum").double().cpu().numpy()
        pe = K.pre_errors(evs[li], wts[li], ts, tabs, TAU_S, tau32) if li > 0 else None
        g_ref, g_abs, pe_ref, pe_abs = ref_layer_backward(refs[li], err_in.clone(), want_pre=li > 0)
        st = assert_sum_close(g, g_ref, g_abs, what=f"{variant} layer {li + 1} gradient")
        report.append(f"L{li + 1} gradient: {st[0]} entries, {st[1]} need the sum|terms| part, "
                      f"worst err/tol {st[2]:.3f}")
        if li > 0:
            st = assert_sum_close(pe.double().cpu().numpy(), pe_ref.double().cpu().numpy(),
                                  pe_abs.double().cpu().numpy(), what=f"{variant} layer {li + 1} pre errors")
            report.append(f"L{li + 1} pre errors: {st[0]} entries, {st[1]} need the sum|terms| part, "
                          f"worst err/tol {st[2]:.3f}")
            err_in = pe_ref.contiguous()
            del pe_abs
        torch.cuda.empty_cache()
    print(f"\n[{variant} 784-800-800-10 batch 256, spikes per layer {spikes}] " + "; ".join(report))


@pytest.mark.parametrize("variant", ["literal", "active"])
def test_train_step_equals_kernel_chain_784_800_800_10_batch_256(cuda, variant):
    from bats_gb300.train import FCLayerSpec, FCTrainStep
    t, n_in, ws, thetas, labels = _case(variant, seed=3)
    specs = [FCLayerSpec(n, float(TAU_S), th, th, KP) for n, th in zip(SIZES[1:], thetas)]
    ts = FCTrainStep(B, SIZES[0], 1, specs, [torch.tensor(w) for w in ws], TARGET_TRUE, TARGET_FALSE,
                     learning_rate=3e-3, max_simulation=float(MAX_SIM))
    ts.set_inputs(torch.tensor(t), torch.tensor(labels))
    ts.step()
    torch.cuda.synchronize()
    tau32 = np.float32(2 * TAU_S)
    x = torch.tensor(t, device="cuda")
    chain, evs, wts = [], [], []
    for li, (w, th) in enumerate(zip(ws, thetas)):
        ev = K.sort_events(x, TAU_S, tau32)
        wt = K.transpose_weights(torch.tensor(w, device="cuda"))
        o = K.lif_forward_fc(ev, wt, w.shape[0], KP, TAU_S, th, th, MAX_SIM)
        n_ts = ts.out[li][0]
        assert torch.equal(n_ts, o[0]), f"layer {li + 1}: train-step spike counts differ"
        valid = torch.arange(KP, device="cuda")[None, None, :] < o[0][:, :, None]
        for u, v in zip(ts.out[li][1:], o[1:]):
            assert torch.equal(u[valid], v[valid]), f"layer {li + 1}: train-step forward state differs"
        chain.append(o)
        evs.append(ev)
        wts.append(wt)
        x = o[3]
    err = _count_errors(chain[-1][0], labels)
    pre = {}
    for li in (2, 1, 0):
        n, a, xx, tt, z = chain[li]
        _, c, dtt = K.lif_constants(TAU_S, thetas[li], thetas[li])
        tabs = K.backward_prep(tt, a, xx, z, err, c, tau32, dtt)
        g = K.weights_gradient(evs[li], tt, tabs, SIZES[li], per_sample=False, group=ts.groups[li],
                               reduce="mean").double().cpu().numpy()
        got = ts.grad[li].double().cpu().numpy()
        scale = np.abs(g).max() if g.size else 0.0
        assert np.all(np.abs(got - g) <= 1e-6 * np.abs(g) + 1e-12 * max(scale, 1e-30)), \
            f"layer {li + 1}: train-step gradient differs from the kernel chain"
        if li > 0:
            err = K.pre_errors(evs[li], wts[li], tt, tabs, TAU_S, tau32)
            pre[li] = err
    # The pre-spike errors of layer l are the next layer down's incoming errors, which its reset-error step
    # changes in place (in the train step as in the chain): compared after the whole backward.
    for li, err in pre.items():
        cnt = chain[li - 1][0]
        valid = torch.arange(KP, device="cuda")[None, None, :] < cnt[:, :, None]
        assert torch.equal(ts.pre_err[li][valid], err[valid]), f"layer {li + 1}: train-step pre errors differ"


def test_uneven_batch_slice_vs_reference_kernels(cuda):
    """The uneven-batch configuration (1024-1024-20, max_n_spike 30, weights U(-1, 1), thresholds 0.2 / 1.3,
    inputs over 1024 channels with lognormal event counts, median 200, 20-4000 per sample, times U(0, 0.1) s) on
    a slice of 47 samples at evenly spaced length ranks, the longest included: forward bit-identical to
    the reference kernels with both the per-(tile, sample) and the persistent work-queue forward, and each
    layer's batch-summed gradient and pre-spike errors within 1e-5 |ref| + 1e-5 sum|terms|."""
    if not refkern.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    from tests._helpers import uneven_input
    t_all, n_all, ev_counts = uneven_input(512)
    order = np.argsort(ev_counts, kind="stable")
    pick = np.unique(np.r_[order[np.linspace(0, len(order) - 1, 47).astype(int)], order[-1]])
    t, n_in = np.ascontiguousarray(t_all[pick]), np.ascontiguousarray(n_all[pick])
    assert ev_counts[pick].max() == ev_counts.max() and ev_counts[pick].min() <= 25
    rng = np.random.default_rng(12)
    ws = [rng.uniform(-1, 1, (o, i)).astype(np.float32) for i, o in ((1024, 1024), (1024, 20))]
    thetas = [0.2, 1.3]
    tau32 = np.float32(2 * TAU_S)
    x_ours, x_ref, c_ref = (torch.tensor(t, device="cuda"), torch.tensor(t, device="cuda"),
                            torch.tensor(n_in, device="cuda"))
    ours, refs, evs, wts = [], [], [], []
    for li, (w, th) in enumerate(zip(ws, thetas)):
        ev = K.sort_events(x_ours, TAU_S, tau32)
        wt = K.transpose_weights(torch.tensor(w, device="cuda"))
        o = K.lif_forward_fc(ev, wt, w.shape[0], KP, TAU_S, th, th, MAX_SIM)
        oq = K.lif_forward_fc(ev, wt, w.shape[0], KP, TAU_S, th, th, MAX_SIM, algo=K.FWD_QUEUE)
        L = refkern.RefLIF(torch.tensor(w, device="cuda"), TAU_S, th, th, KP)
        r = L.forward(x_ref, c_ref, MAX_SIM)
        _assert_same_forward(o, r, f"uneven layer {li + 1}")
        _assert_same_forward(oq, r, f"uneven layer {li + 1} (work queue)")
        ours.append(o)
        refs.append(L)
        evs.append(ev)
        wts.append(wt)
        x_ours, x_ref, c_ref = o[3], r[3], r[0]
    spikes = [int(o[0].sum()) for o in ours]
    assert min(spikes) > 100, spikes
    labels = rng.integers(0, 20, len(pick))
    err_in = (torch.where(torch.arange(20, device="cuda")[None, :] == torch.as_tensor(labels, device="cuda")[:, None],
                          15.0, 3.0) - refs[-1].out[0].float())[:, :, None].repeat(1, 1, KP).contiguous()
    report = []
    for li in (1, 0):
        n, a, x, ts, z = ours[li]
        _, c, dtt = K.lif_constants(TAU_S, thetas[li], thetas[li])
        tabs = K.backward_prep(ts, a, x, z, err_in.clone(), c, tau32, dtt)
        n_pre = ws[li].shape[1]
        g = K.weights_gradient(evs[li], ts, tabs, n_pre, per_sample=False,
                               group=max(2, K.default_group(len(pick), ws[li].shape[0], n_pre)),
                               reduce="sum").double().cpu().numpy()
        g_ref, g_abs, pe_ref, pe_abs = ref_layer_backward(refs[li], err_in.clone(), want_pre=li > 0)
        st = assert_sum_close(g, g_ref, g_abs, what=f"uneven layer {li + 1} gradient")
        report.append(f"L{li + 1} gradient: {st[1]}/{st[0]} need sum|terms|, worst {st[2]:.3f}")
        if li > 0:
            pe = K.pre_errors(evs[li], wts[li], ts, tabs, TAU_S, tau32)
            st = assert_sum_close(pe.double().cpu().numpy(), pe_ref.double().cpu().numpy(),
                                  pe_abs.double().cpu().numpy(), what=f"uneven layer {li + 1} pre errors")
            report.append(f"L{li + 1} pre errors: {st[1]}/{st[0]}, worst {st[2]:.3f}")
            err_in = pe_ref.contiguous()
    print(f"\n[uneven 1024-1024-20 slice of {len(pick)}, events {int(ev_counts[pick].min())}-"
          f"{int(ev_counts[pick].max())}, spikes per layer {spikes}] " + "; ".join(report))
