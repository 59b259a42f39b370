"""GPU parity of the exact backward (reset errors, factors, weight gradient, pre-spike errors).

Kernel-level checks use the golden fixtures built from the reference tests' own CPU loops
(tests/golden/*.npz); layer-level checks run the reference's CUDA kernels (oracle/refkern.py) on the
same forward state. Gradients are sums of many signed terms; the tolerance is stated relative to the
sum of the terms' magnitudes (the float64 oracle evaluated with |err|, |f1|, -|f2| for the gradient
and |W|, |err|, |f1|, |f2|, -tau for the pre errors, so that every term is added):
    |g - g_ref| <= 1e-5 * |g_ref| + 1e-5 * G_abs.
Spike-time-level quantities (factors, recurrent errors) use 1e-5 relative.
"""
import os

import numpy as np
import pytest
import torch

from bats_gb300 import kernels as K
from oracle import bats_ref64 as R
from oracle import refkern
from tests._helpers import mnist_like_input, multi_spike_input

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def cu(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), device="cuda", dtype=dtype)


def assert_sum_close(got, ref, abs_scale, rtol=1e-5, what=""):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    tol = rtol * np.abs(ref) + rtol * np.asarray(abs_scale, dtype=np.float64) + 1e-30
    err = np.abs(got - ref)
    worst = np.max(err / tol) if err.size else 0.0
    assert worst <= 1.0, f"{what}: worst error / tolerance = {worst:.3f}"


def leading_only(post_t, f1, f2, err):
    """Zero the factors after a neuron's first inf post time (the kernels stop there)."""
    inf = np.isinf(post_t)
    after = np.cumsum(inf, axis=-1) > 0
    return np.where(after, 0, f1), np.where(after, 0, f2), np.where(after, 0, err)


def test_weights_gradient_and_pre_errors_vs_reference_test_loops(cuda):
    d = load("fc_backward_kernels")
    g = K.compute_weights_gradient(cu(d["f1"]), cu(d["f2"]), cu(d["post_t"]), cu(d["pre_t"]), cu(d["es"]),
                                   cu(d["ee"]), cu(d["errors"])).cpu().numpy()
    pre = (d["pre_t"].astype(np.float64), d["es"].astype(np.float64), d["ee"].astype(np.float64))
    f1, f2, e = leading_only(d["post_t"], d["f1"], d["f2"], d["errors"])
    exp = R.compute_weights_gradient(f1, f2, d["post_t"], pre, e)
    gabs = R.compute_weights_gradient(np.abs(f1), -np.abs(f2), d["post_t"], pre, np.abs(e))
    assert_sum_close(g, exp, gabs, what="weights gradient")
    full = ~np.isinf(d["post_t"]).any(-1)
    assert_sum_close(g[full], d["grad"][full], gabs[full], what="weights gradient vs reference test loop")
    pe = K.propagate_errors_to_pre_spikes(cu(d["f1"]), cu(d["f2"]), cu(d["post_t"]), cu(d["pre_t"]), cu(d["es"]),
                                          cu(d["ee"]), cu(d["weights"]), cu(d["errors"]), float(d["tau_s"]),
                                          float(d["tau"])).cpu().numpy()
    pabs = R.propagate_errors_to_pre_spikes(np.abs(f1), np.abs(f2), d["post_t"], pre, np.abs(d["weights"]),
                                            np.abs(e), float(d["tau_s"]), -float(d["tau"]))
    assert_sum_close(pe, d["pre_errors"], pabs, what="pre errors vs reference test loop")


def test_conv_backward_kernels_vs_reference_test_loops(cuda):
    d = load("conv_backward_kernels")
    g = K.compute_weights_gradient_conv(cu(d["f1"]), cu(d["f2"]), cu(d["post_t"]), cu(d["pre_t"]), cu(d["es"]),
                                        cu(d["ee"]), d["pre_shape"], d["post_shape"], d["filter_shape"],
                                        cu(d["errors"])).cpu().numpy()
    pre = (d["pre_t"].astype(np.float64), d["es"].astype(np.float64), d["ee"].astype(np.float64))
    gabs = R.conv_weights_gradient(np.abs(d["f1"]), -np.abs(d["f2"]), d["post_t"], pre, np.abs(d["errors"]),
                                   tuple(d["filter_shape"]), tuple(d["pre_shape"]))
    assert_sum_close(g, d["grad"], gabs, what="conv gradient")
    pe = K.propagate_errors_to_pre_spikes_conv(cu(d["f1"]), cu(d["f2"]), cu(d["post_t"]), cu(d["pre_t"]), cu(d["es"]),
                                               cu(d["ee"]), cu(d["filters"]), cu(d["errors"]), float(d["tau_s"]),
                                               float(d["tau"]), d["pre_shape"]).cpu().numpy()
    pabs = R.conv_pre_errors(np.abs(d["f1"]), np.abs(d["f2"]), d["post_t"], pre, np.abs(d["filters"]),
                             np.abs(d["errors"]), float(d["tau_s"]), -float(d["tau"]), tuple(d["pre_shape"]))
    assert_sum_close(pe, d["pre_errors"], pabs, what="conv pre errors")


def test_factors_and_recurrent_known_answers(cuda):
    d = load("factors")
    f1, f2 = K.compute_factors(cu(d["spike_times"]), cu(d["a"]), float(d["c"]), cu(d["x"]), cu(d["exp_tau"]),
                               float(d["tau"]))
    np.testing.assert_allclose(f1.cpu().numpy(), d["f1"], rtol=1e-5)
    np.testing.assert_allclose(f2.cpu().numpy(), d["f2"], rtol=1e-5)
    r = load("kat_recurrent")
    e = cu(r["errors"])
    K.propagate_recurrent_errors(cu(r["x"]), cu(r["exp_tau"]), e, float(r["delta_theta_tau"]))
    np.testing.assert_allclose(e.cpu().numpy(), r["expected"], rtol=1e-5, atol=1e-6)


def _layer_case(variant, B=16):
    t, n_in = mnist_like_input(B, seed=1)
    rng = np.random.default_rng(2)
    if variant == "active":
        W1 = rng.uniform(-1, 1, (120, 784)).astype(np.float32)
        W2 = rng.uniform(-1, 1, (10, 120)).astype(np.float32)
        th1, th2 = 0.2, 1.3
    else:
        W1 = rng.normal(0, 1 / np.sqrt(784), (120, 784)).astype(np.float32)
        W2 = rng.normal(0, 1 / np.sqrt(120), (10, 120)).astype(np.float32)
        th1, th2 = 1.0, 1.3
    return t, n_in, W1, W2, th1, th2


@pytest.mark.parametrize("variant", ["active", "literal"])
def test_two_layer_backward_vs_reference_kernels(cuda, variant):
    if not refkern.available():
        pytest.skip("reference kernels not built")
    t, n_in, W1, W2, th1, th2 = _layer_case(variant)
    tau_s, K_post = np.float32(0.13), 30
    tau = np.float32(2 * tau_s)
    # Ours.
    tt = cu(t)
    ev1 = K.sort_events(tt, tau_s, tau)
    wt1 = K.transpose_weights(cu(W1))
    n1, a1, x1, t1, z1 = K.lif_forward_fc(ev1, wt1, 120, K_post, tau_s, th1, th1, 0.2)
    ev2 = K.sort_events(t1, tau_s, tau)
    wt2 = K.transpose_weights(cu(W2))
    n2, a2, x2, t2, z2 = K.lif_forward_fc(ev2, wt2, 10, K_post, tau_s, th2, th2, 0.2)
    labels = np.arange(t.shape[0]) % 10
    _, err2 = K.spike_count_loss(n2, labels=cu(labels, torch.int32), target_true=15, target_false=3, k=K_post)
    err2_ref = err2.clone()
    tau32, c2, dtt2 = K.lif_constants(tau_s, th2, th2)
    tab2 = K.backward_prep(t2, a2, x2, z2, err2, c2, tau32, dtt2, want_factors=True)
    g2 = K.weights_gradient(ev2, t2, tab2, 120, per_sample=True)
    pe2 = K.pre_errors(ev2, wt2, t2, tab2, tau_s, tau32)
    _, c1, dtt1 = K.lif_constants(tau_s, th1, th1)
    e1 = pe2.clone()
    tab1 = K.backward_prep(t1, a1, x1, z1, e1, c1, tau32, dtt1, want_factors=True)
    g1 = K.weights_gradient(ev1, t1, tab1, 784, per_sample=True)
    g1_mean = K.weights_gradient(ev1, t1, tab1, 784, per_sample=False, group=4)
    # Reference kernels on the same inputs.
    L1 = refkern.RefLIF(cu(W1), tau_s, th1, th1, K_post)
    L2 = refkern.RefLIF(cu(W2), tau_s, th2, th2, K_post)
    r1 = L1.forward(tt, cu(n_in, torch.int32), np.float32(0.2))
    r2 = L2.forward(r1[3], r1[0], np.float32(0.2))
    for ours, ref in ((n1, r1[0]), (n2, r2[0])):
        assert torch.equal(ours, ref), "forward spike counts differ from the reference kernels"
    rg2, rpe2 = L2.backward(err2_ref, want_pre=True)
    rg1, _ = L1.backward(rpe2.clone(), want_pre=False)
    torch.cuda.synchronize()
    # Scales from the float64 oracle with absolute values.
    f1_2, f2_2 = tab2.f1.cpu().numpy(), tab2.f2.cpu().numpy()
    e2n = err2.cpu().numpy()
    pre1 = (t1.cpu().numpy().astype(np.float64),) + R.compute_pre_exps(t1.cpu().numpy(), float(tau_s), float(tau32))
    g2abs = R.compute_weights_gradient(np.abs(f1_2), -np.abs(f2_2), t2.cpu().numpy(), pre1, np.abs(e2n))
    assert_sum_close(g2.cpu().numpy(), rg2.cpu().numpy(), g2abs, what="layer 2 gradient")
    p2abs = R.propagate_errors_to_pre_spikes(np.abs(f1_2), np.abs(f2_2), t2.cpu().numpy(), pre1, np.abs(W2),
                                             np.abs(e2n), float(tau_s), -float(tau32))
    assert_sum_close(pe2.cpu().numpy(), rpe2.cpu().numpy(), p2abs, what="layer 2 pre errors")
    f1_1, f2_1 = tab1.f1.cpu().numpy(), tab1.f2.cpu().numpy()
    e1n = e1.cpu().numpy()
    pre0 = (t.astype(np.float64),) + R.compute_pre_exps(t, float(tau_s), float(tau32))
    g1abs = R.compute_weights_gradient(np.abs(f1_1), -np.abs(f2_1), t1.cpu().numpy(), pre0, np.abs(e1n))
    assert_sum_close(g1.cpu().numpy(), rg1.cpu().numpy(), g1abs, what="layer 1 gradient")
    # Batch mean path equals the mean of the per-sample gradients.
    assert_sum_close(g1_mean.cpu().numpy(), g1.mean(0).cpu().numpy(), g1abs.mean(0), rtol=1e-6, what="batch mean")
    if variant == "active":
        assert int(n1.sum()) > 0 and float(g1.abs().sum()) > 0


def test_backward_is_deterministic(cuda):
    t, n_in = multi_spike_input(8, 64, 4, 0.1, seed=5)
    rng = np.random.default_rng(5)
    W = rng.uniform(-1, 1, (96, 64)).astype(np.float32)
    outs = []
    for _ in range(2):
        ev = K.sort_events(cu(t), 0.1, 0.2)
        wt = K.transpose_weights(cu(W))
        n, a, x, ts, z = K.lif_forward_fc(ev, wt, 96, 20, 0.1, 0.1, 0.1)
        err = torch.ones_like(ts)
        tau32, c, dtt = K.lif_constants(0.1, 0.1, 0.1)
        tab = K.backward_prep(ts, a, x, z, err, c, tau32, dtt)
        g = K.weights_gradient(ev, ts, tab, 64, per_sample=False, group=3)
        pe = K.pre_errors(ev, wt, ts, tab, 0.1, tau32)
        outs.append((g.cpu(), pe.cpu()))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("n_post", [10, 20, 32])
def test_narrow_layer_kernels(cuda, n_post):
    """Narrow layers (N_post <= 32): the weight gradient over bucketed events is bit-identical to the
    one over the full event list (same order of every sum), per sample and batch-summed, and
    deterministic; the event-parallel pre errors are deterministic and agree with the float64 oracle on
    the same forward state."""
    import dataclasses
    t, n_in = multi_spike_input(16, 150, 4, 0.1, seed=7)
    rng = np.random.default_rng(7)
    W = (rng.uniform(-0.5, 1.0, (n_post, 150)) * 2).astype(np.float32)
    tau_s, th = 0.1, 0.5
    ev = K.sort_events(cu(t), tau_s, 2 * tau_s)
    wt = K.transpose_weights(cu(W))
    n, a, x, ts, z = K.lif_forward_fc(ev, wt, n_post, 8, tau_s, th, th)
    assert int(n.sum()) > 50
    err = cu(rng.normal(size=ts.shape).astype(np.float32))
    tau32, c, dtt = K.lif_constants(tau_s, th, th)
    tab = K.backward_prep(ts, a, x, z, err, c, tau32, dtt, want_factors=True)
    plain = dataclasses.replace(ev, bucketed=None, bucket_offsets=None)
    for per_sample, group in ((True, None), (False, 4), (False, 16)):
        g_b = K.weights_gradient(ev, ts, tab, 150, per_sample=per_sample, group=group)
        g_again = K.weights_gradient(ev, ts, tab, 150, per_sample=per_sample, group=group)
        g_full = K.weights_gradient(plain, ts, tab, 150, per_sample=per_sample, group=group)
        assert torch.equal(g_b, g_again), "gradient not deterministic"
        assert torch.equal(g_b, g_full), f"bucketed vs full event list (per_sample={per_sample}, group={group})"
    pe = K.pre_errors(ev, wt, ts, tab, tau_s, tau32)
    pe2 = K.pre_errors(ev, wt, ts, tab, tau_s, tau32)
    assert torch.equal(pe, pe2)
    f1, f2 = tab.f1.cpu().numpy(), tab.f2.cpu().numpy()
    e = err.cpu().numpy()
    post = ts.cpu().numpy()
    pre = (t.astype(np.float64),) + R.compute_pre_exps(t, float(np.float32(tau_s)), float(tau32))
    ref = R.propagate_errors_to_pre_spikes(f1, f2, post, pre, W, e, float(np.float32(tau_s)), float(tau32))
    scale = R.propagate_errors_to_pre_spikes(np.abs(f1), np.abs(f2), post, pre, np.abs(W), np.abs(e),
                                             float(np.float32(tau_s)), -float(tau32))
    assert_sum_close(pe.cpu().numpy(), ref, scale, what="narrow pre errors vs oracle")


def test_layer_prep_matches_generic_prep_bit_for_bit(cuda):
    """bats_backward_prep_layer (warp-staged, valid slots only, interleaved suffix sums) against the
    one-thread-per-neuron bats_backward_prep on the same forward state: reset errors, factors, counts and
    every table entry before a neuron's count are identical."""
    t, n_in = multi_spike_input(16, 60, 5, 0.1, seed=11, p_silent=0.1)
    rng = np.random.default_rng(11)
    W = (rng.uniform(-0.3, 1.0, (70, 60)) * 1.5).astype(np.float32)
    tau_s, th = 0.1, 0.2
    ev = K.sort_events(cu(t), tau_s, 2 * tau_s)
    n, a, x, ts, z = K.lif_forward_fc(ev, K.transpose_weights(cu(W)), 70, 30, tau_s, th, th)
    assert int(n.max()) >= 8, "some neurons should spike many times"
    err = cu(rng.normal(size=ts.shape).astype(np.float32))
    tau32, c, dtt = K.lif_constants(tau_s, th, th)
    e1, e2 = err.clone(), err.clone()
    tl = K.backward_prep(ts, a, x, z, e1, c, tau32, dtt, want_factors=True)
    B, N, Kp = ts.shape
    tg = K.BackwardTables(torch.empty_like(ts), torch.empty_like(ts), torch.empty((B, N, Kp + 1, 2), device="cuda"),
                          torch.empty((B, N), dtype=torch.int32, device="cuda"))
    from bats_gb300._lib import call, ptr, stream_ptr
    call("bats_backward_prep", ptr(ts), ptr(a), ptr(x), ptr(z), ptr(e2), B, N, Kp, float(c), float(tau32), float(dtt),
         1, 1, ptr(tg.f1), ptr(tg.f2), ptr(tg.tables), ptr(tg.nvalid), stream_ptr())
    torch.cuda.synchronize()
    assert torch.equal(tl.nvalid, tg.nvalid)
    assert torch.equal(e1, e2)
    assert torch.equal(tl.f1, tg.f1) and torch.equal(tl.f2, tg.f2)
    nv = tl.nvalid.cpu().numpy()
    valid = np.arange(Kp + 1)[None, None, :] < nv[:, :, None]
    a_tab, b_tab = tl.tables.cpu().numpy(), tg.tables.cpu().numpy()
    assert np.array_equal(a_tab[valid].view(np.uint32), b_tab[valid].view(np.uint32))


@pytest.mark.parametrize("case", ["heavy", "irregular"])
def test_counted_prep_matches_layer_prep_bit_for_bit(cuda, case):
    """bats_backward_prep_counted (only the slots below the forward's spike counts, staged compactly in
    rounds of at most 256 per warp) against bats_backward_prep_layer on the same forward state: reset
    errors, counts and every table entry before a neuron's count are identical. "heavy": most neurons
    spike 10-30 times, so warps need several rounds; "irregular": counts past the finite slots, a +inf
    time below a count, negative counts of silent neurons."""
    rng = np.random.default_rng(12)
    if case == "heavy":
        t, n_in = multi_spike_input(8, 80, 8, 0.15, seed=12, p_silent=0.0)
        W = (rng.uniform(0.2, 1.0, (96, 80)) * 2.0).astype(np.float32)
    else:
        t, n_in = multi_spike_input(16, 60, 5, 0.1, seed=13, p_silent=0.1)
        W = (rng.uniform(-0.3, 1.0, (70, 60)) * 1.5).astype(np.float32)
    tau_s, th = 0.1, 0.2
    ev = K.sort_events(cu(t), tau_s, 2 * tau_s)
    n, a, x, ts, z = K.lif_forward_fc(ev, K.transpose_weights(cu(W)), W.shape[0], 30, tau_s, th, th)
    counts = n.clone()
    if case == "heavy":
        assert float(n.float().mean()) >= 10, "most neurons should spike many times"
    else:
        nn = n.cpu().numpy()
        s, i = np.argwhere(nn >= 3)[0]
        ts[s, i, 1] = float("inf")                  # a +inf time below the count
        s2, i2 = np.argwhere(nn <= 20)[1]
        counts[s2, i2] += 5                         # count past the finite slots
        silent = np.argwhere(nn == 0)
        if len(silent):
            counts[silent[0][0], silent[0][1]] = -3  # negative count of a silent neuron
    err = cu(rng.normal(size=ts.shape).astype(np.float32))
    tau32, c, dtt = K.lif_constants(tau_s, th, th)
    e1, e2 = err.clone(), err.clone()
    tl = K.backward_prep(ts, a, x, z, e1, c, tau32, dtt)
    tc = K.backward_prep(ts, a, x, z, e2, c, tau32, dtt, n_spikes=counts)
    torch.cuda.synchronize()
    assert torch.equal(tl.nvalid, tc.nvalid)
    assert torch.equal(e1, e2)
    nv = tl.nvalid.cpu().numpy()
    Kp = ts.shape[2]
    valid = np.arange(Kp + 1)[None, None, :] < nv[:, :, None]
    a_tab, b_tab = tl.tables.cpu().numpy(), tc.tables.cpu().numpy()
    assert np.array_equal(a_tab[valid].view(np.uint32), b_tab[valid].view(np.uint32))


@pytest.mark.parametrize("n_post", [60, 200])
def test_wide_bucketed_gradient_matches_full_event_list(cuda, n_post):
    """The batch-summed and per-sample weight gradient of wide layers over bucketed events (each warp
    walking its samples' bucket events 32 at a time, silent lanes adding zeros) is bit-identical to the one
    over the full event list: buckets with more events than one chunk (32), empty buckets, a silent sample,
    groups that do not divide the batch."""
    import dataclasses
    t, n_in = multi_spike_input(13, 150, 8, 0.1, seed=17, p_silent=0.3)
    t[4] = np.inf  # a silent sample
    rng = np.random.default_rng(17)
    W = (rng.uniform(-0.5, 1.0, (n_post, 150)) * 1.2).astype(np.float32)
    tau_s, th = 0.1, 0.5
    ev = K.sort_events(cu(t), tau_s, 2 * tau_s)
    offs = ev.bucket_offsets.cpu().numpy()
    assert (np.diff(offs, axis=1) > 64).any(), "some bucket should need several chunks"
    assert (np.diff(offs, axis=1) == 0).any(), "some bucket should be empty"
    wt = K.transpose_weights(cu(W))
    n, a, x, ts, z = K.lif_forward_fc(ev, wt, n_post, 12, tau_s, th, th)
    assert int(n.sum()) > 100
    err = cu(rng.normal(size=ts.shape).astype(np.float32))
    tau32, c, dtt = K.lif_constants(tau_s, th, th)
    tab = K.backward_prep(ts, a, x, z, err, c, tau32, dtt)
    plain = dataclasses.replace(ev, bucketed=None, bucket_offsets=None)
    for per_sample, group in ((True, None), (False, 2), (False, 5), (False, 13)):
        g_b = K.weights_gradient(ev, ts, tab, 150, per_sample=per_sample, group=group)
        g_full = K.weights_gradient(plain, ts, tab, 150, per_sample=per_sample, group=group)
        assert torch.equal(g_b, g_full), f"bucketed vs full event list (per_sample={per_sample}, group={group})"
