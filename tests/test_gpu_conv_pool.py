"""GPU parity of the convolutional LIF layer and the 2x2 spike-union pooling against the reference's
CUDA kernels, the reference test loops (golden fixtures) and the float64 oracle."""
import os

import numpy as np
import pytest
import torch

from bats_gb300 import kernels as K
from oracle import bats_ref64 as R
from oracle import refkern
from tests._helpers import conditioned_reference, count_mismatches, leading_mask, mnist_like_input, multi_spike_input

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def cu(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), device="cuda", dtype=dtype)


def conv_case(seed=0, B=6):
    t, n = mnist_like_input(B, seed=seed)
    rng = np.random.default_rng(seed + 10)
    filt = rng.uniform(-1, 1, (15, 5, 5, 1)).astype(np.float32)
    return t, n, filt


def run_conv(t, filt, pre_shape, K_post, tau_s, theta, max_sim):
    ev = K.sort_events(cu(t), np.float32(tau_s), np.float32(2 * tau_s))
    out = K.conv_forward(ev, cu(filt), pre_shape, K_post, tau_s, theta, theta, max_sim)
    torch.cuda.synchronize()
    return [v.cpu().numpy() for v in out], ev


def test_conv_forward_vs_reference_kernels_and_oracle(cuda):
    t, n_in, filt = conv_case()
    pre_shape = (28, 28, 1)
    ours, _ = run_conv(t, filt, pre_shape, 10, 0.13, 0.04, 0.2)
    assert ours[0].sum() > 100
    if refkern.available():
        L = refkern.RefConvLIF(cu(filt), pre_shape, np.float32(0.13), 0.04, 0.04, 10)
        ref = [v.cpu().numpy() for v in L.forward(cu(t), cu(n_in, torch.int32), np.float32(0.2))]
        diff, _ = count_mismatches(ours[0], ref[0])
        assert diff == 0
        same = leading_mask(ref[0], 10)
        for u, v in zip(ours[1:], ref[1:]):
            np.testing.assert_allclose(u[same], v[same], rtol=1e-6)
    o64, bounds, sens = conditioned_reference(t[:2], filt, np.float32(0.13), 0.04, 0.04, 10, np.float32(0.2),
                                              conv=pre_shape)
    d, unexplained = count_mismatches(ours[0][:2], o64[0], bounds)
    assert unexplained == 0
    same = (ours[0][:2] == o64[0])[:, :, None] & leading_mask(o64[0], 10)
    e = np.abs(ours[3][:2][same] - o64[3][same])
    assert np.all(e <= 1e-5 * np.abs(o64[3][same]) + 1e-5 * 0.26 + 20 * sens[same])


def test_pool_forward_and_backward(cuda):
    d = np.load(os.path.join(GOLDEN, "pooling.npz"))
    n, t, i = K.aggregate_spikes_conv(cu(d["n_spikes"], torch.int32), cu(d["spike_times"]), d["pre_shape"])
    n, t, i = n.cpu().numpy(), t.cpu().numpy(), i.cpu().numpy()
    np.testing.assert_array_equal(n, d["out_n"])
    np.testing.assert_array_equal(t, d["out_t"])
    fin = np.isfinite(d["out_t"])
    np.testing.assert_array_equal(i[fin], d["out_idx"][fin])
    assert np.array_equal(np.sort(i.reshape(-1)), np.arange(i.size))
    # Backward: errors land on their source slots.
    rng = np.random.default_rng(0)
    err = rng.normal(size=t.shape).astype(np.float32)
    err[~np.isfinite(t)] = 0
    B, N_pre, Kp = d["spike_times"].shape
    pe = K.pool_backward(cu(err), cu(i, torch.int32), (B, N_pre, Kp)).cpu().numpy()
    np.testing.assert_array_equal(pe, R.pool_backward(err, i, B * N_pre * Kp).reshape(B, N_pre, Kp))


def test_conv_pool_conv_stack_vs_reference_kernels(cuda):
    if not refkern.available():
        pytest.skip("reference kernels not built")
    t, n_in, filt1 = conv_case(seed=3, B=4)
    rng = np.random.default_rng(4)
    filt2 = rng.uniform(-1, 1, (8, 5, 5, 15)).astype(np.float32)
    tau_s = np.float32(0.13)
    ours1, ev1 = run_conv(t, filt1, (28, 28, 1), 4, 0.13, 0.04, 0.2)
    L1 = refkern.RefConvLIF(cu(filt1), (28, 28, 1), tau_s, 0.04, 0.04, 4)
    r1 = L1.forward(cu(t), cu(n_in, torch.int32), np.float32(0.2))
    assert np.array_equal(ours1[0], r1[0].cpu().numpy())
    pn, pt, pidx = K.aggregate_spikes_conv(cu(ours1[0], torch.int32), cu(ours1[3]), (24, 24, 15))
    rn, rt, ridx = refkern.pool_forward(r1[0], r1[3], (24, 24, 15))
    assert torch.equal(pn, rn) and torch.equal(pt, rt)
    ours2, ev2 = run_conv(pt.cpu().numpy(), filt2, (12, 12, 15), 3, 0.13, 0.8, 0.2)
    L2 = refkern.RefConvLIF(cu(filt2), (12, 12, 15), tau_s, 0.8, 0.8, 3)
    r2 = L2.forward(rt, rn, np.float32(0.2))
    assert np.array_equal(ours2[0], r2[0].cpu().numpy())
    same = leading_mask(ours2[0], 3)
    np.testing.assert_allclose(ours2[3][same], r2[3].cpu().numpy()[same], rtol=1e-6)
    # Backward through conv2 with unit errors on every spike.
    err = np.where(np.isfinite(ours2[3]), 1.0, 0.0).astype(np.float32)
    tau32, c2, dtt2 = K.lif_constants(0.13, 0.8, 0.8)
    n2, a2, x2, t2, z2 = (cu(v) if k else cu(v, torch.int32) for k, v in enumerate(ours2))
    e2 = cu(err)
    tabs = K.backward_prep(t2, a2, x2, z2, e2, c2, tau32, dtt2)
    g2, pe2 = K.conv_backward(ev2, cu(filt2), (12, 12, 15), t2, tabs, tau_s, tau32, want_pre_errors=True)
    rg2, rpe2 = L2.backward(cu(err), want_pre=True)
    torch.cuda.synchronize()
    g2, rg2, pe2, rpe2 = (v.cpu().numpy().astype(np.float64) for v in (g2, rg2, pe2, rpe2))
    scale_g = np.abs(rg2).max() + 1e-30
    scale_p = np.abs(rpe2).max() + 1e-30
    assert np.max(np.abs(g2 - rg2)) <= 1e-5 * scale_g, np.max(np.abs(g2 - rg2)) / scale_g
    assert np.max(np.abs(pe2 - rpe2)) <= 1e-5 * scale_p, np.max(np.abs(pe2 - rpe2)) / scale_p


def test_position_grouped_conv_backward_matches_cluster_kernel(cuda):
    """The conv backward over events grouped by input position (bucket width = input channels) gives the
    per-sample filter gradient and the pre-spike errors of the event-ordered cluster kernel, up to the order
    of the sums (1e-5 of the largest entry), on a 12x12x15 -> 5x5x8 layer with multi-spike input."""
    import dataclasses
    t, n_in = multi_spike_input(6, 12 * 12 * 15, 3, 0.2, seed=21, p_silent=0.3)
    rng = np.random.default_rng(21)
    filt = rng.uniform(-1, 1, (8, 5, 5, 15)).astype(np.float32)
    tau_s = np.float32(0.13)
    ev = K.sort_events(cu(t), tau_s, np.float32(2 * tau_s), bucket_width=15)
    assert ev.bucketed is not None and ev.bucket_width == 15
    out = K.conv_forward(ev, cu(filt), (12, 12, 15), 4, 0.13, 0.8, 0.8, 0.2)
    n, a, x, ts, z = out
    assert int(n.sum()) > 50
    err = cu(rng.normal(size=ts.shape).astype(np.float32))
    tau32, c, dtt = K.lif_constants(0.13, 0.8, 0.8)
    tabs = K.backward_prep(ts, a, x, z, err, c, tau32, dtt)
    g1, p1 = K.conv_backward(ev, cu(filt), (12, 12, 15), ts, tabs, tau_s, tau32, want_pre_errors=True)
    plain = dataclasses.replace(ev, bucketed=None, bucket_offsets=None)
    g2, p2 = K.conv_backward(plain, cu(filt), (12, 12, 15), ts, tabs, tau_s, tau32, want_pre_errors=True)
    g1, g2, p1, p2 = (v.cpu().numpy().astype(np.float64) for v in (g1, g2, p1, p2))
    assert np.abs(g1).max() > 0 and np.abs(p1).max() > 0
    assert np.max(np.abs(g1 - g2)) <= 1e-5 * np.abs(g2).max()
    assert np.max(np.abs(p1 - p2)) <= 1e-5 * np.abs(p2).max()
