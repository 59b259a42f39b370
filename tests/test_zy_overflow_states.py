"""Forward parity on states that overflow (run after the other GPU files).

Input spikes later than 88 tau_s overflow exp(t/tau_s) to +inf, so a neuron's a becomes +-inf (or NaN) while b,
built from exp(t/tau) with half the exponent, stays finite. The reference's solver
(bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83) then forms z = 2a/(x + b) = NaN, which passes
its sign and window tests, and records NaN spikes until the buffer is full. Every forward variant must do the
same: the no-crossing screens claim no state with |a| > 2^60. Compared with the reference kernels directly
(the float64 oracle does not overflow there).

The conv layer adds one more effect: the reference's conv loop
(bats/CudaKernels/CuFiles/Inference/compute_spike_times_conv.cu:155-172) adds every event of the sample, with
weight 0 outside the neuron's receptive field, so an overflowing event outside the field still turns the
state into NaN (0 * inf). The conv kernel counts such events as relevant to every neuron."""
import numpy as np
import pytest
import torch

from bats_gb300 import kernels as K
from oracle import refkern
from tests._helpers import leading_mask
from tests.test_gpu_forward import _both_algos, run_ref

pytestmark = pytest.mark.gpu


def test_overflowing_states_match_the_reference_kernels(cuda):
    rng = np.random.default_rng(9)
    B, n_in, n_post, k_post, tau_s = 8, 64, 48, 8, 0.13
    t = np.full((B, n_in, 1), np.inf, np.float32)
    fire = rng.random((B, n_in)) < 0.6
    t[fire, 0] = rng.uniform(11.6, 12.0, int(fire.sum()))       # t / tau_s > 89: exp(t / tau_s) overflows
    early = fire & (rng.random((B, n_in)) < 0.3)
    t[early, 0] = rng.uniform(0.0, 0.01, int(early.sum()))       # some finite states before the overflow
    counts = fire.astype(np.int32)
    W = rng.normal(0.0, 1e-3, (n_post, n_in)).astype(np.float32)  # |b| stays below 2^60
    ref = run_ref(t, counts, W, tau_s, 1.0, 1.0, k_post, np.inf)
    assert np.isnan(ref[3]).any() and np.isneginf(ref[1]).any(), "the case should give NaN spikes from a = -inf"
    lead = leading_mask(ref[0], k_post)
    for out in _both_algos(t, W, tau_s, 1.0, 1.0, k_post, np.inf):
        assert np.array_equal(out[0], ref[0])
        for i, name in ((1, "a"), (2, "x"), (3, "t"), (4, "z")):
            assert np.array_equal(out[i][lead], ref[i][lead], equal_nan=True), name


@pytest.mark.parametrize("case", ["late_only", "mixed"])
def test_conv_overflowing_states_match_the_reference_kernels(cuda, case):
    if not refkern.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    rng = np.random.default_rng(19 if case == "mixed" else 23)
    B, X, Y, C, C_out, fx, fy, k_post, tau_s = 6, 12, 12, 2, 4, 3, 3, 6, np.float32(0.13)
    t = np.full((B, X * Y * C, 1), np.inf, np.float32)
    fire = rng.random(t.shape[:2]) < 0.35
    t[fire, 0] = rng.uniform(11.6, 12.0, int(fire.sum()))        # t / tau_s > 89: exp(t / tau_s) overflows
    if case == "mixed":
        early = fire & (rng.random(t.shape[:2]) < 0.5)
        t[early, 0] = rng.uniform(0.0, 0.01, int(early.sum()))    # finite states, spikes, before the overflow
    counts = np.isfinite(t[:, :, 0]).astype(np.int32)
    filt = rng.uniform(-1, 1, (C_out, fx, fy, C)).astype(np.float32) * (1.0 if case == "mixed" else 1e-3)
    theta = 0.05
    dev = "cuda"
    L = refkern.RefConvLIF(torch.tensor(filt, device=dev), (X, Y, C), tau_s, theta, theta, k_post)
    ref = [v.cpu().numpy() for v in L.forward(torch.tensor(t, device=dev), torch.tensor(counts, device=dev),
                                              np.float32(np.inf))]
    assert np.isnan(ref[3]).any(), "the case should give NaN spikes"
    ev = K.sort_events(torch.tensor(t, device=dev), tau_s, np.float32(2 * tau_s))
    ours = [v.cpu().numpy() for v in K.conv_forward(ev, torch.tensor(filt, device=dev), (X, Y, C), k_post, tau_s,
                                                     theta, theta, np.inf)]
    assert np.array_equal(ours[0], ref[0]), f"spike counts differ at {np.argwhere(ours[0] != ref[0])[:5]}"
    lead = leading_mask(ref[0], k_post)
    for i, name in ((1, "a"), (2, "x"), (3, "t"), (4, "z")):
        assert np.array_equal(ours[i][lead], ref[i][lead], equal_nan=True), name
    if case == "mixed":
        assert np.isfinite(ref[3][lead]).any(), "some spikes should come before the overflow"
