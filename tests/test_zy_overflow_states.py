"""Forward parity on states that overflow (run after the other GPU files).

Input spikes later than 88 tau_s overflow exp(t/tau_s) to +inf, so a neuron's a becomes +-inf (or NaN) while b,
built from exp(t/tau) with half the exponent, stays finite. The reference's solver
(bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83) then forms z = 2a/(x + b) = NaN, which passes
its sign and window tests, and records NaN spikes until the buffer is full. Every forward variant must do the
same: the no-crossing screens claim no state with |a| > 2^60. Compared with the reference kernels directly
(the float64 oracle does not overflow there)."""
import numpy as np
import pytest

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
