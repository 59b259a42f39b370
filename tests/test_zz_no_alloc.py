"""The allocation-free batch-mean weight gradient (bats_weights_gradient_mean_noalloc).

Callers that cannot allocate device memory on their call path (a runtime that owns a fixed arena, a
plugin host that only passes input and output buffers) use this entry point: it keeps its scratch in
a static device array of the library instead of a caller workspace. This test calls it through the C
ABI twice in a row and checks both results against bats_weights_gradient with a caller workspace,
within the tolerance of the backward parity tests (1e-5 relative), and checks that sizes beyond the
static scratch are refused. It sits in its own file, collected last, and passes alone or after the
other tests (the scratch keeps the previous call's contents, which the kernel never reads).
"""
import ctypes

import numpy as np
import pytest
import torch

from bats_gb300 import _lib
from bats_gb300 import kernels as K
from tests._helpers import multi_spike_input

pytestmark = pytest.mark.gpu


def _case(batch, n_pre, n_post, seed):
    t, _ = multi_spike_input(batch, n_pre, 3, 0.1, seed=seed)
    rng = np.random.default_rng(seed)
    W = rng.uniform(-1, 1, (n_post, n_pre)).astype(np.float32)
    ev = K.sort_events(torch.tensor(t, device="cuda"), 0.1, 0.2)
    wt = K.transpose_weights(torch.tensor(W, device="cuda"))
    n, a, x, ts, z = K.lif_forward_fc(ev, wt, n_post, 16, 0.1, 0.1, 0.1)
    err = torch.tensor(rng.uniform(-1, 1, ts.shape).astype(np.float32), device="cuda")
    tau32, c, dtt = K.lif_constants(0.1, 0.1, 0.1)
    tabs = K.backward_prep(ts, a, x, z, err, c, tau32, dtt)
    assert int(n.sum()) > 0
    return ev, ts, tabs


def _noalloc(ev, ts, tabs, n_pre, group, out):
    B, n_post, k_post = ts.shape
    return _lib.load().bats_weights_gradient_mean_noalloc(
        ev.events.data_ptr(), ev.counts.data_ptr(), ev.cap, ts.data_ptr(), tabs.tables.data_ptr(),
        tabs.nvalid.data_ptr(), B, n_post, k_post, n_pre, group, out.data_ptr(),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_noalloc_gradient_matches_workspace_entry_point(cuda):
    cap = int(_lib.load().bats_weights_gradient_noalloc_capacity())
    assert cap == 8 * 1024 * 1024
    ev, ts, tabs = _case(64, 200, 120, seed=11)
    expected = K.weights_gradient(ev, ts, tabs, 200, per_sample=False, group=8).cpu().numpy()
    ev2, ts2, tabs2 = _case(16, 96, 40, seed=12)
    expected2 = K.weights_gradient(ev2, ts2, tabs2, 96, per_sample=False, group=4).cpu().numpy()
    for _ in range(2):  # two calls in a row, with a call of another shape between them
        out = torch.full((120, 200), float("nan"), device="cuda")
        assert _noalloc(ev, ts, tabs, 200, 8, out) == 0
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, expected, rtol=1e-5, atol=0)
        out2 = torch.full((40, 96), float("nan"), device="cuda")
        assert _noalloc(ev2, ts2, tabs2, 96, 4, out2) == 0
        np.testing.assert_allclose(out2.cpu().numpy(), expected2, rtol=1e-5, atol=0)


def test_noalloc_gradient_refuses_oversized_scratch(cuda):
    ev, ts, tabs = _case(8, 32, 16, seed=13)
    out = torch.zeros((16, 32), device="cuda")
    B, n_post, k_post = ts.shape
    # Claim 4 groups of a 2048 x 2048 layer: 16 Mi floats of partial sums > the 8 Mi-float scratch.
    # The size check happens on the host before any launch.
    status = _lib.load().bats_weights_gradient_mean_noalloc(
        ev.events.data_ptr(), ev.counts.data_ptr(), ev.cap, ts.data_ptr(), tabs.tables.data_ptr(),
        tabs.nvalid.data_ptr(), 8, 2048, k_post, 2048, 2, out.data_ptr(),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert status == 3  # BATS_ERR_CAPACITY
    assert b"static scratch" in _lib.load().bats_last_error()


def test_noalloc_gradient_refuses_too_many_groups(cuda):
    """More sample groups than a grid's z dimension holds (65535) are refused on the host, before any launch,
    with a message that says to raise the group size."""
    ev, ts, tabs = _case(8, 32, 16, seed=14)
    out = torch.zeros((16, 32), device="cuda")
    B, n_post, k_post = ts.shape
    # Claim 140000 samples in groups of 2 (70000 groups) of a 1 x 1 layer: the scratch would hold them, the
    # grid would not.
    status = _lib.load().bats_weights_gradient_mean_noalloc(
        ev.events.data_ptr(), ev.counts.data_ptr(), ev.cap, ts.data_ptr(), tabs.tables.data_ptr(),
        tabs.nvalid.data_ptr(), 140000, 1, k_post, 1, 2, out.data_ptr(),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert status == 1  # BATS_ERR_BAD_SHAPE
    assert b"raise group" in _lib.load().bats_last_error()
