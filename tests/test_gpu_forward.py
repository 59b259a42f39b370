"""GPU parity of the forward path (event sort + FC LIF forward) against the reference's CUDA kernels
(oracle/refkern.py) and the float64 oracle.

Tolerances: spike times within 1e-5 relative; spike counts exact except
for neurons whose membrane maximum lies within 1e-5 (relative) of the threshold, identified by the
float64 oracle at theta*(1 -+ 1e-5), which are counted and must stay rare.
"""
import numpy as np
import pytest
import torch

from bats_gb300 import kernels as K
from bats_gb300._lib import BatsError, check_device_status, ptr, stream_ptr
from oracle import bats_ref64 as R
from oracle import refkern
from tests._helpers import (conditioned_reference, count_mismatches, grazing_mask, leading_mask, mnist_like_input,
                            multi_spike_input)

pytestmark = pytest.mark.gpu

RTOL_T = 1e-5


def run_fc(t, W, tau_s, theta, dtheta, K_post, max_sim=np.inf):
    tt = torch.tensor(t, device="cuda")
    ev = K.sort_events(tt, np.float32(tau_s), np.float32(2 * tau_s))
    wt = K.transpose_weights(torch.tensor(W, device="cuda"))
    n, a, x, ts, z = K.lif_forward_fc(ev, wt, W.shape[0], K_post, tau_s, theta, dtheta, max_sim)
    torch.cuda.synchronize()
    return [v.cpu().numpy() for v in (n, a, x, ts, z)], ev


def run_ref(t, n_in, W, tau_s, theta, dtheta, K_post, max_sim=np.inf):
    if not refkern.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    layer = refkern.RefLIF(torch.tensor(W, device="cuda"), tau_s, theta, dtheta, K_post)
    out = layer.forward(torch.tensor(t, device="cuda"), torch.tensor(n_in, device="cuda"), max_sim)
    torch.cuda.synchronize()
    return [v.cpu().numpy() for v in out]


def check_against(ours, ref, bounds, max_unexplained=0, rtol=RTOL_T, what="", fields=("t", "z", "a", "x"), t_atol=0.0,
                  t_sens=None):
    """Counts exact up to grazing neurons; the listed fields within rtol on neurons with equal counts."""
    n, a, x, t, z = ours
    rn, ra, rx, rt, rz = ref
    diff, unexplained = count_mismatches(n, rn, bounds)
    assert unexplained <= max_unexplained, f"{what}: {unexplained} unexplained count mismatches ({diff} total)"
    same = (n == rn)[:, :, None] & leading_mask(rn, t.shape[2])
    got = {"t": t, "z": z, "a": a, "x": x}
    exp = {"t": rt, "z": rz, "a": ra, "x": rx}
    for name in fields:
        u = got[name][same].astype(np.float64)
        v = exp[name][same].astype(np.float64)
        e = np.abs(u - v)
        tol = rtol * np.abs(v) + (t_atol if name == "t" else 0.0)
        if t_sens is not None and name in ("t", "z"):
            # 20x the spike time's sensitivity to a 1e-6 relative change of the neuron state (FP32 rounding
            # of the accumulated sums is a few 1e-7); z = exp(t/tau) inherits it through dz = z dt / tau.
            sens = t_sens[same]
            tol = tol + 20 * (sens if name == "t" else sens * np.abs(v) / 0.26)
        assert not (e > tol).any(), f"{what}: {name} max err {np.max(e - tol):.3e} over tolerance"
    pad = ~leading_mask(n, t.shape[2])
    assert np.isinf(t[pad]).all() and np.isinf(z[pad]).all()
    return diff


# Against the float64 oracle, t = tau ln z turns the relative error of z into an absolute error of
# about tau * 1e-7 per FP32 rounding, so the time tolerance there is 1e-5 relative plus 1e-5 * tau, plus a
# term proportional to the spike time's conditioning (near-tangential crossings).
ORACLE = dict(fields=("t", "z"), t_atol=1e-5 * 0.26)


@pytest.mark.parametrize("seed", [0, 1])
def test_small_multi_spike_vs_oracle_and_reference(cuda, seed):
    t, n_in = multi_spike_input(4, 40, 3, 0.3, seed=seed)
    rng = np.random.default_rng(100 + seed)
    W = rng.normal(0, 1, (16, 40)).astype(np.float32)
    tau_s, theta, dth, Kp = 0.1, 0.1, 0.2, 16
    ours, _ = run_fc(t, W, tau_s, theta, dth, Kp, 0.5)
    o64, bounds, sens = conditioned_reference(t, W, np.float32(tau_s), theta, dth, Kp, np.float32(0.5))
    assert ours[0].sum() > 20, "test input should make the layer spike"
    check_against(ours, o64, bounds, what="vs oracle", t_sens=sens, **ORACLE)
    ref = run_ref(t, n_in, W, tau_s, theta, dth, Kp, 0.5)
    d = check_against(ours, ref, bounds, rtol=1e-6, what="vs reference kernels")
    assert d == 0


@pytest.mark.parametrize("variant", ["literal", "active"])
def test_mnist_config_vs_reference_kernels(cuda, variant):
    """784-800 hidden layer of the spike-count MNIST configuration, batch 50, seed 0."""
    t, n_in = mnist_like_input(50, seed=0)
    rng = np.random.default_rng(0)
    if variant == "literal":
        W = rng.normal(0, 1 / np.sqrt(784), (800, 784)).astype(np.float32)
        theta = 1.0
    else:
        W = rng.uniform(-1, 1, (800, 784)).astype(np.float32)
        theta = 0.2
    ours, ev = run_fc(t, W, 0.13, theta, theta, 30, 0.2)
    ref = run_ref(t, n_in, W, 0.13, theta, theta, 30, 0.2)
    bounds = grazing_mask(t, W.astype(np.float64), np.float32(0.13), theta, theta, 30, np.float32(0.2))
    check_against(ours, ref, bounds, what=f"{variant} vs reference kernels")
    o64, b8, sens = conditioned_reference(t[:8], W, np.float32(0.13), theta, theta, 30, np.float32(0.2))
    check_against([v[:8] for v in ours], o64, b8, what=f"{variant} vs oracle", t_sens=sens, **ORACLE)
    if variant == "active":
        assert ours[0].sum() > 1000
    assert np.array_equal(ev.counts.cpu().numpy(), n_in.sum(1))


def test_sort_events(cuda):
    t, n_in = multi_spike_input(3, 500, 12, 0.1, seed=3)
    ev = K.sort_events(torch.tensor(t, device="cuda"), 0.1, 0.2)
    e = ev.events.cpu().numpy()
    sl = ev.slots.cpu().numpy()
    cnt = ev.counts.cpu().numpy()
    for s in range(3):
        et, ej, es = R.sort_events(t[s:s + 1])[0]
        assert cnt[s] == et.size
        assert np.array_equal(sl[s, :cnt[s]], es)
        assert np.array_equal(e[s, :cnt[s], 0], et.astype(np.float32))
        assert np.array_equal(e[s, :cnt[s], 1].view(np.int32), ej)
        np.testing.assert_allclose(e[s, :cnt[s], 2], np.exp(et / np.float32(0.1)), rtol=2e-6)


@pytest.mark.parametrize("k", [1, 3])
def test_sort_events_small_samples_with_ties(cuda, k):
    """Small samples with many tied times: events, slots and counts equal the oracle's stable sort (ties
    in slot order), and the bucketed copy is the time order grouped stably by pre-neuron bucket, with its
    offsets; samples of 0, 1, 40, 150, 256 and 257 events."""
    rng = np.random.default_rng(31)
    B, N = 6, 300
    t = np.full((B, N, k), np.inf, dtype=np.float32)
    want = [150, 256, 257, 0, 1, 40]
    for s, m in enumerate(want):
        slots = rng.choice(N * k, size=m, replace=False)
        vals = (rng.integers(0, 60, m) * 0.001).astype(np.float32)  # many ties
        t[s].reshape(-1)[slots] = vals
    ev = K.sort_events(torch.tensor(t, device="cuda"), 0.1, 0.2, bucket_width=64)
    torch.cuda.synchronize()
    e = ev.events.cpu().numpy()
    sl = ev.slots.cpu().numpy()
    cnt = ev.counts.cpu().numpy()
    be = ev.bucketed.cpu().numpy()
    bo = ev.bucket_offsets.cpu().numpy()
    assert cnt.tolist() == want
    for s in range(B):
        et, ej, es = R.sort_events(t[s:s + 1])[0]
        c = cnt[s]
        assert np.array_equal(sl[s, :c], es)
        assert np.array_equal(e[s, :c, 0], et.astype(np.float32))
        assert np.array_equal(e[s, :c, 1].view(np.int32), ej)
        bucket = ej // 64
        order = np.argsort(bucket, kind="stable")
        assert np.array_equal(be[s, :c].view(np.uint32), e[s, :c][order].view(np.uint32))
        nb = bo.shape[1] - 1
        assert np.array_equal(bo[s, :nb], np.searchsorted(bucket[order], np.arange(nb), side="left"))
        assert bo[s, nb] == c


@pytest.mark.parametrize("shape,fill", [((2, 1000, 6), (6000, 3000)), ((2, 512, 30), (15360, 4000)),
                                        ((2, 1000, 20), (20000, 5000)), ((2, 5000, 14), (70000, 3000)),
                                        ((2, 1000, 16), (16000, 13000)), ((160, 512, 30), (15360, 7000)),
                                        ((160, 512, 30), (6720, 6721)), ((160, 1000, 1), (1000, 999)),
                                        ((160, 4000, 20), (80000, 4000))])
def test_sort_events_large_sample_uses_global_path(cuda, shape, fill):
    """Samples of every size class of the sort. Layers of more than 1024 slots sort with 512 threads: small
    batches (<= 152 samples) hold up to 16448 items in shared memory with 16-bit slot values (layers of at
    most 65536 slots), 12320 with 32-bit values; larger batches 6720 and 4096 (the boundary exactly: 6720 and
    6721 items). Smaller layers sort with 256 threads (17408 / 13312 / 7680 / 4096 items). Samples above
    that sort in the global workspace. Events and slots equal the oracle's sort; the bucketed copy is each
    bucket's events in time order. The samples not listed in `fill` hold 37 spikes."""
    rng = np.random.default_rng(4)
    B, N, Kp = shape
    t = np.full(shape, np.inf, np.float32)
    fill = tuple(fill) + (37,) * (B - len(fill))
    for s, m in enumerate(fill):  # the first m slots of the sample (in slot order) hold spikes
        flat = np.sort(rng.uniform(0, 1, (N, Kp)), axis=1).astype(np.float32).reshape(-1)
        flat[m:] = np.inf
        t[s] = flat.reshape(N, Kp)
    ev = K.sort_events(torch.tensor(t, device="cuda"), 0.1, 0.2)
    cnt = ev.counts.cpu().numpy()
    assert cnt.tolist() == list(fill)
    e, slots_d = ev.events.cpu().numpy(), ev.slots.cpu().numpy()
    be, bo = ev.bucketed.cpu().numpy(), ev.bucket_offsets.cpu().numpy()
    for s in range(min(B, 3)):
        et, ej, slots = R.sort_events(t[s:s + 1])[0]
        c = cnt[s]
        assert np.array_equal(e[s, :c, 0], et.astype(np.float32))
        assert np.array_equal(slots_d[s, :c], slots)
        bucket = (slots // Kp) // K.BUCKET_WIDTH
        order = np.argsort(bucket, kind="stable")
        assert np.array_equal(be[s, :c].view(np.uint32), e[s, :c][order].view(np.uint32))
        nb = bo.shape[1] - 1
        assert np.array_equal(bo[s, :nb], np.searchsorted(bucket[order], np.arange(nb), side="left"))


def _events_equal(p, q, what):
    cnt = p.counts.cpu().numpy()
    assert np.array_equal(cnt, q.counts.cpu().numpy()), what
    pe, qe = p.events.cpu().numpy(), q.events.cpu().numpy()
    ps, qs = p.slots.cpu().numpy(), q.slots.cpu().numpy()
    pb, qb = p.bucketed.cpu().numpy(), q.bucketed.cpu().numpy()
    assert np.array_equal(p.bucket_offsets.cpu().numpy(), q.bucket_offsets.cpu().numpy()), what
    for s in range(cnt.shape[0]):
        c = cnt[s]
        assert np.array_equal(pe[s, :c].view(np.uint32), qe[s, :c].view(np.uint32)), what
        assert np.array_equal(ps[s, :c], qs[s, :c]), what
        assert np.array_equal(pb[s, :c].view(np.uint32), qb[s, :c].view(np.uint32)), what


@pytest.mark.parametrize("case", ["lif_output", "large", "irregular"])
def test_sort_events_counted_matches_full_scan(cuda, case):
    """The sort given the pre layer's spike counts (reading only the slots below them) returns the same
    events, slots, counts and bucketed copy as the full scan: on a LIF layer's output, above the
    shared-memory capacity, and with counts past K, negative counts, empty samples and non-finite times
    below a count."""
    rng = np.random.default_rng(21)
    if case == "lif_output":
        t, n_in = mnist_like_input(8, seed=3)
        W = rng.uniform(-1, 1, (800, 784)).astype(np.float32)
        (n, _, _, ts, _), _ = run_fc(t, W, 0.13, 0.2, 0.2, 30, 0.2)
        assert n.sum() > 0
        times, counts = ts, n.astype(np.int32)
    elif case == "large":
        times = np.sort(rng.uniform(0, 1, (3, 700, 12)).astype(np.float32), axis=2)
        counts = rng.integers(0, 13, (3, 700)).astype(np.int32)
        counts[0] = 12  # 8400 events: the global-memory path
        times[np.arange(12)[None, None, :] >= counts[:, :, None]] = np.inf
    else:
        times = rng.uniform(0, 1, (4, 50, 5)).astype(np.float32)
        counts = rng.integers(0, 6, (4, 50)).astype(np.int32)
        times[np.arange(5)[None, None, :] >= counts[:, :, None]] = np.inf
        counts[0, :3] = 9      # clamped to K
        counts[0, 3] = -2      # treated as 0 (its slots are all inf)
        times[0, 3] = np.inf
        counts[1] = 0
        times[1] = np.inf      # empty sample
        times[2, 7, 0] = np.inf if counts[2, 7] > 1 else times[2, 7, 0]  # hole below a count
        times[3, 9, :] = np.inf
        counts[3, 9] = 5       # count above the finite slots
    tt = torch.tensor(times, device="cuda")
    full = K.sort_events(tt, np.float32(0.1), np.float32(0.2))
    part = K.sort_events(tt, np.float32(0.1), np.float32(0.2), pre_counts=torch.tensor(counts, device="cuda"))
    torch.cuda.synchronize()
    _events_equal(full, part, case)


def _count_class(c):
    """The logarithmic size class of bats_sample_order (16 per octave, 0 for the longest samples)."""
    key = (np.float32(c + 1).reshape(-1).view(np.uint32) >> 19).astype(np.int64) - (127 << 4)
    return 511 - np.clip(key, 0, 511)


def test_sort_events_counted_ordered_matches_unordered(cuda):
    """The counted sort with its CTAs taking the samples in a given order (longest first from
    bats_sample_order, or a random permutation) returns the events, slots, counts and bucketed copy of the
    unordered sort, on a batch of 400 uneven samples (wider than the resident CTAs), some above the
    shared-memory capacity (the global-memory path), some empty; bats_sample_order ranks the samples by
    descending size class."""
    rng = np.random.default_rng(33)
    B, N, Kp = 400, 700, 12
    times = np.sort(rng.uniform(0, 1, (B, N, Kp)).astype(np.float32), axis=2)
    per_sample = np.minimum(Kp, rng.lognormal(0.5, 0.9, B)).astype(np.float32)
    counts = np.minimum(Kp, rng.poisson(per_sample[:, None], (B, N))).astype(np.int32)
    counts[:5] = Kp        # 8400 events: the global-memory path
    counts[5:9] = 0        # empty samples
    times[np.arange(Kp)[None, None, :] >= counts[:, :, None]] = np.inf
    tt = torch.tensor(times, device="cuda")
    tc = torch.tensor(counts, device="cuda")
    plain = K.sort_events(tt, np.float32(0.1), np.float32(0.2), pre_counts=tc)
    order = K.sample_order(plain.counts)
    perm = torch.tensor(rng.permutation(B).astype(np.int32), device="cuda")
    for what, so in (("longest first", order), ("random", perm)):
        got = K.sort_events(tt, np.float32(0.1), np.float32(0.2), pre_counts=tc, sample_order=so)
        torch.cuda.synchronize()
        _events_equal(plain, got, what)
    o = order.cpu().numpy()
    assert np.array_equal(np.sort(o), np.arange(B))
    cls = _count_class(plain.counts.cpu().numpy()[o])
    assert (np.diff(cls) >= 0).all()
    assert set(o[:5].tolist()) == set(range(5))
    # More samples than the order kernel's 1024 threads, lognormal counts with zeros.
    c3 = np.minimum(rng.lognormal(5, 1.5, 3000), 1e6).astype(np.int32)
    c3[::97] = 0
    o3 = K.sample_order(torch.tensor(c3, device="cuda")).cpu().numpy()
    assert np.array_equal(np.sort(o3), np.arange(3000))
    assert (np.diff(_count_class(c3[o3])) >= 0).all()


def test_edge_cases(cuda):
    rng = np.random.default_rng(9)
    W = rng.uniform(-1, 1, (37, 20)).astype(np.float32)
    # Empty batch input: all outputs silent.
    t = np.full((3, 20, 2), np.inf, dtype=np.float32)
    (n, a, x, ts, z), _ = run_fc(t, W, 0.1, 0.1, 0.1, 5)
    assert (n == 0).all() and np.isinf(ts).all() and np.isinf(z).all()
    # One sample silent, one busy; buffer cap reached; max_simulation cut.
    t, n_in = multi_spike_input(2, 20, 4, 0.2, seed=1, p_silent=0.0)
    t[0] = np.inf
    W2 = np.abs(W) * 3
    ours, _ = run_fc(t, W2, 0.1, 0.05, 0.05, 3)
    assert (ours[0][0] == 0).all() and (ours[0][1] == 3).any()
    ref = run_ref(t, n_in, W2, 0.1, 0.05, 0.05, 3)
    check_against(ours, ref, None, what="cap")
    ours, _ = run_fc(t, W2, 0.1, 0.05, 0.05, 40, 0.1)
    assert np.nanmax(np.where(np.isinf(ours[3]), np.nan, ours[3])) <= np.float32(0.1)
    ref = run_ref(t, n_in, W2, 0.1, 0.05, 0.05, 40, 0.1)
    check_against(ours, ref, None, what="max_simulation")


def _both_algos(t, W, tau_s, theta, dtheta, K_post, max_sim=np.inf):
    tt = torch.tensor(t, device="cuda")
    ev = K.sort_events(tt, np.float32(tau_s), np.float32(2 * tau_s))
    wt = K.transpose_weights(torch.tensor(W, device="cuda"))
    outs = []
    for algo in (K.FWD_TILE, K.FWD_LANES, K.FWD_TILE64, K.FWD_QUEUE, K.FWD_QUEUE64, K.FWD_TILE | K.FWD_STAGE,
                 K.FWD_TILE64 | K.FWD_STAGE, K.FWD_QUEUE | K.FWD_STAGE):
        o = K.lif_forward_fc(ev, wt, W.shape[0], K_post, tau_s, theta, dtheta, max_sim, algo=algo)
        outs.append([v.cpu().numpy() for v in o])
    return outs


def _assert_identical(p, q, what):
    n = p[0]
    assert np.array_equal(n, q[0]), what
    valid = leading_mask(n, p[3].shape[2])
    for name, i in (("a", 1), ("x", 2)):
        assert np.array_equal(p[i][valid].view(np.uint32), q[i][valid].view(np.uint32)), f"{what}: {name}"
    for name, i in (("t", 3), ("z", 4)):
        assert np.array_equal(p[i].view(np.uint32), q[i].view(np.uint32)), f"{what}: {name}"


@pytest.mark.parametrize("case", ["small", "mnist_active", "long_narrow", "long_wide", "cap_and_cut", "mnist_literal",
                                  "quiet_and_spiking"])
def test_event_parallel_kernel_matches_tile_kernel(cuda, case):
    """The warp-per-neuron forward (32 events per step, FWD_LANES), the 64-neuron-tile variant, the
    persistent work-queue kernel (both tile widths) and the per-stage-screen variants (FWD_STAGE: tile, 64-neuron
    tiles, queue) are bit-identical to the tile kernel on
    short and long event streams, narrow and wide layers, a full spike buffer and a max_simulation cut; on
    a long stream it also matches the reference kernels."""
    rng = np.random.default_rng(5)
    if case == "small":
        t, n_in = multi_spike_input(4, 40, 3, 0.3, seed=2)
        W = rng.normal(0, 1, (16, 40)).astype(np.float32)
        args = (0.1, 0.1, 0.2, 16, 0.5)
    elif case == "mnist_active":
        t, n_in = mnist_like_input(16, seed=3)
        W = rng.uniform(-1, 1, (800, 784)).astype(np.float32)
        args = (0.13, 0.2, 0.2, 30, 0.2)
    elif case in ("long_narrow", "long_wide"):
        n_post = 20 if case == "long_narrow" else 512
        t, n_in = multi_spike_input(2, 700, 20, 0.2, seed=4, p_silent=0.1)
        W = ((rng.normal(0, 1, (n_post, 700)) + 1.5) / np.sqrt(700)).astype(np.float32)
        args = (0.13, 1.0, 1.0, 30, np.inf)
    elif case == "mnist_literal":  # the hidden layer of the literal configuration: (almost) no neuron spikes
        t, n_in = mnist_like_input(64, seed=7)
        W = rng.normal(0, 1 / np.sqrt(784), (800, 784)).astype(np.float32)
        args = (0.13, 1.0, 1.0, 30, 0.2)
    elif case == "quiet_and_spiking":  # most stages pass the per-stage screen, some neurons spike late
        t, n_in = multi_spike_input(8, 300, 4, 0.1, seed=8, p_silent=0.3)
        W = ((rng.normal(0, 1, (200, 300)) + np.linspace(-0.5, 1.5, 200)[:, None]) / np.sqrt(300)).astype(np.float32)
        args = (0.13, 1.0, 1.0, 30, np.inf)
    else:
        t, n_in = multi_spike_input(3, 50, 6, 0.2, seed=6, p_silent=0.0)
        W = np.abs(rng.normal(0, 1, (40, 50))).astype(np.float32)
        args = (0.1, 0.05, 0.05, 4, 0.12)
    tile, lanes, tile64, queue, queue64, stage, stage64, queue_stage = _both_algos(t, W, *args)
    if case != "mnist_literal":
        assert tile[0].sum() > 0, "the case should spike"
    if case == "quiet_and_spiking":
        assert 0 < (tile[0] > 0).mean() < 0.9, "some neurons should spike and others stay quiet"
    _assert_identical(tile, lanes, case)
    _assert_identical(tile, tile64, case + " (64-neuron tiles)")
    _assert_identical(tile, queue, case + " (work queue)")
    _assert_identical(tile, queue64, case + " (work queue, 64-neuron tiles)")
    _assert_identical(tile, stage, case + " (per-stage screen)")
    _assert_identical(tile, stage64, case + " (per-stage screen, 64-neuron tiles)")
    _assert_identical(tile, queue_stage, case + " (work queue, per-stage screen)")
    if case == "long_narrow":
        ref = run_ref(t, n_in, W, *args)
        check_against(lanes, ref, None, what="lanes vs reference kernels")


@pytest.mark.parametrize("algo", [K.FWD_TILE, K.FWD_LANES, K.FWD_TILE64, K.FWD_QUEUE, K.FWD_TILE | K.FWD_STAGE])
def test_no_pad_flag_leaves_slots_past_counts(cuda, algo):
    """BATS_FWD_NO_PAD: counts and every value below them are those of the padded forward, and the slots
    past the counts keep what the buffers held (here a sentinel)."""
    t, n_in = mnist_like_input(8, seed=4)
    rng = np.random.default_rng(4)
    W = rng.uniform(-1, 1, (200, 784)).astype(np.float32)
    ev = K.sort_events(torch.tensor(t, device="cuda"), np.float32(0.13), np.float32(0.26))
    wt = K.transpose_weights(torch.tensor(W, device="cuda"))
    ref = K.lif_forward_fc(ev, wt, 200, 30, 0.13, 0.2, 0.2, 0.2, algo=algo)
    outs = (torch.full((8, 200), -7, dtype=torch.int32, device="cuda"),
            *(torch.full((8, 200, 30), 12345.0, device="cuda") for _ in range(4)))
    got = K.lif_forward_fc(ev, wt, 200, 30, 0.13, 0.2, 0.2, 0.2, outs=outs, algo=algo | K.FWD_NO_PAD)
    torch.cuda.synchronize()
    n = ref[0].cpu().numpy()
    assert np.array_equal(n, got[0].cpu().numpy())
    assert n.sum() > 0 and (n < 30).any()
    valid = leading_mask(n, 30)
    for r, g in zip(ref[1:], got[1:]):
        r, g = r.cpu().numpy(), g.cpu().numpy()
        assert np.array_equal(r[valid].view(np.uint32), g[valid].view(np.uint32))
        assert (g[~valid] == 12345.0).all()


def uneven_input(batch, n_in, median, hi, t_max, seed, p_empty=0.05):
    """Samples with lognormal event counts (median `median`, at most `hi`), some of them empty, channels
    uniform over n_in, times U(0, t_max): spike trains (B, n_in, K_in), K_in the largest per-channel count."""
    rng = np.random.default_rng(seed)
    counts = np.clip(np.round(rng.lognormal(np.log(median), 1.0, batch)), 1, hi).astype(np.int64)
    counts[rng.random(batch) < p_empty] = 0
    chans = [rng.integers(0, n_in, c) for c in counts]
    k_in = max(1, max(int(np.bincount(ch, minlength=n_in).max()) if len(ch) else 0 for ch in chans))
    t = np.full((batch, n_in, k_in), np.inf, dtype=np.float32)
    for q, ch in enumerate(chans):
        for j in np.unique(ch):
            m = int((ch == j).sum())
            t[q, j, :m] = np.sort(rng.uniform(0, t_max, m))
    return t, counts


@pytest.mark.parametrize("n_post", [20, 50, 300])
def test_work_queue_forward_on_uneven_batch(cuda, n_post):
    """The persistent work-queue forward on a batch whose samples carry 0 to 600 events (lognormal, some
    empty) is bit-identical to the one-CTA-per-item tile kernel, padded and unpadded, and again on a second
    call with the same workspace (the order kernel resets the queue head): tile widths 32, 64 and 128 with a
    partial last tile, K = 8 so that some neurons fill their spike buffer."""
    t, counts = uneven_input(333, 256, 40, 600, 0.05, seed=9)
    assert (counts == 0).any() and counts.max() > 300
    rng = np.random.default_rng(10)
    W = rng.uniform(-0.5, 1.5, (n_post, 256)).astype(np.float32)
    ev = K.sort_events(torch.tensor(t, device="cuda"), np.float32(0.13), np.float32(0.26))
    wt = K.transpose_weights(torch.tensor(W, device="cuda"))
    args = (n_post, 8, 0.13, 0.2, 0.2, 0.2)
    tile = [v.cpu().numpy() for v in K.lif_forward_fc(ev, wt, *args, algo=K.FWD_TILE)]
    assert tile[0].sum() > 0 and (tile[0] == 8).any(), "the case should spike, some neurons up to K"
    ws = torch.empty(K.queue_workspace_bytes(333), dtype=torch.uint8, device="cuda")
    outs = (torch.empty((333, n_post), dtype=torch.int32, device="cuda"),
            *(torch.empty((333, n_post, 8), device="cuda") for _ in range(4)))
    tau32, c, dtt = K.lif_constants(0.13, 0.2, 0.2)
    for rep, algo in enumerate((K.FWD_QUEUE, K.FWD_QUEUE, K.FWD_QUEUE | K.FWD_STAGE)):
        for o in outs:
            o.fill_(-1)
        K.forward_fc_call(ev, wt, n_post, 8, c, dtt, tau32, 0.2, outs, algo, stream_ptr(), ptr(ws), ws.numel())
        _assert_identical(tile, [v.cpu().numpy() for v in outs], f"work queue, call {rep + 1}")
    K.forward_fc_call(ev, wt, n_post, 8, c, dtt, tau32, 0.2, outs, K.FWD_QUEUE | K.FWD_NO_PAD, stream_ptr(),
                      ptr(ws), ws.numel())
    n = outs[0].cpu().numpy()
    assert np.array_equal(n, tile[0])
    valid = leading_mask(n, 8)
    for i in range(1, 5):
        assert np.array_equal(outs[i].cpu().numpy()[valid].view(np.uint32), tile[i][valid].view(np.uint32))
    check_device_status()


def test_work_queue_forward_rejects_small_workspace(cuda):
    t, _ = mnist_like_input(4, seed=1)
    ev = K.sort_events(torch.tensor(t, device="cuda"), np.float32(0.13), np.float32(0.26))
    wt = K.transpose_weights(torch.tensor(np.ones((8, 784), np.float32), device="cuda"))
    outs = (torch.empty((4, 8), dtype=torch.int32, device="cuda"), *(torch.empty((4, 8, 4), device="cuda")
                                                                      for _ in range(4)))
    ws = torch.empty(16, dtype=torch.uint8, device="cuda")
    tau32, c, dtt = K.lif_constants(0.13, 1.0, 1.0)
    with pytest.raises(BatsError):
        K.forward_fc_call(ev, wt, 8, 4, c, dtt, tau32, 0.2, outs, K.FWD_QUEUE, stream_ptr(), ptr(ws), ws.numel())
