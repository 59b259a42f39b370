"""The serving pattern: continuous batching of variable-length spike-event requests on device-resident
FC networks (bats_gb300.serving). Each request's result is the same alone and in a mixed batch (bit for
bit: samples are independent in every kernel), equal to the layer API's forward on the same input, and
the event-list conversion matches the reference test's known answer."""
import os

import numpy as np
import pytest
import torch

from bats_gb300 import kernels as K
from bats_gb300.serving import InferenceServer, make_network, make_requests, run_poisson, latency_stats
from oracle import bats_ref64 as R

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def net(seed=0):
    return make_network(seed=seed)


def test_event_list_conversion_known_answer(cuda):
    d = np.load(os.path.join(GOLDEN, "kat_convert.npz"))
    t, n = K.convert_to_spike_per_neuron(torch.tensor(d["indices"], dtype=torch.int32, device="cuda"),
                                         torch.tensor(d["times"], dtype=torch.float32, device="cuda"),
                                         int(d["n_neurons"]))
    np.testing.assert_array_equal(n.cpu().numpy(), d["n_spike_per_neuron"])
    np.testing.assert_array_equal(t.cpu().numpy(), d["spike_per_neuron"])
    # Random lists against the oracle, with a capacity smaller than the largest count (dropped, counted).
    rng = np.random.default_rng(0)
    idx = rng.integers(0, 40, (5, 300)).astype(np.int32)
    idx[2, 100:] = -1
    tm = np.sort(rng.uniform(0, 1, (5, 300)), axis=1).astype(np.float32)
    t, n = K.convert_to_spike_per_neuron(torch.tensor(idx, device="cuda"), torch.tensor(tm, device="cuda"), 40)
    et, en = R.convert_to_spike_per_neuron(idx, tm, 40)
    np.testing.assert_array_equal(n.cpu().numpy(), en)
    np.testing.assert_array_equal(t.cpu().numpy(), et.astype(np.float32))
    ovf = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.convert_to_spike_per_neuron(torch.tensor(idx, device="cuda"), torch.tensor(tm, device="cuda"), 40, k_cap=4,
                                  overflow=ovf)
    assert int(ovf) == int(np.maximum(en - 4, 0).sum())


def test_event_list_conversion_multi_window(cuda):
    """Samples longer than the conversion kernel's 1024-event shared-memory windows: ends inside the second
    window, exactly at a window boundary, at the first event, and full rows; the flat (CSR) form with uneven
    lengths; and a layer too wide for shared-memory counts (9000 neurons). All equal the oracle."""
    from bats_gb300._lib import call, ptr, stream_ptr
    rng = np.random.default_rng(4)
    idx = rng.integers(0, 700, (5, 3500)).astype(np.int32)
    idx[1, 1500:] = -1
    idx[2, 1024:] = -1
    idx[3, :] = -1
    tm = np.sort(rng.uniform(0, 0.2, (5, 3500)), axis=1).astype(np.float32)
    idx_d, tm_d = torch.tensor(idx, device="cuda"), torch.tensor(tm, device="cuda")
    t, n = K.convert_to_spike_per_neuron(idx_d, tm_d, 700)
    et, en = R.convert_to_spike_per_neuron(idx, tm, 700)
    np.testing.assert_array_equal(n.cpu().numpy(), en)
    np.testing.assert_array_equal(t.cpu().numpy(), et.astype(np.float32))
    # Flat list: each sample's valid events back to back, offsets between them.
    lens = [int((row >= 0).cumprod().sum()) for row in idx]
    flat_i = np.concatenate([idx[q, :m] for q, m in enumerate(lens)]).astype(np.int32)
    flat_t = np.concatenate([tm[q, :m] for q, m in enumerate(lens)]).astype(np.float32)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    kc = int(en.max())
    ct = torch.empty((5, 700, kc), device="cuda")
    cn = torch.empty((5, 700), dtype=torch.int32, device="cuda")
    fi, ft, fo = (torch.tensor(v, device="cuda") for v in (flat_i, flat_t, off))
    call("bats_events_to_trains_csr", ptr(fi), ptr(ft), ptr(fo), 5, 700, kc, ptr(ct), ptr(cn), None, stream_ptr())
    np.testing.assert_array_equal(cn.cpu().numpy(), en)
    np.testing.assert_array_equal(ct.cpu().numpy(), et.astype(np.float32))
    # Counts in global memory (more neurons than the shared-memory counts hold).
    idx2 = rng.integers(0, 9000, (3, 2600)).astype(np.int32)
    idx2[0, 2000:] = -1
    tm2 = np.sort(rng.uniform(0, 0.2, (3, 2600)), axis=1).astype(np.float32)
    t2, n2 = K.convert_to_spike_per_neuron(torch.tensor(idx2, device="cuda"), torch.tensor(tm2, device="cuda"), 9000)
    et2, en2 = R.convert_to_spike_per_neuron(idx2, tm2, 9000)
    np.testing.assert_array_equal(n2.cpu().numpy(), en2)
    np.testing.assert_array_equal(t2.cpu().numpy(), et2.astype(np.float32))


def test_same_result_alone_and_in_the_mix(cuda):
    ws, specs = net()
    server = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=32, max_lanes=3)
    reqs = make_requests(40, seed=1)
    mixed = server.infer(reqs)
    assert sum(int(r.counts.sum()) > 0 for r in mixed) >= 10, "the network should produce output spikes"
    alone_server = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=1, max_lanes=1)
    for r, m in zip(make_requests(40, seed=1, rid0=1000)[:12], mixed[:12]):
        a = alone_server.infer([r])[0]
        np.testing.assert_array_equal(a.counts, m.counts)
        np.testing.assert_array_equal(a.spike_times, m.spike_times)


def test_serving_matches_layer_forward(cuda):
    """The server's batched path gives the same output as converting + running the layers directly."""
    ws, specs = net()
    reqs = make_requests(6, seed=3)
    server = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=8, max_lanes=2)
    res = server.infer(reqs)
    L = max(len(r.indices) for r in reqs)
    idx = np.full((6, L), -1, np.int32)
    tm = np.zeros((6, L), np.float32)
    for q, r in enumerate(reqs):
        idx[q, :len(r.indices)] = r.indices
        tm[q, :len(r.times)] = r.times
    x, _ = K.convert_to_spike_per_neuron(torch.tensor(idx, device="cuda"), torch.tensor(tm, device="cuda"), 700,
                                         k_cap=32)
    for w, sp in zip(ws, specs):
        ev = K.sort_events(x, np.float32(sp.tau_s), np.float32(2 * sp.tau_s), bucketed=False)
        n, a, xx, t, z = K.lif_forward_fc(ev, K.transpose_weights(torch.tensor(w, device="cuda")), sp.n_neurons,
                                          sp.max_n_spike, sp.tau_s, sp.theta, sp.delta_theta)
        x = t
    for q, r in enumerate(res):
        np.testing.assert_array_equal(r.counts, n[q].cpu().numpy())
        np.testing.assert_array_equal(r.spike_times, x[q].cpu().numpy())


def test_autotuned_variants_give_the_same_results(cuda):
    """Per-bucket kernel choices change speed only: results equal those of the untuned server."""
    ws, specs = net()
    reqs = make_requests(24, seed=5)
    plain = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=8, max_lanes=2).infer(reqs)
    tuned_server = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=8, max_lanes=2)
    table = tuned_server.autotune(reqs)
    assert set(table) == {1, 2, 4, 8}
    tuned = tuned_server.infer(make_requests(24, seed=5, rid0=500))
    for p, q in zip(plain, tuned):
        np.testing.assert_array_equal(p.counts, q.counts)
        np.testing.assert_array_equal(p.spike_times, q.spike_times)


def test_poisson_arrivals_complete_with_latency_stats(cuda):
    ws, specs = net()
    server = InferenceServer(ws, specs, 700, 5000, k_in=32, max_batch=16, max_lanes=3)
    reqs = make_requests(200, seed=2)
    res = run_poisson(server, reqs, rate=2000.0)
    assert len(res) == 200 and not server.rejected
    st = latency_stats(res)
    assert st["p99_ms"] >= st["p50_ms"] > 0
    assert server.batches_launched > 1


def test_intensity_encoding_matches_the_reference_formula(cuda):
    """experiments/mnist/Dataset.py:66-71 in NumPy (float64) vs the device encoder."""
    rng = np.random.default_rng(0)
    px = rng.integers(0, 256, (7, 784)).astype(np.uint8)
    px[0, :10] = 0
    px[1, :10] = 255
    t, n = K.intensity_to_spike_times(torch.tensor(px, device="cuda"))
    ref = (100e-3 * (1 - (px.reshape(7, 784, 1) / 255)))
    ref[ref == 100e-3] = np.inf
    np.testing.assert_array_equal(t.cpu().numpy(), ref.astype(np.float32))
    np.testing.assert_array_equal(n.cpu().numpy(), np.isfinite(ref).astype(np.int32).reshape(7, 784))
