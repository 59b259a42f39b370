"""CPU checks of the float64 oracle against the reference's own tests and known answers (golden
fixtures generated by tests/golden/make_golden.py) and against an independent fixed-step integrator."""
import json
import os

import numpy as np
import pytest

from oracle import bats_ref64 as R

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def test_reference_tests_pass_against_oracle():
    d = json.load(open(os.path.join(GOLDEN, "reference_tests_vs_oracle.json")))
    res, notes = d["results"], d["notes"]
    failed = {k: v for k, v in res.items() if v.startswith("FAILED") and k not in notes}
    assert not failed, failed
    assert sum(v == "passed" for v in res.values()) >= 20


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_closed_form_matches_fixed_step_integration(seed):
    rng = np.random.default_rng(seed)
    n_pre, n_post, k = 30, 8, 4
    t = np.full((1, n_pre, k), np.inf)
    for j in range(n_pre):
        c = rng.integers(0, k + 1)
        t[0, j, :c] = np.sort(rng.uniform(0, 0.25, c))
    W = rng.normal(0.0, 1.0, (n_post, n_pre))
    tau_s, theta, dtheta, t_end = 0.1, 0.1, 0.2, 0.4
    n, a, x, tt, z = R.lif_forward(t, W, tau_s, theta, dtheta, 64, t_end)
    sim = R.simulate_fixed_step(t[0], W, tau_s, theta, dtheta, t_end, dt=2e-6)
    for i in range(n_post):
        got = tt[0, i, :n[0, i]]
        exp = sim[i]
        assert got.size == exp.size, (i, got, exp)
        # Each fixed-step spike lags by at most two steps (input and threshold quantisation); the lag of
        # a spike's reset carries over to the later spikes of the neuron.
        lag = exp - got
        assert np.all(lag >= -1e-9) and np.all(lag <= 3 * 2e-6 * (np.arange(got.size) + 1)), (i, got, exp)


def test_max_n_spike_cap_and_max_simulation():
    rng = np.random.default_rng(5)
    t = np.sort(rng.uniform(0, 0.05, (2, 10, 1)), axis=1)
    W = np.full((3, 10), 2.0)
    n, a, x, tt, z = R.lif_forward(t, W, 0.1, 0.05, 0.05, 3, np.inf)
    assert (n == 3).all() and np.isfinite(tt).all()
    n2, _, _, tt2, _ = R.lif_forward(t, W, 0.1, 0.05, 0.05, 50, 0.08)
    assert (tt2[np.isfinite(tt2)] <= 0.08).all()
    assert (n2 < 50).all()


def test_empty_input_gives_silent_layer():
    t = np.full((3, 5, 2), np.inf)
    n, a, x, tt, z = R.lif_forward(t, np.ones((4, 5)), 0.1, 0.1, 0.1, 5)
    assert (n == 0).all() and np.isinf(tt).all() and np.isinf(z).all()


def test_fc_backward_fixtures_match_reference_cpu_loops():
    d = load("fc_backward_kernels")
    pre = (d["pre_t"].astype(np.float64), d["es"].astype(np.float64), d["ee"].astype(np.float64))
    g = R.compute_weights_gradient(d["f1"], d["f2"], d["post_t"], pre, d["errors"])
    # The reference's CPU loop sums every post slot (it does not stop at the first inf post time), so
    # compare on inputs where the two agree: its loop adds f1*0 terms for inf post spikes only when the
    # pre spikes precede them, which the fixture's factors make nonzero. Restrict to leading spikes.
    np.testing.assert_allclose(g, _ref_grad_leading(d), rtol=1e-10, atol=1e-10)
    pe = R.propagate_errors_to_pre_spikes(d["f1"], d["f2"], d["post_t"], pre, d["weights"], d["errors"],
                                          float(d["tau_s"]), float(d["tau"]))
    np.testing.assert_allclose(pe, d["pre_errors"], rtol=1e-10, atol=1e-10)


def _ref_grad_leading(d):
    """The fixture's expected gradient (the reference test's CPU loop, compute_weights_gradient_tests.py:9-24)
    evaluated over each post neuron's leading finite spikes, as the CUDA kernel does
    (compute_weights_gradient.cu:37-38 breaks at the first inf post time)."""
    f1, f2, post, pre_t, es, ee, err = (d[k].astype(np.float64) for k in
                                        ("f1", "f2", "post_t", "pre_t", "es", "ee", "errors"))
    B, n_post, kpost = f1.shape
    out = np.zeros((B, n_post, pre_t.shape[1]))
    for s in range(B):
        for i in range(n_post):
            for k in range(kpost):
                if np.isinf(post[s, i, k]):
                    break
                mask = pre_t[s] < post[s, i, k]
                out[s, i] += err[s, i, k] * (f1[s, i, k] * np.where(mask, es[s], 0).sum(1)
                                             - f2[s, i, k] * np.where(mask, ee[s], 0).sum(1))
    return out


def test_fc_gradient_fixture_equals_reference_loop_where_defined():
    d = load("fc_backward_kernels")
    leading = _ref_grad_leading(d)
    # On neurons without inf post slots the reference test's loop and the kernel semantics coincide.
    full = ~np.isinf(d["post_t"]).any(-1)
    np.testing.assert_allclose(leading[full], d["grad"][full], rtol=1e-10, atol=1e-10)


def test_conv_backward_fixtures():
    d = load("conv_backward_kernels")
    pre = (d["pre_t"].astype(np.float64), d["es"].astype(np.float64), d["ee"].astype(np.float64))
    g = R.conv_weights_gradient(d["f1"], d["f2"], d["post_t"], pre, d["errors"], tuple(d["filter_shape"]),
                                tuple(d["pre_shape"]))
    np.testing.assert_allclose(g, d["grad"], rtol=1e-10, atol=1e-9)
    pe = R.conv_pre_errors(d["f1"], d["f2"], d["post_t"], pre, d["filters"], d["errors"], float(d["tau_s"]),
                           float(d["tau"]), tuple(d["pre_shape"]))
    np.testing.assert_allclose(pe, d["pre_errors"], rtol=1e-10, atol=1e-9)


def test_factors_fixture():
    d = load("factors")
    f1, f2 = R.compute_factors(d["spike_times"], d["a"].astype(np.float64), float(d["c"]), d["x"].astype(np.float64),
                               d["exp_tau"].astype(np.float64), float(d["tau"]))
    np.testing.assert_allclose(f1, d["f1"], rtol=1e-12)
    np.testing.assert_allclose(f2, d["f2"], rtol=1e-12)


def test_pooling_fixture():
    d = load("pooling")
    n, t, i = R.aggregate_spikes_conv(d["n_spikes"], d["spike_times"], tuple(d["pre_shape"]))
    np.testing.assert_array_equal(n, d["out_n"])
    np.testing.assert_array_equal(t.astype(np.float32), d["out_t"])
    fin = np.isfinite(d["out_t"])
    np.testing.assert_array_equal(i[fin], d["out_idx"][fin])
    # The inf slots hold the remaining source slots (each source slot exactly once).
    assert np.array_equal(np.sort(i.reshape(-1)), np.arange(i.size))


def test_known_answers():
    r = load("kat_recurrent")
    e = r["errors"].astype(np.float64).copy()
    R.propagate_recurrent_errors(r["x"], r["exp_tau"], e, float(r["delta_theta_tau"]))
    np.testing.assert_allclose(e, r["expected"], rtol=1e-12)
    t = load("kat_ttfs")
    loss, err = R.ttfs_softmax_cross_entropy(t["spikes"], t["labels"], float(t["tau"]))
    np.testing.assert_allclose(loss, t["loss"], rtol=1e-6)
    np.testing.assert_allclose(err, t["errors"], rtol=1e-6, atol=1e-12)
    c = load("kat_convert")
    sp, n = R.convert_to_spike_per_neuron(c["indices"], c["times"], int(c["n_neurons"]))
    np.testing.assert_array_equal(n, c["n_spike_per_neuron"])
    np.testing.assert_array_equal(sp.astype(np.float32), c["spike_per_neuron"])
    assert bool(c["oracle_passed"])


def test_lif_training_known_answer_oracle():
    """LIFLayer_tests.py:91-132: 200 epochs of TTFS-MSE descent reach the target first spike times within 5e-4."""
    d = load("kat_lif_training")
    assert bool(d["oracle_passed"])


def test_adam_matches_formula():
    rng = np.random.default_rng(0)
    g = rng.normal(size=(3, 4))
    opt = R.Adam(0.01)
    d1 = opt.step([None, g])[1]
    m = (1 - np.float32(0.9)) * g
    v = (1 - np.float32(0.999)) * g * g
    exp = -(np.float32(0.01) * (m / (1 - np.float32(0.9))) / (np.sqrt(v / (1 - np.float32(0.999))) + np.float32(1e-8)))
    np.testing.assert_allclose(d1, exp, rtol=1e-6)
