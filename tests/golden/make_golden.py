"""Generates the golden fixtures of tests/golden/ from the reference's own unit tests.

Run where a checkout of the reference exists, naming it in BATS_REFERENCE:
    BATS_REFERENCE=<path to the reference checkout> python tests/golden/make_golden.py

The reference's tests (tests/**/*.py of Florian-BACHO/bats) import cupy and the bats package,
neither of which can run without its GPU stack. This script loads the test files themselves with
  * a NumPy stand-in for cupy (arrays get a .get() method),
  * a stand-in bats package whose kernel wrappers, layers, losses and optimizers are the float64
    oracle (oracle/bats_ref64.py),
and then
  1. runs every reference test method against the oracle and records pass/fail
     (reference_tests_vs_oracle.json) - this pins the oracle to the reference's own assertions,
     known-answer arrays and CPU-loop oracles;
  2. evaluates the tests' CPU-loop oracles (pure NumPy methods of the test classes) on seeded
     inputs of the tests' shapes and saves inputs + expected outputs as .npz fixtures, together
     with the known-answer arrays the tests hold, for the GPU parity tests (the machines that run them
     hold no reference checkout).
Tests that need brian2 (the simulator ground truth) are recorded as skipped; the oracle is
cross-checked against a fixed-step integrator instead (tests/test_oracle.py).
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys
import types
import unittest

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import bats_ref64 as R  # noqa: E402

REF = os.environ.get("BATS_REFERENCE", "")


# ---- NumPy stand-in for cupy ----------------------------------------------------------------

class GArray(np.ndarray):
    def get(self):
        return np.asarray(self)


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, GArray):
        return x.view(GArray)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    return x


def _make_cupy():
    cp = types.ModuleType("cupy")

    def array(x, dtype=None, copy=True):
        return np.array(np.asarray(x), dtype=dtype).view(GArray)

    cp.array = array
    cp.asarray = array
    cp.ndarray = np.ndarray

    class _Random:
        def normal(self, loc=0.0, scale=1.0, size=None, dtype=np.float64):
            return np.random.normal(loc, scale, size).astype(dtype).view(GArray)

        def uniform(self, low=0.0, high=1.0, size=None, dtype=np.float64):
            return np.random.uniform(low, high, size).astype(dtype).view(GArray)

    cp.random = _Random()

    def __getattr__(name):
        obj = getattr(np, name)
        if callable(obj) and not isinstance(obj, type):
            def f(*a, **k):
                return _wrap(obj(*[np.asarray(v) if isinstance(v, GArray) else v for v in a], **k))
            return f
        return obj

    cp.__getattr__ = __getattr__
    return cp


# ---- oracle-backed stand-ins of the bats wrappers --------------------------------------------

def _np(x):
    return np.asarray(x)


def w_compute_pre_exps(spike_times, tau_s, tau):
    es, e = R.compute_pre_exps(_np(spike_times), float(tau_s), float(tau))
    return _wrap(es.astype(np.float32)), _wrap(e.astype(np.float32))


def w_get_sorted_spikes_indices(spike_times_per_neuron, n_spike_per_neuron):
    t = _np(spike_times_per_neuron)
    B, N, K = t.shape
    S = int(_np(n_spike_per_neuron).sum(1).max())
    reshaped = t.reshape(B, N * K)
    idx = np.argsort(reshaped, axis=1, kind="stable")[:, :S]
    return (B, N * K), _wrap(idx), _wrap(reshaped)


def w_convert_to_spike_per_neuron(indices, times, n_neurons):
    t, n = R.convert_to_spike_per_neuron(_np(indices), _np(times), int(n_neurons))
    return _wrap(t.astype(np.float32)), _wrap(n)


def w_get_spike_weights(weights, spike_indices):
    w = _np(weights)
    idx = _np(spike_indices)
    return _wrap(np.transpose(w[:, idx], (1, 0, 2)).astype(np.float32))


def w_aggregate_spikes_conv(n_spikes, spike_times, pre_shape, post_shape):
    n, t, i = R.aggregate_spikes_conv(_np(n_spikes), _np(spike_times), tuple(int(v) for v in _np(pre_shape)))
    return _wrap(n), _wrap(t.astype(np.float32)), _wrap(i.astype(np.int32))


def w_compute_factors(spike_times, a, c, x, exp_tau, tau):
    f1, f2 = R.compute_factors(_np(spike_times), _np(a).astype(np.float64), float(c), _np(x).astype(np.float64),
                               _np(exp_tau).astype(np.float64), float(tau))
    return _wrap(f1.astype(np.float32)), _wrap(f2.astype(np.float32))


def w_propagate_recurrent_errors(x, exp_tau, errors, delta_theta_tau):
    e = errors.astype(np.float64)
    R.propagate_recurrent_errors(_np(x), _np(exp_tau), e, float(delta_theta_tau))
    errors[...] = e


def w_compute_weights_gradient(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, errors):
    return _wrap(R.compute_weights_gradient(_np(f1), _np(f2), _np(post_times),
                                            (_np(pre_times), _np(pre_exp_tau_s), _np(pre_exp_tau)), _np(errors)))


def w_propagate_errors_to_pre_spikes(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, weights, errors,
                                     tau_s, tau):
    return _wrap(R.propagate_errors_to_pre_spikes(_np(f1), _np(f2), _np(post_times),
                                                  (_np(pre_times), _np(pre_exp_tau_s), _np(pre_exp_tau)),
                                                  _np(weights), _np(errors), float(tau_s), float(tau)))


def w_compute_weights_gradient_conv(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, pre_shape, post_shape,
                                    filter_shape, errors):
    return _wrap(R.conv_weights_gradient(_np(f1), _np(f2), _np(post_times),
                                         (_np(pre_times), _np(pre_exp_tau_s), _np(pre_exp_tau)), _np(errors),
                                         tuple(int(v) for v in _np(filter_shape)),
                                         tuple(int(v) for v in _np(pre_shape))))


def connectivity(pre_shape, post_shape, filter_shape):
    """(N_post, N_pre) mask of receptive-field pairs of a valid conv."""
    X, Y, C = pre_shape
    Xo, Yo, Co = post_shape
    _, fx, fy, _ = filter_shape
    m = np.zeros((Xo, Yo, Co, X, Y, C), dtype=bool)
    for xo in range(Xo):
        for yo in range(Yo):
            m[xo, yo, :, xo:xo + fx, yo:yo + fy, :] = True
    return m.reshape(Xo * Yo * Co, X * Y * C)


def w_propagate_errors_to_pre_spikes_conv(f1, f2, post_times, pre_times, pre_exp_tau_s, pre_exp_tau, weights, errors,
                                          tau_s, tau, pre_shape, post_shape, filter_shape):
    ps, qs, fs = (tuple(int(v) for v in _np(s)) for s in (pre_shape, post_shape, filter_shape))
    w = _np(weights)
    if w.ndim == 2:  # the test passes a dense (N_post, N_pre) matrix, used on connected pairs only
        dense = np.where(connectivity(ps, qs, fs), w, 0.0)
    else:
        dense = R.conv_dense_weights(w, ps)
    return _wrap(R.propagate_errors_to_pre_spikes(_np(f1), _np(f2), _np(post_times),
                                                  (_np(pre_times), _np(pre_exp_tau_s), _np(pre_exp_tau)),
                                                  dense, _np(errors), float(tau_s), float(tau)))


class OracleInputLayer:
    def __init__(self, n_neurons, name=""):
        self.n_neurons = n_neurons
        self.name = name
        self.trainable = False
        self.spike_trains = (None, None)

    def set_spike_trains(self, t, n):
        self.spike_trains = (_wrap(np.asarray(t, dtype=np.float64)), _wrap(np.asarray(n)))
        RECORD.setdefault("input_layer_sets", []).append((np.array(t, dtype=np.float64), np.array(n)))

    def forward(self, max_simulation, training=False):
        pass


class OracleLIFLayer:
    def __init__(self, previous_layer, n_neurons, tau_s, theta, delta_theta, weight_initializer=None, max_n_spike=32,
                 name=""):
        self.prev = previous_layer
        self.n_neurons = n_neurons
        self.name = name
        self.tau_s, self.theta, self.delta_theta, self.K = float(tau_s), float(theta), float(delta_theta), max_n_spike
        self.tau = 2 * self.tau_s
        w = weight_initializer(n_neurons, previous_layer.n_neurons) if weight_initializer else \
            np.zeros((n_neurons, previous_layer.n_neurons))
        self._w = _wrap(np.asarray(w, dtype=np.float64))
        RECORD.setdefault("lif_layers", []).append(dict(n_neurons=n_neurons, tau_s=self.tau_s, theta=self.theta,
                                                        delta_theta=self.delta_theta, max_n_spike=max_n_spike,
                                                        weights=np.array(self._w)))

    trainable = True

    @property
    def weights(self):
        return self._w

    @weights.setter
    def weights(self, w):
        self._w = _wrap(np.array(w, dtype=np.float64))

    def reset(self):
        pass

    def forward(self, max_simulation, training=False):
        pt, _ = self.prev.spike_trains
        self.max_sim = float(max_simulation)
        self.out = R.lif_forward(np.asarray(pt), np.asarray(self._w), self.tau_s, self.theta, self.delta_theta,
                                 self.K, self.max_sim)
        self.pre = np.asarray(pt)

    @property
    def spike_trains(self):
        n, a, x, t, z = self.out
        return _wrap(t), _wrap(n)

    def backward(self, errors):
        n, a, x, t, z = self.out
        e = np.asarray(errors, dtype=np.float64).copy()
        R.propagate_recurrent_errors(x, z, e, self.delta_theta / self.tau)
        f1, f2 = R.compute_factors(t, a, self.theta / self.tau, x, z, self.tau)
        es, ee = R.compute_pre_exps(self.pre, self.tau_s, self.tau)
        g = R.compute_weights_gradient(f1, f2, t, (self.pre, es, ee), e)
        return _wrap(g), None

    def add_deltas(self, d):
        self._w += np.asarray(d)

    def store(self, dir_path):
        np.save(dir_path / (self.name + "_weights.npy"), np.asarray(self._w))

    def restore(self, dir_path):
        f = dir_path / (self.name + "_weights.npy")
        if f.exists():
            self.weights = np.load(f)


class OracleSpikeCountClassLoss:
    def __init__(self, target_true, target_false):
        self.tt, self.tf = float(np.float32(target_true)), float(np.float32(target_false))

    def _targets(self, n, labels):
        return R.class_targets(np.asarray(labels), np.asarray(n).shape[1], self.tt, self.tf)

    def compute_loss(self, spikes, n, labels):
        return _wrap(R.spike_count_loss(np.asarray(n), self._targets(n, labels), 1)[0])

    def compute_errors(self, spikes, n, labels):
        return _wrap(R.spike_count_loss(np.asarray(n), self._targets(n, labels), np.asarray(spikes).shape[2])[1])

    def compute_loss_and_errors(self, spikes, n, labels):
        loss, err = R.spike_count_loss(np.asarray(n), self._targets(n, labels), np.asarray(spikes).shape[2])
        return _wrap(loss), _wrap(err)


class OracleTTFS:
    def __init__(self, tau):
        self.tau = float(tau)

    def compute_loss(self, spikes, n, labels):
        return _wrap(R.ttfs_softmax_cross_entropy(np.asarray(spikes), np.asarray(labels), self.tau)[0])

    def compute_errors(self, spikes, n, labels):
        return _wrap(R.ttfs_softmax_cross_entropy(np.asarray(spikes), np.asarray(labels), self.tau)[1])

    def compute_loss_and_errors(self, spikes, n, labels):
        return _wrap(R.ttfs_softmax_cross_entropy(np.asarray(spikes), np.asarray(labels), self.tau))


class OracleAdam:
    def __init__(self, learning_rate, beta_1=0.9, beta_2=0.999, epsilon=1e-8):
        self.o = R.Adam(learning_rate, beta_1, beta_2, epsilon)

    def step(self, grads):
        return [None if d is None else _wrap(d) for d in self.o.step([None if g is None else np.asarray(g)
                                                                      for g in grads])]


class OracleGD:
    def __init__(self, learning_rate):
        self.lr = float(np.float32(learning_rate))

    def step(self, grads):
        return [None if g is None else _wrap(-self.lr * np.asarray(g)) for g in grads]


RECORD: dict = {}


def install_fakes():
    sys.modules["cupy"] = _make_cupy()
    sys.modules["brian2"] = types.ModuleType("brian2")
    mods = {}
    for name in ["bats", "bats.CudaKernels", "bats.CudaKernels.Wrappers", "bats.CudaKernels.Wrappers.Inference",
                 "bats.CudaKernels.Wrappers.Backpropagation", "bats.Layers", "bats.Losses", "bats.Optimizers"]:
        mods[name] = types.ModuleType(name)
        sys.modules[name] = mods[name]
    inf = mods["bats.CudaKernels.Wrappers.Inference"]
    inf.compute_pre_exps = w_compute_pre_exps
    inf.get_sorted_spikes_indices = w_get_sorted_spikes_indices
    inf.convert_to_spike_per_neuron = w_convert_to_spike_per_neuron
    inf.get_spike_weights = w_get_spike_weights
    inf.aggregate_spikes_conv = w_aggregate_spikes_conv
    inf.compute_spike_times = None
    inf.compute_spike_times_conv = None
    bp = mods["bats.CudaKernels.Wrappers.Backpropagation"]
    bp.compute_factors = w_compute_factors
    bp.propagate_recurrent_errors = w_propagate_recurrent_errors
    bp.compute_weights_gradient = w_compute_weights_gradient
    bp.propagate_errors_to_pre_spikes = w_propagate_errors_to_pre_spikes
    bp.compute_weights_gradient_conv = w_compute_weights_gradient_conv
    bp.propagate_errors_to_pre_spikes_conv = w_propagate_errors_to_pre_spikes_conv
    bp.compute_bias_gradient = None
    mods["bats.Layers"].InputLayer = OracleInputLayer
    mods["bats.Layers"].LIFLayer = OracleLIFLayer
    mods["bats.Losses"].SpikeCountClassLoss = OracleSpikeCountClassLoss
    mods["bats.Losses"].TTFSSoftmaxCrossEntropy = OracleTTFS
    mods["bats.Optimizers"].AdamOptimizer = OracleAdam
    mods["bats.Optimizers"].GradientDescentOptimizer = OracleGD


def load_test_module(rel):
    path = os.path.join(REF, "tests", rel)
    spec = importlib.util.spec_from_file_location("reftest_" + rel.replace("/", "_")[:-3], path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


TEST_FILES = [
    "CudaKernels/Inference/compute_pre_exps_tests.py",
    "CudaKernels/Inference/convert_to_spike_per_neuron_tests.py",
    "CudaKernels/Inference/get_sorted_spikes_indices_tests.py",
    "CudaKernels/Inference/get_spike_weights_tests.py",
    "CudaKernels/Inference/aggregate_spikes_conv.py",
    "CudaKernels/Inference/compute_spike_times_tests.py",
    "CudaKernels/Inference/compute_spike_times_conv_tests.py",
    "CudaKernels/Backpropagation/compute_factors_tests.py",
    "CudaKernels/Backpropagation/propagate_recurrent_errors_tests.py",
    "CudaKernels/Backpropagation/compute_weights_gradient_tests.py",
    "CudaKernels/Backpropagation/propagate_errors_to_pre_spikes_tests.py",
    "CudaKernels/Backpropagation/compute_weights_gradient_conv_tests.py",
    "CudaKernels/Backpropagation/propagate_errors_to_pre_spikes_conv_tests.py",
    "CudaKernels/Backpropagation/compute_bias_gradient_tests.py",
    "Layers/LIFLayer_tests.py",
    "Losses/SpikeCountLoss_tests.py",
    "Losses/TTFSSoftmaxCrossEntropy_tests.py",
    "Optimizers/AdamOptimizer.py",
    "Optimizers/GradientDescentOptimizer.py",
]

NEEDS_BRIAN2 = {"test_compute_spike_times", "test_forward"}
OUT_OF_SCOPE = {"test_compute_bias_gradient"}  # bias gradient: no layer has a bias


def run_reference_tests():
    results = {}
    for rel in TEST_FILES:
        mod = load_test_module(rel)
        for cname in dir(mod):
            cls = getattr(mod, cname)
            if not (isinstance(cls, type) and issubclass(cls, unittest.TestCase)):
                continue
            for mname in sorted(m for m in dir(cls) if m.startswith("test")):
                key = f"{rel}::{cname}.{mname}"
                if mname in NEEDS_BRIAN2:
                    results[key] = "skipped: needs brian2 (simulator ground truth)"
                    continue
                if mname in OUT_OF_SCOPE:
                    results[key] = "skipped: bias gradient is not on the path"
                    continue
                np.random.seed(1234)
                case = cls(mname)
                res = unittest.TestResult()
                case.run(res)
                if res.wasSuccessful():
                    results[key] = "passed"
                else:
                    err = (res.failures + res.errors)[0][1].strip().splitlines()[-1]
                    results[key] = "FAILED: " + err
                print(f"{results[key][:60]:60s} {key}")
    return results


def make_fixtures():
    """Seeded inputs of the reference tests' shapes with the tests' own CPU-loop oracles' outputs."""
    out = {}
    inst = lambda rel, cname: getattr(load_test_module(rel), cname)("run")  # noqa: E731

    rng = np.random.default_rng(7)
    # compute_weights_gradient_tests.py:26-54 and propagate_errors_to_pre_spikes_tests.py:33-64 shapes.
    B, n_pre, n_post, kpre, kpost, tau_s = 10, 20, 10, 25, 12, 0.1
    tau = 2 * tau_s
    f1 = rng.uniform(0, 1.0, (B, n_post, kpost)).astype(np.float32)
    f2 = rng.uniform(0, 1.0, (B, n_post, kpost)).astype(np.float32)
    pre_t = np.sort(rng.uniform(0, 1.0, (B, n_pre, kpre)), axis=2).astype(np.float32)
    post_t = np.sort(rng.uniform(0, 1.0, (B, n_post, kpost)), axis=2).astype(np.float32)
    # Some silent tails, as the layers produce them.
    pre_t[:, ::3, kpre // 2:] = np.inf
    post_t[:, ::4, kpost // 3:] = np.inf
    es = np.exp(pre_t.astype(np.float64) / tau_s).astype(np.float32)
    ee = np.exp(pre_t.astype(np.float64) / tau).astype(np.float32)
    err = rng.uniform(-1, 1, (B, n_post, kpost)).astype(np.float32)
    w = rng.normal(0, 1, (n_post, n_pre)).astype(np.float32)
    f64 = lambda a: a.astype(np.float64)  # noqa: E731
    t1 = inst("CudaKernels/Backpropagation/compute_weights_gradient_tests.py", "CudaKernelsTests")
    g = t1.compute_weights_gradient_cpu(f64(f1), f64(f2), f64(post_t), f64(pre_t), f64(es), f64(ee), f64(err))
    t2 = inst("CudaKernels/Backpropagation/propagate_errors_to_pre_spikes_tests.py", "CudaKernelsTests")
    pe = t2.propagate_errors_to_pre_spikes(f64(f1), f64(f2), f64(post_t), f64(pre_t), f64(es), f64(ee), f64(w),
                                           f64(err), tau_s, tau)
    np.savez_compressed(os.path.join(HERE, "fc_backward_kernels.npz"), f1=f1, f2=f2, pre_t=pre_t, post_t=post_t,
                        es=es, ee=ee, errors=err, weights=w, tau_s=tau_s, tau=tau, grad=g, pre_errors=pe)
    out["fc_backward_kernels"] = "compute_weights_gradient_tests.py:9-24, propagate_errors_to_pre_spikes_tests.py:9-31"

    # Conv kernels (compute_weights_gradient_conv_tests.py:47-87, propagate_errors_to_pre_spikes_conv_tests.py:49-92).
    B = 2
    pre_shape = np.array([10, 10, 3])
    filter_shape = np.array([2, 5, 5, 3])
    post_shape = np.array([6, 6, 2])
    n_pre, n_post, kpre, kpost = 300, 72, 5, 4
    f1 = rng.uniform(0, 1.0, (B, n_post, kpost)).astype(np.float32)
    f2 = rng.uniform(0, 1.0, (B, n_post, kpost)).astype(np.float32)
    pre_t = np.sort(rng.uniform(0, 1.0, (B, n_pre, kpre)), axis=2).astype(np.float32)
    post_t = np.sort(rng.uniform(0, 1.0, (B, n_post, kpost)), axis=2).astype(np.float32)
    pre_t[:, ::5, 2:] = np.inf
    es = np.exp(pre_t.astype(np.float64) / tau_s).astype(np.float32)
    ee = np.exp(pre_t.astype(np.float64) / tau).astype(np.float32)
    err = rng.uniform(-1, 1, (B, n_post, kpost)).astype(np.float32)
    filt = rng.normal(0, 1, tuple(filter_shape)).astype(np.float32)
    t3 = inst("CudaKernels/Backpropagation/compute_weights_gradient_conv_tests.py", "CudaKernelsTests")
    gc = t3.compute_weights_gradient_conv_cpu(f64(f1), f64(f2), f64(post_t), f64(pre_t), f64(es), f64(ee),
                                              pre_shape, post_shape, filter_shape, f64(err))
    dense = R.conv_dense_weights(filt, tuple(pre_shape))
    t4 = inst("CudaKernels/Backpropagation/propagate_errors_to_pre_spikes_conv_tests.py", "CudaKernelsTests")
    pec = t4.propagate_errors_to_pre_spikes(f64(f1), f64(f2), f64(post_t), f64(pre_t), f64(es), f64(ee), dense,
                                            f64(err), tau_s, tau, pre_shape, post_shape, filter_shape)
    np.savez_compressed(os.path.join(HERE, "conv_backward_kernels.npz"), f1=f1, f2=f2, pre_t=pre_t, post_t=post_t,
                        es=es, ee=ee, errors=err, filters=filt, pre_shape=pre_shape, post_shape=post_shape,
                        filter_shape=filter_shape, tau_s=tau_s, tau=tau, grad=gc, pre_errors=pec)
    out["conv_backward_kernels"] = ("compute_weights_gradient_conv_tests.py:17-45, "
                                    "propagate_errors_to_pre_spikes_conv_tests.py:18-47")

    # Factors (compute_factors_tests.py:9-33).
    a = rng.uniform(0.1, 10.0, (4, 6, 8)).astype(np.float32)
    x = rng.uniform(0.1, 10.0, (4, 6, 8)).astype(np.float32)
    st = np.sort(rng.uniform(0, 1.0, (4, 6, 8)), axis=2).astype(np.float32)
    st[:, ::2, 5:] = np.inf
    z = np.exp(st.astype(np.float64) / 0.2).astype(np.float32)
    t5 = inst("CudaKernels/Backpropagation/compute_factors_tests.py", "CudaKernelsTests")
    ff1, ff2 = t5.compute_f1_f2(f64(a), 1.0 / 0.2, f64(x), f64(z), 0.2)
    ff1 = np.where(np.isinf(st), 0.0, ff1)
    ff2 = np.where(np.isinf(st), 0.0, ff2)
    np.savez_compressed(os.path.join(HERE, "factors.npz"), a=a, x=x, spike_times=st, exp_tau=z, c=1.0 / 0.2, tau=0.2,
                        f1=ff1, f2=ff2)
    out["factors"] = "compute_factors_tests.py:9-12 (0 where no spike: compute_factors.cu:20-26)"

    # Pooling (aggregate_spikes_conv.py:18-61).
    pre_shape = np.array([10, 10, 3])
    idx = rng.integers(0, 300, size=(1, 100))
    tt = np.sort(rng.uniform(0, 1.0, size=(1, 100)), axis=1)
    tt[0, -30:] = np.inf
    idx[0, -30:] = -1
    sp_t, sp_n = R.convert_to_spike_per_neuron(idx, tt, 300)
    sp_t = sp_t.astype(np.float32)
    t6 = inst("CudaKernels/Inference/aggregate_spikes_conv.py", "CudaKernelsTests")
    pn, pt, pi = t6.aggregate_spikes_conv_cpu(sp_n, sp_t, pre_shape, np.array([5, 5, 3]))
    np.savez_compressed(os.path.join(HERE, "pooling.npz"), n_spikes=sp_n, spike_times=sp_t, pre_shape=pre_shape,
                        out_n=pn, out_t=pt, out_idx=pi)
    out["pooling"] = "aggregate_spikes_conv.py:18-61 (reference test file)"

    # Known-answer arrays captured from the test bodies.
    for key in ("kat_recurrent", "kat_ttfs", "kat_convert", "kat_lif_training"):
        if key in CAPTURE:
            np.savez_compressed(os.path.join(HERE, key + ".npz"), **CAPTURE[key])
            out[key] = CAPTURE_SRC[key]
    return out


CAPTURE: dict = {}
CAPTURE_SRC = {
    "kat_recurrent": "propagate_recurrent_errors_tests.py:20-50",
    "kat_ttfs": "TTFSSoftmaxCrossEntropy_tests.py:16-36, 49-68",
    "kat_convert": "convert_to_spike_per_neuron_tests.py:9-37",
    "kat_lif_training": "LIFLayer_tests.py:91-132",
}


def capture_known_answers():
    """Re-run the known-answer tests with recording stand-ins so that their fixed arrays and
    expected results can be saved."""
    inf = sys.modules["bats.CudaKernels.Wrappers.Inference"]
    bp = sys.modules["bats.CudaKernels.Wrappers.Backpropagation"]

    # Recurrent errors: inputs and the test's own CPU-loop result.
    mod = load_test_module("CudaKernels/Backpropagation/propagate_recurrent_errors_tests.py")
    orig = bp.propagate_recurrent_errors

    def rec(x, exp_tau, errors, dtt):
        e0 = np.array(errors, dtype=np.float64)
        ref = e0.copy()
        mod.CudaKernelsTests("run").prop_recurrent_errors(np.asarray(x, dtype=np.float64),
                                                          np.asarray(exp_tau, dtype=np.float64), ref, float(dtt))
        CAPTURE["kat_recurrent"] = dict(x=np.asarray(x), exp_tau=np.asarray(exp_tau), errors=e0, delta_theta_tau=dtt,
                                        expected=ref)
        return orig(x, exp_tau, errors, dtt)

    mod.propagate_recurrent_errors = rec
    unittest.TestResult()
    mod.CudaKernelsTests("test_propagate_recurrent_errors").run(unittest.TestResult())

    # TTFS loss: fixed spikes and labels, expected from the test's CPU functions.
    mod = load_test_module("Losses/TTFSSoftmaxCrossEntropy_tests.py")

    class RecTTFS(OracleTTFS):
        def compute_loss_and_errors(self, spikes, n, labels):
            t = mod.TTFSSoftmaxCrossEntropy_tests("run")
            s64 = np.asarray(spikes, dtype=np.float64)
            CAPTURE["kat_ttfs"] = dict(spikes=np.asarray(spikes), labels=np.asarray(labels), tau=self.tau,
                                       loss=t.compute_loss_cpu(s64, np.asarray(labels), self.tau),
                                       errors=t.compute_errors_cpu(s64, np.asarray(labels), self.tau))
            return super().compute_loss_and_errors(spikes, n, labels)

    mod.TTFSSoftmaxCrossEntropy = RecTTFS
    mod.TTFSSoftmaxCrossEntropy_tests("test_compute_loss_and_errors").run(unittest.TestResult())

    # convert_to_spike_per_neuron: the test holds inputs and the exact expected arrays.
    mod = load_test_module("CudaKernels/Inference/convert_to_spike_per_neuron_tests.py")

    def conv_rec(indices, times, n):
        t, c = w_convert_to_spike_per_neuron(indices, times, n)
        CAPTURE["kat_convert"] = dict(indices=np.asarray(indices), times=np.asarray(times), n_neurons=int(n),
                                      spike_per_neuron=np.asarray(t), n_spike_per_neuron=np.asarray(c))
        return t, c

    mod.convert_to_spike_per_neuron = conv_rec
    res = unittest.TestResult()
    mod.CudaKernelsTests("test_convert_to_spike_per_neuron").run(res)
    CAPTURE["kat_convert"]["oracle_passed"] = res.wasSuccessful()

    # LIF training known answer: record the layer set-up, inputs and targets.
    mod = load_test_module("Layers/LIFLayer_tests.py")
    RECORD.clear()
    captured = {}
    orig_mse = mod.LifLayer_tests.ttfs_mse

    def mse(self, spikes, targets):
        captured["targets"] = np.asarray(targets)
        return orig_mse(self, spikes, targets)

    mod.LifLayer_tests.ttfs_mse = mse
    res = unittest.TestResult()
    mod.LifLayer_tests("test_backward").run(res)
    lif = RECORD["lif_layers"][0]
    t_in, n_in = RECORD["input_layer_sets"][0]
    CAPTURE["kat_lif_training"] = dict(spike_per_neuron=t_in, n_spike_per_neuron=n_in, targets=captured["targets"],
                                       n_post=lif["n_neurons"], tau_s=lif["tau_s"], theta=lif["theta"],
                                       delta_theta=lif["delta_theta"], max_n_spike=lif["max_n_spike"],
                                       weights0=lif["weights"], learning_rate=3e3, n_epoch=200,
                                       max_simulation=np.float32(0.02), atol=5e-4,
                                       oracle_passed=res.wasSuccessful())


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "tests")):
        raise SystemExit("set BATS_REFERENCE to a checkout of the reference (its tests/ folder was not found"
                         + (f" under {REF})" if REF else ")"))
    install_fakes()
    results = run_reference_tests()
    capture_known_answers()
    fixtures = make_fixtures()
    notes = {
        "CudaKernels/Inference/aggregate_spikes_conv.py::CudaKernelsTests.test_aggregate_spikes_conv":
            "counts, times and the source indices of every real spike agree; the test also compares the source "
            "indices of the +inf padding slots, whose order among equal (+inf) keys is whatever np.argsort's "
            "unstable sort returns; the oracle keeps them in concatenation order (stable). Those slots carry no "
            "spike and receive zero error in PoolingLayer.backward.",
    }
    with open(os.path.join(HERE, "reference_tests_vs_oracle.json"), "w") as f:
        json.dump({"results": results, "notes": notes, "fixtures": fixtures}, f, indent=1, sort_keys=True)
    n_pass = sum(v == "passed" for v in results.values())
    print(f"{n_pass}/{len(results)} reference tests passed against the oracle")


if __name__ == "__main__":
    main()
