"""Monitors (bats/Monitors/*.py interface) on CPU tensors: the values the reference's numpy versions give."""
import numpy as np

from bats_gb300.Monitors import (AccuracyMonitor, LossMonitor, MonitorsManager, SilentLabelsMonitor,
                                 SilentNeuronsMonitor, SpikeCountMonitor, ValueMonitor, WeightsNormMonitor)


def test_monitor_values(tmp_path):
    rng = np.random.default_rng(0)
    pred = rng.integers(0, 10, 50)
    tgt = rng.integers(0, 10, 50)
    acc = AccuracyMonitor(export_path=tmp_path / "acc")
    acc.add(pred[:20], tgt[:20])
    acc.add(pred[20:], tgt[20:])
    assert np.isclose(acc.record(1.0), np.mean(pred == tgt) * 100)
    losses = np.array([1.0, np.inf, 3.0, np.nan, 5.0])
    lm = LossMonitor()
    lm.add(losses)
    assert np.isclose(lm.record(1.0), 3.0)
    n_out = rng.integers(0, 3, (50, 10))
    sl = SilentLabelsMonitor()
    sl.add(n_out, tgt)
    assert np.isclose(sl.record(1.0), np.mean(n_out[np.arange(50), tgt] == 0) * 100)
    sn = SilentNeuronsMonitor("h")
    sn.add(n_out[:25])
    sn.add(n_out[25:])
    assert np.isclose(sn.record(1.0), np.mean(n_out.sum(0) == 0) * 100)
    sc = SpikeCountMonitor("h")
    sc.add(n_out)
    assert np.isclose(sc.record(1.0), n_out.sum() / 50)
    W = rng.normal(size=(4, 5)).astype(np.float32)
    wn = WeightsNormMonitor("h")
    wn.add(W)
    assert np.isclose(wn.record(1.0), np.linalg.norm(W), rtol=1e-6)
    v = ValueMonitor(name="lr")
    v.add(0.5)
    assert v.record(1.0) == 0.5
    mgr = MonitorsManager([acc, lm])
    mgr.print(1.0)
    acc.export()
    d = np.load(tmp_path / "acc.npz")
    assert d["values"].shape == (1,)
