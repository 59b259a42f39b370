"""The per-stage no-crossing screen of the FC forward (stage_no_crossing, bats_gb300/csrc/common.cuh) is
conservative: whenever it passes a stage, the reference solver accepts no crossing after any event of the
stage (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83: discriminant formed in double, root
z = 2a / (sqrt(tmp) + b), time tau * __logf(z), accepted in (last event or spike, next event]), for every value
of __logf and of the stage's first exp(t/tau) within their documented error bounds (tests/_float_model.py).
Host emulation in NumPy float32/float64 of both, on random stages chosen so that the screen's bound lies within 10 % of the
threshold (the cases where a loose proof would fail), with states of both signs, times from 0 to past 8 tau,
and windows that end at the next event or never."""
import numpy as np

from tests._float_model import F, expf_range, fmaf, reference_may_accept
from tests._float_model import stage_no_crossing as screen


def test_screen_never_passes_a_stage_with_a_crossing():
    """A broad sweep of random stages (few of which cross at all; the targeted test below builds crossing
    stages at the edge of the proof)."""
    rng = np.random.default_rng(7)
    tau_s = 0.13
    tau = 2 * tau_s
    passed = checked = 0
    for trial in range(10):
        n, sev = 200_000, 8
        theta = F(rng.choice([0.2, 1.0, 1.3]))
        c = F(theta / F(tau))
        t0 = rng.uniform(0.0, 2.5, (n, 1))                       # stage start up to ~10 tau
        dt = np.sort(rng.uniform(0.0, rng.choice([0.001, 0.02, 0.2]), (n, sev + 1)), axis=1)
        t = (t0 + dt).astype(F)                                  # event times of the stage, and the next event
        es = np.exp(t.astype(np.float64) / F(tau_s)).astype(F)
        e = np.exp(t.astype(np.float64) / F(tau)).astype(F)
        scale = rng.uniform(0.05, 3.0, (n, 1)) * np.exp(-t0 / tau)  # keeps V near the threshold
        w = (rng.normal(rng.uniform(-0.5, 1.0, (n, 1)), 1.0, (n, sev)) * scale).astype(F)
        a = (rng.normal(0.0, 1.0, n) * scale[:, 0] * e[:, 0]).astype(F)
        b = (rng.normal(0.5, 1.0, n) * scale[:, 0] * np.sqrt(e[:, 0])).astype(F)
        states_a, states_b = [], []
        aa, bb = a.copy(), b.copy()
        for u in range(sev):
            aa = fmaf(w[:, u], es[:, u], aa)
            bb = fmaf(w[:, u], e[:, u], bb)
            states_a.append(aa)
            states_b.append(bb)
        A, Bm = np.stack(states_a, 1), np.stack(states_b, 1)
        amin, bmax, amag = A.min(1), Bm.max(1), np.abs(A).min(1)
        ok = screen(amin, bmax, amag, aa, bb, expf_range(t[:, 0], tau)[1], c)
        # keep the hard cases: bound within 10 % of the threshold
        x0 = (e[:, 0] * F(1.0 - 2.0 ** -17)).astype(np.float64)
        bound = np.maximum(bmax, 0) / x0 + np.maximum(-amin, 0) / x0 ** 2
        hard = ok & (bound > 0.9 * c)
        passed += int(ok.sum())
        checked += int(hard.sum())
        never_ends = rng.random(n) < 0.3
        for u in range(sev):
            next_t = np.where(never_ends & (u == sev - 1), np.inf, t[:, u + 1]).astype(F)
            spk = reference_may_accept(A[:, u], Bm[:, u], t[:, u], next_t, c, tau, F(np.inf))
            bad = ok & spk
            assert not bad.any(), (f"screen passed a stage whose state {u} crosses: a={A[bad, u][:3]}, "
                                   f"b={Bm[bad, u][:3]}, t={t[bad, u][:3]}, c={c}")
    assert passed > 250_000 and checked > 2_000, (passed, checked)


def _crossing_stages(rng, n, tau_s, sev=8):
    """Stages whose state crosses the threshold just after the first event: a > 0 and b with
    b^2 = 4ac (1 + delta), the smaller root z1 = x_first (1 + eps), eps from 1e-7 (inside the screen's
    2^-17 margin) to 5e-2; the later events carry zero weight, so every state of the stage is (a, b)."""
    tau = 2 * tau_s
    theta = F(rng.choice([0.2, 1.0, 1.3]))
    c = F(theta / F(tau))
    delta = rng.uniform(1e-4, 0.05, n)
    t_first = rng.uniform(0.0, 2.0, n)
    x_first = np.exp(t_first / tau)
    eps = np.exp(rng.uniform(np.log(1e-7), np.log(5e-2), n))
    z1 = x_first * (1 + eps)
    s = np.sqrt(delta / (1 + delta))
    b = 2 * c * z1 / (1 - s)
    a = b * b / (4 * c * (1 + delta))
    t = np.empty((n, sev + 1))
    t[:, 0] = t_first
    span = rng.uniform(5e-4, 0.2, n)
    t[:, 1:] = (t_first + tau * np.log1p(eps) + 1e-6)[:, None] + np.sort(rng.uniform(0, 1, (n, sev)), 1) * span[:, None]
    t = t.astype(F)
    e = np.exp(t.astype(np.float64) / F(tau)).astype(F)
    A = np.repeat(a.astype(F)[:, None], sev, 1)
    Bm = np.repeat(b.astype(F)[:, None], sev, 1)
    return c, tau, t, e, A, Bm


def test_screen_rejects_stages_that_cross_just_after_their_first_event():
    """Almost every such stage crosses in the reference solver's arithmetic, and the screen passes none of those; a
    screen that took its bound from the stage's end instead of its start (a planted mistake, applied to the
    emulation only) passes some, which shows the cases reach the proof's edge."""
    rng = np.random.default_rng(3)
    planted_caught = 0
    for _ in range(5):
        c, tau, t, e, A, Bm = _crossing_stages(rng, 200_000, 0.13)
        spk = reference_may_accept(A[:, 0], Bm[:, 0], t[:, 0], t[:, 1], c, tau, F(np.inf))
        assert spk.mean() > 0.9  # the rest cross within a float ulp of the event and are rounded to it
        ok = screen(A.min(1), Bm.max(1), np.abs(A).min(1), A[:, -1], Bm[:, -1], expf_range(t[:, 0], tau)[1], c)
        assert not (ok & spk).any(), "the screen passed a stage that crosses"
        wrong = screen(A.min(1), Bm.max(1), np.abs(A).min(1), A[:, -1], Bm[:, -1], e[:, -1], c)
        planted_caught += int((wrong & spk).sum())
    assert planted_caught > 0
