"""The per-event no-crossing screen of the FC forward (no_crossing, bats_gb300/csrc/common.cuh) is conservative:
whenever it claims that the reference solver accepts no crossing after an event, no value of __expf and
__logf within their documented error bounds lets the reference accept one
(bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83; the solve is called with the event's time
as the last spike and the next event's time as the window's end, :118-134).

Host emulation (tests/_float_model.py) on states built with a root just outside the window — the edge of the
proof — with the event table's exp(t/tau) taken at the end of its error interval that makes the screen claim
the most. Each test also plants a too-small margin in the emulated screen and checks that the cases catch it."""
import numpy as np

from tests._float_model import (F, expf_range, logf_range, no_crossing, reference_may_accept, reference_root,
                                states_with_root_near, ulp32)

TAUS = (F(0.02), F(0.26), F(2.0))
THETAS = (0.2, 1.0, 1.3)
NO_T = F(-np.inf)


def _right_cases(rng, n, tau, theta, x_lo, x_hi, u_lo, u_hi, delta_lo):
    """States whose smaller root lies u (in units of 2^-20, relative) right of the lowest value __expf may
    give for the next event's exp(t/tau), t/tau uniform in [x_lo, x_hi)."""
    c = F(F(theta) / tau)
    t_next = (rng.uniform(x_lo, x_hi, n) * np.float64(tau)).astype(F)
    e_lo, _ = expf_range(t_next, tau)
    u = rng.uniform(u_lo, u_hi, n) * 2.0 ** -20
    delta = np.exp(rng.uniform(np.log(delta_lo), 0.0, n))
    a, b = states_with_root_near(e_lo.astype(np.float64), u, delta, c)
    return c, t_next, e_lo, a, b


def test_right_of_window_claims_are_never_accepted():
    rng = np.random.default_rng(11)
    claims = planted = 0
    for tau in TAUS:
        for theta in THETAS:
            c, t_next, e_lo, a, b = _right_cases(rng, 300_000, tau, theta, 0.2, 8.2, -2.0, 12.0, 1e-6)
            may = reference_may_accept(a, b, NO_T, t_next, c, tau, F(np.inf))
            claim = no_crossing(a, b, 0.0, e_lo, c, left=False)
            assert not (claim & may).any(), "the screen claimed a window in which the reference may spike"
            claims += int(claim.sum())
            planted += int((no_crossing(a, b, 0.0, e_lo, c, widen=2.0 ** -20, left=False) & may).sum())
    assert claims > 100_000, claims
    assert planted > 0, "a widening of 2^-20 should be too small"


def test_right_of_window_near_eight_tau():
    """Windows ending just below 8 tau, where the root can pass e^8 and __logf's 3 ulp double: the screen's
    limit Z < 2980 keeps them out; the limit Z < 2981 (a planted mistake) claims some the reference may
    accept."""
    rng = np.random.default_rng(12)
    planted = 0
    for tau in TAUS:
        for theta in THETAS:
            c, t_next, e_lo, a, b = _right_cases(rng, 400_000, tau, theta, 8 - 6e-6, 8 + 3e-7, 2.5, 5.0, 1e-2)
            may = reference_may_accept(a, b, NO_T, t_next, c, tau, F(np.inf))
            assert not (no_crossing(a, b, 0.0, e_lo, c, left=False) & may).any()
            planted += int((no_crossing(a, b, 0.0, e_lo, c, cap=2981.0, left=False) & may).sum())
    assert planted > 0, "the limit Z < 2981 should let a claim through"


def test_window_ending_at_max_simulation():
    """Last event of the sample (next event at +inf): the window ends at max_sim, whose exp(max_sim/tau) the
    library rounds from double."""
    rng = np.random.default_rng(13)
    claims = 0
    for tau in TAUS:
        for theta in THETAS:
            n = 200_000
            c = F(F(theta) / tau)
            max_sim = F(rng.uniform(0.2, 8.0) * np.float64(tau))
            e_max = F(np.exp(np.float64(max_sim) / np.float64(tau)))
            u = rng.uniform(-2.0, 12.0, n) * 2.0 ** -20
            delta = np.exp(rng.uniform(np.log(1e-6), 0.0, n))
            a, b = states_with_root_near(np.full(n, np.float64(e_max)), u, delta, c)
            may = reference_may_accept(a, b, NO_T, F(np.inf), c, tau, max_sim)
            claim = no_crossing(a, b, 0.0, F(np.inf), c, e_max=e_max, left=False)
            assert not (claim & may).any()
            claims += int(claim.sum())
    assert claims > 50_000, claims


def test_left_of_window_claims_are_never_accepted():
    """States whose smaller root lies just before the event (Z_lo between the roots), or whose larger root does
    (both roots before it), with the event's exp(t/tau) at the top of __expf's interval. Half the roots lie
    within 6 x 2^-20 of the event, where a margin of 2^-21 (planted) is too small; the screen's 2^-17 is
    eight times what the model needs."""
    rng = np.random.default_rng(14)
    claims = planted = 0
    for tau in TAUS:
        for theta in THETAS:
            for larger in (False, True):
                n = 200_000
                c = F(F(theta) / tau)
                t_ev = (rng.uniform(0.2, 8.05, n) * np.float64(tau)).astype(F)
                _, e_hi = expf_range(t_ev, tau)
                u = np.where(rng.random(n) < 0.5, rng.uniform(-24.0, 2.0, n), rng.uniform(-6.0, 2.0, n)) * 2.0 ** -20
                delta = np.exp(rng.uniform(np.log(1e-6), 0.0, n))
                a, b = states_with_root_near(e_hi.astype(np.float64), u, delta, c, larger=larger)
                may = reference_may_accept(a, b, t_ev, F(np.inf), c, tau, F(np.inf))
                claim = no_crossing(a, b, e_hi, F(np.inf), c)
                assert not (claim & may).any(), "the screen claimed a crossing the reference may accept"
                claims += int(claim.sum())
                planted += int((no_crossing(a, b, e_hi, F(np.inf), c, margin=2.0 ** -21) & may).sum())
    assert claims > 200_000, claims
    assert planted > 0, "a left margin of 2^-21 should be too small"


def test_model_reproduces_the_root_and_brackets_the_log():
    """Sanity of the model itself: the emulated root of a state built with a known root is within 2^-21 of it,
    and the __logf interval contains the exact logarithm and is a few ulp wide."""
    rng = np.random.default_rng(15)
    c = F(1.0 / 0.26)
    x = np.exp(rng.uniform(0.0, 8.0, 10_000))
    a, b = states_with_root_near(x, 0.0, np.full(10_000, 0.3), c)
    ok, z = reference_root(a, b, c)
    assert ok.all()
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    z1 = 2 * a64 / (b64 + np.sqrt(b64 * b64 - 4 * a64 * np.float64(c)))
    assert np.all(np.abs(z / z1 - 1) < 2.0 ** -21)
    lo, hi = logf_range(z)
    l = np.log(z.astype(np.float64))
    assert np.all(lo <= l) and np.all(hi >= l)
    assert np.all((hi.astype(np.float64) - lo) <= 8 * ulp32(l.astype(F)) + 2 * 2.0 ** -21.41)


def test_conv_right_of_window_claims_are_never_accepted():
    """The conv layer's screen (right-of-window test with the float discriminant's extra slack; no left test)
    against the conv solver (compute_spike_times_conv.cu:59-77) under every evaluation order of its float
    discriminant, with roots from near-tangent (delta 1e-9) to far apart (1e6). The slack and the widening
    together carry the margin: a screen with a widening of 2^-20 and no slack (a planted mistake) claims some
    windows the reference may accept."""
    rng = np.random.default_rng(16)
    claims = planted = 0
    for tau in TAUS:
        for theta in THETAS:
            n = 200_000
            c = F(F(theta) / tau)
            t_next = (rng.uniform(0.2, 8.2, n) * np.float64(tau)).astype(F)
            e_lo, _ = expf_range(t_next, tau)
            u = rng.uniform(-2.0, 12.0, n) * 2.0 ** -20
            delta = np.exp(rng.uniform(np.log(1e-9), np.log(1e6), n))
            a, b = states_with_root_near(e_lo.astype(np.float64), u, delta, c)
            may = reference_may_accept(a, b, NO_T, t_next, c, tau, F(np.inf), conv=True)
            claim = no_crossing(a, b, 0.0, e_lo, c, conv=True)
            assert not (claim & may).any(), "the conv screen claimed a window in which the reference may spike"
            claims += int(claim.sum())
            planted += int((no_crossing(a, b, 0.0, e_lo, c, conv=True, widen=2.0 ** -20, conv_slack=0.0) & may).sum())
    assert claims > 100_000, claims
    assert planted > 0, "a widening of 2^-20 without the slack should be too small"


def test_sweep_script_runs_clean_at_small_size():
    """tests/screen_sweep.py (the same checks with c and tau drawn over wide ranges, for large host runs)
    finds no violation on a small run."""
    import json
    import os
    import subprocess
    import sys
    script = os.path.join(os.path.dirname(os.path.abspath(__file__)), "screen_sweep.py")
    r = subprocess.run([sys.executable, script, "--cases-per-kind", "250000", "--workers", "2", "--seed", "7"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    kinds = json.loads(r.stdout.strip().splitlines()[-1])["kinds"]
    assert all(k["violations"] == 0 and k["claims"] > 0 for k in kinds.values()), kinds
