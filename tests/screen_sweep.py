"""Large randomized sweep of the no-crossing screens (bats_gb300/csrc/common.cuh) against the host model of the
reference solver and of the intrinsics' documented error bounds (tests/_float_model.py): the checks of
tests/test_event_screen.py and tests/test_stage_screen.py, with the threshold c = theta/tau and tau drawn
log-uniformly over wide ranges instead of the networks' constants, and far more cases than a unit test runs.

    python tests/screen_sweep.py [--cases-per-kind N] [--workers W] [--seed S]

Prints one JSON line: per kind of case, the cases drawn, the screen's claims, and the claims the reference
may contradict (violations; every count must be 0). Runs on the host only, in spawned worker processes."""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from tests._float_model import (F, expf_range, fmaf, no_crossing, reference_may_accept,  # noqa: E402
                                stage_no_crossing, states_with_root_near)

KINDS = ("right", "right_8tau", "max_sim", "left", "conv", "stage")
CHUNK = 250_000


def _draw_c_tau(rng):
    tau = F(np.exp(rng.uniform(np.log(1e-3), np.log(10.0))))
    c = F(np.exp(rng.uniform(np.log(2.0 ** -30), np.log(2.0 ** 16))))
    return c, tau


def _delta(rng, n, lo=1e-9, hi=1e6):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def _chunk(kind, rng, n):
    """(claims, violations) of one chunk of one kind."""
    c, tau = _draw_c_tau(rng)
    with np.errstate(all="ignore"):
        if kind in ("right", "right_8tau", "conv"):
            lo, hi = (8 - 6e-6, 8 + 3e-7) if kind == "right_8tau" else (0.0, 8.2)
            t_next = (rng.uniform(lo, hi, n) * np.float64(tau)).astype(F)
            e_lo, _ = expf_range(t_next, tau)
            u = rng.uniform(-2.0, 12.0, n) * 2.0 ** -20
            ok = np.isfinite(e_lo) & (e_lo > 0)
            a, b = states_with_root_near(np.where(ok, e_lo, F(1)).astype(np.float64), u, _delta(rng, n), c)
            conv = kind == "conv"
            may = reference_may_accept(a, b, F(-np.inf), t_next, c, tau, F(np.inf), conv=conv)
            claim = ok & no_crossing(a, b, 0.0, e_lo, c, left=False, conv=conv)
        elif kind == "max_sim":
            max_sim = F(rng.uniform(0.0, 8.2) * np.float64(tau))
            e_max = F(np.exp(np.float64(max_sim) / np.float64(tau)))
            u = rng.uniform(-2.0, 12.0, n) * 2.0 ** -20
            a, b = states_with_root_near(np.full(n, np.float64(e_max)), u, _delta(rng, n), c)
            may = reference_may_accept(a, b, F(-np.inf), F(np.inf), c, tau, max_sim)
            claim = no_crossing(a, b, 0.0, F(np.inf), c, e_max=e_max, left=False)
        elif kind == "left":
            t_ev = (rng.uniform(0.0, 8.05, n) * np.float64(tau)).astype(F)
            _, e_hi = expf_range(t_ev, tau)
            u = rng.uniform(-24.0, 2.0, n) * 2.0 ** -20
            larger = rng.random() < 0.5
            a, b = states_with_root_near(e_hi.astype(np.float64), u, _delta(rng, n), c, larger=larger)
            may = reference_may_accept(a, b, t_ev, F(np.inf), c, tau, F(np.inf))
            claim = no_crossing(a, b, e_hi, F(np.inf), c)
        else:  # stage: random 8-event stages whose bound lies near the threshold (states scaled by c / c_ref,
            # times by tau / tau_ref, which keeps bound / c and t / tau)
            sev, tau_ref = 8, 0.26
            theta = rng.choice([0.2, 1.0, 1.3])
            ratio = np.float64(c) / (theta / tau_ref)
            t0 = rng.uniform(0.0, 2.5, (n, 1))
            dt = np.sort(rng.uniform(0.0, rng.choice([0.001, 0.02, 0.2]), (n, sev + 1)), axis=1)
            t = ((t0 + dt) * (np.float64(tau) / tau_ref)).astype(F)
            es = np.exp(t.astype(np.float64) / (np.float64(tau) / 2)).astype(F)
            e = np.exp(t.astype(np.float64) / np.float64(tau)).astype(F)
            scale = rng.uniform(0.05, 3.0, (n, 1)) * np.exp(-t0 / tau_ref) * ratio
            w = (rng.normal(rng.uniform(-0.5, 1.0, (n, 1)), 1.0, (n, sev)) * scale).astype(F)
            aa = (rng.normal(0.0, 1.0, n) * scale[:, 0] * e[:, 0]).astype(F)
            bb = (rng.normal(0.5, 1.0, n) * scale[:, 0] * np.sqrt(e[:, 0])).astype(F)
            A, Bm = [], []
            for k in range(sev):
                aa = fmaf(w[:, k], es[:, k], aa)
                bb = fmaf(w[:, k], e[:, k], bb)
                A.append(aa)
                Bm.append(bb)
            A, Bm = np.stack(A, 1), np.stack(Bm, 1)
            _, e_hi = expf_range(t[:, 0], tau)
            claim = stage_no_crossing(A.min(1), Bm.max(1), np.abs(A).min(1), aa, bb, e_hi, c)
            never_ends = rng.random(n) < 0.3
            may = np.zeros(n, dtype=bool)
            for k in range(sev):
                next_t = np.where(never_ends & (k == sev - 1), np.inf, t[:, k + 1]).astype(F)
                may |= reference_may_accept(A[:, k], Bm[:, k], t[:, k], next_t, c, tau, F(np.inf))
    return int(claim.sum()), int((claim & may).sum())


def _worker(args):
    kind, seed, n_chunks = args
    rng = np.random.default_rng(seed)
    claims = bad = 0
    for _ in range(n_chunks):
        cl, v = _chunk(kind, rng, CHUNK)
        claims += cl
        bad += v
    return kind, n_chunks * CHUNK, claims, bad


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases-per-kind", type=int, default=2_000_000)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    chunks = max(1, args.cases_per_kind // CHUNK)
    per_task = max(1, chunks // max(1, args.workers))
    tasks, s = [], args.seed * 1_000_003
    for kind in KINDS:
        left = chunks
        while left > 0:
            k = min(per_task, left)
            tasks.append((kind, s, k))
            s += 1
            left -= k
    t0 = time.time()
    out = {k: {"cases": 0, "claims": 0, "violations": 0} for k in KINDS}
    with mp.get_context("spawn").Pool(args.workers) as pool:
        for kind, n, cl, v in pool.imap_unordered(_worker, tasks):
            out[kind]["cases"] += n
            out[kind]["claims"] += cl
            out[kind]["violations"] += v
    print(json.dumps({"kinds": out, "seconds": round(time.time() - t0, 1), "workers": args.workers,
                      "c_range": [2.0 ** -30, 2.0 ** 16], "tau_range": [1e-3, 10.0]}))
    return 0 if all(o["violations"] == 0 for o in out.values()) else 1


if __name__ == "__main__":
    sys.exit(main())
