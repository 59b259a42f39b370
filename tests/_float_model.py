"""Host model of the float arithmetic that decides whether the reference solver accepts a crossing, for the
tests of the no-crossing screens (bats_gb300/csrc/common.cuh).

The reference's solver (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83) forms the root
z = 2a / (sqrt(tmp) + b) from IEEE operations, which NumPy reproduces bit for bit, and takes the spike time
tau * __logf(z); the event table holds x = __expf(t / tau). __expf and __logf are fast intrinsics whose
exact results are not reproduced here: the model takes every value their documented error bounds allow
(CUDA C++ Programming Guide, intrinsic functions: __expf within 2 + floor(|1.173 x|) ulp; __logf within
2^-21.41 absolute for x in [0.5, 2], else within 3 ulp), so that a screen that holds against the model
holds for any GPU that meets those bounds."""
from __future__ import annotations

import numpy as np

F = np.float32


def fmaf(x, y, z):
    """float32 fused multiply-add (the product of two floats is exact in double; one rounding to float)."""
    return (np.asarray(x, F).astype(np.float64) * np.asarray(y, F).astype(np.float64)
            + np.asarray(z, F).astype(np.float64)).astype(F)


def ulp32(v):
    """Spacing of float32 at |v| (the distance to the next float away from zero)."""
    v = np.abs(np.asarray(v, F))
    return (np.nextafter(v, F(np.inf)) - v).astype(np.float64)


def _float_at_least(v):
    """Smallest float32 >= v (v float64)."""
    f = v.astype(F)
    return np.where(f.astype(np.float64) < v, np.nextafter(f, F(np.inf)), f)


def _float_at_most(v):
    f = v.astype(F)
    return np.where(f.astype(np.float64) > v, np.nextafter(f, F(-np.inf)), f)


def expf_range(t, tau):
    """(lo, hi): the float32 values __expf(t / tau) may take, t float32, tau float."""
    with np.errstate(all="ignore"):
        x = (np.asarray(t, F) / F(tau)).astype(F)                 # IEEE division
        e = np.exp(x.astype(np.float64))
        k = 2 + np.floor(np.abs(1.173 * x.astype(np.float64)))
        u = ulp32(e.astype(F))
        return _float_at_least(e - k * u), _float_at_most(e + k * u)


def logf_range(z):
    """(lo, hi): the float32 values __logf(z) may take, z > 0 float32."""
    with np.errstate(all="ignore"):
        zd = np.asarray(z, F).astype(np.float64)
        l = np.log(zd)
        err = np.where((zd >= 0.5) & (zd <= 2.0), 2.0 ** -21.41, 3.0 * ulp32(np.abs(l).astype(F)))
        return _float_at_least(l - err), _float_at_most(l + err)


def reference_root(a, b, c):
    """(ok, z): the reference's root z = 2a / (sqrt(tmp) + b) with tmp = (float)((double)fl(b*b) - 4.0*a*c),
    and whether the solver goes on to the log (tmp >= 0, a non-zero denominator, z >= 0)."""
    with np.errstate(all="ignore"):
        a, b = np.asarray(a, F), np.asarray(b, F)
        b2 = (b * b).astype(F)
        tmp = (b2.astype(np.float64) - 4.0 * a.astype(np.float64) * np.float64(F(c))).astype(F)
        ok = ~(tmp < 0)
        x = np.sqrt(np.where(ok, tmp, F(0))).astype(F)
        den = (x + b).astype(F)
        ok &= den != 0
        z = ((F(2) * a).astype(F) / np.where(den == 0, F(1), den)).astype(F)
        ok &= ~(z < 0)
        return ok, z


def reference_roots_conv(a, b, c):
    """[(ok, z)] of the conv solver (compute_spike_times_conv.cu:59-71), whose discriminant
    b * b - 4 * a * c is formed in float: once per evaluation order a compiler may choose (two roundings, or
    either product fused into the subtraction)."""
    with np.errstate(all="ignore"):
        a, b = np.asarray(a, F), np.asarray(b, F)
        c = F(c)
        p = ((F(4) * a).astype(F) * c).astype(F)
        b2 = (b * b).astype(F)
        tmps = [(b2 - p).astype(F),
                fmaf(b, b, -p),
                fmaf(-(F(4) * a).astype(F), np.full_like(a, c), b2)]
        out = []
        for tmp in tmps:
            ok = ~(tmp < 0)
            x = np.sqrt(np.where(ok, tmp, F(0))).astype(F)
            den = (x + b).astype(F)
            ok = ok & (den != 0)
            z = ((F(2) * a).astype(F) / np.where(den == 0, F(1), den)).astype(F)
            out.append((ok & ~(z < 0), z))
        return out


def reference_may_accept(a, b, last_t, next_t, c, tau, max_sim, conv=False):
    """True where the reference solver accepts the crossing after the event for some __logf value within its
    bound: spike time tau * L (one IEEE product) in (last_t, min(next_t, max_sim)]. conv: the conv solver,
    for any of its discriminant's evaluation orders."""
    roots = reference_roots_conv(a, b, c) if conv else [reference_root(a, b, c)]
    may = np.zeros(np.shape(a), dtype=bool)
    with np.errstate(all="ignore"):
        for ok, z in roots:
            l_lo, l_hi = logf_range(np.where(ok & (z > 0), z, F(1)))
            t_lo = (F(tau) * l_lo).astype(F)
            t_hi = (F(tau) * l_hi).astype(F)
            zero = ok & (z == 0)                                  # log(0) = -inf: never after the event
            may |= ok & ~zero & (t_hi > np.asarray(last_t, F)) & (t_lo <= F(max_sim)) & (
                t_lo <= np.asarray(next_t, F))
    return may


def no_crossing(a, b, e_start, e_next, c, e_max=np.inf, widen=1.5 * 2.0 ** -19, cap=2980.0, margin=2.0 ** -17,
                left=True, conv=False, conv_slack=2.0 ** -23):
    """The per-event screen, operation for operation (conv: the conv layer's form, which adds conv_slack * B2 / c
    to the error bound and has no left test); widen, cap, margin and conv_slack are parameters so that a test
    can plant a mistake in the model."""
    with np.errstate(all="ignore"):
        a, b = np.asarray(a, F), np.asarray(b, F)
        c = np.asarray(c, F)
        ab = np.abs(b)
        usable = (c > 0) & (ab >= F(2.0 ** -60)) & (ab <= F(2.0 ** 60)) & (np.abs(a) <= F(2.0 ** 60))
        p_hi = ((F(4) * a).astype(F) * c).astype(F)
        b2 = (b * b).astype(F)
        level1 = (a <= 0) | (b < 0) | (b2 < p_hi)
        cc = np.full_like(a, c)
        z = (np.fmin(np.asarray(e_next, F), np.asarray(e_max, F)) * F(1.0 + widen)).astype(F)  # fminf: NaN-skipping
        q = fmaf(fmaf(cc, z, -b), z, a)
        err = (F(2.0 ** -21) * fmaf(fmaf(cc, z, b), z, a)).astype(F)
        if conv:
            err = fmaf((F(conv_slack) * b2).astype(F), np.full_like(a, (F(1) / c).astype(F)), err)  # k.inv_c
        right = (z < F(cap)) & (((F(2) * c) * z).astype(F) < (b * F(1.0 - 2.0 ** -21)).astype(F)) & (q > err)
        left_w = np.zeros_like(right)
        if left and not conv:
            zl = (np.asarray(e_start, F) * F(1.0 - margin)).astype(F)
            ql = fmaf(fmaf(cc, zl, -b), zl, a)
            errl = (F(2.0 ** -21) * fmaf(fmaf(cc, zl, b), zl, a)).astype(F)
            left_w = (zl > 0) & (zl < F(2981)) & (
                (ql < -errl) | ((ql > errl) & (((F(2) * c) * zl).astype(F) > (b * F(1.0 + 2.0 ** -21)).astype(F))))
        return usable & (level1 | right | left_w)


def stage_no_crossing(amin, bmax, amag, a_last, b_last, e_first, c):
    """The per-stage screen, operation for operation."""
    with np.errstate(all="ignore"):
        c = np.asarray(c, F)
        x0 = (np.asarray(e_first, F) * F(1.0 - 2.0 ** -17)).astype(F)
        lhs = fmaf(np.fmax(bmax, F(0)), x0, np.fmax(-np.asarray(amin, F), F(0)))  # fmaxf: NaN-skipping
        rhs = (((c * F(1.0 - 2.0 ** -19)).astype(F) * x0).astype(F) * x0).astype(F)
        fin = (np.abs(a_last) <= F(2.0 ** 120)) & (np.abs(b_last) <= F(2.0 ** 120))
        return ((c >= F(2.0 ** -40)) & (c <= F(2.0 ** 20)) & (x0 > 0) & (x0 < F(2981)) & (amag >= F(2.0 ** -60))
                & fin & (lhs < rhs))


def states_with_root_near(x, rel, delta, c, larger=False):
    """float32 states (a, b) of c z^2 - b z + a whose smaller root (larger root if larger) lies at
    x (1 + rel), with roots separated by b^2 = 4ac (1 + delta)."""
    s = np.sqrt(delta / (1 + delta))
    root = x * (1 + rel)
    b = 2 * np.float64(c) * root / ((1 + s) if larger else (1 - s))
    a = b * b / (4 * np.float64(c) * (1 + delta))
    return a.astype(F), b.astype(F)
