"""The host restatements of the no-crossing screens (tests/_float_model.py), on which the screen tests and the
sweep rest, give the same answers as the device source itself: bats_gb300/csrc/common.cuh is compiled for the
host (g++, no floating-point contraction; the screens contain no product-plus-sum that nvcc could fuse, so
the host build performs the device's float operations), with stand-ins for the few device-only names the
rest of the header uses, and its no_crossing (FC and conv forms) and stage_no_crossing are evaluated on
millions of inputs: states at the edges of the proofs, and random operands of every magnitude, sign and
class (zeros, subnormals, infinities, NaN)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests._float_model import F, expf_range, no_crossing, stage_no_crossing, states_with_root_near

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
// Host stand-ins for the device-only names that common.cuh uses outside the screens.
#define __fmul_rn(x, y) ((x) * (y))
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
template <class T> static inline T __shfl_xor_sync(unsigned, T v, int, int = 32) { return v; }
static const uint3 threadIdx = {0, 0, 0};
#include "common.cuh"

// stdin: int32 mode, int64 n, then the fields as float32 arrays of n; stdout: n bytes (0/1).
// mode 0: no_crossing<FC, left test>(a, b, e_start, e_next; c, e_max); mode 1: the conv form (same fields);
// mode 2: stage_no_crossing(amin, bmax, amag, a_last, b_last, e_first; c); mode 3: whether no_crossing_at with
// event_window(e_start, e_next) agrees with no_crossing (bit 0: with the left test, bit 1: without; bit 2: the
// conv form, no_crossing_conv_at with conv_window(e_next)).
int main() {
    int mode;
    long long n;
    if (std::fread(&mode, 4, 1, stdin) != 1 || std::fread(&n, 8, 1, stdin) != 1) return 2;
    const int nf = mode == 2 ? 7 : 6;
    std::vector<float> f((size_t)nf * n);
    if (std::fread(f.data(), 4, f.size(), stdin) != f.size()) return 3;
    std::vector<unsigned char> out(n);
    for (long long i = 0; i < n; ++i) {
        const float* v = f.data();
        bats::SolveConst k{};
        k.c = v[(mode == 2 ? 6 : 4) * n + i];
        k.tau = 1.0f;
        k.e_max = mode == 2 ? INFINITY : v[5 * n + i];
        k.inv_c = k.c > 0.0f ? 1.0f / k.c : 0.0f;
        k.fast = k.c > 0.0f;
        bool r;
        if (mode == 3) {
            // no_crossing_at with the stage's precomputed window against no_crossing, with and without the left
            // test: 1 | 2 when both agree.
            const bats::EventWindow w = bats::event_window(v[2 * n + i], v[3 * n + i], k);
            const bool left = bats::no_crossing_at<true>(v[i], v[n + i], w, k) ==
                              bats::no_crossing<false, true>(v[i], v[n + i], v[2 * n + i], v[3 * n + i], k);
            const bool right = bats::no_crossing_at<false>(v[i], v[n + i], w, k) ==
                               bats::no_crossing<false, false>(v[i], v[n + i], v[2 * n + i], v[3 * n + i], k);
            // bit 2: the conv form with its window from conv_window(e_next) against no_crossing<true>.
            const bool conv = bats::no_crossing_conv_at(v[i], v[n + i], bats::conv_window(v[3 * n + i], k), k) ==
                              bats::no_crossing<true>(v[i], v[n + i], 0.0f, v[3 * n + i], k);
            out[i] = (left ? 1 : 0) | (right ? 2 : 0) | (conv ? 4 : 0);
            continue;
        }
        if (mode == 0) r = bats::no_crossing<false>(v[i], v[n + i], v[2 * n + i], v[3 * n + i], k);
        else if (mode == 1) r = bats::no_crossing<true>(v[i], v[n + i], v[2 * n + i], v[3 * n + i], k);
        else r = bats::stage_no_crossing(v[i], v[n + i], v[2 * n + i], v[3 * n + i], v[4 * n + i], v[5 * n + i], k);
        out[i] = r;
    }
    std::fwrite(out.data(), 1, out.size(), stdout);
    return 0;
}
'''


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
        if os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


@pytest.fixture(scope="module")
def screen_exe(tmp_path_factory):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("no host C++ compiler or CUDA headers")
    d = tmp_path_factory.mktemp("screen_src")
    src, exe = d / "screen.cpp", d / "screen"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "bats_gb300", "csrc"),
                    "-I", inc, "-o", str(exe), str(src)], check=True)
    return str(exe)


def _run(exe, mode, fields):
    n = len(fields[0])
    payload = (np.int32(mode).tobytes() + np.int64(n).tobytes()
               + b"".join(np.ascontiguousarray(x, dtype=F).tobytes() for x in fields))
    r = subprocess.run([exe], input=payload, capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return np.frombuffer(r.stdout, dtype=np.uint8).astype(bool)


def _run_raw(exe, mode, fields):
    n = len(fields[0])
    payload = (np.int32(mode).tobytes() + np.int64(n).tobytes()
               + b"".join(np.ascontiguousarray(x, dtype=F).tobytes() for x in fields))
    r = subprocess.run([exe], input=payload, capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return np.frombuffer(r.stdout, dtype=np.uint8)


def _wild(rng, n):
    """float32 operands of every magnitude and sign, with zeros, subnormals, infinities and NaN mixed in."""
    x = (np.exp(rng.uniform(np.log(1e-44), np.log(3e38), n)) * rng.choice([-1.0, 1.0], n)).astype(F)
    special = np.array([0.0, -0.0, 1e-45, -1e-45, 1e-40, np.inf, -np.inf, np.nan, 1.0, 2981.0, 2980.0,
                        2.0 ** -60, 2.0 ** 60, 2.0 ** 120, 2.0 ** -40, 2.0 ** 20], dtype=F)
    pick = rng.random(n) < 0.1
    x[pick] = rng.choice(special, int(pick.sum()))
    return x


def _edge_states(rng, n):
    """States with a root within a few 2^-20 of the window's end or start, over wide c and tau."""
    tau = F(np.exp(rng.uniform(np.log(1e-3), np.log(10.0))))
    c = np.full(n, F(np.exp(rng.uniform(np.log(2.0 ** -30), np.log(2.0 ** 16)))), dtype=F)
    x = np.where(rng.random(n) < 0.1, rng.uniform(8 - 4e-4, 8 + 1e-4, n), rng.uniform(0.0, 8.2, n))  # 8 tau band
    t = (x * np.float64(tau)).astype(F)
    e_lo, e_hi = expf_range(t, tau)
    u = rng.uniform(-24.0, 12.0, n) * 2.0 ** -20
    delta = np.exp(rng.uniform(np.log(1e-9), np.log(1e6), n))
    a, b = states_with_root_near(e_lo.astype(np.float64), u, delta, c[0], larger=bool(rng.random() < 0.5))
    e_max = np.where(rng.random(n) < 0.5, F(np.inf), e_lo).astype(F)
    e_next = np.where(rng.random(n) < 0.3, F(np.inf), e_lo).astype(F)
    return a, b, e_hi, e_next, c, e_max


@pytest.mark.parametrize("mode", [0, 1])
def test_event_screen_model_equals_the_device_source(screen_exe, mode):
    rng = np.random.default_rng(40 + mode)
    parts = [_edge_states(rng, 100_000) for _ in range(20)]
    fields = [np.concatenate([p[i] for p in parts]) for i in range(6)]
    n = 1_000_000
    wild = [_wild(rng, n), _wild(rng, n), np.abs(_wild(rng, n)), np.abs(_wild(rng, n)),
            np.abs(_wild(rng, n)), np.abs(_wild(rng, n))]
    fields = [np.concatenate([f, w]) for f, w in zip(fields, wild)]
    got = _run(screen_exe, mode, fields)
    a, b, e_start, e_next, c, e_max = fields
    want = no_crossing(a, b, e_start, e_next, c, e_max=e_max, conv=mode == 1)
    assert want.sum() > 100_000 and (~want).sum() > 100_000
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, [tuple(float(f[i]) for f in fields) for i in bad[:5]]


def test_precomputed_window_screen_equals_the_event_screen(screen_exe):
    """The forward's tile kernels form each event's window constants once per stage (event_window) and test
    every neuron with no_crossing_at; that must give no_crossing's answer on every input, with and without the
    left-of-window test, so the kernels' results stay those of the per-event form. The same for the conv
    kernel's window constants, formed once per staged event (conv_window, no_crossing_conv_at)."""
    rng = np.random.default_rng(60)
    parts = [_edge_states(rng, 100_000) for _ in range(10)]
    fields = [np.concatenate([p[i] for p in parts]) for i in range(6)]
    n = 1_000_000
    wild = [_wild(rng, n), _wild(rng, n), np.abs(_wild(rng, n)), np.abs(_wild(rng, n)),
            np.abs(_wild(rng, n)), np.abs(_wild(rng, n))]
    fields = [np.concatenate([f, w]) for f, w in zip(fields, wild)]
    n_all = len(fields[0])
    payload_ok = _run_raw(screen_exe, 3, fields)
    assert payload_ok.size == n_all
    bad = np.flatnonzero(payload_ok != 7)
    assert bad.size == 0, [(int(payload_ok[i]),) + tuple(float(f[i]) for f in fields) for i in bad[:5]]


def test_stage_screen_model_equals_the_device_source(screen_exe):
    rng = np.random.default_rng(50)
    n = 1_000_000
    c = np.exp(rng.uniform(np.log(2.0 ** -45), np.log(2.0 ** 22), n)).astype(F)
    e_first = np.exp(rng.uniform(0.0, 8.1, n)).astype(F)
    x0 = (e_first * F(1.0 - 2.0 ** -17)).astype(F).astype(np.float64)
    # bound near the threshold: b_max / x0 + max(-a_min, 0) / x0^2 ~ c (1 +- 1e-5)
    split = rng.uniform(0.0, 1.0, n)
    target = c.astype(np.float64) * x0 * x0 * (1 + rng.uniform(-1e-5, 1e-5, n))
    bmax = (split * target / x0).astype(F)
    amin = (-(1 - split) * target).astype(F)
    amag = np.abs(_wild(rng, n))
    a_last, b_last = _wild(rng, n), _wild(rng, n)
    near = [amin, bmax, amag, a_last, b_last, e_first, c]
    wild = [_wild(rng, n), _wild(rng, n), np.abs(_wild(rng, n)), _wild(rng, n), _wild(rng, n),
            np.abs(_wild(rng, n)), np.abs(_wild(rng, n))]
    fields = [np.concatenate([x, w]) for x, w in zip(near, wild)]
    got = _run(screen_exe, 2, fields)
    want = stage_no_crossing(*fields)
    assert want.sum() > 50_000 and (~want).sum() > 50_000
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, [tuple(float(f[i]) for f in fields) for i in bad[:5]]
