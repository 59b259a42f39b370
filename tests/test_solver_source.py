"""The crossing solver of the forward kernels (solve_crossings, bats_gb300/csrc/common.cuh; FC and conv forms),
compiled for the host, gives bit for bit the results of the reference's solver loops
(bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83 and compute_spike_times_conv.cu:59-90, whose
discriminant is formed in float; restated below in plain C from its
behaviour: discriminant (float)(fl(b*b) - 4.0*a*c) in double, x = sqrtf, z = 2a / (x + b), t = tau * log z,
accepted in (last, min(next, max_sim)], reset b -= (delta_theta/tau) z, at most K spikes). Both sides use the
host's logf and expf, which lie within the documented error bounds of __logf and __expf, so the check covers
what the screens may skip (no_crossing must never drop a spike the loop accepts), the FP64-free
discriminant, the window tests, the reset and the K cap. Both are compiled without floating-point
contraction, the same policy on both sides (on the GPU, nvcc and the reference's runtime compiler both
contract the reset). Cases: roots within a few 2^-20 of the window's start or end, windows near 8 tau,
strongly driven neurons that spike several times in one window, and operands of every magnitude, sign and
class."""
import os
import shutil
import subprocess

import pytest

from tests.test_screen_source import _cuda_include

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <cuda_runtime.h>
// Host stand-ins for the device-only names that common.cuh uses.
#define __fmul_rn(x, y) ((x) * (y))
#define __logf(x) logf(x)
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
template <class T> static inline T __shfl_xor_sync(unsigned, T v, int, int = 32) { return v; }
static const uint3 threadIdx = {0, 0, 0};
#include "common.cuh"

// The reference's per-event solver loop, restated from its behaviour (conv: the conv layer's loop, whose
// discriminant is formed in float).
template <bool CONV>
static bool reference_solve(float c, float dtt, float tau, float max_sim, float a, float& b, float last, float next,
                            int& n, int K, float* ao, float* xo, float* to, float* zo) {
    while (true) {
        const float bb = b * b;
        float tmp = CONV ? bb - 4 * a * c : (float)((double)bb - 4.0 * (double)a * (double)c);
        if (tmp < 0) return false;
        const float x = sqrtf(tmp);
        tmp = x + b;
        if (tmp == 0.0f) return false;
        const float z = 2 * a / tmp;
        if (z < 0) return false;
        tmp = tau * logf(z);
        if (tmp <= last || tmp > max_sim || tmp > next) return false;
        ao[n] = a; xo[n] = x; to[n] = tmp; zo[n] = z;
        last = tmp;
        b -= dtt * z;
        n++;
        if (n >= K) return true;
    }
}

static bool same(float x, float y) { uint32_t a, b; std::memcpy(&a, &x, 4); std::memcpy(&b, &y, 4); return a == b; }

template <bool CONV>
static int run(long long N) {
    std::mt19937_64 rng(2024);
    std::uniform_real_distribution<double> U(0, 1);
    auto logu = [&](double lo, double hi) { return std::exp(std::log(lo) + U(rng) * (std::log(hi) - std::log(lo))); };
    const float specials[] = {0.0f, -0.0f, 1e-45f, 1e-38f, INFINITY, -INFINITY, NAN, 1.0f, -1.0f, 3e38f};
    long long bad = 0, spikes = 0, screened = 0, multi = 0;
    for (long long q = 0; q < N; ++q) {
        const float tau = (float)logu(1e-3, 10.0);
        const float c = (float)logu(std::ldexp(1.0, -20), std::ldexp(1.0, 12));
        const float dtt = (float)(c * U(rng) * 2.0);
        const float max_sim = U(rng) < 0.5 ? INFINITY : (float)(tau * U(rng) * 9.0);
        const double xt = (q % 8 == 0) ? 8.0 + (U(rng) - 0.8) * 5e-4 : U(rng) * 8.2;
        const float t_ev = (float)(tau * xt);
        const float next = U(rng) < 0.3 ? INFINITY : (float)(t_ev + tau * logu(1e-7, 1.0));
        const float e_ev = expf(t_ev / tau), e_nx = expf(next / tau);
        double x = e_ev;
        float a, b;
        switch (q % 4) {
            case 0: {  // a root within a few 2^-20 of the window's start or end
                const double edge = (U(rng) < 0.5 || !std::isfinite(e_nx)) ? (double)e_ev : (double)e_nx;
                const double delta = logu(1e-9, 1e6), s = std::sqrt(delta / (1 + delta));
                const double root = edge * (1 + (U(rng) - 0.5) * std::ldexp(48.0, -20));
                const double bd = (U(rng) < 0.5) ? 2 * c * root / (1 - s) : 2 * c * root / (1 + s);
                b = (float)bd;
                a = (float)(bd * bd / (4.0 * c * (1 + delta)));
                break;
            }
            case 1: {  // strongly driven: crosses soon after the event, several times after resets
                const double bd = 2 * c * x * (1 + logu(1e-6, 30.0));
                b = (float)bd;
                a = (float)(bd * bd / (4.0 * c) * (1 - U(rng)));
                break;
            }
            case 2:
                a = (float)((U(rng) < 0.5 ? -1 : 1) * logu(1e-30, 1e30));
                b = (float)((U(rng) < 0.7 ? 1 : -1) * logu(1e-30, 1e30));
                break;
            default:
                a = U(rng) < 0.5 ? specials[rng() % 10] : (float)((U(rng) - 0.3) * 100);
                b = U(rng) < 0.5 ? specials[rng() % 10] : (float)((U(rng) - 0.3) * 100);
                break;
        }
        bats::SolveConst k{};
        k.c = c; k.dtt = dtt; k.tau = tau; k.max_sim = max_sim;
        const double em = std::exp((double)max_sim / (double)tau);
        k.e_max = std::isfinite(em) && em < 3.0e38 ? (float)em : INFINITY;
        k.inv_c = 1.0f / c;
        k.fast = true;
        const int K = 1 + (int)(rng() % 30), n0 = (int)(rng() % K);
        float ao1[32], xo1[32], to1[32], zo1[32], ao2[32], xo2[32], to2[32], zo2[32];
        std::memset(ao1, 0, sizeof ao1); std::memcpy(ao2, ao1, sizeof ao1);
        std::memcpy(xo1, ao1, sizeof ao1); std::memcpy(xo2, ao1, sizeof ao1);
        std::memcpy(to1, ao1, sizeof ao1); std::memcpy(to2, ao1, sizeof ao1);
        std::memcpy(zo1, ao1, sizeof ao1); std::memcpy(zo2, ao1, sizeof ao1);
        float b1 = b, b2 = b;
        int n1 = n0, n2 = n0;
        const bool r1 = reference_solve<CONV>(c, dtt, tau, max_sim, a, b1, t_ev, next, n1, K, ao1, xo1, to1, zo1);
        if (bats::no_crossing<CONV>(a, b, e_ev, e_nx, k)) ++screened;
        const bool r2 = bats::solve_crossings<CONV>(a, b2, t_ev, next, e_ev, e_nx, k, n2, K, ao2, xo2, to2, zo2);
        bool ok = r1 == r2 && n1 == n2 && same(b1, b2);
        for (int i = n0; ok && i < n1; ++i)
            ok = same(ao1[i], ao2[i]) && same(xo1[i], xo2[i]) && same(to1[i], to2[i]) && same(zo1[i], zo2[i]);
        spikes += n1 - n0;
        multi += n1 - n0 >= 2;
        if (!ok) {
            if (bad < 5) std::printf("mismatch a=%a b=%a c=%a tau=%a t=%a next=%a: n %d/%d\n", a, b, c, tau, t_ev, next, n1, n2);
            ++bad;
        }
    }
    std::printf("%lld mismatches of %lld; spikes %lld; multi %lld; screened %lld\n", bad, N, spikes, multi, screened);
    return bad != 0;
}

int main(int argc, char** argv) {
    const long long N = std::atoll(argv[1]);
    return std::atoi(argv[2]) ? run<true>(N) : run<false>(N);
}
'''


@pytest.mark.parametrize("conv", [0, 1], ids=["fc", "conv"])
def test_solver_matches_the_reference_loop(tmp_path, conv):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("no host C++ compiler or CUDA headers")
    src, exe = tmp_path / "solver.cpp", tmp_path / "solver"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "bats_gb300", "csrc"),
                    "-I", inc, "-o", str(exe), str(src)], check=True)
    r = subprocess.run([str(exe), "4000000", str(conv)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    assert words[0] == "0", r.stdout
    spikes, multi, screened = int(words[5].rstrip(";")), int(words[7].rstrip(";")), int(words[9])
    assert spikes > 500_000 and multi > 50_000 and screened > 1_000_000, r.stdout


MERGED = PROGRAM.split("\nstatic bool same(")[0] + r'''
static bool same(float x, float y) { uint32_t a, b; std::memcpy(&a, &x, 4); std::memcpy(&b, &y, 4); return a == b; }

// Conv layer: the reference visits every event of the sample, with weight 0 outside the neuron's receptive
// field, and solves each window (t_i, t_{i+1}] (compute_spike_times_conv.cu:155-172); the conv kernel visits
// only the relevant events and solves the merged window between them, then (t_last, inf). An event outside
// the field is relevant when one of its exponentials is not finite (0 * inf is NaN in the reference's sums).
// argv[2] = 1 plants the old mistake: outside events are never relevant.
// argv[3] = 1 uses the plain restatement of the reference's solver on the reference side (else the device
// solver there too, which isolates the window merging).
int main(int argc, char** argv) {
    const long long N = std::atoll(argv[1]);
    const bool old_rule = argc > 2 && std::atoi(argv[2]) != 0;
    const bool plain_ref = argc > 3 && std::atoi(argv[3]) != 0;
    long long overflow_cases = 0;
    std::mt19937_64 rng(77);
    std::uniform_real_distribution<double> U(0, 1);
    std::normal_distribution<double> G(0, 1);
    long long bad = 0, spikes = 0;
    for (long long q = 0; q < N; ++q) {
        const int E = 1 + (int)(rng() % 60), K = 1 + (int)(rng() % 12);
        const float tau_s = (float)(0.02 + U(rng) * 0.3), tau = 2 * tau_s;
        const float theta = (float)(0.05 + U(rng) * 1.5), c = theta / tau, dtt = (float)(U(rng) * 2 * theta) / tau;
        const float max_sim = U(rng) < 0.5 ? INFINITY : (float)(U(rng) * 0.4);
        float t[64], es[64], e[64], w[64];
        bool rel[64];
        // One case in four reaches past 88 tau_s, where expf(t / tau_s) overflows to +inf (and past 177 tau_s,
        // where expf(t / tau) does too), with max_sim = inf half the time as above.
        const bool late = q % 4 == 3;
        for (int i = 0; i < E; ++i) t[i] = late ? (float)(tau_s * (80.0 + U(rng) * 110.0)) : (float)(U(rng) * 0.3);
        std::sort(t, t + E);
        if (q % 5 == 0) for (int i = 1; i < E; i += 3) t[i] = t[i - 1];   // ties
        const double scale = std::exp(G(rng));
        for (int i = 0; i < E; ++i) {
            es[i] = expf(t[i] / tau_s); e[i] = expf(t[i] / tau);
            rel[i] = U(rng) < 0.35;
            w[i] = (float)((G(rng) + 0.8) * scale);
        }
        bats::SolveConst k{};
        k.c = c; k.dtt = dtt; k.tau = tau; k.max_sim = max_sim;
        const double em = std::exp((double)max_sim / (double)tau);
        k.e_max = std::isfinite(em) && em < 3.0e38 ? (float)em : INFINITY;
        k.inv_c = 1.0f / c; k.fast = true;
        float ao1[16], xo1[16], to1[16], zo1[16], ao2[16], xo2[16], to2[16], zo2[16];
        bool any_inf = false;
        for (int i = 0; i < E; ++i) any_inf |= !std::isfinite(es[i]);
        overflow_cases += any_inf;
        // the reference's loop over every event
        float a = 0, b = 0;
        int n1 = 0;
        for (int i = 0; i < E; ++i) {
            const float wi = rel[i] ? w[i] : 0.0f;
            a += wi * es[i];
            b += wi * e[i];
            const float next = i + 1 < E ? t[i + 1] : INFINITY;
            const bool full = plain_ref
                ? reference_solve<true>(c, dtt, tau, max_sim, a, b, t[i], next, n1, K, ao1, xo1, to1, zo1)
                : bats::solve_crossings<true>(a, b, t[i], next, 0.0f, i + 1 < E ? e[i + 1] : INFINITY, k, n1, K,
                                              ao1, xo1, to1, zo1);
            if (full) break;
        }
        // the conv kernel's loop over the relevant events only
        float a2 = 0, b2 = 0, last = 0;
        int n2 = 0;
        bool has_prev = false, done = false;
        for (int i = 0; i < E && !done; ++i) {
            const bool finite = std::isfinite(es[i]) && std::isfinite(e[i]);
            if (!rel[i] && (finite || old_rule)) continue;
            if (has_prev) {
                done = bats::solve_crossings_conv_at(a2, b2, last, t[i], bats::conv_window(e[i], k), k, n2, K, ao2,
                                                     xo2, to2, zo2);
                if (done) break;
            }
            const float wi = rel[i] ? w[i] : 0.0f;
            a2 += wi * es[i];
            b2 += wi * e[i];
            last = t[i];
            has_prev = true;
        }
        if (has_prev && !done) bats::solve_crossings<true>(a2, b2, last, INFINITY, 0.0f, INFINITY, k, n2, K, ao2, xo2, to2, zo2);
        bool ok = n1 == n2;
        for (int i = 0; ok && i < n1; ++i)
            ok = same(ao1[i], ao2[i]) && same(xo1[i], xo2[i]) && same(to1[i], to2[i]) && same(zo1[i], zo2[i]);
        spikes += n1;
        if (!ok) { if (bad < 5) std::printf("mismatch q=%lld n %d/%d\n", q, n1, n2); ++bad; }
    }
    std::printf("%lld mismatches of %lld; spikes %lld; overflow %lld\n", bad, N, spikes, overflow_cases);
    return bad != 0;
}
'''


def test_conv_merged_windows_match_the_reference_loop(tmp_path):
    """Solving the merged windows between a neuron's relevant events gives the same spikes, bit for bit, as the
    reference's per-event windows over every event of the sample (ties included), also when inputs later than
    88 tau_s overflow exp(t/tau_s): events outside the field with a non-finite exponential count as relevant
    (weight 0, as the reference adds them). Without that rule the overflowing cases differ."""
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("no host C++ compiler or CUDA headers")
    src, exe = tmp_path / "merged.cpp", tmp_path / "merged"
    src.write_text(MERGED.replace("#include <random>", "#include <random>\n#include <algorithm>"))
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "bats_gb300", "csrc"),
                    "-I", inc, "-o", str(exe), str(src)], check=True)
    r = subprocess.run([str(exe), "400000", "0", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    assert words[0] == "0" and int(words[5].rstrip(";")) > 200_000 and int(words[7]) > 50_000, r.stdout
    # The same check with the device solver on both sides (window merging alone).
    r = subprocess.run([str(exe), "400000", "0", "0"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.split()[0] == "0", r.stdout + r.stderr
    # A planted mistake: outside events never relevant, as before overflowing exponentials were handled.
    r = subprocess.run([str(exe), "400000", "1", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and int(r.stdout.split("mismatches")[0].split()[-1]) > 1000, r.stdout
