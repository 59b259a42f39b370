"""The forward kernel's replay skips the solver after a spike for events whose first-pass screen ruled a
crossing out (bats_gb300/csrc/fc_forward.cu, forward_tile_item). The first pass evaluated
no_crossing<false, false> on the state (a, b_p) accumulated without this stage's resets; a reset lowers b
(b -= (delta_theta/tau) z, z > 0) and the later FMAs b = fma(w, e, b) are monotone in b, so the replayed state
is (a, b) with b <= b_p and the same a. The claim is that the reference solver
(bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83) then accepts no crossing in the window either,
provided (a, b) is in the screen's range (2^-60 <= |b| <= 2^60, |a| <= 2^60): every step of the reference's
root is monotone in b (fl(b*b), the discriminant, sqrtf, x + b, 2a / (x + b)), so its z can only grow as b
falls, and the screen's margin covers __logf's documented error at any larger z.

This test checks the claim on the host against the plain-C restatement of the reference solver (host logf
within __logf's bounds), on states built at the screen's edges (roots just right of the window end, states
just outside level 1) and random ones, lowered by resets of every size; and it checks that the reverse
(b raised instead of lowered, a planted mistake) breaks it."""
import os
import shutil
import subprocess

import pytest

from tests.test_screen_source import _cuda_include
from tests.test_solver_source import PROGRAM

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

TRANSFER = PROGRAM.split("\nstatic bool same(")[0] + r'''
#include <algorithm>
static bool usable(float a, float b) {
    const float ab = fabsf(b);
    return ab >= 0x1p-60f && ab <= 0x1p60f && fabsf(a) <= 0x1p60f;
}

int main(int argc, char** argv) {
    const long long N = std::atoll(argv[1]);
    const bool raise = std::atoi(argv[2]) != 0;   // planted mistake: b moved up instead of down
    std::mt19937_64 rng(99);
    std::uniform_real_distribution<double> U(0, 1);
    auto logu = [&](double lo, double hi) { return std::exp(std::log(lo) + U(rng) * (std::log(hi) - std::log(lo))); };
    long long claimed = 0, checked = 0, bad = 0;
    for (long long q = 0; q < N; ++q) {
        const float tau = (float)logu(1e-3, 10.0);
        const float c = (float)logu(std::ldexp(1.0, -20), std::ldexp(1.0, 12));
        const float dtt = (float)(c * U(rng) * 2.0);
        const float max_sim = U(rng) < 0.5 ? INFINITY : (float)(tau * U(rng) * 9.0);
        const double xt = (q % 8 == 0) ? 8.0 + (U(rng) - 0.8) * 5e-4 : U(rng) * 8.2;
        const float t_ev = (float)(tau * xt);
        const float next = U(rng) < 0.2 ? INFINITY : (float)(t_ev + tau * logu(1e-7, 1.0));
        const float e_ev = expf(t_ev / tau), e_nx = expf(next / tau);
        float a, b;
        if (q % 3 == 0 && std::isfinite(e_nx)) {
            // The smaller root a few 2^-20 right of the window end: what the right-of-window test claims.
            const double delta = logu(1e-9, 1e6), s = std::sqrt(delta / (1 + delta));
            const double root = (double)e_nx * (1 + logu(1e-7, 1e-3));
            const double bd = 2 * c * root / (1 + s);
            b = (float)bd;
            a = (float)(bd * bd / (4.0 * c * (1 + delta)));
        } else if (q % 3 == 1) {
            // Just outside or inside level 1 (b^2 near 4ac).
            const double bd = logu(1e-20, 1e20);
            b = (float)bd;
            a = (float)(bd * bd / (4.0 * c) * (1 + (U(rng) - 0.5) * 1e-5));
        } else {
            a = (float)((U(rng) < 0.2 ? -1 : 1) * logu(1e-30, 1e30));
            b = (float)((U(rng) < 0.2 ? -1 : 1) * logu(1e-30, 1e30));
        }
        bats::SolveConst k{};
        k.c = c; k.dtt = dtt; k.tau = tau; k.max_sim = max_sim;
        const double em = std::exp((double)max_sim / (double)tau);
        k.e_max = std::isfinite(em) && em < 3.0e38 ? (float)em : INFINITY;
        k.inv_c = 1.0f / c;
        k.fast = true;
        if (!bats::no_crossing<false, false>(a, b, e_ev, e_nx, k)) continue;
        ++claimed;
        for (int r = 0; r < 8; ++r) {
            float b2 = b;
            switch (r) {
                case 0: b2 = nextafterf(b, raise ? INFINITY : -INFINITY); break;
                case 1: b2 = b * (raise ? 1.0f + 0x1p-20f : 1.0f - 0x1p-20f); break;
                default: {
                    // One or more resets b -= dtt * z with z a crossing value of the window or beyond.
                    const float z = (float)(e_ev * logu(1.0, 1e3));
                    const int resets = 1 + (int)(rng() % 3);
                    for (int i = 0; i < resets; ++i) b2 = raise ? b2 + dtt * z : b2 - dtt * z;
                    if (r >= 5) b2 = raise ? b2 + (float)logu(1e-6, 1e3) * fabsf(b) : b2 - (float)logu(1e-6, 1e3) * fabsf(b);
                }
            }
            if (!usable(a, b2)) continue;
            ++checked;
            float ao[32], xo[32], to[32], zo[32];
            int n = 0;
            float bb = b2;
            reference_solve<false>(c, dtt, tau, max_sim, a, bb, t_ev, next, n, 30, ao, xo, to, zo);
            if (n != 0) {
                if (bad < 5) std::printf("spike after transfer: a=%a b=%a b2=%a c=%a t=%a next=%a\n", a, b, b2, c, t_ev, next);
                ++bad;
            }
        }
    }
    std::printf("%lld violations; claimed %lld; checked %lld\n", bad, claimed, checked);
    return bad != 0;
}
'''


def _build(tmp_path):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("no host C++ compiler or CUDA headers")
    src, exe = tmp_path / "transfer.cpp", tmp_path / "transfer"
    src.write_text(TRANSFER)
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "bats_gb300", "csrc"),
                    "-I", inc, "-o", str(exe), str(src)], check=True)
    return exe


def test_screen_claims_survive_lowering_b(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "3000000", "0"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.strip().splitlines()[-1].split()
    assert words[0] == "0" and int(words[3].rstrip(";")) > 500_000 and int(words[5]) > 2_000_000, r.stdout


def test_raising_b_instead_is_caught(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "3000000", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and int(r.stdout.strip().splitlines()[-1].split()[0]) > 1000, r.stdout
