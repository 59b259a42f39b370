"""FP64-free evaluations (bats_gb300/csrc/disc.cuh) against the double expressions they replace, bit for
bit, on the host:
* the FC solver's discriminant (float)((double)fl(b*b) - 4.0*a*c)
  (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:57): random operands over the solver's ranges,
  near-tangential cases (b^2 ~ 4ac), mixed signs, and adversarial cases whose exact value lies at or near a
  midpoint between floats, at or next to powers of two, where rounding twice (to double, then to float)
  differs from rounding once;
* the optimizers' bias-corrected moments (float)((double)m / (1 - beta^t)): bias corrections of Adam's
  and NAdam's betas over thousands of steps, random and power-of-two numerators, and numerators placed at
  float midpoints of the quotient."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include "disc.cuh"
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <random>
static long long bad = 0, total = 0, fast = 0;
static void check(float b2, float a, float c) {
    float x = bats::fc_discriminant(b2, a, c), y = bats::fc_discriminant_ref64(b2, a, c);
    uint32_t xi, yi; std::memcpy(&xi, &x, 4); std::memcpy(&yi, &y, 4);
    ++total;
    if (xi != yi) { if (bad < 5) std::printf("mismatch b2=%a a=%a c=%a got %a want %a\n", b2, a, c, x, y); ++bad; }
}
int main(int argc, char** argv) {
    const long long n = std::atoll(argv[1]);
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0, 1);
    auto logu = [&](double lo, double hi) { return (float)std::exp(std::log(lo) + U(rng) * (std::log(hi) - std::log(lo))); };
    for (long long q = 0; q < n; ++q) {
        float c = logu(1e-2, 1e2), a, b;
        switch (q % 4) {
            case 0: a = logu(1e-6, 1e6); b = logu(1e-6, 1e6); break;
            case 1: a = logu(1e-3, 1e4); b = (float)(std::sqrt(4.0 * a * c) * (1 + (U(rng) - 0.5) * 1e-5)); break;
            case 2: a = logu(1e-3, 1e4); b = (float)(std::sqrt(4.0 * a * c) * (1 + (U(rng) - 0.5) * 1e-2)); break;
            default: a = (float)((U(rng) - 0.5) * 100); b = (float)((U(rng) - 0.5) * 100); break;
        }
        check(b * b, a, c);
        int e0 = (int)(U(rng) * 20) - 10;
        float b2 = q % 3 == 0 ? std::ldexp(1.0f, e0)
                 : q % 3 == 1 ? std::nextafter(std::ldexp(1.0f, e0), (q & 8) ? 0.0f : 10.0f)
                              : (float)std::ldexp(1.0 + U(rng), e0);
        float cc = (q % 5 == 0) ? 1.0f : (float)(0.5 + U(rng));
        double p = std::ldexp(1.0 + U(rng), e0 - 20 - (int)(U(rng) * 40));
        if (q & 16) p = std::ldexp(1.0, e0 - 24) * (1.0 + (U(rng) - 0.5) * std::ldexp(1.0, -(int)(U(rng) * 30)));
        if (q & 32) p = -p;
        check(b2, (float)(p / (4.0 * cc)), cc);
    }
    // Quotients x / d (d > 0) near float midpoints.
    for (long long q = 0; q < n; ++q) {
        double d = q % 2 ? 1.0 - std::pow(0.999, 1 + (int)(U(rng) * 5000)) : 1.0 - std::pow(0.9, 1 + (int)(U(rng) * 200));
        float x = (float)((U(rng) - 0.5) * std::pow(10.0, (U(rng) - 0.5) * 16));
        if (q % 3 == 0) {
            float m = (float)std::ldexp(1.0 + U(rng), (int)(U(rng) * 30) - 15);
            double mid = (double)m + std::ldexp((double)std::nextafter(m, 1e30f) - (double)m, -1);
            x = (float)(mid * d);
        }
        float hi, lo;
        bats::reciprocal_pair(d, hi, lo);
        float a = bats::quotient_f64_to_f32(x, hi, lo, d), b = bats::quotient_ref64(x, d);
        uint32_t ai, bi; std::memcpy(&ai, &a, 4); std::memcpy(&bi, &b, 4);
        ++total;
        if (ai != bi) { if (bad < 5) std::printf("quotient mismatch x=%a d=%a got %a want %a\n", x, d, a, b); ++bad; }
    }
    // Special values.
    const float sp[] = {0.0f, -0.0f, 1e-45f, 1e-30f, 1e30f, 3e38f, INFINITY, -INFINITY, NAN, 1.0f, -1.0f};
    for (float x : sp) for (float y : sp) for (float z : sp) check(x, y, z);
    std::printf("%lld mismatches of %lld\n", bad, total);
    return bad != 0;
}
'''


def test_fc_discriminant_bit_exact(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "disc_test.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "disc_test"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "bats_gb300", "csrc"),
                    "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe), "3000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().startswith("0 mismatches"), out.stdout
