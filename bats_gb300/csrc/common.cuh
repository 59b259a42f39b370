// Shared definitions for the BATS sm_103a kernels.
//
// Data layouts in HBM (all row-major, FP32 unless noted):
//   spike trains      times (B, N, K), +inf after the neuron's n spikes; counts (B, N) int32
//   solver state      a, x, post_exp_tau (B, N, K), valid for k < n
//   sorted events     Event (B, cap) per sample, cap = N_pre * K_pre, ev_count (B) int32
//   transposed weights wt (N_pre, ld) with ld >= N_post, ld % 4 == 0 (16-byte rows)
//   suffix tables     tab (B, N_post, K_post + 1) float2 = (sum err*f1, sum err*f2) over k >= p
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#define BATS_INF __int_as_float(0x7f800000)

namespace bats {

// One pre-synaptic spike of one sample, sorted by time. 16 bytes so that a warp reads it as a
// single broadcast vector load from shared memory.
struct __align__(16) Event {
    float t;   // spike time
    int j;     // pre-synaptic neuron index
    float es;  // __expf(t / tau_s)
    float e;   // __expf(t / tau)
};

// Order-preserving map of an IEEE float onto uint32 (negative values flipped).
__device__ __forceinline__ uint32_t float_to_key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_to_float(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Constants of the crossing search of one layer.
struct SolveConst {
    float c;        // theta / tau
    float dtt;      // delta_theta / tau
    float tau;
    float max_sim;
    float e_max;    // exp(max_sim / tau), +inf when unbounded
    bool fast;      // c > 0: the provable rejections below are valid
};

// True when the reference solver provably finds no crossing in the window (t_last, t_next] for the
// state (a, b), so the exact evaluation can be skipped without changing any result:
//   * a <= 0 or b < 0 (with b^2 a normal float): the reference's x = sqrt(tmp) satisfies x >= |b|
//     (a <= 0) or x <= |b| (a > 0, b < 0), because sqrt(fl(b^2)) == |b| in binary floating point;
//     then x + b == 0, or z = 2a/(x + b) <= 0, and the log of a non-positive z is rejected.
//   * a > 0 and fl(b*b) < fl(4a*c): b^2 - 4ac < 0 in every evaluation order (double, float, fused).
//   * otherwise an approximate root z_f = 2a/(b + sq), sq ~ sqrt(fl(b^2 - 4ac)), is compared with the
//     window [exp(t_last/tau), min(exp(t_next/tau), exp(max_sim/tau))] in z = exp(t/tau) space with a
//     relative margin m that bounds |z_f - z| for the reference's root z: with
//     err_D = 2^-23 b^2 + 2^-24 |D_f| >= |D_f - D| (D = fl(b^2) - 4ac, a > 0, b > 0, 4ac <= fl(b^2)),
//     |sq - sqrt(D)| <= d = min(err_D / sq, sqrt(err_D)) + 2^-21 sq, so z_f is within d / (b + sq - d) of
//     the exact root; the reference's own rounding of x, x + b and 2a/(x + b), the approximate
//     reciprocal and square roots used here, __expf of the window ends and __logf of the root are all
//     below 2^-19 relative together, and m = d / (b + sq - d) + 2^-16 covers them. A root outside the
//     widened window gives a spike time tau*ln(z) outside (t_last, min(t_next, max_sim)], which the
//     reference rejects.
__device__ __forceinline__ bool no_crossing(float a, float b, float e_last, float e_next, const SolveConst& k) {
    if (!k.fast) return false;
    const float ab = fabsf(b);
    if (!(ab >= 0x1p-60f && ab <= 0x1p60f)) return false;
    if (a <= 0.0f || b < 0.0f) return true;
    if (!(a <= 0x1p60f)) return false;
    const float p_hi = __fmul_rn(__fmul_rn(4.0f, a), k.c);
    const float B2 = __fmul_rn(b, b);
    if (B2 < p_hi) return true;
    const float Df = fmaf(b, b, -p_hi);
    const float err_d = fmaf(0x1p-23f, B2, 0x1p-24f * fabsf(Df));
    const float rs = Df > 0.0f ? rsqrtf(Df) : 0.0f;
    const float sq = Df * rs;  // 0 when Df <= 0
    const float d_sqrt = err_d * rsqrtf(err_d);
    const float d = (Df > 0.0f ? fminf(err_d * rs, d_sqrt) : d_sqrt) + 0x1p-21f * sq;
    const float den = b + sq;
    if (!(den > 2.0f * d)) return false;
    const float m = __fdividef(d, den - d) + 0x1p-16f;
    const float zf = __fdividef(2.0f * a, den);
    return zf > fminf(e_next, k.e_max) * (1.0f + m) || zf < e_last * (1.0f - m);
}

// Threshold-crossing solver of the current-based LIF neuron after an input event.
//
// The neuron state is a = sum w*exp(t_i/tau_s), b = sum w*exp(t_i/tau) - (dtheta/tau)*sum z_k,
// c = theta/tau. The next crossing is z = 2a / (b + sqrt(b^2 - 4ac)), t = tau*ln z, accepted in
// the window (last_t, min(next_t, max_sim)]. Each accepted spike applies the reset
// b -= (dtheta/tau) * z and the search repeats until no crossing remains or k_post spikes
// have been written. Returns true when the spike buffer is full. e_last/e_next are exp(t/tau) of
// the window ends (used only by no_crossing).
//
// The arithmetic after the no_crossing test is kept operation for operation identical to the
// reference solver (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83 for the FC layer,
// compute_spike_times_conv.cu:59-90 for the conv layer, whose discriminant is evaluated in float
// instead of double), so that spike times agree bit for bit.
template <bool CONV>
__device__ __forceinline__ bool solve_crossings(float a, float& b, float last_t, float next_t, float e_last,
                                                float e_next, const SolveConst& k, int& n, int k_post,
                                                float* __restrict__ a_out, float* __restrict__ x_out,
                                                float* __restrict__ t_out, float* __restrict__ z_out) {
    while (true) {
        if (no_crossing(a, b, e_last, e_next, k)) return false;
        float tmp;
        if (CONV) {
            tmp = b * b - 4 * a * k.c;
        } else {
            tmp = (float)((double)__fmul_rn(b, b) - 4.0 * (double)a * (double)k.c);
        }
        if (tmp < 0) return false;
        const float x_tmp = sqrtf(tmp);
        tmp = x_tmp + b;
        if (tmp == 0.0f) return false;
        const float inside_log = 2 * a / tmp;
        if (inside_log < 0) return false;
        tmp = k.tau * __logf(inside_log);
        if (tmp <= last_t || tmp > k.max_sim || tmp > next_t) return false;
        a_out[n] = a;
        x_out[n] = x_tmp;
        t_out[n] = tmp;
        z_out[n] = inside_log;
        last_t = tmp;
        e_last = inside_log;
        b -= k.dtt * inside_log;
        n++;
        if (n >= k_post) return true;
    }
}

// Sum over the 32 lanes of v[e] for e = 0..31, leaving lane l with the total for e = l.
// 31 shuffles instead of 32 separate butterflies; the summation order is fixed.
__device__ __forceinline__ float warp_transpose_reduce32(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int q = 0; q < off; ++q) {
            const float send = upper ? v[q] : v[q + off];
            const float keep = upper ? v[q + off] : v[q];
            v[q] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0];
}

}  // namespace bats
