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

// Threshold-crossing solver of the current-based LIF neuron after an input event.
//
// The neuron state is a = sum w*exp(t_i/tau_s), b = sum w*exp(t_i/tau) - (dtheta/tau)*sum z_k,
// c = theta/tau. The next crossing is z = 2a / (b + sqrt(b^2 - 4ac)), t = tau*ln z, accepted in
// the window (last_t, min(next_t, max_sim)]. Each accepted spike applies the reset
// b -= (dtheta/tau) * z and the search repeats until no crossing remains or k_post spikes
// have been written. Returns true when the spike buffer is full.
//
// The arithmetic of the slow path is kept operation for operation identical to the reference
// solver (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83 for the FC layer,
// compute_spike_times_conv.cu:59-90 for the conv layer, whose discriminant is evaluated in
// float instead of double), so that spike times agree bit for bit. The fast path in front of it
// only returns false in cases where the reference provably returns false:
//   * a <= 0 and b^2 a normal float: sqrt(fl(b^2)) == |b| in binary floating point, so
//     x + b >= 0 and either x + b == 0 or 2a/(x+b) <= 0 (log(-0) = -inf is rejected too);
//   * a > 0 and fl(b*b) < fl(4a*c): then b^2 - 4ac < 0 in every evaluation order (double,
//     float, or either fused form), so the discriminant test fails.
template <bool CONV>
__device__ __forceinline__ bool solve_crossings(float a, float& b, float last_t, float next_t,
                                                float c, float dtt, float tau, float max_sim,
                                                int& n, int k_post,
                                                float* __restrict__ a_out, float* __restrict__ x_out,
                                                float* __restrict__ t_out, float* __restrict__ z_out) {
    while (true) {
        const float B2 = __fmul_rn(b, b);
        const float ab = fabsf(b);
        if (c > 0.0f && ab >= 0x1p-60f && ab <= 0x1p60f) {
            if (a <= 0.0f) return false;
            const float p_hi = __fmul_rn(__fmul_rn(4.0f, a), c);
            if (B2 < p_hi) return false;
        }
        float tmp;
        if (CONV) {
            tmp = b * b - 4 * a * c;
        } else {
            tmp = (float)((double)B2 - 4.0 * (double)a * (double)c);
        }
        if (tmp < 0) return false;
        const float x_tmp = sqrtf(tmp);
        tmp = x_tmp + b;
        if (tmp == 0.0f) return false;
        const float inside_log = 2 * a / tmp;
        if (inside_log < 0) return false;
        tmp = tau * __logf(inside_log);
        if (tmp <= last_t || tmp > max_sim || tmp > next_t) return false;
        a_out[n] = a;
        x_out[n] = x_tmp;
        t_out[n] = tmp;
        z_out[n] = inside_log;
        last_t = tmp;
        b -= dtt * inside_log;
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
