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
#include "disc.cuh"

#define BATS_INF __int_as_float(0x7f800000)

namespace bats {

// First statement of every kernel (programmatic dependent launch): let the next kernel in the stream launch
// its CTAs now (they wait in their own prologue), then wait until the grids this one depends on have
// completed and their writes are visible. Both are no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_prologue() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

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
    float inv_c;    // 1 / c
    bool fast;      // c > 0: the provable rejections below are valid
};

// True when the reference solver provably accepts no crossing in the window (t_last, t_next] for the
// state (a, b), so that its exact evaluation can be skipped without changing any result. With
// B2 = fl(b*b), D = B2 - 4ac and (|b| a normal float, |a| <= 2^60, c > 0; a state below -2^60 can
// overflow 2a and the discriminant, where the reference's z = 2a/(x + b) is NaN and accepted as a spike):
//   * a <= 0 or b < 0: the reference's x = sqrt(tmp) satisfies x >= |b| (a <= 0) or x <= |b|
//     (a > 0, b < 0), because sqrt(fl(b^2)) == |b| in binary floating point; then x + b == 0, or
//     z = 2a/(x + b) <= 0, and the log of a non-positive z is rejected.
//   * a > 0 and B2 < fl(4a*c): D < 0 in every evaluation order (double, float, fused), so the
//     discriminant test fails.
//   * otherwise (a, b > 0) the reference's root z = 2a/(x + b) lies within 2^-21 (relative) of the
//     smaller root z1 of Q(z) = c z^2 - sqrt(B2) z + a (the FC discriminant is formed in double, so tmp
//     is D to 2^-24 relative; the conv discriminant, formed in float, is D to 2^-22 B2 absolute, which
//     bounds z by the root of Q with a lowered by 2^-24 B2 / c). The sign of Q at a point Z is known
//     when the evaluated Q(Z) exceeds its rounding error (2^-21 of the sum of its terms' magnitudes;
//     plus 2^-23 B2 / c for conv) in magnitude.
//     - Right of the window: Z_hi = min(exp(t_next/tau), exp(max_sim/tau)), widened by 2^-19 + 2^-20.
//       If Z_hi lies left of the vertex of Q (2c Z_hi < sqrt(B2)) and Q(Z_hi) > 0 beyond its error bound
//       (whose 2^-21 relative slack adds at least 2^-20 more), then Z_hi < z1: the spike time tau ln z
//       exceeds t_next or max_sim, and the reference rejects it. The margin covers the documented error
//       bounds of __expf (2 + floor(1.173 |x|) ulp, in the event table's exp(t_next/tau)) and of __logf
//       (3 ulp), the root's and the roundings of t/tau and of tau * ln z, for Z_hi < 2980: a root that
//       close to Z_hi then lies below e^8, where 3 ulp of the logarithm are 1.5 x 2^-20 (from e^8 = 2980.96
//       on they double, and a window ending in [2980, 2981) could be claimed wrongly).
//     - Left of the window (FC only; e_start = exp(t_event/tau) of the window's first event, 0 to skip):
//       Z_lo = e_start (1 - 2^-17). If Q(Z_lo) < 0 (Z_lo between the roots), or Q(Z_lo) > 0 with Z_lo
//       right of the vertex (both roots below it), then z1 < Z_lo: the spike time tau ln z lies before
//       the event (the margin 2^-17 covers __expf, __logf and the root), and the reference rejects it
//       as not after the last spike or event. Strongly driven neurons that were reset meet this after
//       most events.
//     The left test is used for Z_lo < 2981 (about 8 tau), where the root's bound holds; its 2^-17 margin
//     also covers the doubled __logf error of a root in [e^8, 2981).
//     LEFT = false leaves the left test out (a cheaper first screen; the solver applies it).
//     No square root or division is needed.
template <bool CONV, bool LEFT = !CONV>
__device__ __forceinline__ bool no_crossing(float a, float b, float e_start, float e_next, const SolveConst& k) {
    const float ab = fabsf(b);
    const bool usable = k.fast && ab >= 0x1p-60f && ab <= 0x1p60f && fabsf(a) <= 0x1p60f;
    const float p_hi = __fmul_rn(__fmul_rn(4.0f, a), k.c);
    const float B2 = __fmul_rn(b, b);
    const bool level1 = a <= 0.0f || b < 0.0f || B2 < p_hi;
    const float Z = fminf(e_next, k.e_max) * (1.0f + 0x1.8p-19f);
    const float q = fmaf(fmaf(k.c, Z, -b), Z, a);                 // (cZ - b) Z + a
    float err = 0x1p-21f * fmaf(fmaf(k.c, Z, b), Z, a);           // |rounding| + |sqrt(B2) - b| Z
    if (CONV) err = fmaf(0x1p-23f * B2, k.inv_c, err);
    const bool right_of_window = Z < 2980.0f && (2.0f * k.c) * Z < b * (1.0f - 0x1p-21f) && q > err;
    bool left_of_window = false;
    if (LEFT && !CONV) {
        const float Zl = e_start * (1.0f - 0x1p-17f);
        const float ql = fmaf(fmaf(k.c, Zl, -b), Zl, a);
        const float errl = 0x1p-21f * fmaf(fmaf(k.c, Zl, b), Zl, a);
        left_of_window = Zl > 0.0f && Zl < 2981.0f &&
                         (ql < -errl || (ql > errl && (2.0f * k.c) * Zl > b * (1.0f + 0x1p-21f)));
    }
    return usable && (level1 || right_of_window || left_of_window);
}

// The window constants of one event for no_crossing_at, formed once per stage for all neurons of a tile by
// the same float operations as no_crossing: Z and (2c) Z of the right-of-window test ((2c) Z = +inf where the
// test does not apply, Z >= 2980), and Zl and (2c) Zl of the left-of-window test (NaN where it does not apply:
// every comparison with them is false). no_crossing_at<LEFT>(a, b, event_window(e_start, e_next, k), k) ==
// no_crossing<false, LEFT>(a, b, e_start, e_next, k) for every a, b.
struct __align__(16) EventWindow {
    float Z, tcZ, Zl, tcZl;
};
__device__ __forceinline__ EventWindow event_window(float e_start, float e_next, const SolveConst& k) {
    EventWindow w;
    w.Z = fminf(e_next, k.e_max) * (1.0f + 0x1.8p-19f);
    w.tcZ = w.Z < 2980.0f ? (2.0f * k.c) * w.Z : BATS_INF;
    const float zl = e_start * (1.0f - 0x1p-17f);
    w.Zl = (zl > 0.0f && zl < 2981.0f) ? zl : __int_as_float(0x7fc00000);
    w.tcZl = (2.0f * k.c) * w.Zl;
    return w;
}
template <bool LEFT>
__device__ __forceinline__ bool no_crossing_at(float a, float b, const EventWindow& w, const SolveConst& k) {
    const float ab = fabsf(b);
    const bool usable = k.fast && ab >= 0x1p-60f && ab <= 0x1p60f && fabsf(a) <= 0x1p60f;
    const float p_hi = __fmul_rn(__fmul_rn(4.0f, a), k.c);
    const float B2 = __fmul_rn(b, b);
    const bool level1 = a <= 0.0f || b < 0.0f || B2 < p_hi;
    const float q = fmaf(fmaf(k.c, w.Z, -b), w.Z, a);
    const float err = 0x1p-21f * fmaf(fmaf(k.c, w.Z, b), w.Z, a);
    const bool right_of_window = w.tcZ < b * (1.0f - 0x1p-21f) && q > err;
    bool left_of_window = false;
    if (LEFT) {
        const float ql = fmaf(fmaf(k.c, w.Zl, -b), w.Zl, a);
        const float errl = 0x1p-21f * fmaf(fmaf(k.c, w.Zl, b), w.Zl, a);
        left_of_window = ql < -errl || (ql > errl && w.tcZl > b * (1.0f + 0x1p-21f));
    }
    return usable && (level1 || right_of_window || left_of_window);
}

// Screen of a run of consecutive events (FC layer, tau = 2 tau_s): true when the reference solver provably
// accepts no crossing after any event of the run, given the run's states (a_u, b_u) only through
// amin = min_u a_u and bmax = max_u b_u, and e_first = exp(t/tau) of the run's first event.
// With x = exp(t/tau), the crossing condition c x^2 - b x + a = 0 reads V(x) = b/x - a/x^2 = c. For
// x >= X0 = e_first (1 - 2^-17) every state satisfies V_u(x) <= max(bmax, 0)/X0 + max(-amin, 0)/X0^2,
// a bound that decreases in x. If it lies below c (1 - 2^-20), then for each state either
//   * the maximum of V_u over x > 0 is below c (1 - 2^-20), so b_u^2 < 4 a_u c (1 - 2^-20) (or a_u <= 0 or
//     b_u <= 0, whose roots the reference rejects by sign, as in no_crossing), and the reference's
//     discriminant, fl(b^2) - 4ac with fl(b^2) <= b^2 (1 + 2^-24), is negative; or
//   * V_u reaches c only left of X0 (V_u is unimodal), so both roots lie below e_first (1 - 2^-17): the
//     reference's root z (within 2^-21 of the smaller root), after __logf, gives a time before the event,
//     which it rejects — the margin of the left-of-window test of no_crossing.
// The test is evaluated multiplied through by X0^2 > 0: fma(max(bmax, 0), X0, max(-amin, 0)) < c' X0 X0 with
// c' = c (1 - 2^-19), whose roundings (a few units of 2^-24) stay inside the 2^-20 margin; the same margin
// covers the reference's fl(b^2) in place of b^2 (a 2^-24 change of b moves V by at most 2^-24 c right of
// X0, where b/x < c). As for no_crossing, the run must start before 8 tau (X0 < 2981) and every |a_u| must
// be at least 2^-60 (amag = min_u |a_u|), so that the discriminant's rounding is relative; with
// 2^-40 <= c <= 2^20, a state whose roots exist then has 2^-49 < b < c X0 and a < c X0^2 / 4 < 2^42, inside
// the range where no_crossing's bound on the computed root holds. fminf/fmaxf
// skip NaN, so the run's last state (a_last, b_last) must be finite: a non-finite state stays non-finite
// through the later events of the run, and the reference turns it into a NaN spike. No division or square
// root.
__device__ __forceinline__ bool stage_no_crossing(float amin, float bmax, float amag, float a_last, float b_last,
                                                  float e_first, const SolveConst& k) {
    const float x0 = e_first * (1.0f - 0x1p-17f);
    const float lhs = fmaf(fmaxf(bmax, 0.0f), x0, fmaxf(-amin, 0.0f));
    const float rhs = (k.c * (1.0f - 0x1p-19f)) * x0 * x0;
    return k.fast && k.c >= 0x1p-40f && k.c <= 0x1p20f && x0 > 0.0f && x0 < 2981.0f && amag >= 0x1p-60f &&
           fabsf(a_last) <= 0x1p120f &&
           fabsf(b_last) <= 0x1p120f && lhs < rhs;
}

// Threshold-crossing solver of the current-based LIF neuron after an input event.
//
// The neuron state is a = sum w*exp(t_i/tau_s), b = sum w*exp(t_i/tau) - (dtheta/tau)*sum z_k,
// c = theta/tau. The next crossing is z = 2a / (b + sqrt(b^2 - 4ac)), t = tau*ln z, accepted in
// the window (last_t, min(next_t, max_sim)]. Each accepted spike applies the reset
// b -= (dtheta/tau) * z and the search repeats until no crossing remains or k_post spikes
// have been written. Returns true when the spike buffer is full. e_start and e_next are exp(t/tau) of
// the window's first event and of the next event, used only by no_crossing (e_start 0: not known).
//
// The arithmetic after the no_crossing test gives results bit-identical to the reference solver
// (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:53-83 for the FC layer,
// compute_spike_times_conv.cu:59-90 for the conv layer, whose discriminant is evaluated in float
// instead of double): the FC discriminant through fc_discriminant, which reproduces the reference's
// double expression without FP64 on its common path, everything else operation for operation.
template <bool CONV, typename Screen>
__device__ __forceinline__ bool solve_crossings_screened(float a, float& b, float last_t, float next_t,
                                                         Screen no_crossing_here, const SolveConst& k, int& n,
                                                         int k_post, float* __restrict__ a_out,
                                                         float* __restrict__ x_out, float* __restrict__ t_out,
                                                         float* __restrict__ z_out) {
    while (true) {
        if (no_crossing_here(a, b)) return false;
        float tmp;
        if (CONV) {
            tmp = b * b - 4 * a * k.c;
        } else {
            tmp = fc_discriminant(__fmul_rn(b, b), a, k.c);  // == (float)((double)fl(b*b) - 4.0*a*c)
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
        b -= k.dtt * inside_log;
        n++;
        if (n >= k_post) return true;
    }
}

template <bool CONV>
__device__ __forceinline__ bool solve_crossings(float a, float& b, float last_t, float next_t, float e_start,
                                                float e_next, const SolveConst& k, int& n, int k_post,
                                                float* __restrict__ a_out, float* __restrict__ x_out,
                                                float* __restrict__ t_out, float* __restrict__ z_out) {
    return solve_crossings_screened<CONV>(
        a, b, last_t, next_t, [&](float a_, float b_) { return no_crossing<CONV>(a_, b_, e_start, e_next, k); }, k,
        n, k_post, a_out, x_out, t_out, z_out);
}

// The conv form of the right-of-window constants, formed once per staged event (the window that ends at it):
// Z = min(e_next, e_max)(1 + 1.5 2^-19) and (2c) Z, +inf where the test does not apply (Z >= 2980), by the
// float operations of no_crossing<true>. no_crossing_conv_at(a, b, conv_window(e_next, k), k) ==
// no_crossing<true>(a, b, 0, e_next, k) for every a, b.
__device__ __forceinline__ float2 conv_window(float e_next, const SolveConst& k) {
    const float Z = fminf(e_next, k.e_max) * (1.0f + 0x1.8p-19f);
    return make_float2(Z, Z < 2980.0f ? (2.0f * k.c) * Z : BATS_INF);
}
__device__ __forceinline__ bool no_crossing_conv_at(float a, float b, float2 zw, const SolveConst& k) {
    const float ab = fabsf(b);
    const bool usable = k.fast && ab >= 0x1p-60f && ab <= 0x1p60f && fabsf(a) <= 0x1p60f;
    const float p_hi = __fmul_rn(__fmul_rn(4.0f, a), k.c);
    const float B2 = __fmul_rn(b, b);
    const bool level1 = a <= 0.0f || b < 0.0f || B2 < p_hi;
    const float q = fmaf(fmaf(k.c, zw.x, -b), zw.x, a);
    float err = 0x1p-21f * fmaf(fmaf(k.c, zw.x, b), zw.x, a);
    err = fmaf(0x1p-23f * B2, k.inv_c, err);
    const bool right_of_window = zw.y < b * (1.0f - 0x1p-21f) && q > err;
    return usable && (level1 || right_of_window);
}
// solve_crossings<true> with the window's constants from conv_window.
__device__ __forceinline__ bool solve_crossings_conv_at(float a, float& b, float last_t, float next_t, float2 zw,
                                                        const SolveConst& k, int& n, int k_post,
                                                        float* __restrict__ a_out, float* __restrict__ x_out,
                                                        float* __restrict__ t_out, float* __restrict__ z_out) {
    return solve_crossings_screened<true>(
        a, b, last_t, next_t, [&](float a_, float b_) { return no_crossing_conv_at(a_, b_, zw, k); }, k, n, k_post,
        a_out, x_out, t_out, z_out);
}

// solve_crossings<false> with the event's window constants formed once per stage (event_window).
__device__ __forceinline__ bool solve_crossings_at(float a, float& b, float last_t, float next_t, const EventWindow& w,
                                                const SolveConst& k, int& n, int k_post,
                                                float* __restrict__ a_out, float* __restrict__ x_out,
                                                float* __restrict__ t_out, float* __restrict__ z_out) {
    while (true) {
        if (no_crossing_at<true>(a, b, w, k)) return false;
        float tmp;
        tmp = fc_discriminant(__fmul_rn(b, b), a, k.c);  // == (float)((double)fl(b*b) - 4.0*a*c)
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
        b -= k.dtt * inside_log;
        n++;
        if (n >= k_post) return true;
    }
}

// Position of one post neuron's spike train relative to a time-ordered scan of pre spikes: p = first
// post spike with t_p > the current pre-spike time, with its suffix-table entry AB = (SA_p, SB_p)
// ((0, 0) once p reaches the neuron's n valid spikes). The entry after the current one is loaded ahead,
// so an advance does not wait on a global load.
struct PostCursor {
    const float* tp;
    const float2* tb;
    int n, p;
    float tn, tn1;
    float2 AB, AB1;
    __device__ __forceinline__ void init(const float* tp_, const float2* tb_, int n_) {
        tp = tp_;
        tb = tb_;
        n = n_;
        p = 0;
        tn = n > 0 ? tp[0] : BATS_INF;
        AB = n > 0 ? tb[0] : make_float2(0.0f, 0.0f);
        tn1 = n > 1 ? tp[1] : BATS_INF;
        AB1 = n > 1 ? tb[1] : make_float2(0.0f, 0.0f);
    }
    // The same state as init() from the neuron's cursor head (first two spike times, first two table entries;
    // +inf and zeros past n), which the backward prep writes for every (sample, neuron) in one coalesced array.
    __device__ __forceinline__ void init_head(const float* tp_, const float2* tb_, int n_, float2 ht, float4 hab) {
        tp = tp_;
        tb = tb_;
        n = n_;
        p = 0;
        tn = ht.x;
        tn1 = ht.y;
        AB = make_float2(hab.x, hab.y);
        AB1 = make_float2(hab.z, hab.w);
    }
    __device__ __forceinline__ void advance_past(float t) {
        while (tn <= t) {
            ++p;
            tn = tn1;
            AB = AB1;
            const bool more = p + 1 < n;
            tn1 = more ? tp[p + 1] : BATS_INF;
            AB1 = more ? tb[p + 1] : make_float2(0.0f, 0.0f);
        }
    }
    __device__ __forceinline__ bool valid() const { return p < n; }
};

// Sum over the 32 lanes of v[e] for e = 0..N-1 (N = 32 or 16), leaving lane l with the total for
// e = l mod N. N - 1 shuffles (N for N = 16: the two half-warps are added last) instead of N separate
// butterflies; the summation order is fixed.
template <int N>
__device__ __forceinline__ float warp_transpose_reduce(float (&v)[N]) {
    static_assert(N == 32 || N == 16, "32 or 16 values per lane");
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = N / 2; off >= 1; off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int q = 0; q < off; ++q) {
            const float send = upper ? v[q] : v[q + off];
            const float keep = upper ? v[q + off] : v[q];
            v[q] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    if (N == 16) v[0] += __shfl_xor_sync(0xffffffffu, v[0], 16);
    return v[0];
}

}  // namespace bats
