// Discriminant of the fully-connected crossing solver without FP64 arithmetic on the common path.
//
// The reference evaluates tmp = (float)((double)fl(b*b) - 4.0 * (double)a * (double)c)
// (bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:57): the product 4ac is exact in double,
// the difference is rounded once to double and then to float. GB300's FP64 rate is a small fraction of
// its FP32 rate, and in strongly driven layers this line runs after most input events, so it is
// computed here from FP32 error-free transformations:
//   P = 4a*c = ph + pl exactly (ph = fl(4a*c), pl = fma(4a, c, -ph)),
//   B2 - ph = s + e exactly (TwoSum), e - pl = u + f exactly, s + u = r + g exactly,
// so V = B2 - 4ac = r + g + f exactly and r = fl(s + u). If |g| + |f| stays below half an ulp of r by
// a margin of 2^-20 of that half ulp (which is far larger than double's rounding of V, 2^-53 |V|),
// then both fl(V) and fl(fl_double(V)) equal r. Otherwise (V near a midpoint between floats, or
// operands outside the ranges where the transformations are exact) the double expression itself is
// evaluated. The result is bit-identical to the reference's expression for every input.
#pragma once

#if defined(__CUDACC__)
#define BATS_HD __host__ __device__ __forceinline__
#else
#define BATS_HD inline
#endif

#if defined(__CUDA_ARCH__)
#define BATS_FADD(x, y) __fadd_rn((x), (y))
#define BATS_FMUL(x, y) __fmul_rn((x), (y))
#define BATS_FMA(x, y, z) __fmaf_rn((x), (y), (z))
#define BATS_F2I(x) __float_as_int(x)
#define BATS_I2F(x) __int_as_float(x)
#else
#include <cmath>
#include <cstring>
#define BATS_FADD(x, y) ((x) + (y))
#define BATS_FMUL(x, y) ((x) * (y))
#define BATS_FMA(x, y, z) std::fma((x), (y), (z))
static inline int bats_f2i_host(float x) { int i; std::memcpy(&i, &x, 4); return i; }
static inline float bats_i2f_host(int i) { float x; std::memcpy(&x, &i, 4); return x; }
#define BATS_F2I(x) bats_f2i_host(x)
#define BATS_I2F(x) bats_i2f_host(x)
#endif

namespace bats {

// Exact error of x + y (Knuth's TwoSum; no overflow assumed): x + y = s + err.
BATS_HD float two_sum_err(float x, float y, float s) {
    const float bv = BATS_FADD(s, -x);
    const float av = BATS_FADD(s, -bv);
    return BATS_FADD(BATS_FADD(x, -av), BATS_FADD(y, -bv));
}

// The reference's (float)((double)b2 - 4.0 * (double)a * (double)c), b2 = fl(b*b). Kept out of line on
// the device so that the common path carries no FP64 instruction.
#if defined(__CUDA_ARCH__)
__device__ __noinline__
#else
inline
#endif
float fc_discriminant_ref64(float b2, float a, float c) {
    return (float)((double)b2 - 4.0 * (double)a * (double)c);
}

BATS_HD float fc_discriminant(float b2, float a, float c) {
    const float a4 = BATS_FMUL(4.0f, a);
    const float ph = BATS_FMUL(a4, c);
    const float pl = BATS_FMA(a4, c, -ph);
    const float s = BATS_FADD(b2, -ph);
    const float e = two_sum_err(b2, -ph, s);
    const float u = BATS_FADD(e, -pl);
    const float f = two_sum_err(e, -pl, u);
    const float r = BATS_FADD(s, u);
    const float g = two_sum_err(s, u, r);
    const float ab2 = b2 < 0.0f ? -b2 : b2;
    const float aph = ph < 0.0f ? -ph : ph;
    const float ar = r < 0.0f ? -r : r;
    // Ranges where every step above is exact and r is a normal float well above the subnormals:
    // |b2|, |ph| < 2^120 (no overflow in the sums); 4a*c exactly zero or |ph| >= 2^-90 (pl exact);
    // |r| >= 2^-90.
    const bool in_range = ab2 < 0x1p120f && aph < 0x1p120f && (a4 == 0.0f || c == 0.0f || aph >= 0x1p-90f) &&
                          ar >= 0x1p-90f;
    // Half the spacing of the floats around r: 2^(exponent(r) - 24), halved on the side towards zero
    // when r is a power of two (the spacing below a power of two is half the spacing above it).
    const int rbits = BATS_F2I(ar);
    float lim = BATS_I2F((rbits & 0x7f800000) - (24 << 23));
    const float d = BATS_FADD(g, f);
    const bool toward_zero = (r > 0.0f) ? (d < 0.0f) : (d > 0.0f);
    if ((rbits & 0x007fffff) == 0 && toward_zero) lim = BATS_FMUL(lim, 0.5f);
    const float ag = g < 0.0f ? -g : g;
    const float af = f < 0.0f ? -f : f;
    const bool safe = in_range && BATS_FADD(ag, af) < BATS_FMUL(lim, 1.0f - 0x1p-20f);
    if (safe) return r;
    return fc_discriminant_ref64(b2, a, c);
}

// (float)((double)x / d) for d > 0 given 1/d ~= r_hi + r_lo (two floats, relative error <= 2^-47), without
// FP64 on the common path: x * (r_hi + r_lo) is formed as r + g (r = the float nearest to it, g its exact
// remainder), which lies within 2^-46 |x/d| of the quotient; if |g| plus that bound (and double's own
// rounding of x/d) stays below half the float spacing around r, both roundings of x/d give r. A zero x
// gives the zero of its sign. Otherwise (near a midpoint, tiny quotients, d not positive) the double
// division itself is evaluated.
#if defined(__CUDA_ARCH__)
__device__ __noinline__
#else
inline
#endif
float quotient_ref64(float x, double d) {
    return (float)((double)x / d);
}

BATS_HD float quotient_f64_to_f32(float x, float r_hi, float r_lo, double d) {
    if (x == 0.0f && r_hi > 0.0f) return x;  // +-0 / d = +-0 for d > 0 (zero gradients are common)
    const float p_hi = BATS_FMUL(x, r_hi);
    const float p_lo = BATS_FMA(x, r_hi, -p_hi);
    const float t = BATS_FMA(x, r_lo, p_lo);
    const float r = BATS_FADD(p_hi, t);
    const float g = two_sum_err(p_hi, t, r);
    const float ar = r < 0.0f ? -r : r;
    const bool in_range = ar >= 0x1p-90f && ar < 0x1p120f && r_hi > 0.0f;
    const int rbits = BATS_F2I(ar);
    float lim = BATS_I2F((rbits & 0x7f800000) - (24 << 23));
    const bool toward_zero = (r > 0.0f) ? (g < 0.0f) : (g > 0.0f);
    if ((rbits & 0x007fffff) == 0 && toward_zero) lim = BATS_FMUL(lim, 0.5f);
    const float ag = g < 0.0f ? -g : g;
    const bool safe = in_range && BATS_FADD(ag, BATS_FMUL(0x1p-44f, ar)) < BATS_FMUL(lim, 1.0f - 0x1p-20f);
    if (safe) return r;
    return quotient_ref64(x, d);
}

// The float pair (hi, lo) with hi + lo ~= 1/d to about 2^-48 relative, for quotient_f64_to_f32.
BATS_HD void reciprocal_pair(double d, float& hi, float& lo) {
    const double r = 1.0 / d;
    hi = (float)r;
    lo = (float)(r - (double)hi);
}

}  // namespace bats
