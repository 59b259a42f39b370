// Losses, Adam, weight transpose and the elementwise pre-spike exponentials.
//
// Losses:  bats/Losses/SpikeCountLoss.py:7-38, SpikeCountClassLoss.py:8-33,
//          TTFSSoftmaxCrossEntropy.py:7-56, SpikeTimeLoss.py:7-47
// Adam:    bats/Optimizers/AdamOptimizer.py:7-55 (+ LIFLayer.add_deltas, bats/Layers/LIFLayer.py:112-113)
// Exps:    bats/CudaKernels/CuFiles/Inference/compute_pre_exps.cu:2-22
#include "common.cuh"
#include "abi_util.h"

namespace bats {

__global__ void pre_exps_kernel(const float* __restrict__ t, long long n, float tau_s, float tau,
                                float* __restrict__ es, float* __restrict__ e) {
    pdl_prologue();
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const float v = t[q];
        es[q] = __expf(v / tau_s);
        e[q] = __expf(v / tau);
    }
}

// One warp per sample. counts may be int32 or float32 (count_is_float); targets (B, N) or,
// when labels is given, target_false everywhere and target_true at the label.
__global__ void spike_count_loss_kernel(const void* __restrict__ counts, int count_is_float,
                                        const float* __restrict__ targets, const int* __restrict__ labels,
                                        float target_true, float target_false, int batch, int n, int k,
                                        float* __restrict__ loss, float* __restrict__ errors) {
    pdl_prologue();
    const int warps = blockDim.x >> 5;
    const int s = blockIdx.x * warps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= batch) return;
    const int label = labels ? labels[s] : -1;
    float acc = 0.0f;
    for (int q = lane; q < n; q += 32) {
        const long long idx = (long long)s * n + q;
        const float cnt = count_is_float ? reinterpret_cast<const float*>(counts)[idx]
                                         : (float)reinterpret_cast<const int*>(counts)[idx];
        const float tgt = labels ? (q == label ? target_true : target_false) : targets[idx];
        const float d = tgt - cnt;
        acc += d * d;
        if (errors) {
            float* eo = errors + idx * k;
            for (int kk = 0; kk < k; ++kk) eo[kk] = d;
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && loss) loss[s] = acc / 2;
}

__device__ __forceinline__ float nan_to_num_f(float v) {
    if (isnan(v)) return 0.0f;
    if (isinf(v)) return v > 0 ? 3.402823466e38f : -3.402823466e38f;
    return v;
}

// Softmax cross-entropy of the first spike times. exp(-t/tau) is evaluated as the reference's
// generated kernel does: the division by the literal tau happens in double.
__global__ void ttfs_sce_kernel(const float* __restrict__ spikes, const int* __restrict__ labels, int batch, int n,
                                int k, double tau_literal, float tau_f, float* __restrict__ loss,
                                float* __restrict__ errors) {
    pdl_prologue();
    const int warps = blockDim.x >> 5;
    const int s = blockIdx.x * warps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= batch) return;
    const int label = labels[s];
    float sum = 0.0f;
    for (int q = lane; q < n; q += 32) {
        const float t0 = spikes[((long long)s * n + q) * k];
        sum += __expf((float)(-(double)t0 / tau_literal));
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    for (int q = lane; q < n; q += 32) {
        const long long idx = (long long)s * n + q;
        const float t0 = spikes[idx * k];
        const float ex = __expf((float)(-(double)t0 / tau_literal));
        if (loss && q == label) loss[s] = -__logf(ex / sum);
        if (errors) {
            float ns = -ex / sum;
            if (q == label) ns += 1;
            ns /= tau_f;
            float* eo = errors + idx * k;
            eo[0] = nan_to_num_f(ns);
            for (int kk = 1; kk < k; ++kk) eo[kk] = 0.0f;
        }
    }
}

// Mean squared error on first spike times with silent neurons (inf) replaced by 1.0.
// mode 0: loss only; 1: errors = spikes_copy - targets; 2: loss and errors = spikes - targets
// (the reference's compute_loss_and_errors subtracts from the uncopied spikes).
// Targets are modified in place (inf -> 1.0) like the reference.
__global__ void spike_time_loss_kernel(const float* __restrict__ spikes, float* __restrict__ targets, int batch, int n,
                                       int k, int mode, float* __restrict__ loss, float* __restrict__ errors) {
    pdl_prologue();
    const int warps = blockDim.x >> 5;
    const int s = blockIdx.x * warps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= batch) return;
    float acc = 0.0f;
    for (int q = lane; q < n; q += 32) {
        const long long base = ((long long)s * n + q) * k;
        for (int kk = 0; kk < k; ++kk) {
            float tg = targets[base + kk];
            if (isinf(tg)) {
                tg = 1.0f;
                targets[base + kk] = tg;
            }
            const float sp = spikes[base + kk];
            const float spc = isinf(sp) ? 1.0f : sp;
            if (kk == 0) {
                const float d = tg - spc;
                acc += d * d;
            }
            if (errors && mode >= 1) errors[base + kk] = (mode == 1 ? spc : sp) - tg;
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && loss && mode != 1) loss[s] = acc / 2;
}

// Adam (AdamOptimizer.step) for one tensor: m, v updated in place; the delta is written to
// `delta` and/or added to `w` (Network.apply_deltas); when wt is given, w's new value is also
// written transposed into wt (n_pre, ld) for the forward kernels.
__global__ void adam_kernel(const float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                            long long count, float beta_1, float one_minus_beta_1, float beta_2,
                            float one_minus_beta_2, double bias1, double bias2, const double* __restrict__ powers,
                            float r1_hi, float r1_lo, float r2_hi, float r2_lo,
                            float lr, float eps, float* __restrict__ delta, float* __restrict__ w, float* __restrict__ wt, int n_post,
                            int n_pre, int ld) {
    pdl_prologue();
    if (powers) {
        // State written by adam_powers_kernel: beta^t (double) and the reciprocal pairs of 1 - beta^t.
        bias1 = 1.0 - powers[0];
        bias2 = 1.0 - powers[1];
        const float4 rp = *reinterpret_cast<const float4*>(powers + 2);
        r1_hi = rp.x;
        r1_lo = rp.y;
        r2_hi = rp.z;
        r2_lo = rp.w;
    }
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < count;
         q += (long long)gridDim.x * blockDim.x) {
        const float g = grad[q];
        const float nm = beta_1 * m[q] + one_minus_beta_1 * g;
        const float nv = beta_2 * v[q] + one_minus_beta_2 * g * g;
        m[q] = nm;
        v[q] = nv;
        // (float)((double)nm / (1 - beta_1^t)), (float)((double)nv / (1 - beta_2^t)) without FP64 division
        // (the double is only formed on the rare fallback path).
        const float m_hat = quotient_f64_to_f32(nm, r1_hi, r1_lo, bias1);
        const float v_hat = quotient_f64_to_f32(nv, r2_hi, r2_lo, bias2);
        const float d = -(lr * m_hat / (sqrtf(v_hat) + eps));
        if (delta) delta[q] = d;
        if (w) {
            const float nw = w[q] + d;
            w[q] = nw;
            if (wt) {
                const int i = (int)(q / n_pre), j = (int)(q % n_pre);
                wt[(long long)j * ld + i] = nw;
            }
        }
    }
}

// adam_kernel for a weight matrix with its transposed copy: CTA per 32 x 32 tile (block 32 x 8), rows read
// and written along j, the tile transposed through shared memory so that the copy wt (n_pre, ld) is written
// along i too (the per-element transposed store of adam_kernel touches one 32-byte sector per element).
// The arithmetic per element is adam_kernel's.
__global__ void __launch_bounds__(256)
adam_tiled_kernel(const float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v, float beta_1,
                  float one_minus_beta_1, float beta_2, float one_minus_beta_2, double bias1, double bias2,
                  const double* __restrict__ powers, float r1_hi, float r1_lo, float r2_hi, float r2_lo, float lr,
                  float eps, float* __restrict__ delta, float* __restrict__ w, float* __restrict__ wt, int n_post,
                  int n_pre, int ld) {
    pdl_prologue();
    __shared__ float tile[32][33];
    if (powers) {
        bias1 = 1.0 - powers[0];
        bias2 = 1.0 - powers[1];
        const float4 rp = *reinterpret_cast<const float4*>(powers + 2);
        r1_hi = rp.x;
        r1_lo = rp.y;
        r2_hi = rp.z;
        r2_lo = rp.w;
    }
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = j0 + tx;
    // All four rows' operands are loaded before the arithmetic, so that their latencies overlap.
    float g_in[4], m_in[4], v_in[4], w_in[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty + 8 * r;
        if (i < n_post && j < n_pre) {
            const long long q = (long long)i * n_pre + j;
            g_in[r] = grad[q];
            m_in[r] = m[q];
            v_in[r] = v[q];
            w_in[r] = w[q];
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty + 8 * r;
        if (i < n_post && j < n_pre) {
            const long long q = (long long)i * n_pre + j;
            const float g = g_in[r];
            const float nm = beta_1 * m_in[r] + one_minus_beta_1 * g;
            const float nv = beta_2 * v_in[r] + one_minus_beta_2 * g * g;
            m[q] = nm;
            v[q] = nv;
            const float m_hat = quotient_f64_to_f32(nm, r1_hi, r1_lo, bias1);
            const float v_hat = quotient_f64_to_f32(nv, r2_hi, r2_lo, bias2);
            const float d = -(lr * m_hat / (sqrtf(v_hat) + eps));
            if (delta) delta[q] = d;
            const float nw = w_in[r] + d;
            w[q] = nw;
            tile[ty + 8 * r][tx] = nw;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int jj = j0 + ty + 8 * r;  // row of wt
        const int ii = i0 + tx;          // column of wt
        if (jj < n_pre && ii < n_post) wt[(long long)jj * ld + ii] = tile[tx][ty + 8 * r];
    }
}

// beta_1^t, beta_2^t kept on the device so that a captured step can advance t without host input.
__global__ void adam_powers_kernel(double* powers, float beta_1, float beta_2) {
    pdl_prologue();
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        powers[0] *= (double)beta_1;
        powers[1] *= (double)beta_2;
        float4 rp;
        reciprocal_pair(1.0 - powers[0], rp.x, rp.y);
        reciprocal_pair(1.0 - powers[1], rp.z, rp.w);
        *reinterpret_cast<float4*>(powers + 2) = rp;
    }
}

// out (cols, ld) = in (rows, cols) transposed, 32x32 shared-memory tiles.
__global__ void transpose_kernel(const float* __restrict__ in, int rows, int cols, float* __restrict__ out, int ld) {
    pdl_prologue();
    __shared__ float tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int r = by + yy, cc = bx + threadIdx.x;
        if (r < rows && cc < cols) tile[yy][threadIdx.x] = in[(long long)r * cols + cc];
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int cc = bx + yy, r = by + threadIdx.x;
        if (cc < cols && r < rows) out[(long long)cc * ld + r] = tile[threadIdx.x][yy];
    }
}

__global__ void add_inplace_kernel(float* __restrict__ w, const float* __restrict__ d, long long count,
                                   float* __restrict__ wt, int n_pre, int ld) {
    pdl_prologue();
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < count;
         q += (long long)gridDim.x * blockDim.x) {
        const float nw = w[q] + d[q];
        w[q] = nw;
        if (wt) wt[(q % n_pre) * (long long)ld + q / n_pre] = nw;
    }
}

}  // namespace bats

static unsigned grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 16) b = 152LL * 16;
    if (b < 1) b = 1;
    return (unsigned)b;
}

extern "C" int bats_compute_pre_exps(const float* times, long long count, float tau_s, float tau, float* exp_tau_s,
                                     float* exp_tau, cudaStream_t stream) {
    BATS_REQUIRE(count >= 0, BATS_ERR_BAD_SHAPE, "compute_pre_exps: bad shape");
    if (count == 0) return BATS_OK;
    BATS_REQUIRE(times && exp_tau_s && exp_tau, BATS_ERR_NULL, "compute_pre_exps: null pointer");
    BATS_CUDA(bats::launch(bats::pre_exps_kernel, grid_for(count, 256), 256, 0, stream, times, count, tau_s, tau,
        exp_tau_s, exp_tau));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_spike_count_loss(const void* counts, int count_is_float, const float* targets, const int* labels,
                                     float target_true, float target_false, int batch, int n, int k, float* loss,
                                     float* errors, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n >= 0 && k >= 0, BATS_ERR_BAD_SHAPE, "spike_count_loss: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(counts && (targets || labels), BATS_ERR_NULL, "spike_count_loss: null pointer");
    const int warps = 4;
    BATS_CUDA(bats::launch(bats::spike_count_loss_kernel, (batch + warps - 1) / warps, warps * 32, 0, stream, counts,
        count_is_float, targets, labels, target_true, target_false, batch, n, k, loss, errors));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_ttfs_softmax_cross_entropy(const float* spikes, const int* labels, int batch, int n, int k,
                                               double tau, float* loss, float* errors, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n >= 0 && k >= 1, BATS_ERR_BAD_SHAPE, "ttfs_sce: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(spikes && labels, BATS_ERR_NULL, "ttfs_sce: null pointer");
    const int warps = 4;
    BATS_CUDA(bats::launch(bats::ttfs_sce_kernel, (batch + warps - 1) / warps, warps * 32, 0, stream, spikes, labels,
        batch, n, k, tau, (float)tau, loss, errors));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_spike_time_loss(const float* spikes, float* targets, int batch, int n, int k, int mode,
                                    float* loss, float* errors, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n >= 0 && k >= 1 && mode >= 0 && mode <= 2, BATS_ERR_BAD_SHAPE,
                 "spike_time_loss: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(spikes && targets, BATS_ERR_NULL, "spike_time_loss: null pointer");
    const int warps = 4;
    BATS_CUDA(bats::launch(bats::spike_time_loss_kernel, (batch + warps - 1) / warps, warps * 32, 0, stream, spikes,
        targets, batch, n, k, mode, loss, errors));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_adam_step(const float* grad, float* m, float* v, long long count, float beta_1, float beta_2,
                              float epsilon, float learning_rate, double bias_correction_1,
                              double bias_correction_2, float* delta, float* weights, float* weights_t, int n_post,
                              int n_pre, int ld, cudaStream_t stream) {
    BATS_REQUIRE(count >= 0, BATS_ERR_BAD_SHAPE, "adam_step: bad shape");
    if (count == 0) return BATS_OK;
    BATS_REQUIRE(grad && m && v && (delta || weights), BATS_ERR_NULL, "adam_step: null pointer");
    BATS_REQUIRE(!weights_t || ((long long)n_post * n_pre == count && ld >= n_post), BATS_ERR_BAD_SHAPE,
                 "adam_step: transposed copy needs n_post*n_pre == count");
    float r1h, r1l, r2h, r2l;
    bats::reciprocal_pair(bias_correction_1, r1h, r1l);
    bats::reciprocal_pair(bias_correction_2, r2h, r2l);
    if (weights && weights_t) {
        dim3 grid((n_pre + 31) / 32, (n_post + 31) / 32), block(32, 8);
        BATS_CUDA(bats::launch(bats::adam_tiled_kernel, grid, block, 0, stream, grad, m, v, beta_1,
            (float)(1.0 - (double)beta_1), beta_2, (float)(1.0 - (double)beta_2), bias_correction_1, bias_correction_2,
            nullptr, r1h, r1l, r2h, r2l, learning_rate, epsilon, delta, weights, weights_t, n_post, n_pre, ld));
    } else {
        BATS_CUDA(bats::launch(bats::adam_kernel, grid_for(count, 256), 256, 0, stream, grad, m, v, count, beta_1,
            (float)(1.0 - (double)beta_1), beta_2, (float)(1.0 - (double)beta_2), bias_correction_1, bias_correction_2,
            nullptr, r1h, r1l, r2h, r2l, learning_rate, epsilon, delta, weights, weights_t, n_post, n_pre, ld));
    }
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_adam_powers_advance(double* powers, float beta_1, float beta_2, cudaStream_t stream) {
    BATS_REQUIRE(powers, BATS_ERR_NULL, "adam_powers_advance: null pointer");
    BATS_CUDA(bats::launch(bats::adam_powers_kernel, 1, 32, 0, stream, powers, beta_1, beta_2));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_adam_step_device(const float* grad, float* m, float* v, long long count, float beta_1,
                                     float beta_2, float epsilon, float learning_rate, const double* powers,
                                     float* weights, float* weights_t, int n_post, int n_pre, int ld,
                                     cudaStream_t stream) {
    BATS_REQUIRE(count >= 0, BATS_ERR_BAD_SHAPE, "adam_step_device: bad shape");
    if (count == 0) return BATS_OK;
    BATS_REQUIRE(grad && m && v && weights && powers, BATS_ERR_NULL, "adam_step_device: null pointer");
    BATS_REQUIRE(!weights_t || ((long long)n_post * n_pre == count && ld >= n_post), BATS_ERR_BAD_SHAPE,
                 "adam_step_device: transposed copy needs n_post*n_pre == count");
    if (weights_t) {
        dim3 grid((n_pre + 31) / 32, (n_post + 31) / 32), block(32, 8);
        BATS_CUDA(bats::launch(bats::adam_tiled_kernel, grid, block, 0, stream, grad, m, v, beta_1,
            (float)(1.0 - (double)beta_1), beta_2, (float)(1.0 - (double)beta_2), 0.0, 0.0, powers, 0.0f, 0.0f, 0.0f,
            0.0f, learning_rate, epsilon, nullptr, weights, weights_t, n_post, n_pre, ld));
    } else {
        BATS_CUDA(bats::launch(bats::adam_kernel, grid_for(count, 256), 256, 0, stream, grad, m, v, count, beta_1,
            (float)(1.0 - (double)beta_1), beta_2, (float)(1.0 - (double)beta_2), 0.0, 0.0, powers, 0.0f, 0.0f, 0.0f,
            0.0f, learning_rate, epsilon, nullptr, weights, weights_t, n_post, n_pre, ld));
    }
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_transpose(const float* in, int rows, int cols, float* out, int ld, cudaStream_t stream) {
    BATS_REQUIRE(rows >= 0 && cols >= 0 && ld >= rows, BATS_ERR_BAD_SHAPE, "transpose: bad shape");
    if (rows == 0 || cols == 0) return BATS_OK;
    BATS_REQUIRE(in && out, BATS_ERR_NULL, "transpose: null pointer");
    dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    BATS_CUDA(bats::launch(bats::transpose_kernel, grid, dim3(32, 8), 0, stream, in, rows, cols, out, ld));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_copy_device(void* dst, const void* src, size_t bytes, cudaStream_t stream) {
    if (bytes == 0) return BATS_OK;
    BATS_REQUIRE(dst && src, BATS_ERR_NULL, "copy_device: null pointer");
    BATS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, stream));
    return BATS_OK;
}

extern "C" int bats_add_deltas(float* weights, const float* delta, long long count, float* weights_t, int n_pre,
                               int ld, cudaStream_t stream) {
    BATS_REQUIRE(count >= 0, BATS_ERR_BAD_SHAPE, "add_deltas: bad shape");
    if (count == 0) return BATS_OK;
    BATS_REQUIRE(weights && delta, BATS_ERR_NULL, "add_deltas: null pointer");
    BATS_REQUIRE(!weights_t || n_pre > 0, BATS_ERR_BAD_SHAPE, "add_deltas: n_pre");
    BATS_CUDA(bats::launch(bats::add_inplace_kernel, grid_for(count, 256), 256, 0, stream, weights, delta, count,
        weights_t, n_pre, ld));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}
