// NAdam and the synaptic-scaling gradient regularizers.
//
// NAdam replaces the three CuPy element-wise kernels of bats/Optimizers/NAdamOptimizer.py:6-20 and its
// step (:35-58) with one pass over the tensor. The regularizers are the reference's
// bats/CudaKernels/CuFiles/Regularization/apply_weights_synaptic_scaling.cu and
// apply_label_weights_synaptic_scaling.cu: they push the per-sample gradient of silent neurons towards
// larger weights, by factor * |w|.
#include <cmath>
#include "abi_util.h"
#include "common.cuh"

namespace bats {

// m, v updated in place (update_m_kernel / update_v_kernel); m_hat, v_hat = m / (1 - beta_1^t),
// v / (1 - beta_2^t) with the corrections in double and the results rounded to float (the host scalars
// of the reference are float64); delta = -(lr / (sqrt(v_hat) + eps)) *
// (beta_1 m_hat + (1 - beta_1) g / (1 - beta_1^t)) with the correction passed as float32, as the
// reference's compute_deltas_kernel receives it.
__global__ void nadam_kernel(const float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                             long long count, float beta_1, float one_minus_beta_1, float beta_2,
                             float one_minus_beta_2, double bias1, double bias2, float bias1_f, float r1_hi,
                             float r1_lo, float r2_hi, float r2_lo, float lr, float eps, float* __restrict__ delta) {
    pdl_prologue();
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < count;
         q += (long long)gridDim.x * blockDim.x) {
        const float g = grad[q];
        const float nm = beta_1 * m[q] + one_minus_beta_1 * g;
        const float nv = beta_2 * v[q] + one_minus_beta_2 * g * g;
        m[q] = nm;
        v[q] = nv;
        const float m_hat = quotient_f64_to_f32(nm, r1_hi, r1_lo, bias1);  // (float)((double)nm / bias1)
        const float v_hat = quotient_f64_to_f32(nv, r2_hi, r2_lo, bias2);
        delta[q] = -(lr / (sqrtf(v_hat) + eps)) * (beta_1 * m_hat + one_minus_beta_1 * g / bias1_f);
    }
}

// gradient[s, i, j] -= factor * |W[i, j]| for every sample whose silent ratio reaches the threshold and
// every post neuron i that did not spike in it (apply_weights_synaptic_scaling.cu:2-25).
__global__ void weights_synaptic_scaling_kernel(const float* __restrict__ w, const float* __restrict__ silent_ratios,
                                                const int* __restrict__ n_spikes, float* __restrict__ gradient,
                                                int batch, int n_post, int n_pre, float threshold, float factor) {
    pdl_prologue();
    const long long total = (long long)batch * n_post * n_pre;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const long long si = q / n_pre;  // sample * n_post + post
        const int j = (int)(q % n_pre);
        const int s = (int)(si / n_post), i = (int)(si % n_post);
        if (silent_ratios[s] < threshold) continue;
        if (n_spikes[si] > 0) continue;
        gradient[q] -= factor * fabsf(w[(long long)i * n_pre + j]);
    }
}

// gradient[s, label_s, j] -= factor * |W[label_s, j]| unless the label neuron spiked
// (apply_label_weights_synaptic_scaling.cu:2-20). The reference reads the spike count as
// n_spike_per_neuron[label], i.e. in the first sample's row; that indexing is kept.
__global__ void label_weights_synaptic_scaling_kernel(const float* __restrict__ w, const float* __restrict__ labels,
                                                      const int* __restrict__ n_spikes, float* __restrict__ gradient,
                                                      int batch, int n_post, int n_pre, float factor) {
    pdl_prologue();
    const long long total = (long long)batch * n_pre;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(q / n_pre), j = (int)(q % n_pre);
        const int label = (int)labels[s];
        if (label < 0 || label >= n_post) continue;  // not a neuron of the layer: nothing to scale
        if (n_spikes[label] > 0) continue;
        gradient[((long long)s * n_post + label) * n_pre + j] -= factor * fabsf(w[(long long)label * n_pre + j]);
    }
}

static int grid_for(long long count, int threads) {
    const long long blocks = (count + threads - 1) / threads;
    return (int)(blocks < 152LL * 16 ? (blocks < 1 ? 1 : blocks) : 152LL * 16);
}

}  // namespace bats

extern "C" int bats_nadam_step(const float* grad, float* m, float* v, long long count, float beta_1, float beta_2,
                               float epsilon, float learning_rate, double bias_correction_1,
                               double bias_correction_2, float* delta, cudaStream_t stream) {
    BATS_REQUIRE(count >= 0, BATS_ERR_BAD_SHAPE, "nadam_step: bad shape");
    if (count == 0) return BATS_OK;
    BATS_REQUIRE(grad && m && v && delta, BATS_ERR_NULL, "nadam_step: null pointer");
    float r1h, r1l, r2h, r2l;
    bats::reciprocal_pair(bias_correction_1, r1h, r1l);
    bats::reciprocal_pair(bias_correction_2, r2h, r2l);
    BATS_CUDA(bats::launch(bats::nadam_kernel, bats::grid_for(count, 256), 256, 0, stream, grad, m, v, count, beta_1,
        (float)(1.0 - (double)beta_1), beta_2, (float)(1.0 - (double)beta_2), bias_correction_1, bias_correction_2,
        (float)bias_correction_1, r1h, r1l, r2h, r2l, learning_rate, epsilon, delta));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_weights_synaptic_scaling(const float* weights, const float* silent_ratios, const int* n_spikes,
                                             float* gradient, int batch, int n_post, int n_pre, float threshold,
                                             float factor, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0, BATS_ERR_BAD_SHAPE, "weights_synaptic_scaling: bad shape");
    const long long total = (long long)batch * n_post * n_pre;
    if (total == 0) return BATS_OK;
    BATS_REQUIRE(weights && silent_ratios && n_spikes && gradient, BATS_ERR_NULL,
                 "weights_synaptic_scaling: null pointer");
    BATS_CUDA(bats::launch(bats::weights_synaptic_scaling_kernel, bats::grid_for(total, 256), 256, 0, stream, weights,
        silent_ratios, n_spikes, gradient, batch, n_post, n_pre, threshold, factor));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_label_weights_synaptic_scaling(const float* weights, const float* labels, const int* n_spikes,
                                                   float* gradient, int batch, int n_post, int n_pre, float factor,
                                                   cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0, BATS_ERR_BAD_SHAPE,
                 "label_weights_synaptic_scaling: bad shape");
    const long long total = (long long)batch * n_pre;
    if (total == 0 || n_post == 0) return BATS_OK;
    BATS_REQUIRE(weights && labels && n_spikes && gradient, BATS_ERR_NULL,
                 "label_weights_synaptic_scaling: null pointer");
    BATS_CUDA(bats::launch(bats::label_weights_synaptic_scaling_kernel, bats::grid_for(total, 256), 256, 0, stream,
        weights, labels, n_spikes, gradient, batch, n_post, n_pre, factor));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}
