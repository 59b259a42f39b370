// Exact multi-spike backward of a LIF layer, event-driven and linear in the number of spikes.
//
// Replaces propagate_recurrent_errors, compute_factors, compute_weights_gradient and
// propagate_errors_to_pre_spikes (bats/CudaKernels/CuFiles/Backpropagation/*.cu and the wrappers in
// bats/CudaKernels/Wrappers/Backpropagation/*.py).
//
// For a post neuron i with spikes t_0 < ... < t_{n-1}, errors err_k, factors f1_k, f2_k, define the
// suffix sums  SA_p = sum_{k>=p} err_k f1_k,  SB_p = sum_{k>=p} err_k f2_k.  For a pre spike at time
// tau_m of neuron j, let p = first k with t_k > tau_m. Then
//   dL/dW[i, j]     += exp(tau_m/tau_s) SA_p - exp(tau_m/tau) SB_p          (summed over m of j)
//   dL/dtau_m       += W[i, j] (SA_p exp(tau_m/tau_s)/tau_s - SB_p exp(tau_m/tau)/tau)   (summed over i)
// which is the reference's per-(post spike, pre neuron) merge
// (compute_weights_gradient.cu:36-45) and per-(pre spike, post neuron) loop
// (propagate_errors_to_pre_spikes.cu:41-53) regrouped around the time-sorted events of the
// forward pass: one pointer per post neuron advances monotonically while the events are scanned,
// so each (event, post neuron) pair costs O(1) and no 4-D temporary is built.
//
// The suffix sums are accumulated in the reference's order (ascending k from p, fused
// multiply-add), so SA_p equals the reference's cumul_f1 for the same pre spike bit for bit.
#include "common.cuh"
#include "abi_util.h"

namespace bats {

// One thread per (sample, post neuron): recurrent (reset) errors in place, factors, suffix tables.
//   recurrent: propagate_recurrent_errors.cu:17-22   factors: compute_factors.cu:20-30
__global__ void bwd_prep_kernel(const float* __restrict__ t, const float* __restrict__ a, const float* __restrict__ x,
                                const float* __restrict__ z, float* __restrict__ err, long long total, int K, float c,
                                float tau, float dtt, int do_recurrent, int do_factors,
                                float* __restrict__ f1, float* __restrict__ f2, float2* __restrict__ tab,
                                int* __restrict__ nvalid) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long base = idx * K;
    if (do_recurrent) {
        float cum = 0.0f;
        for (int k = K - 1; k >= 0; --k) {
            const float zk = z[base + k];
            if (isinf(zk)) continue;
            const float ek = err[base + k] + cum * zk;
            err[base + k] = ek;
            cum += ek * dtt / x[base + k];
        }
    }
    int n = K;
    for (int k = 0; k < K; ++k) {
        const float tk = t[base + k];
        if (n == K && isinf(tk)) n = k;
        if (do_factors) {
            float v1, v2;
            if (isinf(tk)) {
                v1 = 0.0f;
                v2 = 0.0f;
            } else {
                const float xk = x[base + k];
                v1 = tau / a[base + k] * (1 + z[base + k] * c / xk);
                v2 = tau / xk;
            }
            f1[base + k] = v1;
            f2[base + k] = v2;
        }
    }
    if (nvalid) nvalid[idx] = n;
    if (tab) {
        float2* tb = tab + idx * (K + 1);
        for (int p = 0; p < n; ++p) {
            float sa = 0.0f, sb = 0.0f;
            for (int k = p; k < n; ++k) {
                const float ek = err[base + k];
                sa += ek * f1[base + k];
                sb += ek * f2[base + k];
            }
            tb[p] = make_float2(sa, sb);
        }
        tb[n] = make_float2(0.0f, 0.0f);
    }
}

constexpr int BWD_CHUNK = 128;

// Weight gradient. Grid (post tiles, pre chunks, sample groups); each thread owns one post
// neuron column of a shared-memory [JC][TILE] gradient tile, so no atomics are needed and the
// per-group result is deterministic. With one sample per group the output is the reference's
// per-sample gradient (B, N_post, N_pre); with larger groups it is a partial batch sum.
template <int TILE, int JC>
__global__ void __launch_bounds__(TILE)
bwd_grad_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                const float* __restrict__ post_t, const float2* __restrict__ tab, const int* __restrict__ nvalid,
                int n_post, int k_post, int n_pre, int batch, int group, float* __restrict__ out) {
    __shared__ float G[JC][TILE + 1];
    __shared__ Event sev[BWD_CHUNK];
    const int tid = threadIdx.x;
    const int i = blockIdx.x * TILE + tid;
    const bool active = i < n_post;
    const int J0 = blockIdx.y * JC;
    const int g = blockIdx.z;
    for (int q = tid; q < JC * (TILE + 1); q += TILE) (&G[0][0])[q] = 0.0f;

    const int s_begin = g * group;
    const int s_end = min(batch, s_begin + group);
    for (int s = s_begin; s < s_end; ++s) {
        const long long pn = (long long)s * n_post + (active ? i : 0);
        const int n = active ? nvalid[pn] : 0;
        const float* tp = post_t + pn * k_post;
        const float2* tb = tab + pn * (k_post + 1);
        int p = 0;
        float2 AB = n > 0 ? tb[0] : make_float2(0.0f, 0.0f);
        float tn = n > 0 ? tp[0] : BATS_INF;
        const int E = ev_count[s];
        const Event* evs = ev + (long long)s * ev_cap;
        for (int m0 = 0; m0 < E; m0 += BWD_CHUNK) {
            const int cnt = min(BWD_CHUNK, E - m0);
            __syncthreads();
            for (int q = tid; q < cnt; q += TILE) sev[q] = evs[m0 + q];
            __syncthreads();
            for (int m = 0; m < cnt; ++m) {
                const Event e = sev[m];
                const int jj = e.j - J0;
                if (jj < 0 || jj >= JC) continue;
                while (tn <= e.t) {
                    ++p;
                    if (p < n) {
                        AB = tb[p];
                        tn = tp[p];
                    } else {
                        AB = make_float2(0.0f, 0.0f);
                        tn = BATS_INF;
                    }
                }
                if (p < n) G[jj][tid] += fmaf(e.es, AB.x, -(e.e * AB.y));
            }
        }
    }
    __syncthreads();
    // Write-out, coalesced along j.
    const long long obase = (long long)g * n_post * n_pre;
    for (int q = tid; q < TILE * JC; q += TILE) {
        const int ii = q / JC, jj = q % JC;
        const int gi = blockIdx.x * TILE + ii, gj = J0 + jj;
        if (gi < n_post && gj < n_pre) out[obase + (long long)gi * n_pre + gj] = G[jj][ii];
    }
}

// Sum of per-group partial gradients in a fixed order, divided by `divisor` (1 or the batch).
__global__ void reduce_groups_kernel(const float* __restrict__ partial, long long per_group, int groups,
                                     float divisor, float* __restrict__ out) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < per_group;
         q += (long long)gridDim.x * blockDim.x) {
        float acc = 0.0f;
        for (int g = 0; g < groups; ++g) acc += partial[(long long)g * per_group + q];
        out[q] = acc / divisor;
    }
}

// Errors of the pre-synaptic spikes. Grid (post tiles, B). Per event, each thread forms the
// reference's term w * (SA e_s / tau_s - SB e / tau) for its post neuron; the sum over the tile is
// a fixed-order warp transpose-reduction (31 shuffles per 32 events) followed by a cross-warp sum.
// Per-tile partial sums go to partial[(s, m, tile)] and are summed in tile order by
// pre_err_scatter_kernel, which writes them to the event's (neuron, slot).
template <int TILE>
__global__ void __launch_bounds__(TILE)
bwd_pre_err_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                   const float* __restrict__ wt, int ld, const float* __restrict__ post_t,
                   const float2* __restrict__ tab, const int* __restrict__ nvalid, int n_post, int k_post,
                   float tau_s, float tau, float* __restrict__ partial, int n_tiles) {
    constexpr int WARPS = TILE / 32;
    __shared__ Event sev[BWD_CHUNK];
    __shared__ float sred[WARPS][BWD_CHUNK];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s = blockIdx.y;
    const int i = blockIdx.x * TILE + tid;
    const bool active = i < n_post;
    const long long pn = (long long)s * n_post + (active ? i : 0);
    const int n = active ? nvalid[pn] : 0;
    const float* tp = post_t + pn * k_post;
    const float2* tb = tab + pn * (k_post + 1);
    const float* wcol = wt + (active ? i : 0);
    int p = 0;
    float2 AB = n > 0 ? tb[0] : make_float2(0.0f, 0.0f);
    float tn = n > 0 ? tp[0] : BATS_INF;
    const int E = ev_count[s];
    const Event* evs = ev + (long long)s * ev_cap;
    for (int m0 = 0; m0 < E; m0 += BWD_CHUNK) {
        const int cnt = min(BWD_CHUNK, E - m0);
        __syncthreads();
        for (int q = tid; q < cnt; q += TILE) sev[q] = evs[m0 + q];
        __syncthreads();
        for (int r = 0; r < cnt; r += 32) {
            float v[32];
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int mm = min(r + q, cnt - 1);
                v[q] = __ldg(wcol + (long long)sev[mm].j * ld);
            }
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                float term = 0.0f;
                if (r + q < cnt) {
                    const Event e = sev[r + q];
                    while (tn <= e.t) {
                        ++p;
                        if (p < n) {
                            AB = tb[p];
                            tn = tp[p];
                        } else {
                            AB = make_float2(0.0f, 0.0f);
                            tn = BATS_INF;
                        }
                    }
                    if (p < n) term = v[q] * (AB.x * e.es / tau_s - AB.y * e.e / tau);
                }
                v[q] = term;
            }
            const float red = warp_transpose_reduce32(v);
            sred[warp][r + lane] = red;
        }
        __syncthreads();
        for (int q = tid; q < cnt; q += TILE) {
            float acc = 0.0f;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) acc += sred[w][q];
            partial[((long long)s * ev_cap + m0 + q) * n_tiles + blockIdx.x] = acc;
        }
    }
}

__global__ void pre_err_scatter_kernel(const float* __restrict__ partial, const int* __restrict__ ev_slot,
                                       const int* __restrict__ ev_count, long long ev_cap, int n_tiles,
                                       long long slots_per_sample, float* __restrict__ pre_err) {
    const int s = blockIdx.y;
    const int E = ev_count[s];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < E; m += gridDim.x * blockDim.x) {
        const float* pp = partial + ((long long)s * ev_cap + m) * n_tiles;
        float acc = 0.0f;
        for (int q = 0; q < n_tiles; ++q) acc += pp[q];
        pre_err[(long long)s * slots_per_sample + ev_slot[(long long)s * ev_cap + m]] = acc;
    }
}

}  // namespace bats

// ---------------------------------------------------------------------------------------------
// C-ABI
constexpr int GRAD_TILE = 128;
constexpr int GRAD_JC = 64;
constexpr int PERR_TILE = 128;

extern "C" int bats_backward_prep(const float* post_times, const float* a, const float* x, const float* post_exp_tau,
                                  float* errors, int batch, int n_post, int k_post, float c, float tau,
                                  float delta_theta_tau, int do_recurrent, int do_factors, float* f1, float* f2,
                                  void* tables, int* nvalid, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0, BATS_ERR_BAD_SHAPE, "backward_prep: bad shape");
    const long long total = (long long)batch * n_post;
    if (total == 0) return BATS_OK;
    BATS_REQUIRE(post_times && errors && (!do_recurrent || (x && post_exp_tau)), BATS_ERR_NULL,
                 "backward_prep: null pointer");
    BATS_REQUIRE(!do_factors || (a && x && post_exp_tau && f1 && f2), BATS_ERR_NULL, "backward_prep: null factor");
    BATS_REQUIRE(!tables || (f1 && f2), BATS_ERR_NULL, "backward_prep: tables need f1/f2");
    const int threads = 128;
    const int blocks = (int)((total + threads - 1) / threads);
    bats::bwd_prep_kernel<<<blocks, threads, 0, stream>>>(post_times, a, x, post_exp_tau, errors, total, k_post, c,
                                                         tau, delta_theta_tau, do_recurrent, do_factors, f1, f2,
                                                         reinterpret_cast<float2*>(tables), nvalid);
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" size_t bats_weights_gradient_workspace_bytes(int batch, int n_post, int n_pre, int group) {
    if (group <= 1 || group >= batch) return 0;
    const long long groups = (batch + group - 1) / group;
    return (size_t)groups * n_post * n_pre * sizeof(float);
}

extern "C" int bats_weights_gradient(const void* events, const int* ev_count, long long ev_cap, const float* post_times,
                                     const void* tables, const int* nvalid, int batch, int n_post, int k_post,
                                     int n_pre, int group, int mean, float* grad, void* workspace,
                                     size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0 && k_post > 0 && group >= 1, BATS_ERR_BAD_SHAPE,
                 "weights_gradient: bad shape");
    if (batch == 0 || n_post == 0 || n_pre == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && post_times && tables && nvalid && grad, BATS_ERR_NULL,
                 "weights_gradient: null pointer");
    dim3 block(GRAD_TILE);
    if (group == 1) {
        // Per-sample gradient (B, N_post, N_pre).
        dim3 grid((n_post + GRAD_TILE - 1) / GRAD_TILE, (n_pre + GRAD_JC - 1) / GRAD_JC, batch);
        bats::bwd_grad_kernel<GRAD_TILE, GRAD_JC><<<grid, block, 0, stream>>>(
            reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, post_times,
            reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, n_pre, batch, 1, grad);
        BATS_CUDA(cudaGetLastError());
        return BATS_OK;
    }
    // Batch mean (N_post, N_pre).
    const int groups = (batch + group - 1) / group;
    float* part = grad;
    if (groups > 1) {
        BATS_REQUIRE(workspace && workspace_bytes >= bats_weights_gradient_workspace_bytes(batch, n_post, n_pre, group),
                     BATS_ERR_WORKSPACE, "weights_gradient: workspace too small");
        part = reinterpret_cast<float*>(workspace);
    }
    dim3 grid((n_post + GRAD_TILE - 1) / GRAD_TILE, (n_pre + GRAD_JC - 1) / GRAD_JC, groups);
    bats::bwd_grad_kernel<GRAD_TILE, GRAD_JC><<<grid, block, 0, stream>>>(
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, post_times,
        reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, n_pre, batch, group, part);
    BATS_CUDA(cudaGetLastError());
    const long long per = (long long)n_post * n_pre;
    const int rb = (int)std::min<long long>((per + 255) / 256, 152LL * 8);
    bats::reduce_groups_kernel<<<rb, 256, 0, stream>>>(part, per, groups, mean ? (float)batch : 1.0f, grad);
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" size_t bats_pre_errors_workspace_bytes(int batch, long long ev_cap, int n_post) {
    const long long tiles = (n_post + PERR_TILE - 1) / PERR_TILE;
    return (size_t)batch * ev_cap * tiles * sizeof(float);
}

extern "C" int bats_pre_errors(const void* events, const int* ev_slot, const int* ev_count, long long ev_cap,
                               const float* weights_t, int ld, const float* post_times, const void* tables,
                               const int* nvalid, int batch, int n_post, int k_post, int n_pre, int k_pre,
                               float tau_s, float tau, float* pre_errors, void* workspace, size_t workspace_bytes,
                               cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0 && k_post > 0 && k_pre > 0 && ld >= n_post,
                 BATS_ERR_BAD_SHAPE, "pre_errors: bad shape");
    if (batch == 0 || n_pre == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_slot && ev_count && pre_errors, BATS_ERR_NULL, "pre_errors: null pointer");
    const long long slots = (long long)n_pre * k_pre;
    BATS_CUDA(cudaMemsetAsync(pre_errors, 0, (size_t)batch * slots * sizeof(float), stream));
    if (n_post == 0) return BATS_OK;
    BATS_REQUIRE(weights_t && post_times && tables && nvalid, BATS_ERR_NULL, "pre_errors: null pointer");
    BATS_REQUIRE(workspace && workspace_bytes >= bats_pre_errors_workspace_bytes(batch, ev_cap, n_post),
                 BATS_ERR_WORKSPACE, "pre_errors: workspace too small");
    const int tiles = (n_post + PERR_TILE - 1) / PERR_TILE;
    float* part = reinterpret_cast<float*>(workspace);
    dim3 grid(tiles, batch);
    bats::bwd_pre_err_kernel<PERR_TILE><<<grid, PERR_TILE, 0, stream>>>(
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, weights_t, ld, post_times,
        reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, tau_s, tau, part, tiles);
    BATS_CUDA(cudaGetLastError());
    dim3 g2((unsigned)std::min<long long>((ev_cap + 255) / 256, 64), batch);
    bats::pre_err_scatter_kernel<<<g2, 256, 0, stream>>>(part, ev_slot, ev_count, ev_cap, tiles, slots, pre_errors);
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// ---------------------------------------------------------------------------------------------
// Allocation-free variant of the batch-mean weight gradient.
//
// Some callers cannot allocate device memory on the path that calls this library: a runtime that
// owns every device allocation up front (a fixed arena or pool it may not grow), a host whose
// plugin interface hands the plugin only input and output buffers, or a caller in a language with
// no CUDA allocator of its own. For them, bats_weights_gradient_mean_noalloc keeps its per-group
// partial sums in this file-scope device array instead of a caller-provided workspace. The array is
// part of the library image, so every GPU that loads the library holds it (32 MiB) until the process
// exits. Every call shares it: two calls whose kernels overlap on the GPU (different streams, or
// different host threads on one device) race on it and must be serialised by the caller. The kernel
// writes every partial it later reads, so nothing has to be cleared between calls.
constexpr long long NOALLOC_GRAD_SCRATCH_FLOATS = 8LL * 1024 * 1024;  // 32 MiB
static __device__ __align__(256) float g_noalloc_grad_scratch[NOALLOC_GRAD_SCRATCH_FLOATS];

#include <mutex>

// Device address of the scratch array, looked up once per device (host code only sees a stand-in
// for the symbol, so the address must come from cudaGetSymbolAddress with that device current).
static int noalloc_scratch_ptr(float** out) {
    static std::mutex mu;
    static float* cache[128] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (dev < 0 || dev >= 128) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_grad_scratch);
        if (e != cudaSuccess) return (int)e;
        cache[dev] = reinterpret_cast<float*>(p);
    }
    *out = cache[dev];
    return (int)cudaSuccess;
}

extern "C" long long bats_weights_gradient_noalloc_capacity(void) { return NOALLOC_GRAD_SCRATCH_FLOATS; }

extern "C" int bats_weights_gradient_mean_noalloc(const void* events, const int* ev_count, long long ev_cap,
                                                  const float* post_times, const void* tables, const int* nvalid,
                                                  int batch, int n_post, int k_post, int n_pre, int group,
                                                  float* grad, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0 && k_post > 0 && group >= 2, BATS_ERR_BAD_SHAPE,
                 "weights_gradient_mean_noalloc: bad shape (group must be >= 2)");
    if (batch == 0 || n_post == 0 || n_pre == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && post_times && tables && nvalid && grad, BATS_ERR_NULL,
                 "weights_gradient_mean_noalloc: null pointer");
    const int groups = (batch + group - 1) / group;
    const long long per = (long long)n_post * n_pre;
    float* part = grad;
    if (groups > 1) {
        BATS_REQUIRE(per <= NOALLOC_GRAD_SCRATCH_FLOATS / groups, BATS_ERR_CAPACITY,
                     "weights_gradient_mean_noalloc: ceil(batch/group) * n_post * n_pre exceeds the 8 Mi-float "
                     "(32 MiB) static scratch; use a larger group or bats_weights_gradient with a workspace");
        BATS_CUDA((cudaError_t)noalloc_scratch_ptr(&part));
    }
    dim3 grid((n_post + GRAD_TILE - 1) / GRAD_TILE, (n_pre + GRAD_JC - 1) / GRAD_JC, groups);
    bats::bwd_grad_kernel<GRAD_TILE, GRAD_JC><<<grid, GRAD_TILE, 0, stream>>>(
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, post_times,
        reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, n_pre, batch, group, part);
    BATS_CUDA(cudaGetLastError());
    const int rb = (int)std::min<long long>((per + 255) / 256, 152LL * 8);
    bats::reduce_groups_kernel<<<rb, 256, 0, stream>>>(part, per, groups, (float)batch, grad);
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}
