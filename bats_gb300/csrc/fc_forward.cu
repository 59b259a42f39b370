// Fully-connected LIF forward: event scan + closed-form threshold crossings.
//
// Replaces get_spike_weights + compute_spike_times
// (bats/CudaKernels/Wrappers/Inference/get_spike_weights.py:9-18,
//  bats/CudaKernels/Wrappers/Inference/compute_spike_times.py:11-32,
//  bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:86-138).
//
// Grid (ceil(N_post / TILE), B): one CTA per (post-neuron tile, sample), one thread per post
// neuron. The sample's sorted events are staged in shared memory in chunks; each event's weight
// row segment wt[j, tile] is read as one coalesced 128-byte line per warp from the transposed
// weights (L2-resident), so the (B, N_post, S) weight gather of the reference is never built.
// The per-thread recurrence is the reference's: a += w*exp(t/tau_s), b += w*exp(t/tau), then the
// crossing search in the window (t_event, t_next_event].
#include "common.cuh"
#include "abi_util.h"

namespace bats {

constexpr int FWD_CHUNK = 256;

template <int TILE, int UNROLL>
__global__ void __launch_bounds__(TILE)
lif_fc_forward_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                      const float* __restrict__ wt, int ld, int n_post, int k_post, float c, float dtt,
                      float tau, float max_sim, int* __restrict__ n_spikes, float* __restrict__ a_out,
                      float* __restrict__ x_out, float* __restrict__ t_out, float* __restrict__ z_out) {
    __shared__ Event sev[FWD_CHUNK + 1];
    const int s = blockIdx.y;
    const int i = blockIdx.x * TILE + threadIdx.x;
    const bool active = i < n_post;
    const int E = ev_count[s];
    const Event* evs = ev + (long long)s * ev_cap;
    const long long obase = ((long long)s * n_post + (active ? i : 0)) * k_post;
    float* ao = a_out + obase;
    float* xo = x_out + obase;
    float* to = t_out + obase;
    float* zo = z_out + obase;
    const float* wcol = wt + (active ? i : 0);

    float a = 0.0f, b = 0.0f;
    int n = 0;
    bool done = !active;
    for (int m0 = 0; m0 < E; m0 += FWD_CHUNK) {
        const int cnt = min(FWD_CHUNK, E - m0);
        __syncthreads();
        if (!__syncthreads_or(!done)) break;
        for (int q = threadIdx.x; q <= cnt; q += TILE) {
            Event e;
            if (m0 + q < E) {
                e = evs[m0 + q];
            } else {
                e.t = BATS_INF; e.j = 0; e.es = 0.0f; e.e = 0.0f;
            }
            sev[q] = e;
        }
        __syncthreads();
        if (done) continue;
        for (int m = 0; m < cnt; m += UNROLL) {
            float w[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const int mm = min(m + u, cnt - 1);
                w[u] = __ldg(wcol + (long long)sev[mm].j * ld);
            }
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                if (m + u < cnt && !done) {
                    const Event e = sev[m + u];
                    a += w[u] * e.es;
                    b += w[u] * e.e;
                    done = solve_crossings<false>(a, b, e.t, sev[m + u + 1].t, c, dtt, tau, max_sim, n, k_post,
                                                  ao, xo, to, zo);
                }
            }
        }
    }
    if (active) {
        n_spikes[(long long)s * n_post + i] = n;
        for (int k = n; k < k_post; ++k) {
            to[k] = BATS_INF;
            zo[k] = BATS_INF;
        }
    }
}

}  // namespace bats

extern "C" int bats_lif_forward_fc(const void* events, const int* ev_count, long long ev_cap, const float* weights_t,
                                   int ld, int batch, int n_post, int k_post, float c, float delta_theta_tau,
                                   float tau, float max_simulation, int* n_spikes, float* a, float* x, float* times,
                                   float* post_exp_tau, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0 && ld >= n_post, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc: bad shape");
    if (batch == 0 || n_post == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && weights_t && n_spikes && a && x && times && post_exp_tau, BATS_ERR_NULL,
                 "lif_forward_fc: null pointer");
    constexpr int TILE = 128;
    dim3 grid((n_post + TILE - 1) / TILE, batch);
    bats::lif_fc_forward_kernel<TILE, 8><<<grid, TILE, 0, stream>>>(
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, weights_t, ld, n_post, k_post, c,
        delta_theta_tau, tau, max_simulation, n_spikes, a, x, times, post_exp_tau);
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}
