// Fully-connected LIF forward: event scan + closed-form threshold crossings.
//
// Replaces get_spike_weights + compute_spike_times
// (bats/CudaKernels/Wrappers/Inference/get_spike_weights.py:9-18,
//  bats/CudaKernels/Wrappers/Inference/compute_spike_times.py:11-32,
//  bats/CudaKernels/CuFiles/Inference/compute_spike_times.cu:86-138).
//
// Grid (ceil(N_post / TILE), B): one CTA per (post-neuron tile, sample). The reference gathers a
// dense (B, N_post, S) weight array first; here a producer warp streams, for every event of the
// sample in time order, the event record and the weight-row segment wt[j, tile] (TILE floats) into a
// ring of shared-memory stages with bulk copies (cp.async.bulk, completing on an mbarrier), running
// up to STAGES * SEV events ahead of the consumers, so no weight load sits on the consumers' path.
// Each consumer thread owns one post neuron and runs the reference's recurrence
// a += w*exp(t/tau_s), b += w*exp(t/tau), crossing search in (t_event, t_next_event].
// Per stage the consumer first accumulates all SEV events and evaluates the provable no-crossing
// test on each intermediate state; only if some event may cross does it replay the stage from its
// saved state with the exact solver. The accumulation is the same FMA sequence either way, so the
// results are those of the reference's one-event-at-a-time loop.
#include <cmath>
#include <limits>
#include "common.cuh"
#include "pipeline.cuh"
#include "abi_util.h"

namespace bats {

template <int TILE, int SEV, int STAGES>
__global__ void __launch_bounds__(TILE + 32)
lif_fc_forward_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                      const float* __restrict__ wt, int ld, int n_post, int k_post, SolveConst sk,
                      int* __restrict__ n_spikes, float* __restrict__ a_out, float* __restrict__ x_out,
                      float* __restrict__ t_out, float* __restrict__ z_out, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using Smem = StreamSmem<TILE, SEV, STAGES>;
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    constexpr int CONSUMER_WARPS = TILE / 32;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int s = blockIdx.y;
    const int tile0 = blockIdx.x * TILE;
    const int E = ev_count[s];
    const int n_stages = (E + SEV - 1) / SEV;
    const Event* evs = ev + (long long)s * ev_cap;
    stream_init(sm, CONSUMER_WARPS);
    __syncthreads();
    if (warp == CONSUMER_WARPS) {
        stream_produce(sm, evs, E, wt, ld, tile0, n_stages, lane, status);
        return;
    }

    // ---- consumer warps: thread = post neuron ----
    const int i = tile0 + tid;
    const bool active = i < n_post;
    const long long obase = ((long long)s * n_post + (active ? i : 0)) * k_post;
    float* ao = a_out + obase;
    float* xo = x_out + obase;
    float* to = t_out + obase;
    float* zo = z_out + obase;
    float a = 0.0f, b = 0.0f;
    int n = 0;
    bool done = !active;
    for (int k = 0; k < n_stages; ++k) {
        const int slot = k % STAGES;
        if (!stream_acquire(sm, k, status)) return;
        const int m0 = k * SEV;
        const int cnt = min(SEV, E - m0);
        const Event* se = sm.evs[slot];
        if (!done) {
            // Pass 1: accumulate the stage's events (the reference's FMA sequence) and mark every event
            // after which a crossing cannot be ruled out. Branch-free, so the per-event tests of the
            // stage overlap; events past the sample's end (last stage) leave the state unchanged.
            float aa = a, bb = b;
            unsigned cand = 0u;
#pragma unroll
            for (int u = 0; u < SEV; ++u) {
                const float4 e4 = *reinterpret_cast<const float4*>(&se[u]);  // (t, j, es, e)
                const float e_nx = se[u + 1].e;
                const float w = sm.rows[slot][u][tid];
                const bool in = u < cnt;
                const float a2 = fmaf(w, e4.z, aa);
                const float b2 = fmaf(w, e4.w, bb);
                aa = in ? a2 : aa;
                bb = in ? b2 : bb;
                const float e_next = (m0 + u + 1 < E) ? e_nx : BATS_INF;
                const bool maybe = !no_crossing<false>(aa, bb, e_next, sk);
                cand |= (in && maybe) ? (1u << u) : 0u;
            }
            if (cand == 0u) {
                a = aa;
                b = bb;
            } else {
                // Pass 2: no crossing is possible before the first marked event, so its state is
                // reached by the plain accumulation; from there on, the reference's event-by-event loop.
                const int first = __ffs(cand) - 1;
                for (int u = 0; u < first; ++u) {
                    const float wu = sm.rows[slot][u][tid];
                    a = fmaf(wu, se[u].es, a);
                    b = fmaf(wu, se[u].e, b);
                }
                for (int u = first; u < cnt; ++u) {
                    const Event e = se[u];
                    const float wu = sm.rows[slot][u][tid];
                    a = fmaf(wu, e.es, a);
                    b = fmaf(wu, e.e, b);
                    const bool has_next = m0 + u + 1 < E;
                    const float t_next = has_next ? se[u + 1].t : BATS_INF;
                    const float e_next = has_next ? se[u + 1].e : BATS_INF;
                    done = solve_crossings<false>(a, b, e.t, t_next, e_next, sk, n, k_post, ao, xo, to, zo);
                    if (done) break;
                }
            }
        }
        stream_release(sm, k);
    }
    if (active) {
        n_spikes[(long long)s * n_post + i] = n;
        for (int q = n; q < k_post; ++q) {
            to[q] = BATS_INF;
            zo[q] = BATS_INF;
        }
    }
}

template <int TILE, int SEV, int STAGES>
static int launch_forward(const void* events, const int* ev_count, long long ev_cap, const float* wt, int ld, int batch,
                          int n_post, int k_post, const SolveConst& sk, int* n_spikes, float* a, float* x,
                          float* times, float* post_exp_tau, int* status, cudaStream_t stream) {
    const size_t smem = sizeof(StreamSmem<TILE, SEV, STAGES>);
    BATS_CUDA((cudaError_t)max_dynamic_smem_set((const void*)lif_fc_forward_kernel<TILE, SEV, STAGES>, (int)smem));
    dim3 grid((n_post + TILE - 1) / TILE, batch);
    lif_fc_forward_kernel<TILE, SEV, STAGES><<<grid, TILE + 32, smem, stream>>>(
        reinterpret_cast<const Event*>(events), ev_count, ev_cap, wt, ld, n_post, k_post, sk, n_spikes, a, x, times,
        post_exp_tau, status);
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

SolveConst make_solve_const(float c, float dtt, float tau, float max_sim) {
    SolveConst k;
    k.c = c;
    k.dtt = dtt;
    k.tau = tau;
    k.max_sim = max_sim;
    const double em = std::exp((double)max_sim / (double)tau);
    k.e_max = std::isfinite(em) && em < 3.0e38 ? (float)em : std::numeric_limits<float>::infinity();
    k.inv_c = c > 0.0f ? 1.0f / c : 0.0f;
    k.fast = c > 0.0f && tau > 0.0f;
    return k;
}

}  // namespace bats

extern "C" int bats_lif_forward_fc(const void* events, const int* ev_count, long long ev_cap, const float* weights_t,
                                   int ld, int batch, int n_post, int k_post, float c, float delta_theta_tau,
                                   float tau, float max_simulation, int* n_spikes, float* a, float* x, float* times,
                                   float* post_exp_tau, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0 && ld >= n_post && ld % 4 == 0, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc: bad shape (ld must be >= n_post and a multiple of 4)");
    if (batch == 0 || n_post == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && weights_t && n_spikes && a && x && times && post_exp_tau, BATS_ERR_NULL,
                 "lif_forward_fc: null pointer");
    BATS_REQUIRE(((uintptr_t)weights_t & 15) == 0 && ((uintptr_t)events & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc: weights_t and events must be 16-byte aligned");
    const bats::SolveConst sk = bats::make_solve_const(c, delta_theta_tau, tau, max_simulation);
    int* status = nullptr;
    BATS_CUDA((cudaError_t)bats::device_status(&status));
    if (n_post <= 32)
        return bats::launch_forward<32, 16, 8>(events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                               n_spikes, a, x, times, post_exp_tau, status, stream);
    if (n_post <= 64)
        return bats::launch_forward<64, 16, 6>(events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                              n_spikes, a, x, times, post_exp_tau, status, stream);
    return bats::launch_forward<128, 16, 6>(events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                           n_spikes, a, x, times, post_exp_tau, status, stream);
}
