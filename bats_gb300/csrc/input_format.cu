// Event-list input format: (neuron index, time) per spike, in order of appearance, index < 0 ending a
// sample -> per-neuron spike trains (B, N, K) + counts (B, N), the layout every layer reads.
//
// Replaces convert_to_spike_per_neuron (bats/CudaKernels/CuFiles/Inference/convert_to_spike_per_neuron.cu:2-26,
// Wrappers/Inference/convert_to_spike_per_neuron.py:20-33): the reference runs one thread per sample
// over its events; here one warp per sample takes 32 events at a time and ranks events of the same
// neuron by __match_any_sync, so every spike lands in the slot of its order of appearance, as in the
// reference. Slots past a neuron's count hold +inf. Spikes beyond k_cap slots are dropped and counted in
// *overflow (the reference sizes K to the batch maximum with a host-side cp.unique loop; callers that
// need the same do so from the counts of a first pass).
#include "common.cuh"
#include "abi_util.h"

namespace bats {

constexpr int CONV_WARPS = 4;
// Per-sample neuron counts are kept in shared memory up to this many neurons (with the event windows below,
// 48 KB in all, no opt-in needed); larger layers keep them in the output counts array.
constexpr int CONV_SMEM_NEURONS = 8000;  // 32 000 B of counts + 16 400 B of windows <= 48 KB
constexpr int CONV_WINDOW = 1024;  // events per shared-memory window (two windows: double buffering)

// One CTA per sample. The sample's events are staged through shared memory in windows of CONV_WINDOW
// (indices and times, coalesced loads by warps 1..3, one window ahead of the ranking). Warp 0 ranks each
// window's events in order of appearance, 32 at a time (events of the same neuron ranked by
// __match_any_sync), writing each spike into its slot, with the per-neuron counts in shared memory when
// SMEM_COUNTS: a 32-event step then waits on shared memory only. Finally all warps set the slots past each
// neuron's count to +inf (row by row, contiguous stores) and write the counts.
template <bool SMEM_COUNTS>
__global__ void __launch_bounds__(CONV_WARPS * 32)
events_to_trains_kernel(const int* __restrict__ indices, const float* __restrict__ times,
                        const int* __restrict__ offsets, int batch, int max_events, int n_neurons, int k_cap,
                        float* __restrict__ out_times, int* __restrict__ out_counts, int* __restrict__ overflow) {
    pdl_prologue();
    extern __shared__ int s_cnt[];
    __shared__ int w_idx[2][CONV_WINDOW];
    __shared__ float w_t[2][CONV_WINDOW];
    __shared__ int s_stop;  // the sample ended (negative or out-of-range index) inside the current window
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s = blockIdx.x;
    const long long tb = (long long)s * n_neurons * k_cap;
    int* cnt = SMEM_COUNTS ? s_cnt : out_counts + (long long)s * n_neurons;
    for (int q = tid; q < n_neurons; q += blockDim.x) cnt[q] = 0;
    // Padded rows (B, max_events), or with offsets the events offsets[s] .. offsets[s + 1] of a flat list.
    const long long first = offsets ? (long long)offsets[s] : (long long)s * max_events;
    const int n_ev = offsets ? offsets[s + 1] - offsets[s] : max_events;
    const int* idx = indices + first;
    const float* tm = times + first;
    const int n_win = (n_ev + CONV_WINDOW - 1) / CONV_WINDOW;
    // Window 0, loaded by every thread.
    for (int q = tid; q < min(n_ev, CONV_WINDOW); q += blockDim.x) {
        w_idx[0][q] = idx[q];
        w_t[0][q] = tm[q];
    }
    if (tid == 0) s_stop = 0;
    __syncthreads();
    int dropped = 0;
    for (int w = 0; w < n_win; ++w) {
        const int buf = w & 1;
        const int m_base = w * CONV_WINDOW;
        const int cnt_w = min(CONV_WINDOW, n_ev - m_base);
        if (warp == 0) {
            for (int m0 = 0; m0 < cnt_w; m0 += 32) {
                const int m = m0 + lane;
                int j = m < cnt_w ? w_idx[buf][m] : -1;
                const float t = m < cnt_w ? w_t[buf][m] : 0.0f;
                // The sample ends at its first negative (or out-of-range) index.
                const unsigned neg = __ballot_sync(0xffffffffu, j < 0 || j >= n_neurons);
                const int stop = neg ? __ffs(neg) - 1 : 32;
                const bool valid = lane < stop;
                if (!valid) j = -1 - lane;  // distinct keys so that invalid lanes never match
                const unsigned peers = __match_any_sync(0xffffffffu, j);
                const int rank = __popc(peers & lanemask_lt());
                int base = 0;
                if (valid && rank == 0) base = cnt[j];
                base = __shfl_sync(0xffffffffu, base, __ffs(peers) - 1);
                if (valid) {
                    const int slot = base + rank;
                    if (slot < k_cap)
                        out_times[tb + (long long)j * k_cap + slot] = t;
                    else
                        ++dropped;
                    if (rank == 0) cnt[j] = min(base + __popc(peers), k_cap);
                }
                __syncwarp();
                if (stop < 32) {
                    if (lane == 0) s_stop = 1;
                    break;
                }
            }
        } else if (w + 1 < n_win) {
            // Warps 1..3: the next window into the other buffer.
            const int nb = m_base + CONV_WINDOW;
            const int cnt_n = min(CONV_WINDOW, n_ev - nb);
            for (int q = tid - 32; q < cnt_n; q += blockDim.x - 32) {
                w_idx[buf ^ 1][q] = idx[nb + q];
                w_t[buf ^ 1][q] = tm[nb + q];
            }
        }
        __syncthreads();
        if (s_stop) break;
    }
    if (warp == 0) {
        for (int o = 16; o >= 1; o >>= 1) dropped += __shfl_xor_sync(0xffffffffu, dropped, o);
        if (lane == 0 && dropped && overflow) atomicAdd(overflow, dropped);
    }
    // +inf past each neuron's spikes; the ranking above wrote only the slots below the counts.
    for (int j = warp; j < n_neurons; j += CONV_WARPS) {
        float* row = out_times + tb + (long long)j * k_cap;
        for (int k = cnt[j] + lane; k < k_cap; k += 32) row[k] = BATS_INF;
    }
    if (SMEM_COUNTS)
        for (int q = tid; q < n_neurons; q += blockDim.x) out_counts[(long long)s * n_neurons + q] = cnt[q];
}

static int launch_events_to_trains(const int* indices, const float* times, const int* offsets, int batch,
                                   int max_events, int n_neurons, int k_cap, float* out_times, int* out_counts,
                                   int* overflow, cudaStream_t stream) {
    if (n_neurons <= CONV_SMEM_NEURONS)
        BATS_CUDA(bats::launch(events_to_trains_kernel<true>, batch, CONV_WARPS * 32, (size_t)n_neurons * sizeof(int),
            stream, indices, times, offsets, batch, max_events, n_neurons, k_cap, out_times, out_counts, overflow));
    else
        BATS_CUDA(bats::launch(events_to_trains_kernel<false>, batch, CONV_WARPS * 32, 0, stream, indices, times,
            offsets, batch, max_events, n_neurons, k_cap, out_times, out_counts, overflow));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// Largest per-neuron spike count of each sample (the K the reference derives on the host).
// Warp per sample; the counts live in a warp-private slice of shared memory when SMEM_COUNTS (else in the
// caller's scratch).
template <bool SMEM_COUNTS>
__global__ void __launch_bounds__(CONV_WARPS * 32)
max_per_neuron_kernel(const int* __restrict__ indices, int batch, int max_events, int n_neurons,
                      int* __restrict__ scratch_counts, int* __restrict__ out_max) {
    pdl_prologue();
    extern __shared__ int s_cnt[];
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * CONV_WARPS + (threadIdx.x >> 5);
    if (s >= batch) return;
    int* cnt = SMEM_COUNTS ? s_cnt + (threadIdx.x >> 5) * n_neurons : scratch_counts + (long long)s * n_neurons;
    for (int q = lane; q < n_neurons; q += 32) cnt[q] = 0;
    __syncwarp();
    const int* idx = indices + (long long)s * max_events;
    int best = 0;
    for (int m0 = 0; m0 < max_events; m0 += 32) {
        const int m = m0 + lane;
        int j = m < max_events ? idx[m] : -1;
        const unsigned neg = __ballot_sync(0xffffffffu, j < 0 || j >= n_neurons);
        const int stop = neg ? __ffs(neg) - 1 : 32;
        const bool valid = lane < stop;
        if (!valid) j = -1 - lane;
        const unsigned peers = __match_any_sync(0xffffffffu, j);
        const int rank = __popc(peers & lanemask_lt());
        int base = 0;
        if (valid && rank == 0) base = cnt[j];
        base = __shfl_sync(0xffffffffu, base, __ffs(peers) - 1);
        if (valid && rank == 0) {
            cnt[j] = base + __popc(peers);
            best = max(best, base + __popc(peers));
        }
        __syncwarp();
        if (stop < 32) break;
    }
    for (int o = 16; o >= 1; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (lane == 0) out_max[s] = best;
}

}  // namespace bats

extern "C" int bats_events_to_trains(const int* indices, const float* times, int batch, int max_events, int n_neurons,
                                     int k_cap, float* out_times, int* out_counts, int* overflow,
                                     cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && max_events >= 0 && n_neurons > 0 && k_cap > 0, BATS_ERR_BAD_SHAPE,
                 "events_to_trains: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(out_times && out_counts && (max_events == 0 || (indices && times)), BATS_ERR_NULL,
                 "events_to_trains: null pointer");
    return bats::launch_events_to_trains(indices, times, nullptr, batch, max_events, n_neurons, k_cap, out_times,
                                         out_counts, overflow, stream);
}

extern "C" int bats_events_to_trains_csr(const int* indices, const float* times, const int* offsets, int batch,
                                         int n_neurons, int k_cap, float* out_times, int* out_counts, int* overflow,
                                         cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_neurons >= 0 && k_cap > 0, BATS_ERR_BAD_SHAPE, "events_to_trains_csr: bad shape");
    if (batch == 0 || n_neurons == 0) return BATS_OK;
    BATS_REQUIRE(indices && times && offsets && out_times && out_counts, BATS_ERR_NULL,
                 "events_to_trains_csr: null pointer");
    return bats::launch_events_to_trains(indices, times, offsets, batch, 0, n_neurons, k_cap, out_times, out_counts,
                                         overflow, stream);
}

extern "C" int bats_events_max_per_neuron(const int* indices, int batch, int max_events, int n_neurons,
                                          int* scratch_counts, int* out_max, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && max_events >= 0 && n_neurons > 0, BATS_ERR_BAD_SHAPE,
                 "events_max_per_neuron: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(scratch_counts && out_max && (max_events == 0 || indices), BATS_ERR_NULL,
                 "events_max_per_neuron: null pointer");
    const int blocks = (batch + bats::CONV_WARPS - 1) / bats::CONV_WARPS;
    if (n_neurons * bats::CONV_WARPS <= 12288)  // 48 KB of warp-private counts
        BATS_CUDA(bats::launch(bats::max_per_neuron_kernel<true>, blocks, bats::CONV_WARPS * 32,
            (size_t)n_neurons * bats::CONV_WARPS * sizeof(int), stream, indices, batch, max_events, n_neurons,
            scratch_counts, out_max));
    else
        BATS_CUDA(bats::launch(bats::max_per_neuron_kernel<false>, blocks, bats::CONV_WARPS * 32, 0, stream, indices,
            batch, max_events, n_neurons, scratch_counts, out_max));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// Intensity (time-to-first-spike) encoding of the reference's MNIST pipeline
// (experiments/mnist/Dataset.py:66-71): one spike per input at t = time_window * (1 - x / max_value),
// evaluated in double as NumPy does, and no spike (+inf, count 0) where t equals time_window (x == 0).
namespace bats {
__global__ void intensity_to_spike_times_kernel(const unsigned char* __restrict__ pixels, long long total,
                                                double time_window, double max_value, float* __restrict__ times,
                                                int* __restrict__ counts) {
    pdl_prologue();
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const double t = time_window * (1.0 - ((double)pixels[q] / max_value));
        const bool spike = t != time_window;
        times[q] = spike ? (float)t : BATS_INF;
        counts[q] = spike ? 1 : 0;
    }
}
}  // namespace bats

extern "C" int bats_intensity_to_spike_times(const unsigned char* pixels, int batch, int n_neurons, double time_window,
                                             double max_value, float* times, int* counts, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_neurons >= 0 && max_value > 0.0, BATS_ERR_BAD_SHAPE,
                 "intensity_to_spike_times: bad shape");
    const long long total = (long long)batch * n_neurons;
    if (total == 0) return BATS_OK;
    BATS_REQUIRE(pixels && times && counts, BATS_ERR_NULL, "intensity_to_spike_times: null pointer");
    const long long blocks = (total + 255) / 256;
    BATS_CUDA(bats::launch(bats::intensity_to_spike_times_kernel,
        (int)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, stream, pixels, total, time_window, max_value, times, counts));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}
