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
//
// Variants, all bit-identical: the stage screen (SCREEN, BATS_FWD_STAGE_SCREEN) first tests a whole
// stage with one membrane bound per neuron (quiet layers); the persistent work-queue kernel
// (bats_lif_forward_fc_queue) runs the same per-item code over (sample, tile) items taken longest
// samples first by resident CTAs (uneven batches); the lanes kernel gives a warp to one (sample, neuron)
// and 32 events at a time (narrow layers, small batches).
#include <algorithm>
#include <cmath>
#include <limits>
#include "common.cuh"
#include "pipeline.cuh"
#include "abi_util.h"

namespace bats {

// Consumer warps' part of one work item (sample s, post neurons tile0 .. tile0 + TILE - 1): thread = post
// neuron. The item's event stages are stages k0 .. k0 + ceil(E / SEV) - 1 of the CTA's ring (k0 = 0 when the
// CTA has one item). Returns false when a wait gave up (the CTA is aborting).
// SCREEN: every full stage first runs only the accumulation, tracking the smallest a and |a| and the largest
// b of its states, and skips the per-event tests when stage_no_crossing rules out a crossing after any of
// its events (quiet neurons: one test per stage instead of one per event); otherwise the stage is
// evaluated as without SCREEN. The FMA sequence is the same either way, so results are bit-identical.
// Each warp forms the window constants of the stage's events once (event_window, lane u for event u) and every
// neuron's per-event test reads them (no_crossing_at: the answers of no_crossing, with fewer instructions).
template <int TILE, int SEV, int STAGES, bool SCREEN = false>
__device__ __forceinline__ bool forward_tile_item(StreamSmem<TILE, SEV, STAGES>& sm, int k0, int s, int tile0, int E,
                                                  int n_post, int k_post, const SolveConst& sk,
                                                  int* __restrict__ n_spikes, float* __restrict__ a_out,
                                                  float* __restrict__ x_out, float* __restrict__ t_out,
                                                  float* __restrict__ z_out, int* status, int pad) {
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int n_stages = (E + SEV - 1) / SEV;
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
    __shared__ EventWindow s_win[TILE / 32][SEV];
    EventWindow* wv = s_win[warp];
    for (int k = 0; k < n_stages; ++k) {
        const int kg = k0 + k;  // the stage's place in the CTA's ring
        const int slot = kg % STAGES;
        if (!stream_acquire(sm, kg, status)) return false;
        const int m0 = k * SEV;
        const int cnt = min(SEV, E - m0);
        const Event* se = sm.evs[slot];
        // The window constants of the stage's events, formed once per warp (lane u: event u).
        if (lane < SEV) {
            const float e_nx = (m0 + lane + 1 < E) ? se[lane + 1].e : BATS_INF;
            wv[lane] = event_window(se[lane].e, e_nx, sk);
        }
        __syncwarp();
        if (!done) {
            // Pass 1: accumulate the stage's events (the reference's FMA sequence) and mark every event
            // after which a crossing cannot be ruled out. Branch-free, so the per-event tests of the
            // stage overlap; events past the sample's end (last stage) leave the state unchanged.
            float aa = a, bb = b;
            unsigned cand = 0u;
            bool screened = false;
            if (SCREEN && m0 + SEV < E) {
                float amin = BATS_INF, bmax = -BATS_INF, amag = BATS_INF;
#pragma unroll
                for (int u = 0; u < SEV; ++u) {
                    const float w = sm.rows[slot][u][tid];
                    aa = fmaf(w, se[u].es, aa);
                    bb = fmaf(w, se[u].e, bb);
                    amin = fminf(amin, aa);
                    amag = fminf(amag, fabsf(aa));
                    bmax = fmaxf(bmax, bb);
                }
                screened = stage_no_crossing(amin, bmax, amag, aa, bb, se[0].e, sk);
                if (!screened) {
                    aa = a;
                    bb = b;
                }
            }
            if (screened) {
                // no event of the stage can cross: aa, bb hold the state after the stage
            } else if (m0 + SEV < E) {
                // A full stage followed by more events (every stage but the last): no bounds to select on.
#pragma unroll
                for (int u = 0; u < SEV; ++u) {
                    const float4 e4 = *reinterpret_cast<const float4*>(&se[u]);  // (t, j, es, e)
                    const float w = sm.rows[slot][u][tid];
                    aa = fmaf(w, e4.z, aa);
                    bb = fmaf(w, e4.w, bb);
                    cand |= no_crossing_at<false>(aa, bb, wv[u], sk) ? 0u : (1u << u);
                }
            } else {
#pragma unroll
                for (int u = 0; u < SEV; ++u) {
                    const float4 e4 = *reinterpret_cast<const float4*>(&se[u]);
                    const float w = sm.rows[slot][u][tid];
                    const bool in = u < cnt;
                    const float a2 = fmaf(w, e4.z, aa);
                    const float b2 = fmaf(w, e4.w, bb);
                    aa = in ? a2 : aa;
                    bb = in ? b2 : bb;
                    const bool maybe = !no_crossing_at<false>(aa, bb, wv[u], sk);
                    cand |= (in && maybe) ? (1u << u) : 0u;
                }
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
                    const float t_next = m0 + u + 1 < E ? se[u + 1].t : BATS_INF;
                    done = solve_crossings_at(a, b, e.t, t_next, wv[u], sk, n, k_post, ao, xo, to, zo);
                    if (done) break;
                }
            }
        }
        stream_release(sm, kg);
    }
    if (active) n_spikes[(long long)s * n_post + i] = n;
    // +inf past each neuron's spikes. The warp's 32 neurons own contiguous rows of k_post slots, so the
    // warp fills them row by row with the lanes along the row (contiguous stores), not lane by neuron.
    const int i0 = tile0 + warp * 32;
    const int rows = pad ? max(0, min(32, n_post - i0)) : 0;
    const long long wbase = ((long long)s * n_post + i0) * k_post;
    for (int r = 0; r < rows; ++r) {
        const int nr = __shfl_sync(0xffffffffu, n, r);
        for (int q = nr + lane; q < k_post; q += 32) {
            t_out[wbase + (long long)r * k_post + q] = BATS_INF;
            z_out[wbase + (long long)r * k_post + q] = BATS_INF;
        }
    }
    return true;
}

template <int TILE, int SEV, int STAGES, bool SCREEN>
__global__ void __launch_bounds__(TILE + 32)
lif_fc_forward_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                      const float* __restrict__ wt, int ld, int n_post, int k_post, SolveConst sk,
                      int* __restrict__ n_spikes, float* __restrict__ a_out, float* __restrict__ x_out,
                      float* __restrict__ t_out, float* __restrict__ z_out, int* __restrict__ status, int pad) {
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using Smem = StreamSmem<TILE, SEV, STAGES>;
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    constexpr int CONSUMER_WARPS = TILE / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
    forward_tile_item<TILE, SEV, STAGES, SCREEN>(sm, 0, s, tile0, E, n_post, k_post, sk, n_spikes, a_out, x_out, t_out,
                                                z_out, status, pad);
}

// Persistent variant over a work queue, for batches whose samples carry very different numbers of events.
// A work item is (sample, post-neuron tile); the items are numbered in the order of `order` (samples by
// descending event count, from work_order_kernel), the tiles of a sample next to each other, and a grid of
// as many CTAs as fit on the GPU at once takes them from a global counter (`head`, zero at launch) until
// none is left: the longest samples start first and the short ones fill the end, instead of the block
// scheduler's fixed index order leaving a long sample for last. The producer warp claims the next item
// and starts streaming its stages while the consumers finish the current one (the ring's stage count runs
// on across items), so no CTA start-up or pipeline fill sits between items. Items reach the consumers
// through a two-slot mailbox with its own full/empty mbarriers. Each item computes exactly what the
// one-item-per-CTA kernel computes for it, so results are bit-identical to lif_fc_forward_kernel's.
struct WorkItem {
    int s;      // sample, < 0: no work left
    int tile0;  // first post neuron of the tile
    int E;      // events of the sample
    int unused;
};
struct ItemMailbox {
    uint64_t full[2];   // the producer has written item[q] (one arrival)
    uint64_t empty[2];  // every consumer warp has read item[q] (one arrival per warp)
    WorkItem item[2];
};

template <typename Smem>
__host__ __device__ constexpr size_t mailbox_offset() {
    return (sizeof(Smem) + 15) / 16 * 16;
}

template <int TILE, int SEV, int STAGES, bool SCREEN>
__global__ void __launch_bounds__(TILE + 32)
lif_fc_forward_queue_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                            const float* __restrict__ wt, int ld, int n_post, int k_post, SolveConst sk,
                            int* __restrict__ n_spikes, float* __restrict__ a_out, float* __restrict__ x_out,
                            float* __restrict__ t_out, float* __restrict__ z_out, int* __restrict__ status, int pad,
                            const int* __restrict__ order, int* __restrict__ head, int n_tiles, int n_items) {
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using Smem = StreamSmem<TILE, SEV, STAGES>;
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    ItemMailbox& box = *reinterpret_cast<ItemMailbox*>(smem_raw + mailbox_offset<Smem>());
    constexpr int CONSUMER_WARPS = TILE / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int q = 0; q < 2; ++q) {
            mbar_init(&box.full[q], 1);
            mbar_init(&box.empty[q], CONSUMER_WARPS);
        }
    }
    stream_init(sm, CONSUMER_WARPS);  // thread 0: the stage barriers, then the barrier-init fence
    __syncthreads();
    if (warp == CONSUMER_WARPS) {
        int issued = 0;  // stages issued by this CTA so far
        for (int it = 0;; ++it) {
            int item = 0;
            if (lane == 0) item = atomicAdd(head, 1);
            item = __shfl_sync(0xffffffffu, item, 0);
            WorkItem w = {-1, 0, 0, 0};
            if (item < n_items) {
                const int r = item / n_tiles;
                w.s = __ldg(order + r);
                w.tile0 = (item - r * n_tiles) * TILE;
                w.E = __ldg(ev_count + w.s);
            }
            const int q = it & 1;
            const bool ok = mbar_wait(&box.empty[q], ((it >> 1) & 1) ^ 1, &sm.abort, status);
            if (!__all_sync(0xffffffffu, ok)) break;
            if (lane == 0) {
                box.item[q] = w;
                mbar_arrive(&box.full[q]);  // release: the item is visible to the consumers' acquiring wait
            }
            if (w.s < 0) break;
            const int n_stages = (w.E + SEV - 1) / SEV;
            const int done = stream_produce_at(sm, ev + (long long)w.s * ev_cap, w.E, wt, ld, w.tile0, n_stages,
                                               issued, lane, status);
            issued += done;
            if (done < n_stages) break;
        }
        if (sm.abort) stream_drain(sm, issued);
        return;
    }
    int k0 = 0;  // the current item's first stage in the ring
    for (int it = 0;; ++it) {
        const int q = it & 1;
        const bool ok = mbar_wait(&box.full[q], (it >> 1) & 1, &sm.abort, status);
        if (!__all_sync(0xffffffffu, ok)) return;
        const volatile int* vi = reinterpret_cast<const volatile int*>(&box.item[q]);
        const int s = vi[0], tile0 = vi[1], E = vi[2];
        __syncwarp();
        if (lane == 0) mbar_arrive(&box.empty[q]);
        if (s < 0) return;
        if (!forward_tile_item<TILE, SEV, STAGES, SCREEN>(sm, k0, s, tile0, E, n_post, k_post, sk, n_spikes, a_out,
                                                         x_out, t_out, z_out, status, pad))
            return;
        k0 += (E + SEV - 1) / SEV;
    }
}

// Longest-first order of the samples for lif_fc_forward_queue_kernel, and the reset of its queue head. The
// samples are ranked by descending event count in 512 logarithmic classes (16 per octave: the exponent and
// top four mantissa bits of the float count + 1); the order inside a class is whatever the atomics give,
// which changes only the schedule, never a result. One CTA of 1024 threads. head may be null (bats_sample_order:
// the order alone, for the sort of the layer's output spikes).
__device__ __forceinline__ int count_class(int c) {
    const int key = (int)(__float_as_uint((float)(c + 1)) >> 19) - (127 << 4);  // increasing in c, >= 0
    return 511 - min(511, max(0, key));
}

__global__ void __launch_bounds__(1024) work_order_kernel(const int* __restrict__ ev_count, int batch,
                                                          int* __restrict__ head, int* __restrict__ order) {
    pdl_prologue();
    __shared__ int off[512];
    __shared__ int warp_sum[16];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < 512) off[tid] = 0;
    if (tid == 0 && head) *head = 0;
    __syncthreads();
    for (int s = tid; s < batch; s += blockDim.x) atomicAdd(&off[count_class(ev_count[s])], 1);
    __syncthreads();
    // Exclusive scan of the 512 class sizes: 16 warps of 32 classes, then the warp totals.
    int v = 0, incl = 0;
    if (tid < 512) {
        v = off[tid];
        incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += u;
        }
        if (lane == 31) warp_sum[warp] = incl;
    }
    __syncthreads();
    if (tid < 512) {
        int base = 0;
        for (int w = 0; w < warp; ++w) base += warp_sum[w];
        off[tid] = base + incl - v;
    }
    __syncthreads();
    for (int s = tid; s < batch; s += blockDim.x) order[atomicAdd(&off[count_class(ev_count[s])], 1)] = s;
}

// Event-parallel variant for layers with little neuron parallelism (few post neurons, or a small
// batch with long event streams): one warp per (sample, post neuron), the 32 lanes taking 32
// consecutive events. Per block of 32 events:
//   1. the states after each event are formed by the reference's sequential FMA chain
//      (a = fma(w, e^{t/tau_s}, a), b = fma(w, e^{t/tau}, b), event order), every lane running the
//      same chain over the block's (w, exponentials) in warp-private shared memory and keeping the
//      state after its own event;
//   2. every lane evaluates the provable no-crossing test on its own state at once (one ballot);
//   3. candidates are taken in event order by their lane with the exact solver; a spike's reset
//      changes b for the later events of the block, whose b chain is then re-run from the spiking
//      event (a is unaffected by resets) and whose tests are re-evaluated.
// The arithmetic per event is that of the reference's loop, so results are bit-identical to the
// tile kernel's. The warp is latency-bound rather than issue-bound: a 32-event block costs about 230
// instructions for one neuron, against the tile kernel's ~100 per 32 neurons and event, so the
// variant pays off when B * N_post is small against the GPU's ~5000 resident warps.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
lif_fc_forward_lanes_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                            const float* __restrict__ wt, int ld, int n_post, int k_post, SolveConst sk,
                            int* __restrict__ n_spikes, float* __restrict__ a_out, float* __restrict__ x_out,
                            float* __restrict__ t_out, float* __restrict__ z_out, int pad) {
    pdl_prologue();
    __shared__ float4 blk[WARPS][32];  // (w, es, e, -) of the block's events
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int s = blockIdx.y;
    const int i = blockIdx.x * WARPS + warp;
    if (i >= n_post) return;  // whole warp
    const int E = ev_count[s];
    const Event* evs = ev + (long long)s * ev_cap;
    const long long obase = ((long long)s * n_post + i) * k_post;
    float* ao = a_out + obase;
    float* xo = x_out + obase;
    float* to = t_out + obase;
    float* zo = z_out + obase;
    float4* my = blk[warp];
    float a = 0.0f, b = 0.0f;
    int n = 0;
    bool done = false;
    // The next block's event and weight are loaded one block ahead, so that the gather latency overlaps
    // the current block's chain and tests.
    float4 e4_nx = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float w_nx = 0.0f;
    if (lane < E) {
        e4_nx = __ldg(reinterpret_cast<const float4*>(evs + lane));
        w_nx = __ldg(wt + (long long)__float_as_int(e4_nx.y) * ld + i);
    }
    for (int m0 = 0; m0 < E && !done; m0 += 32) {
        const int m = m0 + lane;
        const int cnt = min(32, E - m0);
        const bool in = lane < cnt;
        const float4 e4 = e4_nx;  // (t, j, es, e); zeros past the end
        const float w = w_nx;
        e4_nx = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w_nx = 0.0f;
        if (m + 32 < E) {
            e4_nx = __ldg(reinterpret_cast<const float4*>(evs + m + 32));
            w_nx = __ldg(wt + (long long)__float_as_int(e4_nx.y) * ld + i);
        }
        // Window end: the next event's time and exponential (+inf after the last event).
        float t_nx = __shfl_down_sync(0xffffffffu, e4.x, 1);
        float e_nx = __shfl_down_sync(0xffffffffu, e4.w, 1);
        if (lane == 31 && m0 + 32 < E) {
            const float4 nx = __ldg(reinterpret_cast<const float4*>(evs + m0 + 32));
            t_nx = nx.x;
            e_nx = nx.w;
        }
        if (m + 1 >= E) {
            t_nx = BATS_INF;
            e_nx = BATS_INF;
        }
        // 1. sequential chain; lanes past the block's end carry w = 0, which leaves a and b unchanged.
        my[lane] = make_float4(w, e4.z, e4.w, 0.0f);
        __syncwarp();
        // Lane l stops after event l: its state is the chain's l-th prefix, with no select per step.
        float am = a, bm = b;
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            const float4 q = my[k];
            if (k <= lane) {
                am = fmaf(q.x, q.y, am);
                bm = fmaf(q.x, q.z, bm);
            }
        }
        // 2. provable no-crossing tests of all lanes at once.
        unsigned cand = __ballot_sync(0xffffffffu, in && !no_crossing<false>(am, bm, e4.w, e_nx, sk));
        // 3. candidates in event order.
        while (cand) {
            const int u = __ffs(cand) - 1;
            int spiked = 0;
            int full = 0;
            if (lane == u) {
                const int n0 = n;
                full = solve_crossings<false>(am, bm, e4.x, t_nx, e4.w, e_nx, sk, n, k_post, ao, xo, to, zo) ? 1 : 0;
                spiked = n - n0;
            }
            n = __shfl_sync(0xffffffffu, n, u);
            spiked = __shfl_sync(0xffffffffu, spiked, u);
            if (__shfl_sync(0xffffffffu, full, u)) {
                done = true;
                break;
            }
            if (spiked) {
                float cb2 = __shfl_sync(0xffffffffu, bm, u);
                for (int k = u + 1; k < cnt; ++k) {
                    const float4 q = my[k];
                    cb2 = fmaf(q.x, q.z, cb2);
                    bm = (lane == k) ? cb2 : bm;
                }
                cand = __ballot_sync(0xffffffffu, in && lane > u && !no_crossing<false>(am, bm, e4.w, e_nx, sk));
            } else {
                cand &= cand - 1u;
            }
        }
        a = __shfl_sync(0xffffffffu, am, cnt - 1);
        b = __shfl_sync(0xffffffffu, bm, cnt - 1);
        __syncwarp();
    }
    if (lane == 0) n_spikes[(long long)s * n_post + i] = n;
    for (int q = n + lane; pad && q < k_post; q += 32) {
        to[q] = BATS_INF;
        zo[q] = BATS_INF;
    }
}

template <int WARPS>
static int launch_forward_lanes(const void* events, const int* ev_count, long long ev_cap, const float* wt, int ld,
                                int batch, int n_post, int k_post, const SolveConst& sk, int* n_spikes, float* a,
                                float* x, float* times, float* post_exp_tau, int pad, cudaStream_t stream) {
    dim3 grid((n_post + WARPS - 1) / WARPS, batch);
    BATS_CUDA(bats::launch(lif_fc_forward_lanes_kernel<WARPS>, grid, WARPS * 32, 0, stream,
        reinterpret_cast<const Event*>(events), ev_count, ev_cap, wt, ld, n_post, k_post, sk, n_spikes, a, x, times,
        post_exp_tau, pad));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

template <int TILE, int SEV, int STAGES, bool SCREEN>
static int launch_forward(const void* events, const int* ev_count, long long ev_cap, const float* wt, int ld, int batch,
                          int n_post, int k_post, const SolveConst& sk, int* n_spikes, float* a, float* x,
                          float* times, float* post_exp_tau, int* status, int pad, cudaStream_t stream) {
    const size_t smem = sizeof(StreamSmem<TILE, SEV, STAGES>);
    BATS_CUDA((cudaError_t)max_dynamic_smem_set((const void*)lif_fc_forward_kernel<TILE, SEV, STAGES, SCREEN>,
                                                (int)smem));
    dim3 grid((n_post + TILE - 1) / TILE, batch);
    BATS_CUDA(bats::launch(lif_fc_forward_kernel<TILE, SEV, STAGES, SCREEN>, grid, TILE + 32, smem, stream,
        reinterpret_cast<const Event*>(events), ev_count, ev_cap, wt, ld, n_post, k_post, sk, n_spikes, a, x, times,
        post_exp_tau, status, pad));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// Work-queue launch: the order kernel, then a grid of as many CTAs of the persistent kernel as are resident
// at once on this GPU (at most one per work item).
template <int TILE, int SEV, int STAGES, bool SCREEN>
static int launch_forward_queue(const void* events, const int* ev_count, long long ev_cap, const float* wt, int ld,
                                int batch, int n_post, int k_post, const SolveConst& sk, int* n_spikes, float* a,
                                float* x, float* times, float* post_exp_tau, int* status, int pad, int* order,
                                int* head, cudaStream_t stream) {
    using Smem = StreamSmem<TILE, SEV, STAGES>;
    const size_t smem = mailbox_offset<Smem>() + sizeof(ItemMailbox);
    const void* kern = (const void*)lif_fc_forward_queue_kernel<TILE, SEV, STAGES, SCREEN>;
    BATS_CUDA((cudaError_t)max_dynamic_smem_set(kern, (int)smem));
    int dev = 0, n_sm = 0, per_sm = 0;
    BATS_CUDA(cudaGetDevice(&dev));
    BATS_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    BATS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, lif_fc_forward_queue_kernel<TILE, SEV, STAGES, SCREEN>, TILE + 32, smem));
    const int n_tiles = (n_post + TILE - 1) / TILE;
    BATS_REQUIRE((long long)batch * n_tiles < (1LL << 31), BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc_queue: batch * post-neuron tiles must stay below 2^31");
    const int n_items = batch * n_tiles;
    const int grid = (int)std::min<long long>(n_items, (long long)std::max(1, per_sm) * std::max(1, n_sm));
    BATS_CUDA(bats::launch(work_order_kernel, 1, 1024, 0, stream, ev_count, batch, head, order));
    BATS_CUDA(cudaGetLastError());
    BATS_CUDA(bats::launch(lif_fc_forward_queue_kernel<TILE, SEV, STAGES, SCREEN>, grid, TILE + 32, smem, stream,
        reinterpret_cast<const Event*>(events), ev_count, ev_cap, wt, ld, n_post, k_post, sk, n_spikes, a, x, times,
        post_exp_tau, status, pad, order, head, n_tiles, n_items));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// The stage-screen choice (a run-time flag) mapped onto the kernel template.
template <int TILE, int SEV, int STAGES, typename... Args>
static int launch_tile(bool screen, Args... args) {
    return screen ? launch_forward<TILE, SEV, STAGES, true>(args...)
                  : launch_forward<TILE, SEV, STAGES, false>(args...);
}
template <int TILE, int SEV, int STAGES, typename... Args>
static int launch_queue(bool screen, Args... args) {
    return screen ? launch_forward_queue<TILE, SEV, STAGES, true>(args...)
                  : launch_forward_queue<TILE, SEV, STAGES, false>(args...);
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

static int forward_fc_impl(const void* events, const int* ev_count, long long ev_cap, const float* weights_t, int ld,
                           int batch, int n_post, int k_post, float c, float delta_theta_tau, float tau,
                           float max_simulation, int* n_spikes, float* a, float* x, float* times, float* post_exp_tau,
                           int algo, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0 && ld >= n_post && ld % 4 == 0, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc: bad shape (ld must be >= n_post and a multiple of 4)");
    const int pad = (algo & BATS_FWD_NO_PAD) ? 0 : 1;
    const bool screen = (algo & BATS_FWD_STAGE_SCREEN) != 0;
    algo &= ~(BATS_FWD_NO_PAD | BATS_FWD_STAGE_SCREEN);
    BATS_REQUIRE(algo >= BATS_FWD_AUTO && algo <= BATS_FWD_TILE64, BATS_ERR_BAD_SHAPE, "lif_forward_fc: unknown algo");
    if (batch == 0 || n_post == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && weights_t && n_spikes && a && x && times && post_exp_tau, BATS_ERR_NULL,
                 "lif_forward_fc: null pointer");
    BATS_REQUIRE(((uintptr_t)weights_t & 15) == 0 && ((uintptr_t)events & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc: weights_t and events must be 16-byte aligned");
    const bats::SolveConst sk = bats::make_solve_const(c, delta_theta_tau, tau, max_simulation);
    if (algo == BATS_FWD_AUTO)
        algo = bats_lif_forward_fc_default_algo(batch, n_post, (int)(ev_cap < (1LL << 30) ? ev_cap : (1LL << 30)));
    if (algo == BATS_FWD_LANES)
        return bats::launch_forward_lanes<4>(events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                             n_spikes, a, x, times, post_exp_tau, pad, stream);
    int* status = nullptr;
    BATS_CUDA((cudaError_t)bats::device_status(&status));
    if (algo == BATS_FWD_TILE64)
        return bats::launch_tile<64, 16, 6>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                              n_spikes, a, x, times, post_exp_tau, status, pad, stream);
    if (n_post <= 32)
        return bats::launch_tile<32, 16, 8>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                               n_spikes, a, x, times, post_exp_tau, status, pad, stream);
    if (n_post <= 64)
        return bats::launch_tile<64, 16, 6>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                              n_spikes, a, x, times, post_exp_tau, status, pad, stream);
    // 8-event stages: half the shared memory of 16-event stages, so 7 CTAs (28 consumer warps) fit on an SM
    // instead of 4, and a replay after a possible crossing covers fewer events.
    return bats::launch_tile<128, 8, 6>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                          n_spikes, a, x, times, post_exp_tau, status, pad, stream);
}

extern "C" int bats_lif_forward_fc_default_algo(int batch, int n_post, int ev_cap) {
    (void)ev_cap;
    // Warp per (sample, neuron) when that gives fewer warps than about four per SM sub-partition of a
    // 152-SM GPU, or the layer has so few neurons that the tile kernel would idle most of its lanes.
    const long long warps = (long long)batch * n_post;
    return (n_post <= 16 || warps <= 152LL * 4 * 4) ? BATS_FWD_LANES : BATS_FWD_TILE;
}

extern "C" int bats_lif_forward_fc(const void* events, const int* ev_count, long long ev_cap, const float* weights_t,
                                   int ld, int batch, int n_post, int k_post, float c, float delta_theta_tau,
                                   float tau, float max_simulation, int* n_spikes, float* a, float* x, float* times,
                                   float* post_exp_tau, cudaStream_t stream) {
    return forward_fc_impl(events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, c, delta_theta_tau, tau,
                           max_simulation, n_spikes, a, x, times, post_exp_tau, BATS_FWD_AUTO, stream);
}

extern "C" int bats_lif_forward_fc_algo(const void* events, const int* ev_count, long long ev_cap,
                                        const float* weights_t, int ld, int batch, int n_post, int k_post, float c,
                                        float delta_theta_tau, float tau, float max_simulation, int* n_spikes,
                                        float* a, float* x, float* times, float* post_exp_tau, int algo,
                                        cudaStream_t stream) {
    return forward_fc_impl(events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, c, delta_theta_tau, tau,
                           max_simulation, n_spikes, a, x, times, post_exp_tau, algo, stream);
}

extern "C" int bats_sample_order(const int* ev_count, int batch, int* order, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0, BATS_ERR_BAD_SHAPE, "sample_order: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(ev_count && order, BATS_ERR_NULL, "sample_order: null pointer");
    BATS_CUDA(bats::launch(bats::work_order_kernel, 1, 1024, 0, stream, ev_count, batch, (int*)nullptr, order));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" size_t bats_lif_forward_fc_queue_workspace_bytes(int batch) {
    // The queue head (own 256-byte line), then the sample order.
    return 256 + ((size_t)(batch > 0 ? batch : 0) * sizeof(int) + 255) / 256 * 256;
}

extern "C" int bats_lif_forward_fc_queue(const void* events, const int* ev_count, long long ev_cap,
                                         const float* weights_t, int ld, int batch, int n_post, int k_post, float c,
                                         float delta_theta_tau, float tau, float max_simulation, int* n_spikes,
                                         float* a, float* x, float* times, float* post_exp_tau, int algo,
                                         void* workspace, size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0 && ld >= n_post && ld % 4 == 0, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc_queue: bad shape (ld must be >= n_post and a multiple of 4)");
    const int pad = (algo & BATS_FWD_NO_PAD) ? 0 : 1;
    const bool screen = (algo & BATS_FWD_STAGE_SCREEN) != 0;
    algo &= ~(BATS_FWD_NO_PAD | BATS_FWD_STAGE_SCREEN);
    BATS_REQUIRE(algo == BATS_FWD_AUTO || algo == BATS_FWD_TILE || algo == BATS_FWD_TILE64, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc_queue: algo must be BATS_FWD_AUTO, BATS_FWD_TILE or BATS_FWD_TILE64");
    if (batch == 0 || n_post == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && weights_t && n_spikes && a && x && times && post_exp_tau && workspace,
                 BATS_ERR_NULL, "lif_forward_fc_queue: null pointer");
    BATS_REQUIRE(((uintptr_t)weights_t & 15) == 0 && ((uintptr_t)events & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "lif_forward_fc_queue: weights_t and events must be 16-byte aligned");
    BATS_REQUIRE(((uintptr_t)workspace & 15) == 0 &&
                     workspace_bytes >= bats_lif_forward_fc_queue_workspace_bytes(batch),
                 BATS_ERR_WORKSPACE, "lif_forward_fc_queue: workspace too small or not 16-byte aligned");
    const bats::SolveConst sk = bats::make_solve_const(c, delta_theta_tau, tau, max_simulation);
    int* status = nullptr;
    BATS_CUDA((cudaError_t)bats::device_status(&status));
    int* head = reinterpret_cast<int*>(workspace);
    int* order = reinterpret_cast<int*>(reinterpret_cast<char*>(workspace) + 256);
    if (algo == BATS_FWD_TILE64 || (n_post > 32 && n_post <= 64))
        return bats::launch_queue<64, 16, 6>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post,
                                                    sk, n_spikes, a, x, times, post_exp_tau, status, pad, order, head,
                                                    stream);
    if (n_post <= 32)
        return bats::launch_queue<32, 16, 8>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post,
                                                    sk, n_spikes, a, x, times, post_exp_tau, status, pad, order, head,
                                                    stream);
    return bats::launch_queue<128, 8, 6>(screen, events, ev_count, ev_cap, weights_t, ld, batch, n_post, k_post, sk,
                                                n_spikes, a, x, times, post_exp_tau, status, pad, order, head, stream);
}
