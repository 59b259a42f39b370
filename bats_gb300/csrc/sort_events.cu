// Per-sample time sort of all pre-synaptic spikes of a layer (one CTA per sample).
// The sort runs in shared memory whenever the sample's items fit (up to 17408 items with 16-bit slot
// values for batches of at most 152 samples, 7680 for larger ones), else in a per-sample slice of the
// caller's workspace.
//
// Replaces get_sorted_spikes_indices + the three take_along_axis gathers + compute_pre_exps
// (bats/CudaKernels/Wrappers/Inference/get_sorted_spikes_indices.py:7-17,
//  bats/Layers/LIFLayer.py:66-84, bats/CudaKernels/CuFiles/Inference/compute_pre_exps.cu:2-22).
// The reference sorts every (neuron, slot) of the batch on the device with argpartition after a
// host sync on the largest spike count; here every sample's valid slots (time < +inf) are
// compacted and sorted by a stable LSD radix sort in shared memory (8-bit digits, warp ranks
// from nine ballots per digit), so the event list needs no host sync and no padding to the
// batch maximum. Ties keep slot order, which makes the order deterministic.
//
// CTA b sorts sample b, or sample sample_order[b] when an order is given (the samples longest first: on a
// batch of uneven samples wider than the resident CTAs, the long samples then start in the first wave
// instead of setting the kernel's tail). The order changes the schedule only, never a result.
//
// For the backward pass the same kernel can also emit the events grouped by pre-neuron bucket
// (neuron / bucket_width), each bucket still in time order (one more stable counting pass), with
// the per-sample bucket offsets: the weight-gradient kernel then reads only its bucket's events.
#include "common.cuh"

namespace bats {

constexpr int SORT_BINS = 256;  // digit values of a counting pass; threads tid < SORT_BINS own one bin each
constexpr int SORT_MAX_BUCKETS = 255;
// Threads per CTA: 512 for layers of more than SORT_WIDE_CAP slots (each round of a counting pass ranks 512
// items: 0.88 -> 0.71 ms on the 4096-sample uneven batch's second sort, 0.093 -> 0.081 ms on 800 x 30 slots
// at batch 256), 256 below (samples of a few hundred items, which a larger block only spreads thinner).
constexpr int SORT_WIDE_CAP = 1024;
// Items held in shared memory (two key buffers and two value buffers): slot values are 16-bit when the
// layer has at most 65536 slots (cap = n_pre * k_pre), else 32-bit. Batches of at most SORT_SMALL_BATCH
// samples (no more CTAs than a GB300 has SMs: one CTA per SM costs no parallelism) get as many items as
// 227 KB holds (SortCaps max_u16 / max_u32); larger batches keep two CTAs per SM (u16 / u32 items, at most
// 113 KB with the counters). Samples with more valid slots than that sort in global scratch. The capacities
// leave room for the counters (SortShared: 18.5 KB at 256 threads, 34.9 KB at 512).
constexpr int SORT_SMALL_BATCH = 152;
template <int T>
struct SortCaps;
template <>
struct SortCaps<256> {
    static constexpr int max_u16 = 17408, max_u32 = 13312, u16 = 7680, u32 = 4096;
};
template <>
struct SortCaps<512> {
    static constexpr int max_u16 = 16448, max_u32 = 12320, u16 = 6720, u32 = 4096;
};

template <int T>
struct SortShared {
    int hist[SORT_BINS];
    int base[SORT_BINS];
    int wcnt[T / 32][SORT_BINS];
    int wofs[T / 32][SORT_BINS];
    int warp_tot[T / 32];
};

template <int T>
__device__ __forceinline__ int block_exclusive_flag_scan(bool f, SortShared<T>& sh, int& block_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    const int in_warp = __popc(bal & lanemask_lt());
    if (lane == 0) sh.warp_tot[warp] = __popc(bal);
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < T / 32; ++w) {
        const int c = sh.warp_tot[w];
        off += (w < warp) ? c : 0;
        tot += c;
    }
    __syncthreads();
    block_total = tot;
    return off + in_warp;
}

// Block-wide exclusive scan of one int per thread (in thread order); block_total gets the sum.
template <int T>
__device__ __forceinline__ int block_exclusive_scan(int v, SortShared<T>& sh, int& block_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) sh.warp_tot[warp] = incl;
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < T / 32; ++w) {
        const int c = sh.warp_tot[w];
        off += (w < warp) ? c : 0;
        tot += c;
    }
    __syncthreads();
    block_total = tot;
    return off + incl - v;
}

// Exclusive scan of sh.hist (SORT_BINS bins, one per thread tid < SORT_BINS) into sh.base; clears sh.wcnt.
template <int T>
__device__ __forceinline__ void scan_bins(SortShared<T>& sh) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool bin = tid < SORT_BINS;
    const int v = bin ? sh.hist[tid] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31 && bin) sh.warp_tot[warp] = incl;
    __syncthreads();
    if (bin) {
        int woff = 0;
        for (int w = 0; w < warp; ++w) woff += sh.warp_tot[w];
        sh.base[tid] = woff + incl - v;
#pragma unroll
        for (int w = 0; w < T / 32; ++w) sh.wcnt[w][tid] = 0;
    }
    __syncthreads();
}

// One stable counting pass (digit < 256) of n (key, val) pairs from (ka, va) into (kb, vb), using the
// bin bases already in sh.base. Items are ranked in rounds of T in their current order; inside a warp,
// items of equal digit are ranked by their peer mask (the AND of nine ballots, one per bit of the digit or
// the out-of-range 256: faster here than __match_any_sync), across warps by a per-digit scan.
template <int T, typename V, typename DigitFn>
__device__ __forceinline__ void stable_pass(const uint32_t* ka, const V* va, uint32_t* kb, V* vb, int n,
                                            SortShared<T>& sh, DigitFn digit) {
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int r0 = 0; r0 < n; r0 += T) {
        const int i = r0 + tid;
        const bool valid = i < n;
        uint32_t key = 0;
        V val = 0;
        int d = 256;
        if (valid) {
            key = ka[i];
            val = va[i];
            d = digit(key, (uint32_t)val);
        }
        unsigned peers = 0xffffffffu;
#pragma unroll
        for (int bit = 0; bit < 9; ++bit) {
            const bool on = (d >> bit) & 1;
            const unsigned bal = __ballot_sync(0xffffffffu, on);
            peers &= on ? bal : ~bal;
        }
        const int rank = __popc(peers & lanemask_lt());
        if (valid && rank == 0) sh.wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (tid < SORT_BINS) {
            int off = sh.base[tid];
#pragma unroll
            for (int w = 0; w < T / 32; ++w) {
                sh.wofs[w][tid] = off;
                off += sh.wcnt[w][tid];
                sh.wcnt[w][tid] = 0;
            }
            sh.base[tid] = off;
        }
        __syncthreads();
        if (valid) {
            const int pos = sh.wofs[warp][d] + rank;
            kb[pos] = key;
            vb[pos] = val;
        }
    }
    __syncthreads();
}

// Valid (finite) times among the first pre_counts[j] slots of pre neuron j (loads eight at a time, so that a
// thread's scattered loads are in flight together).
__device__ __forceinline__ int leading_valid(const int* cnt_src, const float* tsrc, int j, int k_pre) {
    const int c = min(max(cnt_src[j], 0), k_pre);
    const float* tj = tsrc + (long long)j * k_pre;
    int v = 0;
    for (int q0 = 0; q0 < c; q0 += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int q = q0 + u;
            if (q < c) v += tj[q] < BATS_INF;
        }
    }
    return v;
}

__device__ __forceinline__ Event make_event(uint32_t key, uint32_t slot, int k_pre, long long sample_off,
                                            const float* exp_s_in, const float* exp_in, float tau_s, float tau) {
    Event e;
    e.t = key_to_float(key);
    e.j = (int)slot / k_pre;
    if (exp_s_in) {
        e.es = exp_s_in[sample_off + slot];
        e.e = exp_in[sample_off + slot];
    } else {
        e.es = __expf(e.t / tau_s);
        e.e = __expf(e.t / tau);
    }
    return e;
}

struct TimeDigit {
    int shift;
    __device__ int operator()(uint32_t key, uint32_t) const { return (int)((key >> shift) & 255u); }
};
struct BucketDigit {
    int div;
    __device__ int operator()(uint32_t, uint32_t slot) const { return (int)slot / div; }
};

// V: type of the slot values (uint16_t when n_slots <= 65536). smem_cap: items held in shared memory.
template <typename V, int T>
__global__ void __launch_bounds__(T)
sort_events_kernel(const float* __restrict__ times, const int* __restrict__ pre_counts, int n_slots, int k_pre,
                   float tau_s, float tau,
                   const float* __restrict__ exp_s_in, const float* __restrict__ exp_in, Event* __restrict__ ev_out,
                   int* __restrict__ slot_out, int* __restrict__ ev_count, Event* __restrict__ ev_bucketed,
                   int* __restrict__ bucket_off, int bucket_width, int n_buckets, long long cap, int smem_cap,
                   unsigned char* __restrict__ scratch, const int* __restrict__ sample_order) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int SORT_THREADS = T, SORT_WARPS = T / 32;
    SortShared<T>& sh = *reinterpret_cast<SortShared<T>*>(smem_raw);
    unsigned char* smem_items = smem_raw + sizeof(SortShared<T>);

    const int s = sample_order ? __ldg(sample_order + blockIdx.x) : (int)blockIdx.x;
    if ((unsigned)s >= gridDim.x) return;  // not a sample of the batch: the order is not a permutation
    const int tid = threadIdx.x;
    const long long sample_off = (long long)s * n_slots;
    const float* tsrc = times + sample_off;

    // Count valid slots first so that the buffers can be chosen. With the pre layer's spike counts, neuron
    // j's valid slots are its first pre_counts[j] (the forward kernels write +inf after them), so only
    // those are read. Otherwise, with 16-byte rows (n_slots % 4 == 0) each warp counts, and later
    // compacts, its own contiguous range of slots, so neither pass needs a block-wide barrier per round.
    int n = 0;
    const int n_pre = n_slots / k_pre;
    const int* cnt_src = pre_counts ? pre_counts + (long long)s * n_pre : nullptr;
    const bool vec = !cnt_src && (n_slots & 3) == 0;
    const int n4 = n_slots >> 2;
    const int per_warp4 = (n4 + SORT_WARPS - 1) / SORT_WARPS;
    const int w_lo = min(n4, (tid >> 5) * per_warp4), w_hi = min(n4, w_lo + per_warp4);
    const float4* t4 = reinterpret_cast<const float4*>(tsrc);
    if (vec) {
        int c = 0;
        for (int q = w_lo + (tid & 31); q < w_hi; q += 32) {
            const float4 v = t4[q];
            c += (v.x < BATS_INF) + (v.y < BATS_INF) + (v.z < BATS_INF) + (v.w < BATS_INF);
        }
        for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if ((tid & 31) == 0) sh.warp_tot[tid >> 5] = c;
        __syncthreads();
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) n += sh.warp_tot[w];
    } else if (cnt_src) {
        int c = 0;
        for (int j = tid; j < n_pre; j += SORT_THREADS) c += leading_valid(cnt_src, tsrc, j, k_pre);
        for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if ((tid & 31) == 0) sh.warp_tot[tid >> 5] = c;
        __syncthreads();
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) n += sh.warp_tot[w];
        __syncthreads();
    } else {
        for (int r0 = 0; r0 < n_slots; r0 += SORT_THREADS) {
            const int slot = r0 + tid;
            n += __syncthreads_count(slot < n_slots && tsrc[slot] < BATS_INF);
        }
    }
    if (n == 0) {
        // No spike in this sample: empty event list (and empty buckets).
        if (tid == 0) ev_count[s] = 0;
        if (ev_bucketed)
            for (int q = tid; q <= n_buckets; q += SORT_THREADS) bucket_off[(long long)s * (n_buckets + 1) + q] = 0;
        return;
    }

    // Two key and two value buffers: in shared memory when the sample's items fit, else in this sample's
    // part of the global scratch (cap items each).
    uint32_t *ka, *kb;
    V *va, *vb;
    {
        const long long room = n <= smem_cap ? smem_cap : cap;
        unsigned char* base = n <= smem_cap ? smem_items : scratch + (long long)s * cap * (8 + 2 * sizeof(V));
        ka = reinterpret_cast<uint32_t*>(base);
        kb = ka + room;
        va = reinterpret_cast<V*>(kb + room);
        vb = va + room;
    }

    // Compaction in slot order (stable).
    if (cnt_src) {
        // Thread per pre neuron, rounds of SORT_THREADS neurons; each copies its leading valid slots.
        int base = 0;
        for (int r0 = 0; r0 < n_pre; r0 += SORT_THREADS) {
            const int j = r0 + tid;
            const int c = j < n_pre ? leading_valid(cnt_src, tsrc, j, k_pre) : 0;
            int tot;
            int pos = base + block_exclusive_scan(c, sh, tot);
            const int slot0 = j * k_pre;
            const int lim = c > 0 ? min(max(cnt_src[j], 0), k_pre) : 0;
            for (int q0 = 0; q0 < lim; q0 += 8) {
                float tv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) tv[u] = q0 + u < lim ? tsrc[slot0 + q0 + u] : BATS_INF;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (tv[u] < BATS_INF) {
                        ka[pos] = float_to_key(tv[u]);
                        va[pos] = (V)(slot0 + q0 + u);
                        ++pos;
                    }
                }
            }
            base += tot;
        }
    } else if (vec) {
        int base = 0;
        for (int w = 0; w < (tid >> 5); ++w) base += sh.warp_tot[w];
        const int lane = tid & 31;
        for (int q0 = w_lo; q0 < w_hi; q0 += 32) {
            const int q = q0 + lane;
            float4 v = make_float4(BATS_INF, BATS_INF, BATS_INF, BATS_INF);
            if (q < w_hi) v = t4[q];
            const int c = (v.x < BATS_INF) + (v.y < BATS_INF) + (v.z < BATS_INF) + (v.w < BATS_INF);
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            int pos = base + incl - c;
            const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (vv[u] < BATS_INF) {
                    ka[pos] = float_to_key(vv[u]);
                    va[pos] = (V)(4 * q + u);
                    ++pos;
                }
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
    } else {
        int base = 0;
        for (int r0 = 0; r0 < n_slots; r0 += SORT_THREADS) {
            const int slot = r0 + tid;
            float t = BATS_INF;
            if (slot < n_slots) t = tsrc[slot];
            const bool f = t < BATS_INF;
            int tot;
            const int pos = block_exclusive_flag_scan(f, sh, tot);
            if (f) {
                ka[base + pos] = float_to_key(t);
                va[base + pos] = (V)slot;
            }
            base += tot;
        }
    }
    __syncthreads();

    if (n <= SORT_THREADS) {
        // One item per thread: its rank is the number of smaller keys plus the equal keys before it in
        // compaction order, which is the stable order of the radix passes below, with one barrier.
        const uint32_t key = tid < n ? ka[tid] : 0u;
        const V val = tid < n ? va[tid] : V(0);
        int rank = 0;
        if (tid < n)
            for (int q = 0; q < n; ++q) {
                const uint32_t kq = ka[q];
                rank += (kq < key || (kq == key && q < tid)) ? 1 : 0;
            }
        if (tid < n) {
            kb[rank] = key;
            vb[rank] = val;
        }
        __syncthreads();
        uint32_t* t0 = ka; ka = kb; kb = t0;
        V* t1 = va; va = vb; vb = t1;
    }
    // LSD radix sort on the time key, 4 passes of 8 bits; passes whose digit is uniform are skipped.
    for (int shift = 0; n > SORT_THREADS && shift < 32; shift += 8) {
        if (tid < SORT_BINS) sh.hist[tid] = 0;
        __syncthreads();
        for (int i = tid; i < n; i += SORT_THREADS) atomicAdd(&sh.hist[(ka[i] >> shift) & 255u], 1);
        __syncthreads();
        if (__syncthreads_or(tid < SORT_BINS && sh.hist[tid] == n)) continue;
        scan_bins<T>(sh);
        stable_pass<T>(ka, va, kb, vb, n, sh, TimeDigit{shift});
        uint32_t* t0 = ka; ka = kb; kb = t0;
        V* t1 = va; va = vb; vb = t1;
    }

    Event* eo = ev_out + (long long)s * cap;
    int* so = slot_out ? slot_out + (long long)s * cap : nullptr;
    for (int m = tid; m < n; m += SORT_THREADS) {
        eo[m] = make_event(ka[m], (uint32_t)va[m], k_pre, sample_off, exp_s_in, exp_in, tau_s, tau);
        if (so) so[m] = (int)va[m];
    }
    if (tid == 0) ev_count[s] = n;

    if (ev_bucketed) {
        // Stable counting pass by pre-neuron bucket over the time-sorted items.
        const int div = k_pre * bucket_width;
        if (tid < SORT_BINS) sh.hist[tid] = 0;
        __syncthreads();
        for (int i = tid; i < n; i += SORT_THREADS) atomicAdd(&sh.hist[(int)va[i] / div], 1);
        __syncthreads();
        scan_bins<T>(sh);
        int* bo = bucket_off + (long long)s * (n_buckets + 1);
        if (tid < n_buckets) bo[tid] = sh.base[tid];
        if (tid == 0) bo[n_buckets] = n;
        __syncthreads();
        stable_pass<T>(ka, va, kb, vb, n, sh, BucketDigit{div});
        Event* be = ev_bucketed + (long long)s * cap;
        for (int m = tid; m < n; m += SORT_THREADS)
            be[m] = make_event(kb[m], (uint32_t)vb[m], k_pre, sample_off, exp_s_in, exp_in, tau_s, tau);
    }
}

}  // namespace bats

// ---------------------------------------------------------------------------------------------
// C-ABI launchers (declared in include/bats_gb300.h).
#include <algorithm>
#include "abi_util.h"

// Shared-memory items and value width for a batch of samples with cap slots each (see SORT_SMALL_BATCH).
template <int T>
static int sort_room(bool small, bool u16) {
    using C = bats::SortCaps<T>;
    return u16 ? (small ? C::max_u16 : C::u16) : (small ? C::max_u32 : C::u32);
}
static void sort_plan(int batch, long long cap, int* smem_cap, bool* u16) {
    *u16 = cap <= 65536;
    const bool small = batch <= bats::SORT_SMALL_BATCH;
    const int room = cap > bats::SORT_WIDE_CAP ? sort_room<512>(small, *u16) : sort_room<256>(small, *u16);
    *smem_cap = (int)std::min<long long>(room, (cap + 31) / 32 * 32);
}

extern "C" size_t bats_sort_events_workspace_bytes(int batch, int n_pre, int k_pre) {
    const long long cap = (long long)n_pre * k_pre;
    int smem_cap;
    bool u16;
    sort_plan(batch, cap, &smem_cap, &u16);
    if (cap <= smem_cap) return 0;
    return (size_t)(batch > 0 ? batch : 0) * (size_t)cap * (u16 ? 12 : 16);
}

template <typename V, int T>
static cudaError_t launch_sort(const float* pre_times, const int* pre_counts, int batch, long long cap, int k_pre,
                               float tau_s, float tau, const float* exp_tau_s, const float* exp_tau, void* ev_out,
                               int* slot_out, int* ev_count, void* ev_bucketed, int* bucket_offsets, int bucket_width,
                               int n_buckets, int smem_cap, unsigned char* scratch, const int* sample_order,
                               cudaStream_t stream) {
    const size_t smem = sizeof(bats::SortShared<T>) + (size_t)smem_cap * (8 + 2 * sizeof(V));
    cudaError_t e = (cudaError_t)bats::max_dynamic_smem_set((const void*)bats::sort_events_kernel<V, T>, (int)smem);
    if (e != cudaSuccess) return e;
    return bats::launch(bats::sort_events_kernel<V, T>, batch, T, smem, stream, pre_times, pre_counts, (int)cap, k_pre,
                        tau_s, tau, exp_tau_s, exp_tau, reinterpret_cast<bats::Event*>(ev_out), slot_out, ev_count,
                        reinterpret_cast<bats::Event*>(ev_bucketed), bucket_offsets, bucket_width, n_buckets, cap,
                        smem_cap, scratch, sample_order);
}
#define SORT_ARGS pre_times, pre_counts, batch, cap, k_pre, tau_s, tau, exp_tau_s, exp_tau, ev_out, slot_out, \
                  ev_count, ev_bucketed, bucket_offsets, bucket_width, n_buckets, smem_cap, scratch, sample_order, \
                  stream

static int sort_events_impl(const float* pre_times, const int* pre_counts, int batch, int n_pre, int k_pre,
                            float tau_s, float tau, const float* exp_tau_s, const float* exp_tau, void* ev_out,
                            int* slot_out, int* ev_count, void* ev_bucketed, int* bucket_offsets, int bucket_width,
                            const int* sample_order, void* workspace, size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_pre >= 0 && k_pre > 0, BATS_ERR_BAD_SHAPE, "sort_events: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(pre_times && ev_out && ev_count, BATS_ERR_NULL, "sort_events: null pointer");
    BATS_REQUIRE((exp_tau_s == nullptr) == (exp_tau == nullptr), BATS_ERR_NULL, "sort_events: give both exps or none");
    const long long cap = (long long)n_pre * k_pre;
    BATS_REQUIRE(cap < (1LL << 30), BATS_ERR_CAPACITY, "sort_events: n_pre*k_pre too large");
    int n_buckets = 0;
    if (ev_bucketed) {
        BATS_REQUIRE(bucket_offsets && bucket_width > 0, BATS_ERR_NULL, "sort_events: bucket outputs");
        n_buckets = (n_pre + bucket_width - 1) / bucket_width;
        BATS_REQUIRE(n_buckets <= bats::SORT_MAX_BUCKETS, BATS_ERR_CAPACITY,
                     "sort_events: more than 255 pre-neuron buckets (n_pre > 255 * bucket_width)");
    }
    const size_t need = bats_sort_events_workspace_bytes(batch, n_pre, k_pre);
    BATS_REQUIRE(workspace_bytes >= need && (need == 0 || workspace), BATS_ERR_WORKSPACE,
                 "sort_events: workspace too small");
    int smem_cap;
    bool u16;
    sort_plan(batch, cap, &smem_cap, &u16);
    unsigned char* scratch = reinterpret_cast<unsigned char*>(workspace);
    const bool wide = cap > bats::SORT_WIDE_CAP;
    cudaError_t err;
    if (u16)
        err = wide ? launch_sort<uint16_t, 512>(SORT_ARGS) : launch_sort<uint16_t, 256>(SORT_ARGS);
    else
        err = wide ? launch_sort<uint32_t, 512>(SORT_ARGS) : launch_sort<uint32_t, 256>(SORT_ARGS);
    BATS_CUDA(err);
    return BATS_OK;
}

extern "C" int bats_sort_events(const float* pre_times, int batch, int n_pre, int k_pre, float tau_s,
                                float tau, const float* exp_tau_s, const float* exp_tau, void* ev_out, int* slot_out,
                                int* ev_count, void* ev_bucketed, int* bucket_offsets, int bucket_width,
                                void* workspace, size_t workspace_bytes, cudaStream_t stream) {
    return sort_events_impl(pre_times, nullptr, batch, n_pre, k_pre, tau_s, tau, exp_tau_s, exp_tau, ev_out, slot_out,
                            ev_count, ev_bucketed, bucket_offsets, bucket_width, nullptr, workspace, workspace_bytes,
                            stream);
}

extern "C" int bats_sort_events_counted(const float* pre_times, const int* pre_counts, int batch, int n_pre,
                                        int k_pre, float tau_s, float tau, const float* exp_tau_s,
                                        const float* exp_tau, void* ev_out, int* slot_out, int* ev_count,
                                        void* ev_bucketed, int* bucket_offsets, int bucket_width, void* workspace,
                                        size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(pre_counts || batch == 0, BATS_ERR_NULL, "sort_events_counted: null pre_counts");
    return sort_events_impl(pre_times, pre_counts, batch, n_pre, k_pre, tau_s, tau, exp_tau_s, exp_tau, ev_out,
                            slot_out, ev_count, ev_bucketed, bucket_offsets, bucket_width, nullptr, workspace,
                            workspace_bytes, stream);
}

extern "C" int bats_sort_events_counted_ordered(const float* pre_times, const int* pre_counts, int batch, int n_pre,
                                                int k_pre, float tau_s, float tau, const float* exp_tau_s,
                                                const float* exp_tau, void* ev_out, int* slot_out, int* ev_count,
                                                void* ev_bucketed, int* bucket_offsets, int bucket_width,
                                                const int* sample_order, void* workspace, size_t workspace_bytes,
                                                cudaStream_t stream) {
    BATS_REQUIRE(pre_counts || batch == 0, BATS_ERR_NULL, "sort_events_counted_ordered: null pre_counts");
    BATS_REQUIRE(sample_order || batch == 0, BATS_ERR_NULL, "sort_events_counted_ordered: null sample_order");
    return sort_events_impl(pre_times, pre_counts, batch, n_pre, k_pre, tau_s, tau, exp_tau_s, exp_tau, ev_out,
                            slot_out, ev_count, ev_bucketed, bucket_offsets, bucket_width, sample_order, workspace,
                            workspace_bytes, stream);
}
