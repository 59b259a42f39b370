// mbarrier + bulk-copy (TMA engine, non-tensor form) helpers in inline PTX for sm_90+/sm_103a.
//
// Every wait is bounded: after BATS_WAIT_NS of global time it gives up, raises the CTA abort flag and
// the global status word, and returns false, so a lost copy or a missing arrival never hangs the GPU.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bats {

constexpr unsigned long long BATS_WAIT_NS = 2000000000ull;  // give up after 2 s of waiting
constexpr uint32_t BATS_SUSPEND_NS = 2000;                   // per try_wait: sleep until the phase completes,
                                                             // at most this long
constexpr int BATS_STATUS_TIMEOUT = 1;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// One test of the phase; the thread may be suspended (not issuing) until the phase completes or the
// hint expires, so that waiting warps leave the issue slots to the working ones.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(BATS_SUSPEND_NS)
        : "memory");
    return ok != 0;
}

// Bounded wait on one phase of an mbarrier. `abort` is a CTA-shared flag raised by any thread that
// gives up; `status` (may be null) receives BATS_STATUS_TIMEOUT. Ends after BATS_WAIT_NS of global time.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort, int* status) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 15) == 0) {
            if (*abort) return false;
            if (global_ns() - t0 > BATS_WAIT_NS) break;
        }
    }
    *abort = 1;
    if (status) atomicOr(status, BATS_STATUS_TIMEOUT);
    return false;
}

// Bulk copy global -> shared, completing `bytes` transactions on `bar`. src/dst 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace bats

// ---------------------------------------------------------------------------------------------
// Event stream: a producer warp copies, stage by stage, SEV time-sorted event records (plus the next
// one, for the window end) and their weight-row segments wt[j, tile0 : tile0 + TILE] into a ring of
// STAGES shared-memory stages; consumer warps acquire a stage (full barrier), read it, and release it
// (empty barrier, one arrival per consumer warp). Used by the forward and error-propagation kernels.
#include "common.cuh"

namespace bats {

template <int TILE, int SEV, int STAGES>
struct StreamSmem {
    float rows[STAGES][SEV][TILE];
    Event evs[STAGES][SEV + 1];
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
    int abort;
};

template <int TILE, int SEV, int STAGES>
__device__ __forceinline__ void stream_init(StreamSmem<TILE, SEV, STAGES>& sm, int consumer_warps) {
    if (threadIdx.x == 0) {
        for (int q = 0; q < STAGES; ++q) {
            mbar_init(&sm.full[q], 1);
            mbar_init(&sm.empty[q], consumer_warps);
        }
        sm.abort = 0;
        fence_barrier_init();
    }
}

// After an abort: bounded waits for the copies of the last STAGES issued stages (of `issued` in all), so
// that no bulk copy into shared memory is in flight when the CTA exits.
template <int TILE, int SEV, int STAGES>
__device__ __forceinline__ void stream_drain(StreamSmem<TILE, SEV, STAGES>& sm, int issued) {
    for (int k = max(0, issued - STAGES); k < issued; ++k) {
        volatile int dummy = 0;
        mbar_wait(&sm.full[k % STAGES], (k / STAGES) & 1, &dummy, nullptr);
    }
}

// Stages of pre-neuron indices the producer loads ahead. Its loop issues a stage in far less time than a
// global load takes, so with one stage of look-ahead every stage waited for its load; eight stages cover it.
constexpr int STREAM_PREFETCH = 8;

// Producer of stages k0 .. k0 + n_stages - 1 of the ring (k0 = 0: one work item per CTA; persistent kernels
// continue the running stage count of earlier items, so slot and phase follow it). Lane u issues the row
// copy of the stage's event u (SEV <= 32); the pre-neuron indices of the next STREAM_PREFETCH stages are in
// flight in registers (a ring indexed statically by unrolling). Returns the number of stages whose copies
// were issued: n_stages, or fewer when a wait gave up (the CTA abort flag is then raised; drain with
// stream_drain).
template <int TILE, int SEV, int STAGES>
__device__ __forceinline__ int stream_produce_at(StreamSmem<TILE, SEV, STAGES>& sm, const Event* __restrict__ evs,
                                                 int E, const float* __restrict__ wt, int ld, int tile0,
                                                 int n_stages, int k0, int lane, int* status) {
    static_assert(SEV <= 32, "one event per producer lane");
    constexpr int D = STREAM_PREFETCH;
    const uint32_t row_bytes = (uint32_t)min(TILE, ld - tile0) * 4u;
    int jr[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const int m = d * SEV + lane;
        jr[d] = (lane < SEV && m < E) ? __ldg(&evs[m].j) : 0;
    }
    for (int kb = 0; kb < n_stages; kb += D) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const int k = kb + d;
            if (k >= n_stages) break;
            const int kg = k0 + k;
            const int slot = kg % STAGES;
            const int j = jr[d];
            const int m_ahead = (k + D) * SEV + lane;
            jr[d] = (lane < SEV && m_ahead < E) ? __ldg(&evs[m_ahead].j) : 0;
            const bool ok = mbar_wait(&sm.empty[slot], ((kg / STAGES) & 1) ^ 1, &sm.abort, status);
            if (!__all_sync(0xffffffffu, ok)) return k;
            const int m0 = k * SEV;
            const int cnt = min(SEV, E - m0);
            const int cnt_ev = min(SEV + 1, E - m0);
            if (lane == 0)
                mbar_arrive_expect_tx(&sm.full[slot], (uint32_t)cnt_ev * 16u + (uint32_t)cnt * row_bytes);
            __syncwarp();
            if (lane == 0) bulk_copy_g2s(&sm.evs[slot][0], evs + m0, (uint32_t)cnt_ev * 16u, &sm.full[slot]);
            if (lane < cnt)
                bulk_copy_g2s(&sm.rows[slot][lane][0], wt + (long long)j * ld + tile0, row_bytes, &sm.full[slot]);
        }
    }
    return n_stages;
}

// Producer warp body of a CTA with one work item. Never returns with copies in flight into shared memory.
template <int TILE, int SEV, int STAGES>
__device__ __forceinline__ void stream_produce(StreamSmem<TILE, SEV, STAGES>& sm, const Event* __restrict__ evs, int E,
                                               const float* __restrict__ wt, int ld, int tile0, int n_stages,
                                               int lane, int* status) {
    const int issued = stream_produce_at(sm, evs, E, wt, ld, tile0, n_stages, 0, lane, status);
    if (sm.abort) stream_drain(sm, issued);
}

// Consumer side: wait for stage k (all lanes of the warp agree on the outcome).
template <int TILE, int SEV, int STAGES>
__device__ __forceinline__ bool stream_acquire(StreamSmem<TILE, SEV, STAGES>& sm, int k, int* status) {
    const bool ok = mbar_wait(&sm.full[k % STAGES], (k / STAGES) & 1, &sm.abort, status);
    return __all_sync(0xffffffffu, ok);
}

template <int TILE, int SEV, int STAGES>
__device__ __forceinline__ void stream_release(StreamSmem<TILE, SEV, STAGES>& sm, int k) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&sm.empty[k % STAGES]);
}

}  // namespace bats
