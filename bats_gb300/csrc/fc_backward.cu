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
#include "pipeline.cuh"
#include "abi_util.h"

namespace bats {

// Asynchronous 4- and 8-byte global -> shared copies (cp.async): every copy of a staging loop is in
// flight at once, with no register round trip; cp_async_wait_all() waits for the thread's copies.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }


// One thread per (sample, post neuron): recurrent (reset) errors in place, factors, suffix tables.
//   recurrent: propagate_recurrent_errors.cu:17-22   factors: compute_factors.cu:20-30
__global__ void bwd_prep_kernel(const float* __restrict__ t, const float* __restrict__ a, const float* __restrict__ x,
                                const float* __restrict__ z, float* __restrict__ err, long long total, int K, float c,
                                float tau, float dtt, int do_recurrent, int do_factors,
                                float* __restrict__ f1, float* __restrict__ f2, float2* __restrict__ tab,
                                int* __restrict__ nvalid) {
    pdl_prologue();
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

// Layer-path variant of bwd_prep_kernel for K <= 32, for spike trains produced by the forward kernels
// (times and post_exp_tau finite exactly on a neuron's leading spikes). Each warp handles 32 neurons:
// their K-slot rows are contiguous in memory, so they are staged through shared memory with
// coalesced loads and stores; a warp whose neurons are all silent only reads the spike times. The
// arithmetic per neuron is that of bwd_prep_kernel (the reference's order). f1/f2 are written only
// when requested.
constexpr int PREP_WARPS = 2;
constexpr int PREP_KS = 33;  // padded row stride (conflict-free)

__global__ void __launch_bounds__(PREP_WARPS * 32)
bwd_prep_layer_kernel(const float* __restrict__ t, const float* __restrict__ a, const float* __restrict__ x,
                      const float* __restrict__ z, float* __restrict__ err, long long total, int K, float c, float tau,
                      float dtt, float* __restrict__ f1, float* __restrict__ f2, float2* __restrict__ tab,
                      int* __restrict__ nvalid) {
    pdl_prologue();
    extern __shared__ float prep_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* sT = prep_smem + warp * 5 * 32 * PREP_KS;
    float* sZ = sT + 32 * PREP_KS;
    float* sX = sZ + 32 * PREP_KS;
    float* sA = sX + 32 * PREP_KS;
    float* sE = sA + 32 * PREP_KS;
    const long long nb = ((long long)blockIdx.x * PREP_WARPS + warp) * 32;
    if (nb >= total) return;
    const int cnt = (int)min(32LL, total - nb);
    const long long base = nb * K;
    const int nk = cnt * K;
    for (int q = lane; q < nk; q += 32) cp_async4(sT + (q / K) * PREP_KS + q % K, t + base + q);
    cp_async_wait_all();
    __syncwarp();
    int n = 0;
    if (lane < cnt) {
        n = K;
        for (int k = 0; k < K; ++k)
            if (isinf(sT[lane * PREP_KS + k])) {
                n = k;
                break;
            }
        nvalid[nb + lane] = n;
    }
    const int K1 = K + 1;
    __shared__ int sN[PREP_WARPS][32];
    sN[warp][lane] = n;
    if (!__any_sync(0xffffffffu, n > 0)) {
        // Silent neurons: nothing to read or write but zero factors (no table entry is ever read past n).
        if (f1)
            for (int q = lane; q < nk; q += 32) {
                f1[base + q] = 0.0f;
                f2[base + q] = 0.0f;
            }
        return;
    }
    __syncwarp();
    // Only the leading valid slots of each neuron are read (and written back below).
    for (int q = lane; q < nk; q += 32) {
        const int r = q / K, k = q % K;
        if (k >= sN[warp][r]) continue;
        const int o = r * PREP_KS + k;
        cp_async4(sZ + o, z + base + q);
        cp_async4(sX + o, x + base + q);
        cp_async4(sA + o, a + base + q);
        cp_async4(sE + o, err + base + q);
    }
    cp_async_wait_all();
    __syncwarp();
    if (lane < cnt) {
        float* rt = sT + lane * PREP_KS;
        float* rz = sZ + lane * PREP_KS;
        float* rx = sX + lane * PREP_KS;
        float* ra = sA + lane * PREP_KS;
        float* re = sE + lane * PREP_KS;
        // Reset errors, last spike first (propagate_recurrent_errors.cu:17-22).
        float cum = 0.0f;
        for (int k = n - 1; k >= 0; --k) {
            const float ek = re[k] + cum * rz[k];
            re[k] = ek;
            cum += ek * dtt / rx[k];
        }
        // Factors (compute_factors.cu:27-30); f1 replaces a, f2 replaces z.
        for (int k = 0; k < K; ++k) {
            float v1 = 0.0f, v2 = 0.0f;
            if (k < n) {
                const float xk = rx[k];
                v1 = tau / ra[k] * (1 + rz[k] * c / xk);
                v2 = tau / xk;
            }
            ra[k] = v1;
            rz[k] = v2;
        }
        // Suffix tables in the reference's accumulation order (each SA_p, SB_p summed upwards from k = p);
        // four p at a time so that their eight accumulation chains overlap. (SA_p, SB_p) into (t, x) rows.
        for (int p0 = 0; p0 < n; p0 += 4) {
            float sa[4] = {0.0f, 0.0f, 0.0f, 0.0f}, sb[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (int k = p0; k < n; ++k) {
                const float ek = re[k], fa = ra[k], fb = rz[k];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (k >= p0 + u) {
                        sa[u] += ek * fa;
                        sb[u] += ek * fb;
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (p0 + u < n) {
                    rt[p0 + u] = sa[u];
                    rx[p0 + u] = sb[u];
                }
            }
        }
    }
    __syncwarp();
    for (int q = lane; q < nk; q += 32) {
        const int r = q / K, k = q % K;
        const int o = r * PREP_KS + k;
        if (k < sN[warp][r]) err[base + q] = sE[o];
        if (f1) {
            f1[base + q] = sA[o];
            f2[base + q] = sZ[o];
        }
    }
    // Table entries p < n only: the consumers never read an entry at or past a neuron's count.
    const int nt = cnt * K1;
    for (int q = lane; q < nt; q += 32) {
        const int r = q / K1, p = q % K1;
        if (p < sN[warp][r]) tab[nb * K1 + q] = make_float2(sT[r * PREP_KS + p], sX[r * PREP_KS + p]);
    }
}

// Layer-path prep given the forward's spike counts: only each neuron's leading min(n_spikes, K) slots
// are read (the forward writes +inf past them), so silent slots cost nothing. A warp handles 32 neurons
// and stages their valid slots compactly in shared memory (at most PREPC_CAP per round; a round takes
// the next lanes whose slots fit), then each lane runs bwd_prep_layer_kernel's arithmetic on its
// neuron, so errors, tables and counts are identical to it (n = the first +inf time below the count,
// or the count).
constexpr int PREPC_WARPS = 4;
constexpr int PREPC_CAP = 256;

struct PrepCompact {
    float t[PREPC_CAP], z[PREPC_CAP], x[PREPC_CAP], a[PREPC_CAP], e[PREPC_CAP];
    unsigned char owner[PREPC_CAP];
};

__global__ void __launch_bounds__(PREPC_WARPS * 32)
bwd_prep_counted_kernel(const float* __restrict__ t, const int* __restrict__ n_spikes, const float* __restrict__ a,
                        const float* __restrict__ x, const float* __restrict__ z, float* __restrict__ err,
                        long long total, int K, float c, float tau, float dtt, float2* __restrict__ tab,
                        int* __restrict__ nvalid, float2* __restrict__ head_t, float4* __restrict__ head_ab) {
    pdl_prologue();
    __shared__ PrepCompact sm_all[PREPC_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    PrepCompact& sm = sm_all[warp];
    const long long nb = ((long long)blockIdx.x * PREPC_WARPS + warp) * 32;
    if (nb >= total) return;
    const int cnt = (int)min(32LL, total - nb);
    const int K1 = K + 1;
    const int n_in = lane < cnt ? min(max(n_spikes[nb + lane], 0), K) : 0;
    // Inclusive prefix of the counts over the warp's lanes.
    int incl = n_in;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int excl = incl - n_in;
    int r0 = 0, base = 0;
    while (r0 < 32) {
        const unsigned in_round = __ballot_sync(0xffffffffu, lane >= r0 && incl - base <= PREPC_CAP);
        const int r1 = 32 - __clz(in_round);
        const int V = __shfl_sync(0xffffffffu, incl, r1 - 1) - base;
        const bool mine = lane >= r0 && lane < r1;
        const int off = excl - base;  // this lane's first compact entry (valid when mine)
        if (mine)
            for (int k = 0; k < n_in; ++k) sm.owner[off + k] = (unsigned char)lane;
        __syncwarp();
        for (int q0 = 0; q0 < V; q0 += 32) {
            const int q = q0 + lane;
            const int r = q < V ? sm.owner[q] : 0;
            const int ro = __shfl_sync(0xffffffffu, excl, r) - base;
            if (q < V) {
                const long long src = (nb + r) * K + (q - ro);
                cp_async4(sm.t + q, t + src);
                cp_async4(sm.z + q, z + src);
                cp_async4(sm.x + q, x + src);
                cp_async4(sm.a + q, a + src);
                cp_async4(sm.e + q, err + src);
            }
        }
        cp_async_wait_all();
        __syncwarp();
        int n = 0;
        float h_t0 = BATS_INF, h_t1 = BATS_INF;  // the cursor head's spike times (read before the tables overwrite them)
        if (mine) {
            float* rt = sm.t + off;
            float* rz = sm.z + off;
            float* rx = sm.x + off;
            float* ra = sm.a + off;
            float* re = sm.e + off;
            n = n_in;
            for (int k = 0; k < n_in; ++k)
                if (isinf(rt[k])) {
                    n = k;
                    break;
                }
            h_t0 = n > 0 ? rt[0] : BATS_INF;
            h_t1 = n > 1 ? rt[1] : BATS_INF;
            float cum = 0.0f;
            for (int k = n - 1; k >= 0; --k) {
                const float ek = re[k] + cum * rz[k];
                re[k] = ek;
                cum += ek * dtt / rx[k];
            }
            for (int k = 0; k < n; ++k) {
                const float xk = rx[k];
                ra[k] = tau / ra[k] * (1 + rz[k] * c / xk);
                rz[k] = tau / xk;
            }
            for (int p0 = 0; p0 < n; p0 += 4) {
                float sa[4] = {0.0f, 0.0f, 0.0f, 0.0f}, sb[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                for (int k = p0; k < n; ++k) {
                    const float ek = re[k], fa = ra[k], fb = rz[k];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (k >= p0 + u) {
                            sa[u] += ek * fa;
                            sb[u] += ek * fb;
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (p0 + u < n) {
                        rt[p0 + u] = sa[u];
                        rx[p0 + u] = sb[u];
                    }
                }
            }
        }
        if (mine && lane < cnt) {
            nvalid[nb + lane] = n;
            if (head_t) {
                // Cursor head: what PostCursor::init reads from this row, in one coalesced record per pair.
                const float* ra = sm.t + off;
                const float* rb = sm.x + off;
                head_t[nb + lane] = make_float2(h_t0, h_t1);
                head_ab[nb + lane] = make_float4(n > 0 ? ra[0] : 0.0f, n > 0 ? rb[0] : 0.0f, n > 1 ? ra[1] : 0.0f,
                                                 n > 1 ? rb[1] : 0.0f);
            }
        }
        __syncwarp();
        for (int q0 = 0; q0 < V; q0 += 32) {
            const int q = q0 + lane;
            const int r = q < V ? sm.owner[q] : 0;
            const int ro = __shfl_sync(0xffffffffu, excl, r) - base;
            const int nr = __shfl_sync(0xffffffffu, n, r);
            const int k = q - ro;
            if (q < V && k < nr) {
                err[(nb + r) * K + k] = sm.e[q];
                tab[(nb + r) * K1 + k] = make_float2(sm.t[q], sm.x[q]);
            }
        }
        __syncwarp();
        r0 = r1;
        base += V;
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
    pdl_prologue();
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
        PostCursor cur;
        cur.init(tp, tb, n);
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
                cur.advance_past(e.t);
                if (cur.valid()) G[jj][tid] += fmaf(e.es, cur.AB.x, -(e.e * cur.AB.y));
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

// Weight gradient over bucketed events: blockIdx.y is a pre-neuron bucket of JC neurons and the CTA reads only
// that bucket's events of each sample (bats_sort_events with bucket_width == JC), in time order, instead of
// filtering the whole event list; ownership as bwd_grad_kernel. The CTA's warps are independent of one another:
// a warp owns 32 post neurons (columns of the shared-memory gradient tile), zeroes them, reads the bucket's
// events of each sample of its group itself, 32 at a time into its own slice of shared memory, skips the
// samples in which none of its own neurons spiked, and writes its columns and their zero flag out itself. There
// is no barrier in the kernel, so a warp waiting on a sample's cursor loads does not hold the others back. Every
// (i, j) entry receives its terms in the order bwd_grad_kernel adds them (events in time order, samples in
// group order): the results are bit-identical to it.
template <int TILE, int JC>
__global__ void __launch_bounds__(TILE)
bwd_grad_warp_kernel(const Event* __restrict__ ev_b, const int* __restrict__ boff, int n_buckets, long long ev_cap,
                     const float* __restrict__ post_t, const float2* __restrict__ tab, const int* __restrict__ nvalid,
                     int n_post, int k_post, int n_pre, int batch, int group, float* __restrict__ out,
                     int* __restrict__ flags, const float2* __restrict__ head_t, const float4* __restrict__ head_ab) {
    pdl_prologue();
    constexpr int WARPS = TILE / 32;
    static_assert(JC == 32, "the write-out puts a bucket's pre neurons on the lanes");
    __shared__ float G[JC][TILE + 1];
    __shared__ Event sev[WARPS][32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int w0 = blockIdx.x * TILE + warp * 32;  // the warp's first post neuron
    if (w0 >= n_post) return;                      // the last tile's warps past the layer
    const int i = w0 + lane;
    const bool active = i < n_post;
    const int bucket = blockIdx.y;
    const int J0 = bucket * JC;
    const int g = blockIdx.z;
    for (int jj = 0; jj < JC; ++jj) G[jj][tid] = 0.0f;  // the warp's own columns: no other warp touches them
    Event* wev = sev[warp];
    const int s_begin = g * group;
    const int s_end = min(batch, s_begin + group);
    bool worked = false;  // warp-uniform: some sample had events in the bucket and a spike in this warp
    for (int s0 = s_begin; s0 < s_end; s0 += 32) {
        // Up to 32 samples at once: lane q reads sample s0 + q's bucket range, and bit q of spk says whether any
        // of the warp's neurons spiked in it (independent loads, issued together).
        const int ws = min(32, s_end - s0);
        int beg_l = 0, end_l = 0;
        if (lane < ws) {
            const int* bo = boff + (long long)(s0 + lane) * (n_buckets + 1);
            beg_l = bo[bucket];
            end_l = bo[bucket + 1];
        }
        unsigned spk = 0u;
        for (int q = 0; q < ws; ++q) {
            const int nq = active ? nvalid[(long long)(s0 + q) * n_post + i] : 0;
            spk |= __ballot_sync(0xffffffffu, nq > 0) ? (1u << q) : 0u;
        }
        for (int q = 0; q < ws; ++q) {
            const int beg = __shfl_sync(0xffffffffu, beg_l, q), end = __shfl_sync(0xffffffffu, end_l, q);
            if (beg >= end || !((spk >> q) & 1u)) continue;
            worked = true;
            const int s = s0 + q;
            const long long pn = (long long)s * n_post + (active ? i : 0);
            const int n = active ? nvalid[pn] : 0;
            PostCursor cur;
            if (head_t)
                cur.init_head(post_t + pn * k_post, tab + pn * (k_post + 1), n, head_t[pn], head_ab[pn]);
            else
                cur.init(post_t + pn * k_post, tab + pn * (k_post + 1), n);
            const Event* evs = ev_b + (long long)s * ev_cap;
            for (int m0 = beg; m0 < end; m0 += 32) {
                const int cnt = min(32, end - m0);
                __syncwarp();
                if (lane < cnt) wev[lane] = evs[m0 + lane];
                __syncwarp();
                {
                    // Four events at a time: terms in event order, the four shared-memory updates issued with all
                    // loads first when the four pre neurons differ. Lanes of silent neurons and lanes past their
                    // neuron's last spike add 0, which leaves every entry unchanged (an entry starts at +0 and a
                    // sum is -0 only when both addends are), so the adds need no predicate.
                    int m = 0;
                    for (; m + 4 <= cnt; m += 4) {
                        float v[4];
                        int jj[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const Event e = wev[m + u];
                            cur.advance_past(e.t);
                            jj[u] = e.j - J0;
                            v[u] = cur.valid() ? fmaf(e.es, cur.AB.x, -(e.e * cur.AB.y)) : 0.0f;
                        }
                        const bool distinct = jj[0] != jj[1] && jj[0] != jj[2] && jj[0] != jj[3] && jj[1] != jj[2] &&
                                              jj[1] != jj[3] && jj[2] != jj[3];
                        if (distinct) {
                            float gg[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u) gg[u] = G[jj[u]][tid];
#pragma unroll
                            for (int u = 0; u < 4; ++u) G[jj[u]][tid] = gg[u] + v[u];
                        } else {
#pragma unroll
                            for (int u = 0; u < 4; ++u) G[jj[u]][tid] += v[u];
                        }
                    }
                    for (; m < cnt; ++m) {
                        const Event e = wev[m];
                        cur.advance_past(e.t);
                        if (cur.valid()) G[e.j - J0][tid] += fmaf(e.es, cur.AB.x, -(e.e * cur.AB.y));
                    }
                }
            }
        }
    }
    // Flag and write-out per warp, for its own 32 columns, with no barrier among the CTA's warps: a warp that
    // finished its samples leaves without waiting for the others.
    __syncwarp();
    if (flags) {
        // One flag per (group, bucket, 32 post neurons); a partial that is all zero is not written and the
        // reduction skips it.
        if (lane == 0) flags[((long long)g * gridDim.y + blockIdx.y) * ((n_post + 31) >> 5) + (w0 >> 5)] = worked;
        if (!worked) return;
    }
    const long long obase = (long long)g * n_post * n_pre;
    const int gj = J0 + lane;  // lanes over the bucket's pre neurons: each store is one 128-byte row segment
    if (gj < n_pre) {
        const int cols = min(32, n_post - w0);
        for (int c = 0; c < cols; ++c) out[obase + (long long)(w0 + c) * n_pre + gj] = G[lane][warp * 32 + c];
    }
}

// Sum of per-group partial gradients in a fixed order, divided by `divisor` (1 or the batch).
// With `flags` (one per group, pre bucket and post tile of the gradient kernel's grid; 0 = that partial tile
// is all zero and was not written), only the written partials are added. Grid (column blocks, row blocks):
// rows are post neurons, columns pre neurons, so the tile and bucket of an element need no division.
__global__ void reduce_groups_kernel(const float* __restrict__ partial, int n_rows, int n_cols, int groups,
                                     float divisor, float* __restrict__ out, const int* __restrict__ flags,
                                     int tile_shift, int jc_shift, int tiles, int buckets) {
    pdl_prologue();
    const long long per_group = (long long)n_rows * n_cols;
    const long long fstride = (long long)tiles * buckets;
    for (int i = blockIdx.y; i < n_rows; i += gridDim.y) {
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n_cols; j += gridDim.x * blockDim.x) {
            const long long q = (long long)i * n_cols + j;
            const int* fl = flags ? flags + (j >> jc_shift) * tiles + (i >> tile_shift) : nullptr;
            // Loads four partials ahead of the (in-order) additions, so that they are in flight together.
            float acc = 0.0f;
            int g = 0;
            for (; g + 4 <= groups; g += 4) {
                const bool f0 = !fl || fl[g * fstride], f1 = !fl || fl[(g + 1) * fstride];
                const bool f2 = !fl || fl[(g + 2) * fstride], f3 = !fl || fl[(g + 3) * fstride];
                const float p0 = f0 ? partial[(long long)g * per_group + q] : 0.0f;
                const float p1 = f1 ? partial[(long long)(g + 1) * per_group + q] : 0.0f;
                const float p2 = f2 ? partial[(long long)(g + 2) * per_group + q] : 0.0f;
                const float p3 = f3 ? partial[(long long)(g + 3) * per_group + q] : 0.0f;
                if (f0) acc += p0;
                if (f1) acc += p1;
                if (f2) acc += p2;
                if (f3) acc += p3;
            }
            for (; g < groups; ++g)
                if (!fl || fl[g * fstride]) acc += partial[(long long)g * per_group + q];
            out[q] = acc / divisor;
        }
    }
}

// Batch-mean weight gradient from the group partials, fused with the Adam update of the weights: CTA per
// 32 x 32 tile of the (n_post, n_pre) matrix (block 32 x 8, four rows per thread), as the tiled Adam kernel.
// Per element, the written partials are summed in group order and divided by the batch exactly as
// reduce_groups_kernel does, and the Adam update is adam_tiled_kernel's (the bias corrections from the
// device-side powers); the new weights are also written transposed (through shared memory) into wt, and the
// gradient into grad_out when given. Results are bit-identical to bats_weights_gradient followed by
// bats_adam_step_device, without the gradient's round trip through memory and one launch fewer.
constexpr int REDUCE_SMEM_FLAGS = 2048;

__global__ void __launch_bounds__(256)
reduce_adam_tiled_kernel(const float* __restrict__ partial, const int* __restrict__ flags, int groups,
                         int tile_shift, int jc_shift, int tiles, int buckets, float divisor,
                         float* __restrict__ grad_out, float* __restrict__ m, float* __restrict__ v, float beta_1,
                         float one_minus_beta_1, float beta_2, float one_minus_beta_2,
                         const double* __restrict__ powers, float lr, float eps, float* __restrict__ w,
                         float* __restrict__ wt, int n_post, int n_pre, int ld) {
    pdl_prologue();
    __shared__ float tile[32][33];
    __shared__ unsigned char s_fl[REDUCE_SMEM_FLAGS];
    const double bias1 = 1.0 - powers[0];
    const double bias2 = 1.0 - powers[1];
    const float4 rp = *reinterpret_cast<const float4*>(powers + 2);
    const long long per_group = (long long)n_post * n_pre;
    const long long fstride = (long long)tiles * buckets;
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = j0 + tx;
    // The gradient kernel's tiles (post neurons) and buckets (pre neurons) are multiples of 32 and aligned,
    // so this 32 x 32 tile lies in one (tile, bucket) cell and its flags are the same for every element:
    // they are read once into shared memory (up to REDUCE_SMEM_FLAGS groups; beyond, per element).
    const int* fl_cta = flags ? flags + (j0 >> jc_shift) * tiles + (i0 >> tile_shift) : nullptr;
    const bool fl_shared = fl_cta && groups <= REDUCE_SMEM_FLAGS;
    if (fl_shared)
        for (int gg = ty * 32 + tx; gg < groups; gg += 256) s_fl[gg] = fl_cta[gg * fstride] != 0;
    __syncthreads();
    // The four rows' m, v and W are loaded before any arithmetic, so that their DRAM latencies overlap (the
    // whole grid is resident at once; each thread otherwise waited for one row after another).
    float m_in[4], v_in[4], w_in[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int i = i0 + ty + 8 * r;
        if (i < n_post && j < n_pre) {
            const long long q = (long long)i * n_pre + j;
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
            const int* fl = flags ? flags + (j >> jc_shift) * tiles + (i >> tile_shift) : nullptr;
            auto has = [&](int gg) -> bool { return !fl || (fl_shared ? s_fl[gg] != 0 : fl[gg * fstride] != 0); };
            float acc = 0.0f;
            int gg = 0;
            for (; gg + 4 <= groups; gg += 4) {
                const bool f0 = has(gg), f1 = has(gg + 1);
                const bool f2 = has(gg + 2), f3 = has(gg + 3);
                const float p0 = f0 ? partial[(long long)gg * per_group + q] : 0.0f;
                const float p1 = f1 ? partial[(long long)(gg + 1) * per_group + q] : 0.0f;
                const float p2 = f2 ? partial[(long long)(gg + 2) * per_group + q] : 0.0f;
                const float p3 = f3 ? partial[(long long)(gg + 3) * per_group + q] : 0.0f;
                if (f0) acc += p0;
                if (f1) acc += p1;
                if (f2) acc += p2;
                if (f3) acc += p3;
            }
            for (; gg < groups; ++gg)
                if (has(gg)) acc += partial[(long long)gg * per_group + q];
            const float g = acc / divisor;
            if (grad_out) grad_out[q] = g;
            const float nm = beta_1 * m_in[r] + one_minus_beta_1 * g;
            const float nv = beta_2 * v_in[r] + one_minus_beta_2 * g * g;
            m[q] = nm;
            v[q] = nv;
            const float m_hat = quotient_f64_to_f32(nm, rp.x, rp.y, bias1);
            const float v_hat = quotient_f64_to_f32(nv, rp.z, rp.w, bias2);
            const float d = -(lr * m_hat / (sqrtf(v_hat) + eps));
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

// Errors of the pre-synaptic spikes. Grid (post tiles, B), TILE consumer threads (one per post
// neuron) + one producer warp. As in the forward kernel, the producer streams the sample's events and
// their weight-row segments wt[j, tile] into shared-memory stages with bulk copies; a stage holds SEV
// (16) events. Each consumer forms the reference's per-(pre spike, post neuron) term
// w * (SA e_s / tau_s - SB e / tau) for its neuron (SA, SB the suffix sums of the post neuron after the event,
// the 1/tau_s and 1/tau factors applied as reciprocals), as the reference does before it sums over post
// neurons. The terms are summed over the warp by one fixed-order transpose-reduction (16 shuffles per 16
// events), then over the tile's warps, into partial[(s, m, tile)]; pre_err_scatter_kernel sums the tiles in
// order and writes the result to the event's (neuron, slot).
template <int TILE, int SEV, int STAGES>
__global__ void __launch_bounds__(TILE + 32, 4)
bwd_pre_err_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                   const float* __restrict__ wt, int ld, const float* __restrict__ post_t,
                   const float2* __restrict__ tab, const int* __restrict__ nvalid, int n_post, int k_post,
                   float inv_tau_s, float inv_tau, float* __restrict__ partial, int n_tiles,
                   int* __restrict__ status) {
    pdl_prologue();
    constexpr int WARPS = TILE / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    using Smem = StreamSmem<TILE, SEV, STAGES>;
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    __shared__ float sred[2][WARPS][SEV];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s = blockIdx.y;
    const int tile0 = blockIdx.x * TILE;
    const int E = ev_count[s];
    const int n_stages = (E + SEV - 1) / SEV;
    const Event* evs = ev + (long long)s * ev_cap;
    stream_init(sm, WARPS);
    __syncthreads();
    if (warp == WARPS) {
        stream_produce(sm, evs, E, wt, ld, tile0, n_stages, lane, status);
        return;
    }
    const int i = tile0 + tid;
    const bool active = i < n_post;
    const long long pn = (long long)s * n_post + (active ? i : 0);
    const int n = active ? nvalid[pn] : 0;
    const float* tp = post_t + pn * k_post;
    const float2* tb = tab + pn * (k_post + 1);
    PostCursor cur;
    cur.init(tp, tb, n);
    for (int k = 0; k < n_stages; ++k) {
        const int slot = k % STAGES;
        if (!stream_acquire(sm, k, status)) return;
        const int m0 = k * SEV;
        const int cnt = min(SEV, E - m0);
        // Per event: w (SA e_s / tau_s - SB e / tau) for this neuron, zero once its cursor is past its last spike
        // (and for lanes past the layer's last neuron, whose weight slots hold no data); events past the sample's
        // end only feed sums that are not written.
        float v[SEV];
#pragma unroll
        for (int q = 0; q < SEV; ++q) {
            const float4 e4 = *reinterpret_cast<const float4*>(&sm.evs[slot][q]);  // (t, j, es, e)
            if (q < cnt) cur.advance_past(e4.x);
            const float w = sm.rows[slot][q][tid];
            const float c1 = e4.z * inv_tau_s, c2 = e4.w * inv_tau;
            v[q] = cur.valid() ? w * fmaf(cur.AB.x, c1, -(cur.AB.y * c2)) : 0.0f;  // 0 for lanes past n_post
        }
        stream_release(sm, k);
        const float r = warp_transpose_reduce<SEV>(v);
        float* dst = partial + ((long long)s * ev_cap + m0) * n_tiles + blockIdx.x;
        if (WARPS == 1) {
            if (lane < cnt) dst[(long long)lane * n_tiles] = r;
        } else {
            if (lane < SEV) sred[k & 1][warp][lane] = r;
            asm volatile("bar.sync 1, %0;" ::"r"(TILE) : "memory");
            if (warp == 0 && lane < cnt) {
                float sum = 0.0f;
#pragma unroll
                for (int w = 0; w < WARPS; ++w) sum += sred[k & 1][w][lane];
                dst[(long long)lane * n_tiles] = sum;
            }
        }
    }
}

// ---- Narrow layers (N_post <= 32): event-parallel pre-spike errors ----------------------------------
// With few post neurons, one thread per post neuron leaves most lanes idle and the per-sample CTA
// serial over all events; here lanes take events instead, and every lane runs over the (few) post
// neurons. The sample's post-spike times, suffix tables and counts are staged in shared memory.
// (The weight gradient of narrow layers keeps the thread-per-neuron merge of bwd_grad_warp_kernel,
// which costs a few instructions per event for all neurons at once, with more sample groups instead.)

// Post-spike position of every post neuron for a pre spike at time t: p = number of valid post spikes
// with t_k <= t (the first k with t_k > t), by binary search over the neuron's leading valid spikes.
__device__ __forceinline__ int post_position(const float* __restrict__ tk, int n, float t) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (tk[mid] <= t) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Shared-memory copy of one sample's post-neuron data: times (N_post, K), tables (N_post, K + 1),
// counts (N_post), issued as asynchronous copies (cp.async, no register round trip, all in flight at
// once); the caller waits with cp_async_wait_all() and a barrier.
__device__ __forceinline__ void stage_post(const float* __restrict__ post_t, const float2* __restrict__ tab,
                                           const int* __restrict__ nvalid, int s, int n_post, int k_post,
                                           float* st, float2* stab, int* snv) {
    const long long pn0 = (long long)s * n_post;
    for (int q = threadIdx.x; q < n_post * k_post; q += blockDim.x) cp_async4(st + q, post_t + pn0 * k_post + q);
    for (int q = threadIdx.x; q < n_post * (k_post + 1); q += blockDim.x)
        cp_async8(stab + q, tab + pn0 * (k_post + 1) + q);
    for (int q = threadIdx.x; q < n_post; q += blockDim.x) cp_async4(snv + q, nvalid + pn0 + q);
}

// Pre-spike errors, thread per event: sum over post neurons i (in order) of w_ij * SA_i(p) and
// w_ij * SB_i(p), then * e^{t/tau_s}/tau_s and * e^{t/tau}/tau, written to the event's slot.
__global__ void __launch_bounds__(128)
bwd_pre_err_narrow_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_slot,
                          const int* __restrict__ ev_count, long long ev_cap, const float* __restrict__ wt, int ld,
                          const float* __restrict__ post_t, const float2* __restrict__ tab,
                          const int* __restrict__ nvalid, int n_post, int k_post, long long slots_per_sample,
                          float tau_s, float tau, float* __restrict__ pre_err) {
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float2* stab = reinterpret_cast<float2*>(smem_raw);
    float* st = reinterpret_cast<float*>(stab + n_post * (k_post + 1));
    int* snv = reinterpret_cast<int*>(st + n_post * k_post);
    const int s = blockIdx.y;
    const int E = ev_count[s];
    if ((long long)blockIdx.x * blockDim.x >= E) return;  // whole CTA
    stage_post(post_t, tab, nvalid, s, n_post, k_post, st, stab, snv);
    cp_async_wait_all();
    __syncthreads();
    // The sample's events, strided over the CTAs of its row of the grid.
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < E; m += gridDim.x * blockDim.x) {
        const long long em = (long long)s * ev_cap + m;
        const Event e = ev[em];
        const float* wrow = wt + (long long)e.j * ld;
        float sa = 0.0f, sb = 0.0f;
        for (int i = 0; i < n_post; ++i) {
            const int n = snv[i];
            const int p = post_position(st + i * k_post, n, e.t);
            if (p < n) {
                const float w = __ldg(wrow + i);
                const float2 AB = stab[i * (k_post + 1) + p];
                sa += w * AB.x;
                sb += w * AB.y;
            }
        }
        pre_err[(long long)s * slots_per_sample + ev_slot[em]] = sa * e.es / tau_s - sb * e.e / tau;
    }
}

// Sums the per-tile partials of each event in tile order and writes the sum to the event's slot.
__global__ void pre_err_scatter_kernel(const float* __restrict__ partial, const Event* __restrict__ ev,
                                       const int* __restrict__ ev_slot, const int* __restrict__ ev_count,
                                       long long ev_cap, int n_tiles, long long slots_per_sample, float tau_s,
                                       float tau, float* __restrict__ pre_err) {
    pdl_prologue();
    const int s = blockIdx.y;
    const int E = ev_count[s];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < E; m += gridDim.x * blockDim.x) {
        const long long em = (long long)s * ev_cap + m;
        const float* pp = partial + em * n_tiles;
        float sum = 0.0f;
        for (int q = 0; q < n_tiles; ++q) sum += pp[q];
        pre_err[(long long)s * slots_per_sample + ev_slot[em]] = sum;
    }
}

}  // namespace bats

// ---------------------------------------------------------------------------------------------
// C-ABI
constexpr int GRAD_TILE = 128;
constexpr int GRAD_JC = BATS_GRAD_BUCKET_WIDTH;  // 16.5 KB gradient tile: 11 CTAs of 128 threads per SM
constexpr int GRAD_FLAG_TILE = 32;               // post neurons per partial flag (one gradient warp's columns)

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
    BATS_CUDA(bats::launch(bats::bwd_prep_kernel, blocks, threads, 0, stream, post_times, a, x, post_exp_tau, errors,
        total, k_post, c, tau, delta_theta_tau, do_recurrent, do_factors, f1, f2, reinterpret_cast<float2*>(tables),
        nvalid));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_backward_prep_layer(const float* post_times, const float* a, const float* x,
                                        const float* post_exp_tau, float* errors, int batch, int n_post, int k_post,
                                        float c, float tau, float delta_theta_tau, float* f1, float* f2, void* tables,
                                        int* nvalid, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0, BATS_ERR_BAD_SHAPE, "backward_prep_layer: bad shape");
    const long long total = (long long)batch * n_post;
    if (total == 0) return BATS_OK;
    BATS_REQUIRE(post_times && a && x && post_exp_tau && errors && tables && nvalid &&
                     ((f1 == nullptr) == (f2 == nullptr)),
                 BATS_ERR_NULL, "backward_prep_layer: null pointer");
    if (k_post > 32) {
        BATS_REQUIRE(f1 && f2, BATS_ERR_NULL, "backward_prep_layer: f1/f2 buffers are required when k_post > 32");
        return bats_backward_prep(post_times, a, x, post_exp_tau, errors, batch, n_post, k_post, c, tau,
                                  delta_theta_tau, 1, 1, f1, f2, tables, nvalid, stream);
    }
    const long long warps = (total + 31) / 32;
    const int blocks = (int)((warps + bats::PREP_WARPS - 1) / bats::PREP_WARPS);
    const size_t smem = (size_t)bats::PREP_WARPS * 5 * 32 * bats::PREP_KS * sizeof(float);
    BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::bwd_prep_layer_kernel, (int)smem));
    BATS_CUDA(bats::launch(bats::bwd_prep_layer_kernel, blocks, bats::PREP_WARPS * 32, smem, stream, post_times, a, x,
        post_exp_tau, errors, total, k_post, c, tau, delta_theta_tau, f1, f2, reinterpret_cast<float2*>(tables),
        nvalid));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// Cursor heads of `pairs` (sample, neuron) pairs: the first two spike times (float2 per pair), then, from the
// next 16-byte boundary, the first two suffix-table entries (float4 per pair).
struct CursorHeads {
    float2* t;
    float4* ab;
};
static size_t heads_times_bytes(long long pairs) { return ((size_t)pairs * sizeof(float2) + 15) & ~(size_t)15; }
static CursorHeads cursor_heads_of(const void* base, long long pairs) {
    if (!base) return {nullptr, nullptr};
    char* b = static_cast<char*>(const_cast<void*>(base));
    return {reinterpret_cast<float2*>(b), reinterpret_cast<float4*>(b + heads_times_bytes(pairs))};
}
extern "C" size_t bats_cursor_heads_bytes(int batch, int n_post) {
    const long long pairs = (long long)std::max(batch, 0) * std::max(n_post, 0);
    return heads_times_bytes(pairs) + (size_t)pairs * sizeof(float4);
}

extern "C" int bats_backward_prep_counted(const float* post_times, const int* n_spikes, const float* a, const float* x,
                                          const float* post_exp_tau, float* errors, int batch, int n_post, int k_post,
                                          float c, float tau, float delta_theta_tau, void* tables, int* nvalid,
                                          void* cursor_heads, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && k_post > 0, BATS_ERR_BAD_SHAPE, "backward_prep_counted: bad shape");
    BATS_REQUIRE(((uintptr_t)cursor_heads & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "backward_prep_counted: cursor_heads not 16-byte aligned");
    BATS_REQUIRE(k_post <= 32, BATS_ERR_BAD_SHAPE, "backward_prep_counted: k_post > 32 (use bats_backward_prep_layer)");
    const long long total = (long long)batch * n_post;
    if (total == 0) return BATS_OK;
    BATS_REQUIRE(post_times && n_spikes && a && x && post_exp_tau && errors && tables && nvalid, BATS_ERR_NULL,
                 "backward_prep_counted: null pointer");
    const long long warps = (total + 31) / 32;
    const int blocks = (int)((warps + bats::PREPC_WARPS - 1) / bats::PREPC_WARPS);
    const CursorHeads h = cursor_heads_of(cursor_heads, total);
    BATS_CUDA(bats::launch(bats::bwd_prep_counted_kernel, blocks, bats::PREPC_WARPS * 32, 0, stream, post_times,
        n_spikes, a, x, post_exp_tau, errors, total, k_post, c, tau, delta_theta_tau, reinterpret_cast<float2*>(tables),
        nvalid, h.t, h.ab));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

// Post neurons per gradient CTA: two independent warps (the same warps per SM as four, 2.6 % faster on an
// 800 x 800 layer than 128-neuron CTAs); one warp for narrow layers.
static int grad_tile_for(int n_post) { return n_post <= 32 ? 32 : 64; }

static int log2_pow2(int v) { return 31 - __builtin_clz((unsigned)v); }

// Sum of the group partials (groups, n_post, n_pre) into out, ~8 CTAs of 256 threads per SM.
static cudaError_t launch_reduce(const float* part, int n_post, int n_pre, int groups, float divisor, float* out,
                                 const int* flags, int tile, int tiles, int buckets, cudaStream_t stream) {
    const int gx = (n_pre + 255) / 256;
    const int gy = (int)std::min<long long>(n_post, std::max<long long>(1, 152LL * 8 / gx));
    return bats::launch(bats::reduce_groups_kernel, dim3(gx, gy), 256, 0, stream, part, n_post, n_pre, groups, divisor,
                        out, flags, log2_pow2(tile), log2_pow2(GRAD_JC), tiles, buckets);
}

// Partials (groups, n_post, n_pre) floats, then (256-byte aligned) one int flag per partial tile.
static size_t grad_partials_bytes(long long groups, int n_post, int n_pre) {
    return ((size_t)groups * n_post * n_pre * sizeof(float) + 255) & ~(size_t)255;
}

extern "C" size_t bats_weights_gradient_workspace_bytes(int batch, int n_post, int n_pre, int group) {
    if (group <= 1 || group >= batch) return 0;
    const long long groups = (batch + group - 1) / group;
    const long long flag_tiles = (n_post + GRAD_FLAG_TILE - 1) / GRAD_FLAG_TILE, buckets = (n_pre + GRAD_JC - 1) / GRAD_JC;
    return grad_partials_bytes(groups, n_post, n_pre) + (size_t)groups * flag_tiles * buckets * sizeof(int);
}

template <int TILE>
static cudaError_t launch_grad(const void* events, const int* ev_count, const void* ev_b, const int* boff,
                               int n_buckets, long long ev_cap, const float* post_times, const void* tables,
                               const int* nvalid, const void* heads, int batch, int n_post, int k_post, int n_pre,
                               int group, int groups, float* out, int* flags, cudaStream_t stream) {
    dim3 grid((n_post + TILE - 1) / TILE, (n_pre + GRAD_JC - 1) / GRAD_JC, groups);
    const CursorHeads h = cursor_heads_of(heads, (long long)batch * n_post);
    if (ev_b)
        return bats::launch(bats::bwd_grad_warp_kernel<TILE, GRAD_JC>, grid, TILE, 0, stream,
                            reinterpret_cast<const bats::Event*>(ev_b), boff, n_buckets, ev_cap, post_times,
                            reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, n_pre, batch, group, out,
                            flags, (const float2*)h.t, (const float4*)h.ab);
    return bats::launch(bats::bwd_grad_kernel<TILE, GRAD_JC>, grid, TILE, 0, stream,
                        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, post_times,
                        reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, n_pre, batch, group, out);
}

extern "C" int bats_weights_gradient(const void* events, const int* ev_count, const void* events_bucketed,
                                     const int* bucket_offsets, long long ev_cap, const float* post_times,
                                     const void* tables, const int* nvalid, const void* cursor_heads, int batch,
                                     int n_post, int k_post, int n_pre, int group, int mean, float* grad, void* workspace,
                                     size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0 && k_post > 0 && group >= 1, BATS_ERR_BAD_SHAPE,
                 "weights_gradient: bad shape");
    BATS_REQUIRE(((uintptr_t)cursor_heads & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "weights_gradient: cursor_heads not 16-byte aligned");
    if (batch == 0 || n_post == 0 || n_pre == 0) return BATS_OK;
    BATS_REQUIRE(post_times && tables && nvalid && grad &&
                     ((events && ev_count) || (events_bucketed && bucket_offsets)),
                 BATS_ERR_NULL, "weights_gradient: null pointer");
    const int n_buckets = (n_pre + GRAD_JC - 1) / GRAD_JC;
    const int groups = group == 1 ? batch : (batch + group - 1) / group;
    BATS_REQUIRE(groups <= 65535, BATS_ERR_BAD_SHAPE,
                 "weights_gradient: more than 65535 sample groups (the grid's z limit); raise group");
    float* part = grad;
    int* flags = nullptr;  // all-zero partial tiles are skipped (bucketed kernel, partials in the workspace)
    if (group > 1 && groups > 1) {
        BATS_REQUIRE(workspace && workspace_bytes >= bats_weights_gradient_workspace_bytes(batch, n_post, n_pre, group),
                     BATS_ERR_WORKSPACE, "weights_gradient: workspace too small");
        part = reinterpret_cast<float*>(workspace);
        if (events_bucketed)
            flags = reinterpret_cast<int*>(static_cast<char*>(workspace) + grad_partials_bytes(groups, n_post, n_pre));
    }
    const int tile = grad_tile_for(n_post);
    if (tile == 32)
        BATS_CUDA(launch_grad<32>(events, ev_count, events_bucketed, bucket_offsets, n_buckets, ev_cap, post_times,
                                  tables, nvalid, cursor_heads, batch, n_post, k_post, n_pre, group, groups, part,
                                  flags, stream));
    else if (tile == 64)
        BATS_CUDA(launch_grad<64>(events, ev_count, events_bucketed, bucket_offsets, n_buckets, ev_cap, post_times,
                                  tables, nvalid, cursor_heads, batch, n_post, k_post, n_pre, group, groups, part,
                                  flags, stream));
    else
        BATS_CUDA(launch_grad<128>(events, ev_count, events_bucketed, bucket_offsets, n_buckets, ev_cap, post_times,
                                   tables, nvalid, cursor_heads, batch, n_post, k_post, n_pre, group, groups, part,
                                   flags, stream));
    if (group == 1) return BATS_OK;  // per-sample gradient (B, N_post, N_pre)
    BATS_CUDA(launch_reduce(part, n_post, n_pre, groups, mean ? (float)batch : 1.0f, grad, flags, GRAD_FLAG_TILE,
                            (n_post + GRAD_FLAG_TILE - 1) / GRAD_FLAG_TILE, n_buckets, stream));
    return BATS_OK;
}

extern "C" int bats_weights_gradient_adam(const void* events, const int* ev_count, const void* events_bucketed,
                                          const int* bucket_offsets, long long ev_cap, const float* post_times,
                                          const void* tables, const int* nvalid, const void* cursor_heads, int batch,
                                          int n_post, int k_post, int n_pre, int group, float* grad, float* m, float* v,
                                          float beta_1,
                                          float beta_2, float epsilon, float learning_rate, const double* powers,
                                          float* weights, float* weights_t, int ld, void* workspace,
                                          size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0 && k_post > 0 && group >= 2 && ld >= n_post,
                 BATS_ERR_BAD_SHAPE, "weights_gradient_adam: bad shape (group >= 2, ld >= n_post)");
    BATS_REQUIRE(((uintptr_t)cursor_heads & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "weights_gradient_adam: cursor_heads not 16-byte aligned");
    if (batch == 0 || n_post == 0 || n_pre == 0) return BATS_OK;
    BATS_REQUIRE(post_times && tables && nvalid && m && v && powers && weights && weights_t &&
                     ((events && ev_count) || (events_bucketed && bucket_offsets)),
                 BATS_ERR_NULL, "weights_gradient_adam: null pointer");
    const int n_buckets = (n_pre + GRAD_JC - 1) / GRAD_JC;
    const int groups = (batch + group - 1) / group;
    BATS_REQUIRE(groups <= 65535, BATS_ERR_BAD_SHAPE,
                 "weights_gradient_adam: more than 65535 sample groups (the grid's z limit); raise group");
    float* part = grad;
    int* flags = nullptr;
    if (groups > 1) {
        BATS_REQUIRE(workspace && workspace_bytes >= bats_weights_gradient_workspace_bytes(batch, n_post, n_pre, group),
                     BATS_ERR_WORKSPACE, "weights_gradient_adam: workspace too small");
        part = reinterpret_cast<float*>(workspace);
        if (events_bucketed)
            flags = reinterpret_cast<int*>(static_cast<char*>(workspace) + grad_partials_bytes(groups, n_post, n_pre));
    } else {
        BATS_REQUIRE(grad, BATS_ERR_NULL, "weights_gradient_adam: one group (group >= batch) needs grad");
    }
    const int tile = grad_tile_for(n_post);
    if (tile == 32)
        BATS_CUDA(launch_grad<32>(events, ev_count, events_bucketed, bucket_offsets, n_buckets, ev_cap, post_times,
                                  tables, nvalid, cursor_heads, batch, n_post, k_post, n_pre, group, groups, part,
                                  flags, stream));
    else if (tile == 64)
        BATS_CUDA(launch_grad<64>(events, ev_count, events_bucketed, bucket_offsets, n_buckets, ev_cap, post_times,
                                  tables, nvalid, cursor_heads, batch, n_post, k_post, n_pre, group, groups, part,
                                  flags, stream));
    else
        BATS_CUDA(launch_grad<128>(events, ev_count, events_bucketed, bucket_offsets, n_buckets, ev_cap, post_times,
                                   tables, nvalid, cursor_heads, batch, n_post, k_post, n_pre, group, groups, part,
                                   flags, stream));
    dim3 grid((n_pre + 31) / 32, (n_post + 31) / 32), block(32, 8);
    if (grad && groups > 1 && (long long)grid.x * grid.y < 2 * 152) {
        // Few weight tiles (a narrow layer) for many partials: the tile grid would leave most SMs idle while
        // each thread sums the groups; the row-parallel reduction into grad, then the tiled Adam, is faster
        // and computes the same values.
        BATS_CUDA(launch_reduce(part, n_post, n_pre, groups, (float)batch, grad, flags, GRAD_FLAG_TILE,
                                (n_post + GRAD_FLAG_TILE - 1) / GRAD_FLAG_TILE, n_buckets, stream));
        return bats_adam_step_device(grad, m, v, (long long)n_post * n_pre, beta_1, beta_2, epsilon, learning_rate,
                                     powers, weights, weights_t, n_post, n_pre, ld, stream);
    }
    BATS_CUDA(bats::launch(bats::reduce_adam_tiled_kernel, grid, block, 0, stream, part, flags, groups,
        log2_pow2(GRAD_FLAG_TILE), log2_pow2(GRAD_JC), (n_post + GRAD_FLAG_TILE - 1) / GRAD_FLAG_TILE, n_buckets,
        (float)batch, grad, m, v, beta_1,
        (float)(1.0 - (double)beta_1), beta_2, (float)(1.0 - (double)beta_2), powers, learning_rate, epsilon, weights,
        weights_t, n_post, n_pre, ld));
    return BATS_OK;
}

extern "C" size_t bats_pre_errors_workspace_bytes(int batch, long long ev_cap, int n_post) {
    if (n_post <= 32) return 0;  // narrow layers: event-parallel kernel, no partials
    const int tile = n_post <= 32 ? 32 : (n_post <= 64 ? 64 : 128);
    const long long tiles = (n_post + tile - 1) / tile;
    return (size_t)batch * ev_cap * tiles * sizeof(float);
}

template <int TILE>
static int launch_pre_err(const void* events, const int* ev_count, long long ev_cap, const float* wt, int ld,
                          const float* post_times, const void* tables, const int* nvalid, int batch, int n_post,
                          int k_post, float tau_s, float tau, float* part, int* status, cudaStream_t stream) {
    constexpr int SEV = 16, STAGES = 4;  // 33 KB of stages: six CTAs per SM (six stages measured 17 % slower)
    const int tiles = (n_post + TILE - 1) / TILE;
    const size_t smem = sizeof(bats::StreamSmem<TILE, SEV, STAGES>);
    BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::bwd_pre_err_kernel<TILE, SEV, STAGES>,
                                                      (int)smem));
    dim3 grid(tiles, batch);
    BATS_CUDA(bats::launch(bats::bwd_pre_err_kernel<TILE, SEV, STAGES>, grid, TILE + 32, smem, stream,
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, wt, ld, post_times,
        reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, 1.0f / tau_s, 1.0f / tau, part, tiles, status));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_pre_errors(const void* events, const int* ev_slot, const int* ev_count, long long ev_cap,
                               const float* weights_t, int ld, const float* post_times, const void* tables,
                               const int* nvalid, int batch, int n_post, int k_post, int n_pre, int k_pre,
                               float tau_s, float tau, float* pre_errors, void* workspace, size_t workspace_bytes,
                               cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_post >= 0 && n_pre >= 0 && k_post > 0 && k_pre > 0 && ld >= n_post && ld % 4 == 0,
                 BATS_ERR_BAD_SHAPE, "pre_errors: bad shape");
    if (batch == 0 || n_pre == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_slot && ev_count && pre_errors, BATS_ERR_NULL, "pre_errors: null pointer");
    const long long slots = (long long)n_pre * k_pre;
    BATS_CUDA(cudaMemsetAsync(pre_errors, 0, (size_t)batch * slots * sizeof(float), stream));
    if (n_post == 0) return BATS_OK;
    BATS_REQUIRE(weights_t && post_times && tables && nvalid, BATS_ERR_NULL, "pre_errors: null pointer");
    BATS_REQUIRE(((uintptr_t)weights_t & 15) == 0 && ((uintptr_t)events & 15) == 0, BATS_ERR_BAD_SHAPE,
                 "pre_errors: weights_t and events must be 16-byte aligned");
    if (n_post <= 32) {
        const size_t smem = (size_t)n_post * (k_post + 1) * sizeof(float2) + (size_t)n_post * k_post * sizeof(float) +
                            (size_t)n_post * sizeof(int);
        BATS_REQUIRE(smem <= 160 * 1024, BATS_ERR_BAD_SHAPE, "pre_errors: k_post too large for a narrow layer");
        BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::bwd_pre_err_narrow_kernel, (int)smem));
        // At most 8 CTAs per sample (each stages the sample's post data once); empty samples exit at once.
        dim3 grid((unsigned)std::min<long long>((ev_cap + 127) / 128, 8), batch);
        BATS_CUDA(bats::launch(bats::bwd_pre_err_narrow_kernel, grid, 128, smem, stream,
            reinterpret_cast<const bats::Event*>(events), ev_slot, ev_count, ev_cap, weights_t, ld, post_times,
            reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, slots, tau_s, tau, pre_errors));
        BATS_CUDA(cudaGetLastError());
        return BATS_OK;
    }
    BATS_REQUIRE(workspace && workspace_bytes >= bats_pre_errors_workspace_bytes(batch, ev_cap, n_post),
                 BATS_ERR_WORKSPACE, "pre_errors: workspace too small");
    float* part = reinterpret_cast<float*>(workspace);
    int* status = nullptr;
    BATS_CUDA((cudaError_t)bats::device_status(&status));
    int rc;
    int tiles;
    if (n_post <= 32) {
        rc = launch_pre_err<32>(events, ev_count, ev_cap, weights_t, ld, post_times, tables, nvalid, batch, n_post,
                                k_post, tau_s, tau, part, status, stream);
        tiles = (n_post + 31) / 32;
    } else if (n_post <= 64) {
        rc = launch_pre_err<64>(events, ev_count, ev_cap, weights_t, ld, post_times, tables, nvalid, batch, n_post,
                                k_post, tau_s, tau, part, status, stream);
        tiles = (n_post + 63) / 64;
    } else {
        rc = launch_pre_err<128>(events, ev_count, ev_cap, weights_t, ld, post_times, tables, nvalid, batch, n_post,
                                 k_post, tau_s, tau, part, status, stream);
        tiles = (n_post + 127) / 128;
    }
    if (rc != BATS_OK) return rc;
    // A few CTAs per sample, striding over its events (most samples have far fewer events than slots).
    dim3 g2((unsigned)std::min<long long>((ev_cap + 255) / 256, 4), batch);
    BATS_CUDA(bats::launch(bats::pre_err_scatter_kernel, g2, 256, 0, stream, part,
        reinterpret_cast<const bats::Event*>(events), ev_slot, ev_count, ev_cap, tiles, slots, tau_s, tau, pre_errors));
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
// for the symbol, so the address must come from cudaGetSymbolAddress with that device current). The
// cached address belongs to the device's current primary context: after cudaDeviceReset (or any other
// teardown of that context) the library's module is loaded again and the old address is stale, so a
// process that resets a device must not call the allocation-free entry point on it afterwards.
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
    BATS_REQUIRE(groups <= 65535, BATS_ERR_BAD_SHAPE,
                 "weights_gradient_mean_noalloc: more than 65535 sample groups (the grid's z limit); raise group");
    const long long per = (long long)n_post * n_pre;
    float* part = grad;
    if (groups > 1) {
        BATS_REQUIRE(per <= NOALLOC_GRAD_SCRATCH_FLOATS / groups, BATS_ERR_CAPACITY,
                     "weights_gradient_mean_noalloc: ceil(batch/group) * n_post * n_pre exceeds the 8 Mi-float "
                     "(32 MiB) static scratch; use a larger group or bats_weights_gradient with a workspace");
        BATS_CUDA((cudaError_t)noalloc_scratch_ptr(&part));
    }
    dim3 grid((n_post + GRAD_TILE - 1) / GRAD_TILE, (n_pre + GRAD_JC - 1) / GRAD_JC, groups);
    BATS_CUDA(bats::launch(bats::bwd_grad_kernel<GRAD_TILE, GRAD_JC>, grid, GRAD_TILE, 0, stream,
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, post_times,
        reinterpret_cast<const float2*>(tables), nvalid, n_post, k_post, n_pre, batch, group, part));
    BATS_CUDA(cudaGetLastError());
    BATS_CUDA(launch_reduce(part, n_post, n_pre, groups, (float)batch, grad, nullptr, GRAD_TILE, 1, 1, stream));
    return BATS_OK;
}
