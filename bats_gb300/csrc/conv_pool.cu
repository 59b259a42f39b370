// Convolutional LIF layer (valid convolution, stride 1) and 2x2 spike-union pooling.
//
// Neuron layouts follow the reference: a neuron (x, y, c) of a (X, Y, C) layer has index
// (x*Y + y)*C + c; filters are (C_out, fx, fy, C_in) (bats/Layers/ConvLIFLayer.py:20-37).
//
// Forward (replaces compute_spike_times_conv, bats/CudaKernels/CuFiles/Inference/compute_spike_times_conv.cu:93-174):
// the reference tests every event of the sample against every post neuron's receptive field and
// runs the crossing search after each event, relevant or not. Here a CTA owns a spatial tile of
// post positions x all output channels, keeps only the events inside the tile's receptive field,
// and each thread integrates only the events of its own receptive field, searching for crossings
// in (t_prev_relevant, t_this_relevant] before adding the next one. Because the neuron state does
// not change at an irrelevant event and the reference's windows between consecutive events tile
// that interval, this finds the same spikes with the same arithmetic. An event outside the field
// changes the reference's state only when one of its exponentials is not finite (an input later than
// about 88 tau_s overflows exp(t/tau_s)): its weight 0 times +inf is NaN, which the reference's solver
// turns into NaN spikes. Such events are therefore relevant to every neuron, with weight 0 outside the
// field, exactly as the reference adds them.
//
// Backward (replaces compute_weights_gradient_conv and propagate_errors_to_pre_spikes_conv,
// .../Backpropagation/compute_weights_gradient_conv.cu:11-61, propagate_errors_to_pre_spikes_conv.cu:11-89):
// one CTA per sample, one thread per filter tap (c_out, dx, dy); per event the thread looks up the
// post neuron (x-dx, y-dy, c_out), its first spike after the event, and adds the gradient to the
// filter entry it owns (no atomics) and the weighted error term to the event's error.
//
// Pooling (replaces aggregate_spikes_conv + argsort, .../Inference/aggregate_spikes_conv.cu:6-43,
// Wrappers/Inference/aggregate_spikes_conv.py:10-28; backward bats/Layers/PoolingLayer.py:55-66):
// a stable 4-way merge of the children's sorted spike lists, inf slots last in concatenation order.
#include <cooperative_groups.h>
#include "common.cuh"
#include "abi_util.h"

namespace bats {

struct ConvEvent {
    float t, es, e;
    int xyc;  // x | y << 10 | c << 20
};

constexpr int CONV_CHUNK = 256;

__global__ void conv_forward_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_count, long long ev_cap,
                                    const float* __restrict__ W, int X, int Y, int C, int fx, int fy, int C_out,
                                    int Xo, int Yo, int TX, int TY, int tiles_y, int k_post, SolveConst sk,
                                    int w_in_smem, int* __restrict__ n_spikes,
                                    float* __restrict__ a_out, float* __restrict__ x_out, float* __restrict__ t_out,
                                    float* __restrict__ z_out) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ConvEvent* sev = reinterpret_cast<ConvEvent*>(smem_raw);
    float2* szw = reinterpret_cast<float2*>(sev + CONV_CHUNK);  // each kept event's window constants
    int* swarp = reinterpret_cast<int*>(szw + CONV_CHUNK);
    float* sW = reinterpret_cast<float*>(swarp + 32);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    const int s = blockIdx.y;
    const int tx0 = (blockIdx.x / tiles_y) * TX, ty0 = (blockIdx.x % tiles_y) * TY;
    const int nw = C_out * fx * fy * C;
    const float* Wsrc = W;
    if (w_in_smem) {
        for (int q = tid; q < nw; q += blockDim.x) sW[q] = W[q];
        Wsrc = sW;
    }
    const int co = tid % C_out, pl = tid / C_out;
    const int xo = tx0 + pl / TY, yo = ty0 + pl % TY;
    const bool active = pl < TX * TY && xo < Xo && yo < Yo;
    const int n_post = Xo * Yo * C_out;
    const int post = (xo * Yo + yo) * C_out + co;
    const long long obase = ((long long)s * n_post + (active ? post : 0)) * k_post;
    float* ao = a_out + obase;
    float* xo_ = x_out + obase;
    float* to = t_out + obase;
    float* zo = z_out + obase;
    // Receptive field of the whole tile.
    const int rx0 = tx0, rx1 = min(X, tx0 + TX + fx - 1), ry0 = ty0, ry1 = min(Y, ty0 + TY + fy - 1);

    float a = 0.0f, b = 0.0f, last_t = 0.0f;
    bool has_prev = false;
    int n = 0;
    bool done = !active;
    const int E = ev_count[s];
    const Event* evs = ev + (long long)s * ev_cap;
    for (int m0 = 0; m0 < E; m0 += CONV_CHUNK) {
        // Stage the chunk's events that fall in the tile's receptive field, in time order.
        __syncthreads();
        int kept = 0;
        for (int r0 = 0; r0 < CONV_CHUNK && m0 + r0 < E; r0 += blockDim.x) {
            const int q = r0 + tid;
            bool keep = false;
            ConvEvent ce;
            if (q < CONV_CHUNK && m0 + q < E) {
                const Event e = evs[m0 + q];
                const int j = e.j;
                const int cc = j % C, xy = j / C, yy = xy % Y, xx = xy / Y;
                // In the tile's receptive field, or relevant to every neuron (a non-finite exponential).
                keep = (xx >= rx0 && xx < rx1 && yy >= ry0 && yy < ry1) || !(isfinite(e.es) && isfinite(e.e));
                ce.t = e.t;
                ce.es = e.es;
                ce.e = e.e;
                // bit 31: an exponential is not finite (the event is relevant to every neuron)
                ce.xyc = xx | (yy << 10) | (cc << 20) | ((isfinite(e.es) && isfinite(e.e)) ? 0 : (int)0x80000000u);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (lane == 0) swarp[warp] = __popc(bal);
            __syncthreads();
            int off = kept;
            int tot = 0;
            for (int w = 0; w < nwarps; ++w) {
                if (w < warp) off += swarp[w];
                tot += swarp[w];
            }
            if (keep) {
                const int pos = off + __popc(bal & lanemask_lt());
                sev[pos] = ce;
                szw[pos] = conv_window(ce.e, sk);  // the window that ends at this event, once per CTA
            }
            __syncthreads();
            kept += tot;
        }
        __syncthreads();
        if (done) continue;
        for (int m = 0; m < kept && !done; ++m) {
            const ConvEvent e = sev[m];
            const int dx = (e.xyc & 1023) - xo, dy = ((e.xyc >> 10) & 1023) - yo;
            const bool in_field = dx >= 0 && dx < fx && dy >= 0 && dy < fy;
            if (!in_field && e.xyc >= 0) continue;  // weight 0 times a finite value
            if (has_prev) {
                done = solve_crossings_conv_at(a, b, last_t, e.t, szw[m], sk, n, k_post, ao, xo_, to, zo);
                if (done) break;
            }
            const float w = in_field ? Wsrc[((co * fx + dx) * fy + dy) * C + ((e.xyc >> 20) & 2047)] : 0.0f;
            a += w * e.es;
            b += w * e.e;
            last_t = e.t;
            has_prev = true;
        }
    }
    if (active) {
        if (has_prev && !done)
            solve_crossings<true>(a, b, last_t, BATS_INF, 0.0f, BATS_INF, sk, n, k_post, ao, xo_, to, zo);
        n_spikes[(long long)s * n_post + post] = n;
        for (int k = n; k < k_post; ++k) {
            to[k] = BATS_INF;
            zo[k] = BATS_INF;
        }
    }
}

// One CTA per sample; thread q handles filter taps q, q + blockDim, ... of (C_out, fx, fy).
__global__ void conv_backward_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_slot,
                                     const int* __restrict__ ev_count, long long ev_cap, const float* __restrict__ W,
                                     int Y, int C, int fx, int fy, int C_out, int Xo, int Yo,
                                     const float* __restrict__ post_t, const float2* __restrict__ tab,
                                     const int* __restrict__ nvalid, int k_post, float tau_s, float tau,
                                     long long pre_slots, float* __restrict__ grad, float* __restrict__ pre_err) {
    pdl_prologue();
    __shared__ float sred[32][33];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int s = blockIdx.x;
    const int taps = C_out * fx * fy;
    const int n_post = Xo * Yo * C_out;
    const int E = ev_count[s];
    const Event* evs = ev + (long long)s * ev_cap;
    float* gs = grad + (long long)s * taps * C;
    for (int m0 = 0; m0 < E; m0 += 32) {
        const int cnt = min(32, E - m0);
        for (int q = 0; q < cnt; ++q) {
            const Event e = evs[m0 + q];
            const int cc = e.j % C, xy = e.j / C, yy = xy % Y, xx = xy / Y;
            float term = 0.0f;
            for (int tp = tid; tp < taps; tp += blockDim.x) {
                const int co = tp / (fx * fy), dx = (tp / fy) % fx, dy = tp % fy;
                const int xo = xx - dx, yo = yy - dy;
                if (xo < 0 || yo < 0 || xo >= Xo || yo >= Yo) continue;
                const long long pn = (long long)s * n_post + (xo * Yo + yo) * C_out + co;
                const int n = nvalid[pn];
                const float* tp_ = post_t + pn * k_post;
                int p = 0;
                while (p < n && tp_[p] <= e.t) ++p;
                if (p >= n) continue;
                const float2 AB = tab[pn * (k_post + 1) + p];
                gs[(long long)tp * C + cc] += fmaf(e.es, AB.x, -(e.e * AB.y));
                if (pre_err) term += W[(long long)tp * C + cc] * (AB.x * e.es / tau_s - AB.y * e.e / tau);
            }
            if (pre_err) {
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
                if (lane == 0) sred[q][warp] = term;
            }
        }
        if (pre_err) {
            __syncthreads();
            if (tid < cnt) {
                float acc = 0.0f;
                for (int w = 0; w < nwarps; ++w) acc += sred[tid][w];
                pre_err[(long long)s * pre_slots + ev_slot[(long long)s * ev_cap + m0 + tid]] = acc;
            }
            __syncthreads();
        }
    }
}

// Conv backward on a cluster of CONV_BWD_CLUSTER CTAs per sample (thread-block cluster, distributed
// shared memory). Thread = filter tap (co, dx, dy); the sample's events are dealt to the cluster's CTAs in
// groups of 32 (group g to CTA rank g % CONV_BWD_CLUSTER), so that eight times as many CTAs hide the
// latency of the post-spike lookups. Every CTA accumulates its events' gradient terms in a shared-memory
// copy of the per-sample filter gradient (taps x C), in event order; at the end each CTA sums one slice of
// the gradient over the cluster's copies in rank order (deterministic) and writes it. The pre-spike errors
// of a group of events are reduced over the taps inside the CTA that owns the group. Four events are
// processed at a time so that their lookups (binary searches over the post neuron's spike times, table
// entries) are in flight together.
constexpr int CONV_BWD_CLUSTER = 8;
constexpr int CONV_BWD_ILP = 4;

__global__ void __launch_bounds__(1024)
conv_backward_cluster_kernel(const Event* __restrict__ ev, const int* __restrict__ ev_slot,
                             const int* __restrict__ ev_count, long long ev_cap, const float* __restrict__ W, int Y,
                             int C, int fx, int fy, int C_out, int Xo, int Yo, const float* __restrict__ post_t,
                             const float2* __restrict__ tab, const int* __restrict__ nvalid, int k_post,
                             int search_top, float tau_s, float tau, long long pre_slots, float* __restrict__ grad,
                             float* __restrict__ pre_err, int batch, int group) {
    pdl_prologue();
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) float Gs[];  // taps * C
    __shared__ Event sev[32];
    __shared__ float sred[32][33];
    const unsigned rank = cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int taps = C_out * fx * fy;
    const int total = taps * C;
    const int n_post = Xo * Yo * C_out;
    for (int q = tid; q < total; q += blockDim.x) Gs[q] = 0.0f;
    __syncthreads();
    // The cluster's samples (one with group == 1: the per-sample gradient), accumulated in order.
    const int s_end = min(batch, ((int)blockIdx.y + 1) * group);
    for (int s = (int)blockIdx.y * group; s < s_end; ++s) {
    const int E = ev_count[s];
    const Event* evs = ev + (long long)s * ev_cap;
    for (int g = (int)rank; g * 32 < E; g += CONV_BWD_CLUSTER) {
        const int m0 = g * 32;
        const int cnt = min(32, E - m0);
        if (tid < cnt) sev[tid] = evs[m0 + tid];
        __syncthreads();
        for (int q0 = 0; q0 < cnt; q0 += CONV_BWD_ILP) {
            float term[CONV_BWD_ILP];
#pragma unroll
            for (int u = 0; u < CONV_BWD_ILP; ++u) term[u] = 0.0f;
            for (int tp = tid; tp < taps; tp += blockDim.x) {
                const int co = tp / (fx * fy), dx = (tp / fy) % fx, dy = tp % fy;
                long long pn[CONV_BWD_ILP];
                int nv[CONV_BWD_ILP], pos[CONV_BWD_ILP], cc[CONV_BWD_ILP];
                float et[CONV_BWD_ILP];
#pragma unroll
                for (int u = 0; u < CONV_BWD_ILP; ++u) {
                    nv[u] = 0;
                    pos[u] = 0;
                    pn[u] = 0;
                    cc[u] = 0;
                    et[u] = 0.0f;
                    if (q0 + u < cnt) {
                        const Event e = sev[q0 + u];
                        cc[u] = e.j % C;
                        const int xy = e.j / C, yy = xy % Y, xx = xy / Y;
                        const int xo = xx - dx, yo = yy - dy;
                        et[u] = e.t;
                        if (xo >= 0 && yo >= 0 && xo < Xo && yo < Yo) {
                            pn[u] = (long long)s * n_post + (xo * Yo + yo) * C_out + co;
                            nv[u] = nvalid[pn[u]];
                        }
                    }
                }
                // Fixed-depth binary searches, the ILP searches interleaved: pos = #{k < n : t_k <= t}.
                for (int step = search_top; step > 0; step >>= 1) {
#pragma unroll
                    for (int u = 0; u < CONV_BWD_ILP; ++u) {
                        const int cand = pos[u] + step;
                        if (cand <= nv[u] && post_t[pn[u] * k_post + cand - 1] <= et[u]) pos[u] = cand;
                    }
                }
#pragma unroll
                for (int u = 0; u < CONV_BWD_ILP; ++u) {
                    if (pos[u] < nv[u]) {
                        const Event e = sev[q0 + u];
                        const float2 AB = tab[pn[u] * (k_post + 1) + pos[u]];
                        Gs[tp * C + cc[u]] += fmaf(e.es, AB.x, -(e.e * AB.y));
                        if (pre_err) term[u] += W[(long long)tp * C + cc[u]] * (AB.x * e.es / tau_s - AB.y * e.e / tau);
                    }
                }
            }
            if (pre_err) {
#pragma unroll
                for (int u = 0; u < CONV_BWD_ILP; ++u) {
                    float v = term[u];
#pragma unroll
                    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0 && q0 + u < cnt) sred[q0 + u][warp] = v;
                }
            }
        }
        __syncthreads();
        if (pre_err && tid < cnt) {
            float acc = 0.0f;
            for (int w = 0; w < nwarps; ++w) acc += sred[tid][w];
            pre_err[(long long)s * pre_slots + ev_slot[(long long)s * ev_cap + m0 + tid]] = acc;
        }
        __syncthreads();
    }
    }
    cluster.sync();
    const int per = (total + CONV_BWD_CLUSTER - 1) / CONV_BWD_CLUSTER;
    const int q_end = min(total, ((int)rank + 1) * per);
    for (int q = (int)rank * per + tid; q < q_end; q += blockDim.x) {
        float acc = 0.0f;
        for (int r = 0; r < CONV_BWD_CLUSTER; ++r) acc += cluster.map_shared_rank(Gs, r)[q];
        grad[(long long)blockIdx.y * total + q] = acc;
    }
    cluster.sync();  // no CTA leaves while another still reads its shared memory
}

// Conv backward over events grouped by input position (the bucketed copy of the sort with
// bucket_width = C: one bucket per (x, y), time order inside), on a cluster of CONV_BWD_CLUSTER CTAs per
// sample (position groups dealt to the ranks). Thread = filter tap (co, dx, dy). Within a position group
// every tap sees one and the same post neuron (x - dx, y - dy, co), so its spike data is set up once per
// group and followed by a forward-only cursor over the group's time-ordered events, instead of a search
// per (event, tap). A spike's slot (neuron j, k-th spike of j) follows from the order of appearance of j
// in the group. The per-sample gradient copies are combined over the cluster as in
// conv_backward_cluster_kernel; pre errors are reduced over the taps in the CTA that owns the group.
__global__ void __launch_bounds__(1024)
conv_backward_grouped_kernel(const Event* __restrict__ ev_b, const int* __restrict__ boff, int n_pos,
                             long long ev_cap, const float* __restrict__ W, int Y, int C, int fx, int fy, int C_out,
                             int Xo, int Yo, int k_pre, const float* __restrict__ post_t,
                             const float2* __restrict__ tab, const int* __restrict__ nvalid, int k_post,
                             float tau_s, float tau, long long pre_slots, float* __restrict__ grad,
                             float* __restrict__ pre_err, int batch, int group, int w_in_smem) {
    pdl_prologue();
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) float Gs[];  // taps * C, then C spike counters
    __shared__ Event sev[32];
    __shared__ float sred[32][33];
    __shared__ int sslot[32];
    __shared__ int scc[32];
    const float inv_tau_s = 1.0f / tau_s, inv_tau = 1.0f / tau;  // the error terms' factors, as reciprocals
    const unsigned rank = cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int taps = C_out * fx * fy;
    const int total = taps * C;
    int* kcount = reinterpret_cast<int*>(Gs + total);
    const int n_post = Xo * Yo * C_out;
    for (int q = tid; q < total; q += blockDim.x) Gs[q] = 0.0f;
    // The filters, for the pre-spike error terms: in shared memory after the counters when they fit (a
    // thread's weight reads are C floats apart, one cache sector per lane from global memory).
    const float* Wk = W;
    if (w_in_smem) {
        float* sWf = reinterpret_cast<float*>(kcount + C);
        for (int q = tid; q < total; q += blockDim.x) sWf[q] = W[q];
        Wk = sWf;
    }
    // At most one tap per thread here (taps <= blockDim checked by the launcher).
    const int tp = tid;
    const bool has_tap = tp < taps;
    const int co = has_tap ? tp / (fx * fy) : 0, dx = has_tap ? (tp / fy) % fx : 0, dy = has_tap ? tp % fy : 0;
    __syncthreads();
    // The cluster's samples (one with group == 1: the per-sample gradient), accumulated in order.
    const int s_end = min(batch, ((int)blockIdx.y + 1) * group);
    for (int s = (int)blockIdx.y * group; s < s_end; ++s) {
    const int* bo = boff + (long long)s * (n_pos + 1);
    const Event* evs = ev_b + (long long)s * ev_cap;
    for (int g = (int)rank; g < n_pos; g += CONV_BWD_CLUSTER) {
        const int beg = bo[g], end = bo[g + 1];
        if (beg >= end) continue;  // uniform over the CTA
        const int xx = g / Y, yy = g % Y;
        const int xo = xx - dx, yo = yy - dy;
        const bool in = has_tap && xo >= 0 && yo >= 0 && xo < Xo && yo < Yo;
        PostCursor cur;
        const long long pn = in ? (long long)s * n_post + (xo * Yo + yo) * C_out + co : 0;
        cur.init(post_t + pn * k_post, tab + pn * (k_post + 1), in ? nvalid[pn] : 0);
        // Two barriers per chunk: after warp 0 stages it (every thread reads it), and after the error terms are in
        // sred (every thread is done with the chunk's records; the chunk's events then sum the terms). The next
        // chunk's first barrier orders those sums' reads of sred and sslot before anything overwrites them (warp 0
        // sums, then stages; the other warps write sred only after that barrier).
        for (int m0 = beg; m0 < end; m0 += 32) {
            const int cnt = min(32, end - m0);
            if (warp == 0) {
                if (m0 == beg) {  // the position's spike counters per channel: warp 0's alone
                    for (int q = lane; q < C; q += 32) kcount[q] = 0;
                    __syncwarp();
                }
                // Stage the chunk; the spikes' slots: j * k_pre + the order of appearance of j in the group (all
                // events of a position share x and y, so j is fixed by the channel: earlier chunks' counts plus
                // the rank among this chunk's events of the same channel).
                Event e;
                int c = -1;
                if (lane < cnt) {
                    e = evs[m0 + lane];
                    c = e.j % C;
                    sev[lane] = e;
                    scc[lane] = c;
                }
                const unsigned peers = __match_any_sync(0xffffffffu, c);
                const int rank = __popc(peers & lanemask_lt());
                int base = 0;
                if (lane < cnt) base = kcount[c];
                __syncwarp();
                if (lane < cnt) {
                    sslot[lane] = e.j * k_pre + base + rank;
                    if (rank == __popc(peers) - 1) kcount[c] = base + __popc(peers);
                }
            }
            __syncthreads();
            float term[32];
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                term[q] = 0.0f;
                if (q < cnt && in) {
                    const Event e = sev[q];
                    cur.advance_past(e.t);
                    if (cur.valid()) {
                        const int cc = scc[q];
                        Gs[tp * C + cc] += fmaf(e.es, cur.AB.x, -(e.e * cur.AB.y));
                        if (pre_err)
                            term[q] = Wk[tp * C + cc] * (cur.AB.x * e.es * inv_tau_s - cur.AB.y * e.e * inv_tau);
                    }
                }
            }
            if (pre_err) {
                // The chunk's 32 error terms summed over the warp at once (lane q: event q), then over the warps.
                const float v = warp_transpose_reduce<32>(term);
                sred[lane][warp] = v;
            }
            __syncthreads();  // every thread is done with the chunk's records (warp 0 may restage them next)
            if (pre_err && tid < cnt) {
                float acc = 0.0f;
                for (int w = 0; w < nwarps; ++w) acc += sred[tid][w];
                pre_err[(long long)s * pre_slots + sslot[tid]] = acc;
            }
        }
    }
    }
    cluster.sync();
    const int per = (total + CONV_BWD_CLUSTER - 1) / CONV_BWD_CLUSTER;
    const int q_end = min(total, ((int)rank + 1) * per);
    for (int q = (int)rank * per + tid; q < q_end; q += blockDim.x) {
        float acc = 0.0f;
        for (int r = 0; r < CONV_BWD_CLUSTER; ++r) acc += cluster.map_shared_rank(Gs, r)[q];
        grad[(long long)blockIdx.y * total + q] = acc;
    }
    cluster.sync();
}

// Pool forward: one thread per (sample, pooled neuron).
__global__ void pool_forward_kernel(const int* __restrict__ n_spikes, const float* __restrict__ times, int batch, int X,
                                    int Y, int C, int K, int* __restrict__ out_n, float* __restrict__ out_t,
                                    int* __restrict__ out_idx) {
    pdl_prologue();
    const int Xo = X / 2, Yo = Y / 2;
    const long long n_out = (long long)Xo * Yo * C;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)batch * n_out) return;
    const int s = (int)(q / n_out);
    const int o = (int)(q % n_out);
    const int c = o % C, xy = o / C, yo = xy % Yo, xo = xy / Yo;
    long long src[4];
    int cnt[4], pos[4];
    int total = 0;
    for (int ch = 0; ch < 4; ++ch) {
        const int px = 2 * xo + (ch >> 1), py = 2 * yo + (ch & 1);
        const long long pidx = ((long long)s * X + px) * Y * C + (long long)py * C + c;
        src[ch] = pidx * K;
        // Spikes of a child are its leading finite slots.
        int nn = 0;
        while (nn < K && times[src[ch] + nn] < BATS_INF) ++nn;
        cnt[ch] = nn;
        pos[ch] = 0;
        total += n_spikes[pidx];
    }
    const long long obase = q * 4LL * K;
    int w = 0;
    while (true) {
        int best = -1;
        float bt = BATS_INF;
        for (int ch = 0; ch < 4; ++ch) {
            if (pos[ch] < cnt[ch]) {
                const float tt = times[src[ch] + pos[ch]];
                if (best < 0 || tt < bt) {
                    best = ch;
                    bt = tt;
                }
            }
        }
        if (best < 0) break;
        out_t[obase + w] = bt;
        out_idx[obase + w] = (int)(src[best] + pos[best]);
        ++pos[best];
        ++w;
    }
    for (int ch = 0; ch < 4; ++ch) {
        for (int k = cnt[ch]; k < K; ++k) {
            out_t[obase + w] = times[src[ch] + k];
            out_idx[obase + w] = (int)(src[ch] + k);
            ++w;
        }
    }
    out_n[q] = total;
}

__global__ void pool_backward_kernel(const float* __restrict__ errors, const int* __restrict__ idx, long long count,
                                     float* __restrict__ pre_err) {
    pdl_prologue();
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < count;
         q += (long long)gridDim.x * blockDim.x)
        pre_err[idx[q]] = errors[q];
}

}  // namespace bats

// ---------------------------------------------------------------------------------------------
// C-ABI

static void conv_tile(int C_out, int& TX, int& TY) {
    int P = 512 / C_out;
    if (P < 1) P = 1;
    TX = 1;
    while ((TX + 1) * (TX + 1) <= P) ++TX;
    TY = P / TX;
}

extern "C" int bats_conv_forward(const void* events, const int* ev_count, long long ev_cap, const float* weights,
                                 int batch, int X, int Y, int C, int fx, int fy, int C_out, int k_post, float c,
                                 float delta_theta_tau, float tau, float max_simulation, int* n_spikes, float* a,
                                 float* x, float* times, float* post_exp_tau, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && X >= fx && Y >= fy && fx > 0 && fy > 0 && C > 0 && C_out > 0 && k_post > 0 &&
                     X < 1024 && Y < 1024 && C < 2048 && C_out <= 1024,
                 BATS_ERR_BAD_SHAPE, "conv_forward: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_count && weights && n_spikes && a && x && times && post_exp_tau, BATS_ERR_NULL,
                 "conv_forward: null pointer");
    const int Xo = X - fx + 1, Yo = Y - fy + 1;
    int TX, TY;
    conv_tile(C_out, TX, TY);
    const int threads = ((TX * TY * C_out + 31) / 32) * 32;
    const int tiles_x = (Xo + TX - 1) / TX, tiles_y = (Yo + TY - 1) / TY;
    const size_t nw = (size_t)C_out * fx * fy * C;
    const size_t base_smem = bats::CONV_CHUNK * (sizeof(bats::ConvEvent) + sizeof(float2)) + 32 * sizeof(int);
    const int w_in_smem = (base_smem + nw * sizeof(float)) <= 200 * 1024;
    const size_t smem = base_smem + (w_in_smem ? nw * sizeof(float) : 0);
    BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::conv_forward_kernel, (int)smem));
    dim3 grid(tiles_x * tiles_y, batch);
    BATS_CUDA(bats::launch(bats::conv_forward_kernel, grid, threads, smem, stream,
        reinterpret_cast<const bats::Event*>(events), ev_count, ev_cap, weights, X, Y, C, fx, fy, C_out, Xo, Yo, TX, TY,
        tiles_y, k_post, bats::make_solve_const(c, delta_theta_tau, tau, max_simulation), w_in_smem, n_spikes, a, x,
        times, post_exp_tau));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_conv_backward(const void* events, const int* ev_slot, const int* ev_count, long long ev_cap,
                                  const float* weights, int batch, int X, int Y, int C, int fx, int fy, int C_out,
                                  int k_pre, const float* post_times, const void* tables, const int* nvalid,
                                  int k_post, float tau_s, float tau, float* grad_per_sample, float* pre_errors,
                                  cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && X >= fx && Y >= fy && fx > 0 && fy > 0 && C > 0 && C_out > 0 && k_post > 0 &&
                     k_pre > 0,
                 BATS_ERR_BAD_SHAPE, "conv_backward: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_slot && ev_count && weights && post_times && tables && nvalid && grad_per_sample,
                 BATS_ERR_NULL, "conv_backward: null pointer");
    const int Xo = X - fx + 1, Yo = Y - fy + 1;
    const long long taps = (long long)C_out * fx * fy;
    const long long pre_slots = (long long)X * Y * C * k_pre;
    BATS_CUDA(cudaMemsetAsync(grad_per_sample, 0, (size_t)batch * taps * C * sizeof(float), stream));
    if (pre_errors) BATS_CUDA(cudaMemsetAsync(pre_errors, 0, (size_t)batch * pre_slots * sizeof(float), stream));
    int threads = (int)std::min<long long>(1024, ((taps + 31) / 32) * 32);
    const size_t gbytes = (size_t)taps * C * sizeof(float);
    if (gbytes <= 160 * 1024) {
        // Cluster path: the per-sample filter gradient lives in shared memory of every CTA of the cluster.
        BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::conv_backward_cluster_kernel, (int)gbytes));
        int top = 1;
        while (top * 2 <= k_post) top *= 2;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(bats::CONV_BWD_CLUSTER, batch);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = gbytes;
        cfg.stream = stream;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = bats::CONV_BWD_CLUSTER;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1 + (unsigned)bats::pdl_attribute(attr + 1);
        BATS_CUDA(cudaLaunchKernelEx(&cfg, bats::conv_backward_cluster_kernel,
                                     reinterpret_cast<const bats::Event*>(events), ev_slot, ev_count, ev_cap, weights,
                                     Y, C, fx, fy, C_out, Xo, Yo, post_times,
                                     reinterpret_cast<const float2*>(tables), nvalid, k_post, top, tau_s, tau,
                                     pre_slots, grad_per_sample, pre_errors, batch, 1));
        return BATS_OK;
    }
    BATS_CUDA(bats::launch(bats::conv_backward_kernel, batch, threads, 0, stream,
        reinterpret_cast<const bats::Event*>(events), ev_slot, ev_count, ev_cap, weights, Y, C, fx, fy, C_out, Xo, Yo,
        post_times, reinterpret_cast<const float2*>(tables), nvalid, k_post, tau_s, tau, pre_slots, grad_per_sample,
        pre_errors));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_conv_backward_grouped(const void* events_bucketed, const int* bucket_offsets, long long ev_cap,
                                          const float* weights, int batch, int X, int Y, int C, int fx, int fy,
                                          int C_out, int k_pre, const float* post_times, const void* tables,
                                          const int* nvalid, int k_post, float tau_s, float tau,
                                          float* grad_per_sample, float* pre_errors, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && X >= fx && Y >= fy && fx > 0 && fy > 0 && C > 0 && C_out > 0 && k_post > 0 &&
                     k_pre > 0,
                 BATS_ERR_BAD_SHAPE, "conv_backward_grouped: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(events_bucketed && bucket_offsets && weights && post_times && tables && nvalid && grad_per_sample,
                 BATS_ERR_NULL, "conv_backward_grouped: null pointer");
    const long long taps = (long long)C_out * fx * fy;
    BATS_REQUIRE(taps <= 1024 && (long long)X * Y <= 255, BATS_ERR_BAD_SHAPE,
                 "conv_backward_grouped: needs at most 1024 taps and 255 input positions");
    const int Xo = X - fx + 1, Yo = Y - fy + 1;
    const long long pre_slots = (long long)X * Y * C * k_pre;
    const size_t gsmem = (size_t)taps * C * sizeof(float) + (size_t)C * sizeof(int);
    BATS_REQUIRE(gsmem <= 160 * 1024, BATS_ERR_BAD_SHAPE, "conv_backward_grouped: filter gradient too large");
    const int w_in_smem = pre_errors && gsmem + (size_t)taps * C * sizeof(float) <= 200 * 1024;
    const size_t smem = gsmem + (w_in_smem ? (size_t)taps * C * sizeof(float) : 0);
    if (pre_errors) BATS_CUDA(cudaMemsetAsync(pre_errors, 0, (size_t)batch * pre_slots * sizeof(float), stream));
    BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::conv_backward_grouped_kernel, (int)smem));
    const int threads = (int)(((taps + 31) / 32) * 32);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(bats::CONV_BWD_CLUSTER, batch);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = bats::CONV_BWD_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1 + (unsigned)bats::pdl_attribute(attr + 1);
    BATS_CUDA(cudaLaunchKernelEx(&cfg, bats::conv_backward_grouped_kernel,
                                 reinterpret_cast<const bats::Event*>(events_bucketed), bucket_offsets, X * Y, ev_cap,
                                 weights, Y, C, fx, fy, C_out, Xo, Yo, k_pre, post_times,
                                 reinterpret_cast<const float2*>(tables), nvalid, k_post, tau_s, tau, pre_slots,
                                 grad_per_sample, pre_errors, batch, 1, w_in_smem));
    return BATS_OK;
}

// Sum of per-group partial filter gradients (groups, total) in group order, divided by the batch.
namespace bats {
__global__ void conv_grad_reduce_kernel(const float* __restrict__ part, int groups, int total, float batch,
                                        float* __restrict__ grad) {
    pdl_prologue();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total) return;
    float acc = 0.0f;
    for (int g = 0; g < groups; ++g) acc += part[(long long)g * total + q];
    grad[q] = acc / batch;
}
}  // namespace bats

extern "C" size_t bats_conv_backward_adam_workspace_bytes(int batch, int C, int fx, int fy, int C_out, int group) {
    if (batch <= 0 || group <= 0) return 0;
    const long long groups = (batch + group - 1) / group;
    return ((size_t)groups * C_out * fx * fy * C * sizeof(float) + 255) & ~(size_t)255;
}

extern "C" int bats_conv_backward_adam(const void* events, const int* ev_slot, const int* ev_count,
                                       const void* events_bucketed, const int* bucket_offsets, long long ev_cap,
                                       float* weights, int batch, int X, int Y, int C, int fx, int fy, int C_out,
                                       int k_pre, const float* post_times, const void* tables, const int* nvalid,
                                       int k_post, float tau_s, float tau, float* pre_errors, int group, float* grad,
                                       float* m, float* v, float beta_1, float beta_2, float epsilon,
                                       float learning_rate, const double* powers, void* workspace,
                                       size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && X >= fx && Y >= fy && fx > 0 && fy > 0 && C > 0 && C_out > 0 && k_post > 0 &&
                     k_pre > 0 && group >= 1,
                 BATS_ERR_BAD_SHAPE, "conv_backward_adam: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(events && ev_slot && ev_count && weights && post_times && tables && nvalid && grad && m && v && powers,
                 BATS_ERR_NULL, "conv_backward_adam: null pointer");
    const int groups = (batch + group - 1) / group;
    BATS_REQUIRE(groups <= 65535, BATS_ERR_BAD_SHAPE, "conv_backward_adam: more than 65535 sample groups");
    BATS_REQUIRE(workspace && workspace_bytes >= bats_conv_backward_adam_workspace_bytes(batch, C, fx, fy, C_out, group),
                 BATS_ERR_WORKSPACE, "conv_backward_adam: workspace too small");
    const int Xo = X - fx + 1, Yo = Y - fy + 1;
    const long long taps = (long long)C_out * fx * fy;
    const int total = (int)(taps * C);
    const long long pre_slots = (long long)X * Y * C * k_pre;
    float* part = reinterpret_cast<float*>(workspace);
    if (pre_errors) BATS_CUDA(cudaMemsetAsync(pre_errors, 0, (size_t)batch * pre_slots * sizeof(float), stream));
    const bool grouped = events_bucketed && bucket_offsets && taps <= 1024 && (long long)X * Y <= 255 &&
                         (size_t)taps * C * sizeof(float) + (size_t)C * sizeof(int) <= 160 * 1024;
    const size_t gbytes = (size_t)taps * C * sizeof(float) + (grouped ? (size_t)C * sizeof(int) : 0);
    BATS_REQUIRE(gbytes <= 160 * 1024, BATS_ERR_BAD_SHAPE, "conv_backward_adam: filter gradient too large");
    const int threads = (int)std::min<long long>(1024, ((taps + 31) / 32) * 32);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(bats::CONV_BWD_CLUSTER, groups);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = gbytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = bats::CONV_BWD_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1 + (unsigned)bats::pdl_attribute(attr + 1);
    if (grouped) {
        const int w_in_smem = pre_errors && gbytes + (size_t)taps * C * sizeof(float) <= 200 * 1024;
        if (w_in_smem) cfg.dynamicSmemBytes = gbytes + (size_t)taps * C * sizeof(float);
        BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::conv_backward_grouped_kernel,
                                                          (int)cfg.dynamicSmemBytes));
        BATS_CUDA(cudaLaunchKernelEx(&cfg, bats::conv_backward_grouped_kernel,
                                     reinterpret_cast<const bats::Event*>(events_bucketed), bucket_offsets, X * Y,
                                     ev_cap, (const float*)weights, Y, C, fx, fy, C_out, Xo, Yo, k_pre, post_times,
                                     reinterpret_cast<const float2*>(tables), nvalid, k_post, tau_s, tau, pre_slots,
                                     part, pre_errors, batch, group, w_in_smem));
    } else {
        BATS_CUDA((cudaError_t)bats::max_dynamic_smem_set((const void*)bats::conv_backward_cluster_kernel, (int)gbytes));
        int top = 1;
        while (top * 2 <= k_post) top *= 2;
        BATS_CUDA(cudaLaunchKernelEx(&cfg, bats::conv_backward_cluster_kernel,
                                     reinterpret_cast<const bats::Event*>(events), ev_slot, ev_count, ev_cap,
                                     (const float*)weights, Y, C, fx, fy, C_out, Xo, Yo, post_times,
                                     reinterpret_cast<const float2*>(tables), nvalid, k_post, top, tau_s, tau,
                                     pre_slots, part, pre_errors, batch, group));
    }
    BATS_CUDA(bats::launch(bats::conv_grad_reduce_kernel, (total + 255) / 256, 256, 0, stream, part, groups, total,
                           (float)batch, grad));
    BATS_CUDA(cudaGetLastError());
    return bats_adam_step_device(grad, m, v, total, beta_1, beta_2, epsilon, learning_rate, powers, weights, nullptr,
                                 0, 0, 0, stream);
}

extern "C" int bats_pool_forward(const int* n_spikes, const float* times, int batch, int X, int Y, int C, int K,
                                 int* out_n_spikes, float* out_times, int* out_indices, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && X >= 2 && Y >= 2 && C > 0 && K > 0, BATS_ERR_BAD_SHAPE, "pool_forward: bad shape");
    BATS_REQUIRE((long long)batch * X * Y * C * K < (1LL << 31), BATS_ERR_CAPACITY,
                 "pool_forward: indices exceed int32");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(n_spikes && times && out_n_spikes && out_times && out_indices, BATS_ERR_NULL,
                 "pool_forward: null pointer");
    const long long total = (long long)batch * (X / 2) * (Y / 2) * C;
    BATS_CUDA(bats::launch(bats::pool_forward_kernel, (unsigned)((total + 127) / 128), 128, 0, stream, n_spikes, times,
        batch, X, Y, C, K, out_n_spikes, out_times, out_indices));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}

extern "C" int bats_pool_backward(const float* errors, const int* indices, long long count, float* pre_errors,
                                  long long pre_count, cudaStream_t stream) {
    BATS_REQUIRE(count >= 0 && pre_count >= 0, BATS_ERR_BAD_SHAPE, "pool_backward: bad shape");
    if (pre_count > 0) {
        BATS_REQUIRE(pre_errors, BATS_ERR_NULL, "pool_backward: null pointer");
        BATS_CUDA(cudaMemsetAsync(pre_errors, 0, (size_t)pre_count * sizeof(float), stream));
    }
    if (count == 0) return BATS_OK;
    BATS_REQUIRE(errors && indices, BATS_ERR_NULL, "pool_backward: null pointer");
    long long b = (count + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    BATS_CUDA(bats::launch(bats::pool_backward_kernel, (unsigned)b, 256, 0, stream, errors, indices, count,
        pre_errors));
    BATS_CUDA(cudaGetLastError());
    return BATS_OK;
}
