// One inference batch of a fully-connected network in a single call: the host-side request packing
// stays in the caller (flat event list + offsets in pinned memory), everything else is enqueued here on
// one stream with no host synchronisation: host -> device copy of the events, event list -> spike
// trains, per layer the event sort and the LIF forward (kernel variant per layer), and the copy of the
// output layer's counts and spike times (and the overflow count) back to pinned host memory. The
// serving loop (bats_gb300/serving.py) calls it once per batch, so a batch costs one foreign call on
// the host instead of one per kernel.
#include "abi_util.h"

extern "C" int bats_serve_fc_batch(const int* h_indices, const float* h_times, const int* h_offsets, int batch,
                                   int total_events, int* d_indices, float* d_times, int* d_offsets, int n_inputs,
                                   int k_in, float* d_trains, int* d_train_counts, int* d_overflow,
                                   const BatsFcLayer* layers, int n_layers, void* sort_workspace,
                                   size_t sort_workspace_bytes, int* h_out_counts, float* h_out_times,
                                   int* h_overflow, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && total_events >= 0 && n_inputs > 0 && k_in > 0 && n_layers > 0, BATS_ERR_BAD_SHAPE,
                 "serve_fc_batch: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(h_indices && h_times && h_offsets && d_indices && d_times && d_offsets && d_trains &&
                     d_train_counts && d_overflow && layers && h_out_counts && h_out_times && h_overflow,
                 BATS_ERR_NULL, "serve_fc_batch: null pointer");
    if (total_events > 0) {
        BATS_CUDA(cudaMemcpyAsync(d_indices, h_indices, (size_t)total_events * sizeof(int), cudaMemcpyHostToDevice,
                                  stream));
        BATS_CUDA(cudaMemcpyAsync(d_times, h_times, (size_t)total_events * sizeof(float), cudaMemcpyHostToDevice,
                                  stream));
    }
    BATS_CUDA(cudaMemcpyAsync(d_offsets, h_offsets, (size_t)(batch + 1) * sizeof(int), cudaMemcpyHostToDevice,
                              stream));
    BATS_CUDA(cudaMemsetAsync(d_overflow, 0, sizeof(int), stream));
    int rc = bats_events_to_trains_csr(d_indices, d_times, d_offsets, batch, n_inputs, k_in, d_trains,
                                       d_train_counts, d_overflow, stream);
    if (rc != BATS_OK) return rc;
    const float* pre = d_trains;
    for (int l = 0; l < n_layers; ++l) {
        const BatsFcLayer& L = layers[l];
        // The input trains are read whole; a LIF layer's output only below its spike counts.
        if (l == 0)
            rc = bats_sort_events(pre, batch, L.n_pre, L.k_pre, L.tau_s, L.tau, nullptr, nullptr, L.events, L.slots,
                                  L.ev_count, nullptr, nullptr, 0, sort_workspace, sort_workspace_bytes, stream);
        else
            rc = bats_sort_events_counted(pre, layers[l - 1].n_spikes, batch, L.n_pre, L.k_pre, L.tau_s, L.tau,
                                          nullptr, nullptr, L.events, L.slots, L.ev_count, nullptr, nullptr, 0,
                                          sort_workspace, sort_workspace_bytes, stream);
        if (rc != BATS_OK) return rc;
        rc = bats_lif_forward_fc_algo(L.events, L.ev_count, (long long)L.n_pre * L.k_pre, L.weights_t, L.ld, batch,
                                      L.n_post, L.k_post, L.c, L.delta_theta_tau, L.tau, L.max_simulation,
                                      L.n_spikes, L.a, L.x, L.times, L.post_exp_tau,
                                      l + 1 < n_layers ? (L.algo | BATS_FWD_NO_PAD) : L.algo, stream);
        if (rc != BATS_OK) return rc;
        pre = L.times;
    }
    const BatsFcLayer& out = layers[n_layers - 1];
    BATS_CUDA(cudaMemcpyAsync(h_out_counts, out.n_spikes, (size_t)batch * out.n_post * sizeof(int),
                              cudaMemcpyDeviceToHost, stream));
    BATS_CUDA(cudaMemcpyAsync(h_out_times, out.times, (size_t)batch * out.n_post * out.k_post * sizeof(float),
                              cudaMemcpyDeviceToHost, stream));
    BATS_CUDA(cudaMemcpyAsync(h_overflow, d_overflow, sizeof(int), cudaMemcpyDeviceToHost, stream));
    return BATS_OK;
}
