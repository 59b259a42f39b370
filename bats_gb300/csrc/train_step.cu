// One training step of a fully-connected network in a single call (bats_fc_train_step), for callers that
// train through the C ABI instead of the Python layer classes. It enqueues, on one stream and with no host
// synchronisation, exactly the entry-point sequence of the Python train step (bats_gb300/train.py,
// FCTrainStep._build_launches): Adam's powers, per layer the sort (the hidden layers' sorts with the samples
// longest first on batches wider than two CTAs per SM) and the forward, the loss, then per layer from the last
// one the reset-error/factor/table pass, the pre-spike errors and the fused batch-mean gradient + Adam update.
// Same calls, same arguments, so the results are bit-identical to that sequence.
// Reference counterpart: the training iteration of experiments/mnist/train_spike_count.py:143-177.
#include <algorithm>
#include "abi_util.h"

namespace {

constexpr int TRAIN_BUCKET_WIDTH = BATS_GRAD_BUCKET_WIDTH;  // pre-neuron buckets of the gradient kernel (its GRAD_JC)

bool is_queue(int algo) {
    const int base = algo & ~(BATS_FWD_NO_PAD | BATS_FWD_STAGE_SCREEN);
    return base == BATS_FWD_QUEUE || base == BATS_FWD_QUEUE64;
}

// The forward's padding rule of the Python step: hidden layers with k_post <= 32 leave the slots past the
// spike counts as they are (everything that reads them stays below the counts); the output layer (read by
// the loss) and layers with k_post > 32 (whose backward prep scans the times) are padded with +inf.
int pad_flag(const BatsFcTrainLayer* layers, int n_layers, int l) {
    return (l + 1 == n_layers || layers[l].fwd.k_post > 32) ? 0 : BATS_FWD_NO_PAD;
}

// The sample order of the hidden layers' sorts at the workspace's start (its own 256-byte lines; the calls
// share the rest), used when the batch is wider than the sort's resident CTAs (two per SM), as in the Python step.
size_t order_bytes(int batch) { return ((size_t)(batch > 0 ? batch : 0) * sizeof(int) + 255) / 256 * 256; }
bool order_pays(int batch) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return false;
    return batch > 2 * sms;
}

}  // namespace

extern "C" size_t bats_fc_train_step_workspace_bytes(int batch, const BatsFcTrainLayer* layers, int n_layers) {
    if (batch <= 0 || !layers || n_layers <= 0) return 256;
    size_t ws = 256;
    for (int l = 0; l < n_layers; ++l) {
        const BatsFcLayer& F = layers[l].fwd;
        ws = std::max(ws, bats_sort_events_workspace_bytes(batch, F.n_pre, F.k_pre));
        ws = std::max(ws, bats_lif_forward_fc_queue_workspace_bytes(batch));
        ws = std::max(ws, bats_weights_gradient_workspace_bytes(batch, F.n_post, F.n_pre, layers[l].grad_group));
        ws = std::max(ws, bats_pre_errors_workspace_bytes(batch, (long long)F.n_pre * F.k_pre, F.n_post));
    }
    return order_bytes(batch) + ws;
}

extern "C" int bats_fc_train_step(const float* in_times, const int* labels, int batch, BatsFcTrainLayer* layers,
                                  int n_layers, float target_true, float target_false, float beta_1, float beta_2,
                                  float epsilon, float learning_rate, double* powers, float* loss, float* errors,
                                  void* workspace, size_t workspace_bytes, cudaStream_t stream) {
    BATS_REQUIRE(batch >= 0 && n_layers > 0, BATS_ERR_BAD_SHAPE, "fc_train_step: bad shape");
    if (batch == 0) return BATS_OK;
    BATS_REQUIRE(in_times && labels && layers && powers && loss && errors && workspace, BATS_ERR_NULL,
                 "fc_train_step: null pointer");
    for (int l = 0; l < n_layers; ++l) {
        const BatsFcTrainLayer& L = layers[l];
        BATS_REQUIRE(L.grad_group >= 2 && (l == 0 || (L.fwd.n_pre == layers[l - 1].fwd.n_post &&
                                                        L.fwd.k_pre == layers[l - 1].fwd.k_post)),
                     BATS_ERR_BAD_SHAPE, "fc_train_step: layers do not chain, or grad_group < 2");
        BATS_REQUIRE(L.weights && L.adam_m && L.adam_v && L.grad && (!L.events_bucketed == !L.bucket_offsets) &&
                         L.tables && L.nvalid && (l == 0 || L.pre_errors) &&
                         (L.fwd.k_post <= 32 || (L.f1 && L.f2)),
                     BATS_ERR_NULL, "fc_train_step: null layer buffer");
    }
    BATS_REQUIRE(workspace_bytes >= bats_fc_train_step_workspace_bytes(batch, layers, n_layers), BATS_ERR_WORKSPACE,
                 "fc_train_step: workspace too small (bats_fc_train_step_workspace_bytes)");
    int* order = reinterpret_cast<int*>(workspace);
    const bool ordered = order_pays(batch);
    workspace = reinterpret_cast<char*>(workspace) + order_bytes(batch);
    workspace_bytes -= order_bytes(batch);
    int rc = bats_adam_powers_advance(powers, beta_1, beta_2, stream);
    if (rc != BATS_OK) return rc;
    // Forward.
    for (int l = 0; l < n_layers; ++l) {
        const BatsFcTrainLayer& L = layers[l];
        const BatsFcLayer& F = L.fwd;
        if (l == 0)
            rc = bats_sort_events(in_times, batch, F.n_pre, F.k_pre, F.tau_s, F.tau, nullptr, nullptr, F.events,
                                  F.slots, F.ev_count, L.events_bucketed, L.bucket_offsets, TRAIN_BUCKET_WIDTH,
                                  workspace, workspace_bytes, stream);
        else if (!ordered)
            rc = bats_sort_events_counted(layers[l - 1].fwd.times, layers[l - 1].fwd.n_spikes, batch, F.n_pre,
                                          F.k_pre, F.tau_s, F.tau, nullptr, nullptr, F.events, F.slots, F.ev_count,
                                          L.events_bucketed, L.bucket_offsets, TRAIN_BUCKET_WIDTH, workspace,
                                          workspace_bytes, stream);
        else {  // the samples longest first, ranked by the previous layer's input event counts
            rc = bats_sample_order(layers[l - 1].fwd.ev_count, batch, order, stream);
            if (rc != BATS_OK) return rc;
            rc = bats_sort_events_counted_ordered(layers[l - 1].fwd.times, layers[l - 1].fwd.n_spikes, batch,
                                                  F.n_pre, F.k_pre, F.tau_s, F.tau, nullptr, nullptr, F.events,
                                                  F.slots, F.ev_count, L.events_bucketed, L.bucket_offsets,
                                                  TRAIN_BUCKET_WIDTH, order, workspace, workspace_bytes, stream);
        }
        if (rc != BATS_OK) return rc;
        const long long cap = (long long)F.n_pre * F.k_pre;
        const int algo = F.algo | pad_flag(layers, n_layers, l);
        if (is_queue(algo)) {
            const int base = algo & ~(BATS_FWD_NO_PAD | BATS_FWD_STAGE_SCREEN);
            const int tile = base == BATS_FWD_QUEUE64 ? BATS_FWD_TILE64 : BATS_FWD_TILE;
            rc = bats_lif_forward_fc_queue(F.events, F.ev_count, cap, F.weights_t, F.ld, batch, F.n_post, F.k_post,
                                           F.c, F.delta_theta_tau, F.tau, F.max_simulation, F.n_spikes, F.a, F.x,
                                           F.times, F.post_exp_tau,
                                           tile | (algo & (BATS_FWD_NO_PAD | BATS_FWD_STAGE_SCREEN)), workspace,
                                           workspace_bytes, stream);
        } else {
            rc = bats_lif_forward_fc_algo(F.events, F.ev_count, cap, F.weights_t, F.ld, batch, F.n_post, F.k_post,
                                          F.c, F.delta_theta_tau, F.tau, F.max_simulation, F.n_spikes, F.a, F.x,
                                          F.times, F.post_exp_tau, algo, stream);
        }
        if (rc != BATS_OK) return rc;
    }
    // Loss and output errors.
    const BatsFcLayer& O = layers[n_layers - 1].fwd;
    rc = bats_spike_count_loss(O.n_spikes, 0, nullptr, labels, target_true, target_false, batch, O.n_post, O.k_post,
                               loss, errors, stream);
    if (rc != BATS_OK) return rc;
    // Backward, last layer first. The pre-spike errors of layer l read its weights before their update, and
    // become the incoming errors of layer l - 1.
    float* err = errors;
    for (int l = n_layers - 1; l >= 0; --l) {
        const BatsFcTrainLayer& L = layers[l];
        const BatsFcLayer& F = L.fwd;
        // The cursor heads (optional) come from the counted prep only.
        const void* heads = F.k_post <= 32 ? L.cursor_heads : nullptr;
        if (F.k_post <= 32)
            rc = bats_backward_prep_counted(F.times, F.n_spikes, F.a, F.x, F.post_exp_tau, err, batch, F.n_post,
                                            F.k_post, F.c, F.tau, F.delta_theta_tau, L.tables, L.nvalid,
                                            L.cursor_heads, stream);
        else
            rc = bats_backward_prep_layer(F.times, F.a, F.x, F.post_exp_tau, err, batch, F.n_post, F.k_post, F.c,
                                          F.tau, F.delta_theta_tau, L.f1, L.f2, L.tables, L.nvalid, stream);
        if (rc != BATS_OK) return rc;
        const long long cap = (long long)F.n_pre * F.k_pre;
        if (l > 0) {
            rc = bats_pre_errors(F.events, F.slots, F.ev_count, cap, F.weights_t, F.ld, F.times, L.tables, L.nvalid,
                                 batch, F.n_post, F.k_post, F.n_pre, F.k_pre, F.tau_s, F.tau, L.pre_errors, workspace,
                                 workspace_bytes, stream);
            if (rc != BATS_OK) return rc;
        }
        rc = bats_weights_gradient_adam(F.events, F.ev_count, L.events_bucketed, L.bucket_offsets, cap, F.times,
                                        L.tables, L.nvalid, heads, batch, F.n_post, F.k_post, F.n_pre, L.grad_group,
                                        L.grad,
                                        L.adam_m, L.adam_v, beta_1, beta_2, epsilon, learning_rate, powers, L.weights,
                                        const_cast<float*>(F.weights_t), F.ld, workspace, workspace_bytes, stream);
        if (rc != BATS_OK) return rc;
        if (l > 0) err = L.pre_errors;
    }
    return BATS_OK;
}
