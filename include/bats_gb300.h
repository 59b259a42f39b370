/*
 * bats_gb300 — C ABI of the GB300 (sm_103a) kernels for event-based LIF simulation and exact
 * multi-spike error backpropagation (the BATS method).
 *
 * Conventions
 *   - Every pointer is a device pointer owned by the caller (for example a torch tensor's
 *     data_ptr()); the library never allocates device memory. Entry points that need scratch
 *     memory take (workspace, workspace_bytes) and have a *_workspace_bytes() query.
 *   - Every entry point returns a status (BATS_OK == 0); bats_last_error() describes the last
 *     failure of the calling thread. Launches are asynchronous on `stream`.
 *   - Spike trains are (B, N, K) float32 row-major, +inf after the neuron's spikes, with counts
 *     (B, N) int32. Weights of a fully-connected layer are (N_post, N_pre); the forward and
 *     error-propagation kernels read the transposed copy wt (N_pre, ld), ld >= N_post,
 *     ld % 4 == 0 and wt 16-byte aligned (bats_transpose builds it). Conv filters are (C_out, fx, fy, C_in).
 *   - `events` is an array of 16-byte records {float t; int j; float exp(t/tau_s); float exp(t/tau)}
 *     of shape (B, ev_cap), ev_cap = N_pre * K_pre, filled by bats_sort_events.
 *
 * The reference is the CuPy implementation (Florian-BACHO/bats); each entry point names the
 * wrapper(s) in bats/CudaKernels/Wrappers/ (and the .cu kernels under bats/CudaKernels/CuFiles/)
 * whose job it takes over.
 */
#ifndef BATS_GB300_H
#define BATS_GB300_H

#include <stddef.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BATS_ABI_VERSION 1
/* Pre neurons per bucket of the bucketed events that bats_weights_gradient(_adam) and the train step read. */
#define BATS_GRAD_BUCKET_WIDTH 32

#define BATS_OK 0
#define BATS_ERR_BAD_SHAPE 1
#define BATS_ERR_NULL 2
#define BATS_ERR_CAPACITY 3
#define BATS_ERR_WORKSPACE 4
#define BATS_ERR_CUDA 5
#define BATS_ERR_TIMEOUT 6

int bats_abi_version(void);

/* Device-side waits (the mbarrier pipelines of the forward kernels) are bounded: a wait that gives up
 * sets this device's status word and the kernel returns early. Reads it into *out (synchronous), clears
 * it if `clear`, and returns BATS_ERR_TIMEOUT when it was set. */
int bats_read_device_status(int* out, int clear);
const char* bats_status_string(int status);
const char* bats_last_error(void);

/* ---- Inference ------------------------------------------------------------------------------ */

/* exp(t/tau_s), exp(t/tau) elementwise.
 * Replaces compute_pre_exps (bats/CudaKernels/Wrappers/Inference/compute_pre_exps.py:10-18). */
int bats_compute_pre_exps(const float* times, long long count, float tau_s, float tau, float* exp_tau_s,
                          float* exp_tau, cudaStream_t stream);

/* Per-sample time sort of the valid (time < +inf) pre-synaptic spike slots into `events`
 * (B, N_pre*K_pre) plus the slot index n*K_pre+k of each event (slot_out, may be NULL) and the
 * per-sample count. The events' exponentials are __expf(t/tau_s), __expf(t/tau), or gathered from
 * exp_tau_s / exp_tau (B, N_pre, K_pre) when those are given. When events_bucketed is given, the same
 * events are also written grouped by pre-neuron bucket (neuron / bucket_width, at most 255 buckets), time
 * order kept inside each bucket, with bucket_offsets (B, n_buckets + 1) delimiting the buckets.
 * Replaces get_sorted_spikes_indices + take_along_axis + compute_pre_exps
 * (bats/CudaKernels/Wrappers/Inference/get_sorted_spikes_indices.py:7-17; bats/Layers/LIFLayer.py:66-84). */
size_t bats_sort_events_workspace_bytes(int batch, int n_pre, int k_pre);
int bats_sort_events(const float* pre_times, int batch, int n_pre, int k_pre, float tau_s, float tau,
                     const float* exp_tau_s, const float* exp_tau, void* events, int* slot_out, int* ev_count,
                     void* events_bucketed, int* bucket_offsets, int bucket_width, void* workspace,
                     size_t workspace_bytes, cudaStream_t stream);

/* bats_sort_events given the pre layer's spike counts pre_counts (B, N_pre), as the reference's sort receives
 * them (get_sorted_spikes_indices(spike_times_per_neuron, n_spike_per_neuron),
 * bats/CudaKernels/Wrappers/Inference/get_sorted_spikes_indices.py:7). Neuron j's slots q >= pre_counts[s, j]
 * (clamped to [0, K_pre]) must hold +inf, as bats_lif_forward_fc writes them; only the slots below the count
 * are read (and non-finite times among them skipped), so the outputs are identical to bats_sort_events on the
 * same times. */
int bats_sort_events_counted(const float* pre_times, const int* pre_counts, int batch, int n_pre, int k_pre,
                             float tau_s, float tau, const float* exp_tau_s, const float* exp_tau, void* events,
                             int* slot_out, int* ev_count, void* events_bucketed, int* bucket_offsets,
                             int bucket_width, void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* bats_sort_events_counted with the samples taken in the order sample_order (B ints, a permutation of
 * 0 .. B-1): the sort's CTA b works on sample sample_order[b]. The outputs are identical for every order;
 * longest samples first (bats_sample_order) shortens the launch on batches of uneven samples wider than the
 * sort's resident CTAs (two per SM). An entry outside [0, B) leaves its CTA idle. No reference counterpart:
 * the reference sorts the whole batch in one library call. */
int bats_sort_events_counted_ordered(const float* pre_times, const int* pre_counts, int batch, int n_pre,
                                     int k_pre, float tau_s, float tau, const float* exp_tau_s, const float* exp_tau,
                                     void* events, int* slot_out, int* ev_count, void* events_bucketed,
                                     int* bucket_offsets, int bucket_width, const int* sample_order, void* workspace,
                                     size_t workspace_bytes, cudaStream_t stream);

/* The samples ranked longest first by ev_count (B), into order (B ints): by descending count in logarithmic
 * classes (16 per octave), the order inside a class unspecified. One CTA; the order of the work-queue
 * forward (bats_lif_forward_fc_queue). Given the per-sample event counts of a layer's input, it is a close
 * guess of the order of the layer's output spike counts, for bats_sort_events_counted_ordered. */
int bats_sample_order(const int* ev_count, int batch, int* order, cudaStream_t stream);

/* Fully-connected LIF forward: spike counts (B, N_post) and a, x, times, post_exp_tau (B, N_post, K_post);
 * times/post_exp_tau are +inf after the spikes, a/x are undefined there. c = theta/tau,
 * delta_theta_tau = delta_theta/tau. Replaces get_spike_weights + compute_spike_times
 * (bats/CudaKernels/Wrappers/Inference/get_spike_weights.py:9-18, compute_spike_times.py:11-32). */
int bats_lif_forward_fc(const void* events, const int* ev_count, long long ev_cap, const float* weights_t, int ld,
                        int batch, int n_post, int k_post, float c, float delta_theta_tau, float tau,
                        float max_simulation, int* n_spikes, float* a, float* x, float* times, float* post_exp_tau,
                        cudaStream_t stream);

/* Time-to-first-spike encoding of 8-bit intensities (B, N): times (B, N, 1) = time_window * (1 - x / max_value)
 * (in double, then float), +inf and count 0 where x == 0. Replaces Dataset.__to_spikes of the reference's
 * MNIST experiments (experiments/mnist/Dataset.py:66-71). */
int bats_intensity_to_spike_times(const unsigned char* pixels, int batch, int n_neurons, double time_window,
                                  double max_value, float* times, int* counts, cudaStream_t stream);

/* Kernel choice of the FC forward: BATS_FWD_TILE runs one CTA per (post-neuron tile, sample) with a
 * producer warp streaming weight rows (throughput-oriented, large B * N_post); BATS_FWD_LANES runs one warp
 * per (sample, post neuron) with 32 events evaluated in parallel (latency-oriented: few neurons, small
 * batches, long event streams). Both give bit-identical results. BATS_FWD_AUTO picks by
 * bats_lif_forward_fc_default_algo. No counterpart in the reference (it has one kernel shape). */
#define BATS_FWD_AUTO 0
#define BATS_FWD_TILE 1
#define BATS_FWD_LANES 2
#define BATS_FWD_TILE64 3 /* the tile kernel with 64-neuron tiles whatever N_post (more CTAs, less reuse) */
/* OR-ed into `algo`: the slots past each neuron's spikes in times/post_exp_tau are left as they are instead of
 * set to +inf, for outputs read only below the spike counts (bats_sort_events_counted,
 * bats_backward_prep_counted, bats_weights_gradient, bats_pre_errors): the hidden layers of a train step. */
#define BATS_FWD_NO_PAD 0x100
/* OR-ed into `algo` (tile kernels, also those of bats_lif_forward_fc_queue; ignored by BATS_FWD_LANES): each
 * full stage of events first runs the accumulation alone, with one test per neuron and stage that rules out a
 * crossing after any of its events from the smallest a and the largest b of its states (the membrane bound
 * b/x - a/x^2 < theta/tau from the stage's first event on); only stages that fail it get the per-event tests.
 * Faster where most neurons stay far below threshold; results are bit-identical. */
#define BATS_FWD_STAGE_SCREEN 0x200
int bats_lif_forward_fc_default_algo(int batch, int n_post, int ev_cap);
int bats_lif_forward_fc_algo(const void* events, const int* ev_count, long long ev_cap, const float* weights_t,
                             int ld, int batch, int n_post, int k_post, float c, float delta_theta_tau, float tau,
                             float max_simulation, int* n_spikes, float* a, float* x, float* times,
                             float* post_exp_tau, int algo, cudaStream_t stream);

/* The FC forward as one persistent launch over a work queue, for batches whose samples carry very different
 * numbers of events. A first kernel ranks the samples by descending event count (in the workspace, which also
 * holds the queue head it resets); then as many CTAs as fit on the GPU at once take (sample, post-neuron tile)
 * items from the queue, longest samples first, each producer warp streaming its next item while the consumers
 * finish the current one. Outputs, arguments and results are those of bats_lif_forward_fc_algo (bit-identical);
 * algo is BATS_FWD_AUTO or BATS_FWD_TILE (tile width by n_post) or BATS_FWD_TILE64, optionally OR-ed with
 * BATS_FWD_NO_PAD and BATS_FWD_STAGE_SCREEN. The workspace (16-byte aligned,
 * bats_lif_forward_fc_queue_workspace_bytes(batch) bytes) must
 * not be used by another launch until this one ends. Replaces the same reference wrappers as
 * bats_lif_forward_fc (get_spike_weights.py:9-18, compute_spike_times.py:11-32); the reference runs one thread
 * per (sample, neuron) with no scheduling of its own. */
size_t bats_lif_forward_fc_queue_workspace_bytes(int batch);
int bats_lif_forward_fc_queue(const void* events, const int* ev_count, long long ev_cap, const float* weights_t,
                              int ld, int batch, int n_post, int k_post, float c, float delta_theta_tau, float tau,
                              float max_simulation, int* n_spikes, float* a, float* x, float* times,
                              float* post_exp_tau, int algo, void* workspace, size_t workspace_bytes,
                              cudaStream_t stream);

/* Convolutional LIF forward on a (X, Y, C) input with (C_out, fx, fy, C) filters, valid, stride 1.
 * Replaces compute_spike_times_conv (bats/CudaKernels/Wrappers/Inference/compute_spike_times_conv.py:11-35). */
int bats_conv_forward(const void* events, const int* ev_count, long long ev_cap, const float* weights, int batch,
                      int X, int Y, int C, int fx, int fy, int C_out, int k_post, float c, float delta_theta_tau,
                      float tau, float max_simulation, int* n_spikes, float* a, float* x, float* times,
                      float* post_exp_tau, cudaStream_t stream);

/* bats_conv_backward over the events grouped by input position (the bucketed copy of bats_sort_events with
 * bucket_width = C: one bucket per (x, y)); same outputs. For at most 1024 filter taps and 255 input
 * positions. No counterpart in the reference (same results as compute_weights_gradient_conv +
 * propagate_errors_to_pre_spikes_conv, computed from the position-grouped events). */
int bats_conv_backward_grouped(const void* events_bucketed, const int* bucket_offsets, long long ev_cap,
                               const float* weights, int batch, int X, int Y, int C, int fx, int fy, int C_out,
                               int k_pre, const float* post_times, const void* tables, const int* nvalid, int k_post,
                               float tau_s, float tau, float* grad_per_sample, float* pre_errors, cudaStream_t stream);

/* 2x2 spike-union pooling of a (X, Y, C) layer with K slots: counts, times sorted over 4K slots and
 * the flat (batch-global) source slot of every output slot. Replaces aggregate_spikes_conv
 * (bats/CudaKernels/Wrappers/Inference/aggregate_spikes_conv.py:10-28). */
int bats_pool_forward(const int* n_spikes, const float* times, int batch, int X, int Y, int C, int K,
                      int* out_n_spikes, float* out_times, int* out_indices, cudaStream_t stream);

/* Event list -> spike trains: indices/times (B, max_events), index < 0 ends a sample; writes times (B, N, k_cap)
 * (+inf padded, spikes of a neuron in order of appearance) and counts (B, N); spikes beyond k_cap are dropped
 * and added to *overflow (may be NULL). Replaces convert_to_spike_per_neuron
 * (bats/CudaKernels/Wrappers/Inference/convert_to_spike_per_neuron.py:20-33). */
int bats_events_to_trains(const int* indices, const float* times, int batch, int max_events, int n_neurons,
                          int k_cap, float* out_times, int* out_counts, int* overflow, cudaStream_t stream);

/* bats_events_to_trains over a flat event list: sample s owns events offsets[s] .. offsets[s + 1] - 1
 * (offsets: batch + 1 ints, device). No counterpart in the reference (its input is padded). */
int bats_events_to_trains_csr(const int* indices, const float* times, const int* offsets, int batch, int n_neurons,
                              int k_cap, float* out_times, int* out_counts, int* overflow, cudaStream_t stream);

/* Largest per-neuron spike count of each sample of an event list (the K of convert_to_spike_per_neuron,
 * Wrappers/Inference/convert_to_spike_per_neuron.py:11-18). scratch_counts (B, N) holds the running counts
 * when 4 * N ints do not fit the kernel's shared memory (N > 3072); it is left untouched otherwise. */
int bats_events_max_per_neuron(const int* indices, int batch, int max_events, int n_neurons, int* scratch_counts,
                               int* out_max, cudaStream_t stream);

/* ---- Backpropagation ------------------------------------------------------------------------ */

/* Per (sample, post neuron): reset errors in place on `errors` (if do_recurrent), factors f1/f2
 * (if do_factors) and, if `tables` is given, the suffix tables (B, N_post, K_post+1) float2 of
 * (sum_{k>=p} err_k f1_k, sum_{k>=p} err_k f2_k) with the count of leading spikes in nvalid (B, N_post).
 * Replaces propagate_recurrent_errors and compute_factors
 * (bats/CudaKernels/Wrappers/Backpropagation/propagate_recurrent_errors.py:9-16, compute_factors.py:11-22). */
int bats_backward_prep(const float* post_times, const float* a, const float* x, const float* post_exp_tau,
                       float* errors, int batch, int n_post, int k_post, float c, float tau, float delta_theta_tau,
                       int do_recurrent, int do_factors, float* f1, float* f2, void* tables, int* nvalid,
                       cudaStream_t stream);

/* bats_backward_prep (recurrent + factors + tables) for spike trains produced by the forward entry points
 * (post_times and post_exp_tau finite exactly on each neuron's leading spikes): rows staged through shared
 * memory, silent neurons skipped, f1/f2 written only if given (required when k_post > 32). */
int bats_backward_prep_layer(const float* post_times, const float* a, const float* x, const float* post_exp_tau,
                             float* errors, int batch, int n_post, int k_post, float c, float tau,
                             float delta_theta_tau, float* f1, float* f2, void* tables, int* nvalid,
                             cudaStream_t stream);

/* bats_backward_prep_layer given the forward's spike counts n_spikes (B, N_post): only each neuron's first
 * min(n_spikes, K) slots are read (the forward writes +inf past them), valid slots are staged compactly, and
 * errors, tables and nvalid are identical to bats_backward_prep_layer's (nvalid = the first +inf time below
 * the count, or the count). No f1/f2 output; k_post <= 32. Replaces propagate_recurrent_errors and
 * compute_factors (bats/CudaKernels/Wrappers/Backpropagation/propagate_recurrent_errors.py:9-16,
 * compute_factors.py:11-22), which the reference runs over all N_post * K slots.
 * cursor_heads (optional, NULL to skip; 16-byte aligned, bats_cursor_heads_bytes(batch, n_post) bytes):
 * per (sample, neuron) the first two spike times and the first two table entries in one coalesced array,
 * which the weight gradient reads instead of the start of each table row (same results, fewer memory
 * sectors). No counterpart in the reference. */
size_t bats_cursor_heads_bytes(int batch, int n_post);
int bats_backward_prep_counted(const float* post_times, const int* n_spikes, const float* a, const float* x,
                               const float* post_exp_tau, float* errors, int batch, int n_post, int k_post, float c,
                               float tau, float delta_theta_tau, void* tables, int* nvalid, void* cursor_heads,
                               cudaStream_t stream);

/* Weight gradient of a fully-connected layer. group == 1: per-sample gradient (B, N_post, N_pre) like the
 * reference; group > 1: the batch mean (mean != 0) or sum (N_post, N_pre), accumulated per group of samples
 * and reduced in a fixed order (deterministic). Reads the events grouped in pre-neuron buckets of
 * BATS_GRAD_BUCKET_WIDTH (events_bucketed + bucket_offsets from bats_sort_events with bucket_width
 * BATS_GRAD_BUCKET_WIDTH) when given, else filters the
 * time-sorted events (events + ev_count). cursor_heads: NULL, or the array bats_backward_prep_counted wrote
 * with these tables (used with the bucketed events). Replaces compute_weights_gradient (+ the caller's mean
 * over the batch) (bats/CudaKernels/Wrappers/Backpropagation/compute_weights_gradient.py:10-24). */
size_t bats_weights_gradient_workspace_bytes(int batch, int n_post, int n_pre, int group);
int bats_weights_gradient(const void* events, const int* ev_count, const void* events_bucketed,
                          const int* bucket_offsets, long long ev_cap, const float* post_times, const void* tables,
                          const int* nvalid, const void* cursor_heads, int batch, int n_post, int k_post, int n_pre,
                          int group, int mean, float* grad, void* workspace, size_t workspace_bytes,
                          cudaStream_t stream);

/* The batch-mean weight gradient (bats_weights_gradient with group >= 2, mean) and the Adam update of the
 * weights (bats_adam_step_device) in one call: the group partials are summed, divided by the batch and fed to
 * Adam by one tiled kernel, so the gradient needs no round trip through memory; grad (n_post, n_pre) receives
 * it too when not NULL (required when group >= batch, as the one partial lives there). m, v, weights and
 * weights_t (n_pre, ld) are updated in place; powers as for bats_adam_step_device (advanced before the call).
 * For a layer of fewer than 304 32 x 32 weight tiles (a narrow layer) with several partials and grad given, the
 * row-parallel reduction into grad and the tiled Adam run as two kernels instead (more CTAs per partial sum).
 * Results are bit-identical to the two calls. Replaces compute_weights_gradient + the batch mean
 * (bats/CudaKernels/Wrappers/Backpropagation/compute_weights_gradient.py:10-24, train_spike_count.py:167) and
 * AdamOptimizer.step + Network.apply_deltas (bats/Optimizers/AdamOptimizer.py:35-55,
 * bats/Layers/LIFLayer.py:112-113). The weights change, so a caller that propagates errors through this
 * layer (bats_pre_errors) does so before this call. Workspace: bats_weights_gradient_workspace_bytes.
 * cursor_heads as for bats_weights_gradient. */
int bats_weights_gradient_adam(const void* events, const int* ev_count, const void* events_bucketed,
                               const int* bucket_offsets, long long ev_cap, const float* post_times, const void* tables,
                               const int* nvalid, const void* cursor_heads, int batch, int n_post, int k_post,
                               int n_pre, int group, float* grad,
                               float* m, float* v, float beta_1, float beta_2, float epsilon, float learning_rate,
                               const double* powers, float* weights, float* weights_t, int ld, void* workspace,
                               size_t workspace_bytes, cudaStream_t stream);

/* Allocation-free batch mean of bats_weights_gradient (group >= 2), for callers that cannot allocate device
 * memory (a runtime with a fixed arena, a plugin host that passes only input and output buffers). No
 * counterpart in the reference. The per-group partial sums live in a 32 MiB static device array of the
 * library (bats_weights_gradient_noalloc_capacity() floats, held on every GPU that loads the library until
 * exit): ceil(batch/group) * n_post * n_pre must not exceed it (BATS_ERR_CAPACITY otherwise). The first call
 * on a device looks the array's address up (cudaGetSymbolAddress); make that first call before any stream
 * capture. The address is cached per device for the life of the process: after cudaDeviceReset on a device
 * (which tears down the context that holds the array) this entry point must not be called on that device
 * again. All calls share the array, so calls whose kernels overlap on the GPU race and must be serialised
 * by the caller. More than 65535 sample groups (ceil(batch/group)) give BATS_ERR_BAD_SHAPE. */
long long bats_weights_gradient_noalloc_capacity(void);
int bats_weights_gradient_mean_noalloc(const void* events, const int* ev_count, long long ev_cap,
                                       const float* post_times, const void* tables, const int* nvalid, int batch,
                                       int n_post, int k_post, int n_pre, int group, float* grad,
                                       cudaStream_t stream);

/* Errors of the pre-synaptic spikes (B, N_pre, K_pre), zero where there is no spike. Replaces
 * propagate_errors_to_pre_spikes and its (B, N_pre, K_pre, N_post) temporary + sum
 * (bats/CudaKernels/Wrappers/Backpropagation/propagate_errors_to_pre_spikes.py:11-27). */
size_t bats_pre_errors_workspace_bytes(int batch, long long ev_cap, int n_post);
int bats_pre_errors(const void* events, const int* ev_slot, const int* ev_count, long long ev_cap,
                    const float* weights_t, int ld, const float* post_times, const void* tables, const int* nvalid,
                    int batch, int n_post, int k_post, int n_pre, int k_pre, float tau_s, float tau,
                    float* pre_errors, void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Convolutional backward: per-sample filter gradient (B, C_out, fx, fy, C) and, if pre_errors is not
 * NULL, the pre-spike errors (B, X*Y*C, k_pre). Replaces compute_weights_gradient_conv and
 * propagate_errors_to_pre_spikes_conv (bats/CudaKernels/Wrappers/Backpropagation/
 * compute_weights_gradient_conv.py:11-32, propagate_errors_to_pre_spikes_conv.py:11-32). */
int bats_conv_backward(const void* events, const int* ev_slot, const int* ev_count, long long ev_cap,
                       const float* weights, int batch, int X, int Y, int C, int fx, int fy, int C_out, int k_pre,
                       const float* post_times, const void* tables, const int* nvalid, int k_post, float tau_s,
                       float tau, float* grad_per_sample, float* pre_errors, cudaStream_t stream);

/* Pooling backward: pre_errors[indices[q]] = errors[q] (zero elsewhere).
 * Replaces the cp.put scatter of PoolingLayer.backward (bats/Layers/PoolingLayer.py:55-66). */
int bats_pool_backward(const float* errors, const int* indices, long long count, float* pre_errors,
                       long long pre_count, cudaStream_t stream);

/* ---- Losses and optimizer ------------------------------------------------------------------- */

/* loss (B) = 1/2 sum (target - count)^2, errors (B, N, K) = target - count broadcast over K. counts are
 * int32 or float32 (count_is_float). Either targets (B, N) or labels (B) with target_true/target_false.
 * Replaces SpikeCountLoss / SpikeCountClassLoss (bats/Losses/SpikeCountLoss.py:17-38,
 * bats/Losses/SpikeCountClassLoss.py:15-33). loss or errors may be NULL. */
int bats_spike_count_loss(const void* counts, int count_is_float, const float* targets, const int* labels,
                          float target_true, float target_false, int batch, int n, int k, float* loss,
                          float* errors, cudaStream_t stream);

/* Softmax cross-entropy of first-spike times with errors in slot 0.
 * Replaces TTFSSoftmaxCrossEntropy (bats/Losses/TTFSSoftmaxCrossEntropy.py:23-56). */
int bats_ttfs_softmax_cross_entropy(const float* spikes, const int* labels, int batch, int n, int k, double tau,
                                    float* loss, float* errors, cudaStream_t stream);

/* Squared error of first-spike times (mode 0 loss, 1 errors, 2 both); targets modified in place (inf -> 1).
 * Replaces SpikeTimeLoss (bats/Losses/SpikeTimeLoss.py:20-47). */
int bats_spike_time_loss(const float* spikes, float* targets, int batch, int n, int k, int mode, float* loss,
                         float* errors, cudaStream_t stream);

/* One Adam step on one tensor: m, v in place; delta written (if not NULL) and/or added to weights (if not
 * NULL), the new weights also written transposed into weights_t (n_pre, ld) if given.
 * bias_correction_i = 1 - beta_i^t. Replaces AdamOptimizer.step + Network.apply_deltas
 * (bats/Optimizers/AdamOptimizer.py:35-55, bats/Network.py:50-54). */
int bats_adam_step(const float* grad, float* m, float* v, long long count, float beta_1, float beta_2, float epsilon,
                   float learning_rate, double bias_correction_1, double bias_correction_2, float* delta,
                   float* weights, float* weights_t, int n_post, int n_pre, int ld, cudaStream_t stream);

/* Device-side Adam bias-correction state for captured steps, 4 doubles: powers[0..1] *= beta_1, beta_2,
 * then powers[2..3] hold (as four floats) the pairs hi + lo ~= 1 / (1 - beta_i^t) the update kernel divides by.
 * Start from {1, 1, 0, 0}; call once per step before bats_adam_step_device. Replaces the host-side
 * `self.__t += 1` and `beta ** t` of AdamOptimizer.step (bats/Optimizers/AdamOptimizer.py:36, 49-50). */
int bats_adam_powers_advance(double* powers, float beta_1, float beta_2, cudaStream_t stream);

/* bats_adam_step with the bias corrections 1 - powers[i] read from device memory and the delta added to
 * the weights (and their transposed copy) in place. Replaces AdamOptimizer.step + Network.apply_deltas. */
int bats_adam_step_device(const float* grad, float* m, float* v, long long count, float beta_1, float beta_2,
                          float epsilon, float learning_rate, const double* powers, float* weights, float* weights_t,
                          int n_post, int n_pre, int ld, cudaStream_t stream);

/* One NAdam step on one tensor: m, v in place, delta written. bias_correction_i = 1 - beta_i^t.
 * Replaces NAdamOptimizer.step (bats/Optimizers/NAdamOptimizer.py:35-58, kernels :6-20). */
int bats_nadam_step(const float* grad, float* m, float* v, long long count, float beta_1, float beta_2, float epsilon,
                    float learning_rate, double bias_correction_1, double bias_correction_2, float* delta,
                    cudaStream_t stream);

/* Synaptic scaling of the per-sample gradient (B, N_post, N_pre), in place: for samples whose silent ratio is
 * >= threshold, gradient[s, i, :] -= factor * |W[i, :]| for every post neuron i with no spike in s.
 * Replaces apply_weights_synaptic_scaling_kernel
 * (bats/CudaKernels/CuFiles/Regularization/apply_weights_synaptic_scaling.cu:2-25). */
int bats_weights_synaptic_scaling(const float* weights, const float* silent_ratios, const int* n_spikes,
                                  float* gradient, int batch, int n_post, int n_pre, float threshold, float factor,
                                  cudaStream_t stream);

/* Label synaptic scaling, in place: gradient[s, l, :] -= factor * |W[l, :]| with l = (int)labels[s], unless
 * n_spikes[l] > 0 (the reference reads the label's count from the first row of n_spikes; kept as is).
 * Labels outside [0, N_post) are skipped. Replaces apply_label_weights_synaptic_scaling_kernel
 * (bats/CudaKernels/CuFiles/Regularization/apply_label_weights_synaptic_scaling.cu:2-20). */
int bats_label_weights_synaptic_scaling(const float* weights, const float* labels, const int* n_spikes,
                                        float* gradient, int batch, int n_post, int n_pre, float factor,
                                        cudaStream_t stream);

/* weights += delta, optionally refreshing the transposed copy. Replaces LIFLayer.add_deltas
 * (bats/Layers/LIFLayer.py:112-113). */
int bats_add_deltas(float* weights, const float* delta, long long count, float* weights_t, int n_pre, int ld,
                    cudaStream_t stream);

/* out (cols, ld) = in (rows, cols)^T. Builds the transposed weights read by the FC kernels. */
int bats_transpose(const float* in, int rows, int cols, float* out, int ld, cudaStream_t stream);

/* One device-to-device copy of `bytes` bytes, enqueued on `stream` (a memcpy node when the stream is being
 * captured): the train steps copy staged transposed weights with it. */
int bats_copy_device(void* dst, const void* src, size_t bytes, cudaStream_t stream);

/* One fully-connected layer of a served network, for bats_serve_fc_batch: shapes, transposed weights
 * (n_pre, ld), constants as for bats_lif_forward_fc (tau = 2 tau_s, c = theta/tau, delta_theta/tau), the
 * forward kernel variant, and the layer's device buffers for `batch` samples: sorted events
 * (n_pre*k_pre records per sample), their slots and counts, and the outputs (n_spikes (B, n_post);
 * a, x, times, post_exp_tau (B, n_post, k_post)). */
typedef struct BatsFcLayer {
    int n_pre, k_pre, n_post, k_post;
    const float* weights_t;
    int ld;
    float tau_s, tau, c, delta_theta_tau, max_simulation;
    int algo;
    void* events;
    int* slots;
    int* ev_count;
    int* n_spikes;
    float* a;
    float* x;
    float* times;
    float* post_exp_tau;
} BatsFcLayer;

/* One inference batch of an FC network, enqueued on `stream` with no host synchronisation: copies the flat
 * event list (h_indices/h_times, total_events entries) and offsets (batch + 1) from pinned host memory,
 * builds the input spike trains (k_in slots per input neuron, overflow counted in d_overflow), runs every
 * layer's sort and forward, and copies the last layer's counts (B, n_post) and times (B, n_post, k_post)
 * and the overflow count back to pinned host memory. No counterpart in the reference (the serving
 * pattern's batch step). */
int bats_serve_fc_batch(const int* h_indices, const float* h_times, const int* h_offsets, int batch, int total_events,
                        int* d_indices, float* d_times, int* d_offsets, int n_inputs, int k_in, float* d_trains,
                        int* d_train_counts, int* d_overflow, const BatsFcLayer* layers, int n_layers,
                        void* sort_workspace, size_t sort_workspace_bytes, int* h_out_counts, float* h_out_times,
                        int* h_overflow, cudaStream_t stream);

/* Batch-mean filter gradient of a conv layer fused with its Adam update, for a train step: no per-sample
 * gradient is formed. The backward kernel of bats_conv_backward (bats_conv_backward_grouped's when the
 * position-bucketed events are given and the layer fits it) runs on clusters that each accumulate `group`
 * samples into one partial filter gradient in the workspace (bats_conv_backward_adam_workspace_bytes); the
 * partials are summed in group order and divided by the batch into `grad` (C_out, fx, fy, C_in), then Adam
 * (bias corrections from `powers`, as bats_adam_step_device) updates m, v and the filters in place. The
 * pre-spike errors (B, X*Y*C, k_pre), when pre_errors is not NULL, use the filters before the update.
 * Replaces compute_weights_gradient_conv + the batch mean + AdamOptimizer.step + add_deltas
 * (bats/CudaKernels/Wrappers/Backpropagation/compute_weights_gradient_conv.py:11-32,
 * experiments/mnist/train_conv.py, bats/Layers/ConvLIFLayer.py:109-137) and propagate_errors_to_pre_spikes_conv
 * (propagate_errors_to_pre_spikes_conv.py:11-32). */
size_t bats_conv_backward_adam_workspace_bytes(int batch, int C, int fx, int fy, int C_out, int group);
int bats_conv_backward_adam(const void* events, const int* ev_slot, const int* ev_count, const void* events_bucketed,
                            const int* bucket_offsets, long long ev_cap, float* weights, int batch, int X, int Y, int C,
                            int fx, int fy, int C_out, int k_pre, const float* post_times, const void* tables,
                            const int* nvalid, int k_post, float tau_s, float tau, float* pre_errors, int group,
                            float* grad, float* m, float* v, float beta_1, float beta_2, float epsilon,
                            float learning_rate, const double* powers, void* workspace, size_t workspace_bytes,
                            cudaStream_t stream);

/* ---- Training step ---------------------------------------------------------------------------- */

/* Forward kernel choices of bats_fc_train_step beyond BATS_FWD_TILE/LANES/TILE64: the persistent work-queue
 * forward (bats_lif_forward_fc_queue) with 128- or 64-neuron tiles. */
#define BATS_FWD_QUEUE 4
#define BATS_FWD_QUEUE64 5

/* One trainable fully-connected layer of bats_fc_train_step: the forward part as for serving (`fwd`: shapes,
 * transposed weights, which Adam keeps in sync, constants, forward variant, events, slots, counts and outputs
 * for `batch` samples), and the backward and optimizer state, all device buffers owned by the caller:
 *   weights (n_post, n_pre), adam_m, adam_v (same shape), grad (same shape: the last step's batch-mean gradient);
 *   events_bucketed (batch, n_pre*k_pre records) and bucket_offsets (batch, ceil(n_pre/BATS_GRAD_BUCKET_WIDTH)
 *     + 1): the events grouped by pre buckets of BATS_GRAD_BUCKET_WIDTH neurons for the gradient (both NULL: the
 *     gradient reads the time-sorted events);
 *   tables (batch, n_post, k_post + 1, 2 floats), nvalid (batch, n_post): the backward's suffix tables;
 *   cursor_heads (bats_cursor_heads_bytes(batch, n_post) bytes, 16-byte aligned; NULL: not used): written by
 *     the counted prep (k_post <= 32) and read by the gradient;
 *   f1, f2 (batch, n_post, k_post): factors, needed only when k_post > 32 (else may be NULL);
 *   pre_errors (batch, n_pre, k_pre): errors of the layer's input spikes, filled for every layer but the first
 *     (NULL there); they are the incoming errors of the layer below, whose reset-error step changes them;
 *   grad_group: samples per partial gradient (>= 2). */
typedef struct BatsFcTrainLayer {
    BatsFcLayer fwd;
    float* weights;
    float* adam_m;
    float* adam_v;
    float* grad;
    void* events_bucketed;
    int* bucket_offsets;
    void* tables;
    int* nvalid;
    void* cursor_heads;
    float* f1;
    float* f2;
    float* pre_errors;
    int grad_group;
} BatsFcTrainLayer;

/* Workspace of bats_fc_train_step: the sample order of the hidden layers' sorts (batch ints, rounded up to 256
 * bytes), then the largest of the sort, work-queue, gradient and pre-error workspaces of its layers. */
size_t bats_fc_train_step_workspace_bytes(int batch, const BatsFcTrainLayer* layers, int n_layers);

/* One training step of a fully-connected network on device-resident inputs, enqueued on `stream` with no host
 * synchronisation and no allocation, so that it can be called from any language through this ABI (and
 * captured in a CUDA graph): Adam's bias-correction powers advanced on the device (`powers`: 4 doubles,
 * {1, 1, 0, 0} before the first step); per layer the event sort (bucketed copy included; on batches wider than
 * two CTAs per SM the hidden layers' sorts take the samples longest first, bats_sample_order of the previous
 * layer's input event counts) and the LIF forward (hidden layers unpadded); the spike-count class loss (targets target_true / target_false, per-sample loss
 * (batch) and output-layer errors (batch, n_out, k_out)); then per layer from the last one the reset errors,
 * factors and suffix tables, the pre-spike errors (every layer but the first, with the weights before this
 * step's update) and the batch-mean gradient fused with Adam (weights, their transposed copy, m, v, grad).
 * in_times (batch, layers[0].fwd.n_pre, layers[0].fwd.k_pre), labels (batch) int32.
 * Replaces the reference's training iteration (experiments/mnist/train_spike_count.py:143-177: Network.forward,
 * SpikeCountClassLoss.compute_loss_and_errors, Network.backward, the batch mean, AdamOptimizer.step,
 * Network.apply_deltas; bats/Network.py:32-54). Results are those of the same sequence of the entry points it
 * calls. */
int bats_fc_train_step(const float* in_times, const int* labels, int batch, BatsFcTrainLayer* layers, int n_layers,
                       float target_true, float target_false, float beta_1, float beta_2, float epsilon,
                       float learning_rate, double* powers, float* loss, float* errors, void* workspace,
                       size_t workspace_bytes, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BATS_GB300_H */
