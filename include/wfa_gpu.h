/*
 * wfa_gpu.h — C ABI of the GB300 BiWFA aligner (libbiwfa_gb300.so).
 *
 * Two surfaces:
 *   1. A source-compatible subset of WFA2-lib v2.3's aligner API, so code written
 *      against WFA2-lib's BiWFA (gap-affine, wavefront_memory_ultralow) compiles and
 *      runs unchanged. Each declaration cites the WFA2-lib declaration it replaces
 *      (paths relative to WFA2-lib/). Scores and CIGARs are bit-identical to WFA2-lib's
 *      ultralow-memory BiWFA on the same inputs.
 *   2. A batch API (wfg_*) that carries the GPU throughput path: many pairs per call,
 *      one persistent work-stealing kernel, CIGARs returned as SAM-style uint32 runs.
 *
 * Supported configuration: distance_metric = gap_affine, memory_mode =
 * wavefront_memory_ultralow, heuristic = wf_heuristic_none, end-to-end form,
 * match <= 0 (match < 0 via the same penalty transform WFA2-lib applies).
 * Anything else is refused with WF_STATUS_UNSUPPORTED instead of WFA2-lib's exit(1).
 * Input bytes must not contain WFA2-lib's sentinel characters '!' (in the text) or
 * '?' (in the pattern); WFA2-lib's results are undefined there.
 */
#ifndef WFA_GPU_H_
#define WFA_GPU_H_

#include <stdbool.h>
#include <stdint.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
/* wavefront/wfa.h:46-55 */
#define WF_STATUS_ALG_COMPLETED            0
#define WF_STATUS_ALG_PARTIAL              1
#define WF_STATUS_MAX_STEPS_REACHED     -100
#define WF_STATUS_OOM                   -200
#define WF_STATUS_UNATTAINABLE          -300
#define WF_STATUS_OK                      -1
#define WF_STATUS_END_REACHED             -2
#define WF_STATUS_END_UNREACHABLE         -3
/* Added here (no WFA2-lib counterpart): refused configuration, and CUDA errors. */
#define WF_STATUS_UNSUPPORTED           -400
#define WF_STATUS_DEVICE_ERROR          -500

/* ------------------------------------------------------------------ attributes */
/* wavefront/wavefront_penalties.h:42-48 */
typedef enum {
  indel = 0, edit = 1, gap_linear = 2, gap_affine = 3, gap_affine_2p = 4
} distance_metric_t;
/* wavefront/wavefront_attributes.h:49-52 */
typedef enum { compute_score, compute_alignment } alignment_scope_t;
/* wavefront/wavefront_attributes.h:54-58 */
typedef enum { alignment_end2end, alignment_endsfree } alignment_span_t;
/* wavefront/wavefront_attributes.h:59-69 */
typedef struct {
  alignment_span_t span;
  bool extension;
  int pattern_begin_free;
  int pattern_end_free;
  int text_begin_free;
  int text_end_free;
} alignment_form_t;
/* alignment/linear_penalties.h */
typedef struct { int match; int mismatch; int indel; } linear_penalties_t;
/* alignment/affine_penalties.h:38-43 */
typedef struct { int match; int mismatch; int gap_opening; int gap_extension; } affine_penalties_t;
/* alignment/affine2p_penalties.h */
typedef struct {
  int match; int mismatch; int gap_opening1; int gap_extension1; int gap_opening2; int gap_extension2;
} affine2p_penalties_t;
/* wavefront/wavefront_heuristic.h:41-49 */
typedef enum {
  wf_heuristic_none            = 0x0000000000000000ul,
  wf_heuristic_banded_static   = 0x0000000000000001ul,
  wf_heuristic_banded_adaptive = 0x0000000000000002ul,
  wf_heuristic_wfadaptive      = 0x0000000000000004ul,
  wf_heuristic_xdrop           = 0x0000000000000010ul,
  wf_heuristic_zdrop           = 0x0000000000000020ul,
  wf_heuristic_wfmash          = 0x0000000000000040ul,
} wf_heuristic_strategy;
/* wavefront/wavefront_heuristic.h:50-69 */
typedef struct {
  wf_heuristic_strategy strategy;
  int steps_between_cutoffs;
  int min_k; int max_k;
  int min_wavefront_length; int max_distance_threshold;
  int xdrop; int zdrop;
  int steps_wait; int max_sw_score; int max_wf_score; int max_sw_score_offset; int max_sw_score_k;
} wavefront_heuristic_t;
/* wavefront/wavefront_attributes.h:104-109 */
typedef enum {
  wavefront_memory_high = 0, wavefront_memory_med = 1, wavefront_memory_low = 2, wavefront_memory_ultralow = 3,
} wavefront_memory_t;
/* wavefront/wavefront_plot.h (attributes part) */
typedef struct { bool enabled; int resolution_points; int align_level; } wavefront_plot_attr_t;
/* system/profiler_counter.h:42-51 and system/profiler_timer.h:59-65: carried so that the
 * attribute structure below has WFA2-lib's size and field offsets (the timer is never read). */
typedef struct {
  uint64_t total; uint64_t samples; uint64_t min; uint64_t max;
  double m_oldM; double m_newM; double m_oldS; double m_newS;
} profiler_counter_t;
typedef struct {
  struct timespec begin_timer;
  profiler_counter_t time_ns;
  uint64_t accumulated;
} profiler_timer_t;
/* wavefront/wavefront_attributes.h:74-99 */
typedef struct {
  int max_alignment_steps;
  int probe_interval_global;
  int probe_interval_compact;
  uint64_t max_partial_compacts;
  uint64_t max_memory_compact;
  uint64_t max_memory_resident;
  uint64_t max_memory_abort;
  int verbose;
  bool check_alignment_correct;
  profiler_timer_t timer;
  int max_num_threads;
  int min_offsets_per_thread;
} alignment_system_t;
/* wavefront/wavefront_attributes.h:114-133 (mm_allocator is accepted and ignored) */
typedef struct {
  distance_metric_t distance_metric;
  alignment_scope_t alignment_scope;
  alignment_form_t alignment_form;
  linear_penalties_t linear_penalties;
  affine_penalties_t affine_penalties;
  affine2p_penalties_t affine2p_penalties;
  wavefront_heuristic_t heuristic;
  wavefront_memory_t memory_mode;
  void* mm_allocator;
  wavefront_plot_attr_t plot;
  alignment_system_t system;
} wavefront_aligner_attr_t;

/* wavefront/wavefront_attributes.h:138 (defaults as WFA2-lib's: memory_high + wfadaptive;
 * callers of the BiWFA path set memory_mode and heuristic explicitly, as with WFA2-lib). */
extern wavefront_aligner_attr_t wavefront_aligner_attr_default;

/* ------------------------------------------------------------------ results */
/* alignment/cigar.h:44-58. operations[begin_offset .. end_offset) holds 'M' (match),
 * 'X' (mismatch), 'I' (insertion), 'D' (deletion). score is the alignment score
 * (cigar_score_gap_affine of the operations; WFA2-lib leaves INT32_MIN there when
 * the whole alignment took its unidirectional fallback, this library always fills it). */
typedef struct {
  char* operations;
  int max_operations;
  int begin_offset;
  int end_offset;
  int score;
  int end_v;
  int end_h;
  bool has_misms;
  uint32_t* cigar_buffer;
  int cigar_length;
} cigar_t;

struct wavefront_aligner_t;
/* wavefront/wfa.h:61-70 (the two function pointers are never set here) */
typedef struct {
  int status;
  int score;
  bool dropped;
  int num_null_steps;
  uint64_t memory_used;
  void (*wf_align_compute)(struct wavefront_aligner_t* const, const int);
  int (*wf_align_extend)(struct wavefront_aligner_t* const, const int);
} wavefront_align_status_t;

/* wavefront/wfa.h:82-112, byte for byte on LP64 (x86-64, AArch64): the fields WFA2-lib callers
 * read (align_status, alignment_scope, alignment_form, heuristic, memory_mode, cigar, system)
 * sit at WFA2-lib's offsets, so code compiled against WFA2-lib's headers reads them here too.
 * WFA2-lib's internal members that callers do not read are opaque byte regions of their size;
 * the bialigner slot holds this library's private state. */
typedef struct wavefront_aligner_t {
  int align_mode;                     /* wavefront_align_mode_t: 1 (BiWFA) for ultralow memory */
  char* align_mode_tag;
  wavefront_align_status_t align_status;
  uint64_t sequences_[13];            /* wavefront_sequences_t (104 bytes) */
  alignment_scope_t alignment_scope;
  alignment_form_t alignment_form;
  int32_t penalties_[21];             /* wavefront_penalties_t (84 bytes) */
  wavefront_heuristic_t heuristic;
  wavefront_memory_t memory_mode;
  uint64_t wf_components_[12];        /* wavefront_components_t (96 bytes) */
  int component_begin;                /* affine2p_matrix_type: 0 (M) */
  int component_end;
  struct { int score; int k; int32_t offset; } alignment_end_pos;  /* wavefront_pos_t */
  void* bialigner;                    /* private: this library's aligner state */
  cigar_t* cigar;
  bool mm_allocator_own;
  void* mm_allocator;
  void* wavefront_slab;
  void* plot;
  alignment_system_t system;
} wavefront_aligner_t;

/* ------------------------------------------------------------------ WFA2-lib subset */
/* wavefront/wfa.h:125-126; wavefront_aligner.c:421-463. NULL attributes -> defaults.
 * Returns NULL when no CUDA device is usable. An unsupported configuration still
 * returns an aligner whose wavefront_align() reports WF_STATUS_UNSUPPORTED. */
wavefront_aligner_t* wavefront_aligner_new(wavefront_aligner_attr_t* attributes);
/* wavefront/wfa.h:129-130; wavefront_aligner.c:476-503 */
void wavefront_aligner_delete(wavefront_aligner_t* const wf_aligner);
/* wavefront/wfa.h:200-205; wavefront_align.c:578-607. One pair, computed on the GPU.
 * The result stays in wf_aligner->cigar until the next call. */
int wavefront_align(wavefront_aligner_t* const wf_aligner,
                    const char* const pattern, const int pattern_length,
                    const char* const text, const int text_length);
/* wavefront/wfa.h:57-58; wavefront_aligner.c:70-97 */
char* wavefront_align_strerror(const int error_code);
char* wavefront_align_strerror_short(const int error_code);
/* wavefront/wfa.h:136-138 (end-to-end is the only supported span) */
void wavefront_aligner_set_alignment_end_to_end(wavefront_aligner_t* const wf_aligner);
/* wavefront/wfa.h:148-149 */
void wavefront_aligner_set_heuristic_none(wavefront_aligner_t* const wf_aligner);
/* wavefront/wfa.h:176-178 */
void wavefront_aligner_set_max_alignment_steps(wavefront_aligner_t* const wf_aligner,
                                               const int max_alignment_steps);
/* alignment/cigar.h: cigar_sprint (cigar.c:706-740) */
int cigar_sprint(char* const buffer, const cigar_t* const cigar, const bool print_matches);
/* alignment/cigar.h: cigar_score_gap_affine (cigar.c:277-303) */
int cigar_score_gap_affine(const cigar_t* const cigar, const affine_penalties_t* const penalties);
/* alignment/cigar.h: cigar_score_edit (cigar.c:244-259), cigar_score_gap_linear (:260-276),
 * cigar_score_gap_affine2p (:304-342) */
int cigar_score_edit(const cigar_t* const cigar);
int cigar_score_gap_linear(const cigar_t* const cigar, const linear_penalties_t* const penalties);
int cigar_score_gap_affine2p(const cigar_t* const cigar, const affine2p_penalties_t* const penalties);
/* alignment/cigar.h: cigar_get_CIGAR (cigar.c:224-235); SAM BAM op codes, '='/'X' split
 * when show_mismatches. The buffer belongs to the cigar. */
void cigar_get_CIGAR(cigar_t* const cigar, const bool show_mismatches,
                     uint32_t** const cigar_buffer, int* const cigar_length);

/* Batch extension of the WFA2-lib surface (no WFA2-lib counterpart; WFA2-lib callers
 * loop over wavefront_align, align_benchmark.c:546-551). Aligns num_pairs pairs with
 * the aligner's settings in one GPU pass. scores/statuses (host arrays of num_pairs)
 * receive per-pair results; CIGARs are read back with wavefront_batch_cigar. */
int wavefront_align_batch(wavefront_aligner_t* const wf_aligner, const int num_pairs,
                          const char* const* patterns, const int* pattern_lengths,
                          const char* const* texts, const int* text_lengths,
                          int* scores, int* statuses);
/* Runs of pair i of the last wavefront_align_batch: *runs points to *num_runs SAM-style
 * uint32 ops (len<<4 | op, op in {1:I, 2:D, 7:=, 8:X}). Valid until the next call. */
int wavefront_batch_cigar(wavefront_aligner_t* const wf_aligner, const int pair,
                          const uint32_t** runs, int* num_runs);

/* ------------------------------------------------------------------ GB300 batch API */
/* No WFA2-lib counterpart: the throughput path. A context owns one CUDA stream on one
 * device and grow-only device buffers; it is not thread-safe (one per host thread,
 * as WFA2-lib aligners). */
typedef struct wfg_context wfg_context_t;

/* Distances of wfg_config_t.metric: WFA2-lib's gap_affine (default), edit, indel, gap_linear
 * and gap_affine_2p (wavefront/wavefront_penalties.c:39-173). Edit and indel ignore the
 * penalties; gap-linear takes its indel penalty from gap_opening (match <= 0, mismatch > 0,
 * indel > 0); two-piece gap-affine reads (gap_opening, gap_extension) as the first piece and
 * (gap_opening2, gap_extension2) as the second. The score scope (max(x, o+e[, o2+e2]) + 1
 * after the match < 0 transform) may be at most 64; larger penalties are refused with
 * WF_STATUS_UNSUPPORTED. */
typedef enum {
  WFG_METRIC_GAP_AFFINE = 0, WFG_METRIC_EDIT = 1, WFG_METRIC_INDEL = 2, WFG_METRIC_GAP_LINEAR = 3,
  WFG_METRIC_GAP_AFFINE_2P = 4
} wfg_metric_t;

typedef struct {
  int match, mismatch, gap_opening, gap_extension; /* caller's penalties (match <= 0) */
  int score_only;                                  /* 1: score only (compute_score scope) */
  int max_alignment_steps;                         /* <= 0: unlimited (WFA2 default INT_MAX) */
  int metric;                                      /* wfg_metric_t; scores of edit/indel are distances */
  int gap_opening2, gap_extension2;                /* second gap piece (WFG_METRIC_GAP_AFFINE_2P) */
} wfg_config_t;

/* Scheduling policy of wfg_run. */
typedef enum {
  /* pairs sorted by length (descending) and aligned in consecutive launches of as many
   * pairs as the GPU holds at once (one warp per pair); each launch ends with its slowest
   * pair (the plain batched GPU path) */
  WFG_SCHED_PLAIN = 0,
  /* pairs binned and ordered by the score predictor's output, one persistent work-stealing
   * launch per bin, scratch sized from the prediction */
  WFG_SCHED_LEARNED = 1,
  WFG_SCHED_GIVEN = 2,    /* the caller's order (wfg_set_order), one persistent launch */
  /* pairs sorted by length (descending), one persistent launch; pairs with plen + tlen above
   * 32,768 take a multi-warp launch (the retry passes' shape) with rings as wide as the
   * batch's longest pair, concurrent with the single-warp launch of the rest */
  WFG_SCHED_SORTED = 3,
} wfg_sched_t;

typedef struct {
  double kernel_ms;       /* device time of the alignment kernels of the last wfg_run */
  double pack_ms;         /* device time of the packing kernel */
  double total_ms;        /* device time of the whole wfg_run (events on the context's stream) */
  int launches;           /* kernels this library launched in the last wfg_run (packing, alignment
                             passes, and the learned schedule's feature, MLP and binning kernels) */
  int retried_pairs;      /* pairs rerun with a larger arena after a scratch overflow */
  int num_warps;          /* resident warps of the main launch */
  int ring_w;             /* ring width (diagonals) of the main launch */
  int64_t arena_bytes;    /* per-warp arena of the main launch */
  int64_t total_runs;     /* CIGAR runs produced */
  int64_t h2d_bytes, d2h_bytes; /* bytes copied by the last upload / fetch */
  int used_graph;         /* 1 when the last wfg_run's device work ran as one CUDA graph */
  double upload_host_ms;  /* host time of the last wfg_upload before its copies (validation, descriptors) */
  double upload_copy_ms;  /* device time of the last wfg_upload's host-to-device copies */
  int pipeline_chunks;    /* chunks of the last wfg_align_host whose input copy overlapped the
                             alignment (0: uploaded first) */
} wfg_stats_t;

wfg_context_t* wfg_context_create(int device);
void wfg_context_destroy(wfg_context_t* ctx);
/* Last error message of the context (empty string when none). */
const char* wfg_last_error(wfg_context_t* ctx);

/* Upload a batch from host memory: pattern i = seq[p_off[i] .. p_off[i]+plen[i]),
 * text i = seq[t_off[i] .. t_off[i]+tlen[i]) of one host byte buffer of seq_len bytes.
 * Copies to the device and leaves the batch resident until the next upload. */
int wfg_upload(wfg_context_t* ctx, int num_pairs, const char* seq, int64_t seq_len,
               const int64_t* p_off, const int* plen, const int64_t* t_off, const int* tlen);
/* Processing order for WFG_SCHED_GIVEN (num_pairs indices, a permutation). */
int wfg_set_order(wfg_context_t* ctx, const int* order);
/* Predicted scores for WFG_SCHED_LEARNED (host array of num_pairs, WFA penalty units,
 * e.g. from wfg_predict_scores). */
int wfg_set_predictions(wfg_context_t* ctx, const float* predicted_scores);
/* Align the resident batch on the device (pack + align); results stay on the device. */
int wfg_run(wfg_context_t* ctx, const wfg_config_t* cfg, wfg_sched_t sched);
/* Copy results of the last wfg_run to host arrays (any may be NULL). runs receives the
 * dense run buffer (runs_cap entries at most); run_off/run_len index into it. */
int wfg_fetch(wfg_context_t* ctx, int* scores, int* statuses, int64_t* run_off, int* run_len,
              uint32_t* runs, int64_t runs_cap, int64_t* total_runs);
/* Upload + run + fetch in one call (the end-to-end path). Batches of 131,072 pairs or more on
 * WFG_SCHED_SORTED, or on WFG_SCHED_LEARNED with an attached model and a single-warp policy,
 * overlap the input copy with the alignment: the first 1/8 of the pairs (by index) is packed,
 * predicted, ordered and run (first pass) as soon as its bytes are on the device, while the
 * rest is still being copied; the rest then runs as one launch as the head's warps retire, and
 * the retry passes once at the end. This pays when the pairs' bytes lie in the buffer in pair
 * order. Results are the same as upload + run + fetch. */
int wfg_align_host(wfg_context_t* ctx, const wfg_config_t* cfg, wfg_sched_t sched,
                   int num_pairs, const char* seq, int64_t seq_len,
                   const int64_t* p_off, const int* plen, const int64_t* t_off, const int* tlen,
                   int* scores, int* statuses, int64_t* run_off, int* run_len,
                   uint32_t* runs, int64_t runs_cap, int64_t* total_runs);
int wfg_get_stats(wfg_context_t* ctx, wfg_stats_t* stats);
/* Whether wfg_align_host may overlap its input copy with the alignment (default 1). */
int wfg_set_pipeline(wfg_context_t* ctx, int enable);
/* Caps on the first pass's per-warp arena (0 = automatic): ring width in diagonals and
 * leaf store in int32 words. Pairs that do not fit overflow into the retry passes, whose
 * arenas are sized from the batch's longest pair; results never change. */
int wfg_set_arena_limits(wfg_context_t* ctx, int ring_w, int leaf_words);
/* Execution shape of the first pass for WFG_SCHED_PLAIN / WFG_SCHED_GIVEN: group_warps
 * warps cooperate on one pair (1, 4 or 8); ring_in_smem keeps the wavefront rings in
 * shared memory (group_warps > 1; rings of 1024 diagonals, wider pairs overflow into the
 * retry passes). Results never depend on the shape. Default 1, 0. */
int wfg_set_exec_shape(wfg_context_t* ctx, int group_warps, int ring_in_smem);
/* Run wfg_run's device work (order copy, counter reset, packing, every pass, counter
 * read-back) as one CUDA graph: captured on each call and applied to the context's
 * instantiated graph with cudaGraphExecUpdate when the topology is unchanged. enable = 0
 * issues the same work directly on the streams. Default 1. */
int wfg_set_graph(wfg_context_t* ctx, int enable);
/* Warps per pair (1, 4 or 8, HBM rings) of the two retry passes, which realign the pairs that
 * overflowed the first pass's scratch: those are the widest pairs. Default 8. */
int wfg_set_retry_shape(wfg_context_t* ctx, int group_warps);
/* Policy of WFG_SCHED_LEARNED: the pairs with the highest predicted scores, from
 * wide_threshold up and at most one resident wave of the shape, run with wide_warps warps per
 * pair (rings in shared memory when wide_smem and they fit), concurrently with the
 * single-warp launch for the rest (wide_threshold = FLT_MAX: no multi-warp launch); ring
 * widths are ring_margin * the launch's largest predicted score / gap_extension + 64. */
int wfg_set_learned_policy(wfg_context_t* ctx, float wide_threshold, int wide_warps, int wide_smem,
                           float ring_margin);
/* Autotuner for WFG_SCHED_LEARNED (requires an attached model): runs the resident batch
 * with each candidate policy (wide threshold x warps per pair x shared-memory rings, plus
 * "no wide launch"), times the device work with CUDA events, keeps the fastest policy on
 * the context and returns its time (ms) and choice. Results never depend on the policy. */
int wfg_autotune_learned_policy(wfg_context_t* ctx, const wfg_config_t* cfg, float* best_ms,
                                float* best_threshold, int* best_warps, int* best_smem);
/* Write ~bytes of scratch to evict the L2 (between timed runs). */
int wfg_flush_l2(wfg_context_t* ctx, int64_t bytes);
/* Synchronize the context's stream. */
int wfg_synchronize(wfg_context_t* ctx);
/* Page-locked host memory for inputs/outputs (copies to and from it run at full link
 * speed). NULL on failure. */
void* wfg_host_alloc(int64_t bytes);
void wfg_host_free(void* ptr);

/* ------------------------------------------------------------------ learned scheduling */
/* No WFA2-lib counterpart. A small MLP (32 sketch features -> 64 -> 64 -> 1, ReLU, bf16
 * weights, fp32 accumulation) predicts each pair's alignment score from its lengths and
 * 4-mer count differences. WFG_SCHED_LEARNED runs it on the device inside wfg_run to order
 * and bin pairs and size the first pass's scratch; a mispredicted pair overflows into a
 * larger pass, so results never depend on the model. Training runs on the GPU with the
 * library's own forward/backward kernels. */
typedef struct wfg_model wfg_model_t;
#define WFG_MODEL_FEATURES 32
/* Number of fp32 parameters (W1 32x64, b1, W2 64x64, b2, w3, b3). */
int wfg_model_param_count(void);
/* A model on ctx's device, initialised from seed (He-uniform weights, zero biases). */
wfg_model_t* wfg_model_create(wfg_context_t* ctx, uint64_t seed);
void wfg_model_destroy(wfg_model_t* model);
int wfg_model_get_params(wfg_model_t* model, float* params);
int wfg_model_set_params(wfg_model_t* model, const float* params);
/* Features of the resident batch (device); optionally copied to host as bf16 bit patterns
 * (num_pairs x 32 uint16). */
int wfg_features(wfg_context_t* ctx, uint16_t* host_features);
/* Train on the resident batch: targets are alignment scores (host, num_pairs; the model
 * regresses log(1 + |score|)). Minibatches of batch_rows, Adam with learning rate lr,
 * rows shuffled per epoch from seed. epoch_loss (nullable, epochs entries) receives the
 * mean squared error of each epoch. */
int wfg_model_train(wfg_model_t* model, wfg_context_t* ctx, const int* target_scores, int epochs,
                    int batch_rows, float lr, uint64_t seed, float* epoch_loss);
/* Gradient of the mean squared error over all resident pairs for log-targets (host,
 * num_pairs) at the current parameters (for checks against a float64 oracle). */
int wfg_model_gradient(wfg_model_t* model, wfg_context_t* ctx, const float* log_targets,
                       float* grad, float* loss);
/* Predicted scores of the resident batch (kept on the device for WFG_SCHED_LEARNED;
 * optionally copied to host_pred). */
int wfg_model_predict(wfg_model_t* model, wfg_context_t* ctx, float* host_pred);
/* Attach a model to a context: WFG_SCHED_LEARNED then predicts on the device in wfg_run.
 * The context keeps the pointer: attach NULL before destroying the model. */
int wfg_set_model(wfg_context_t* ctx, wfg_model_t* model);

/* Aligning without allocating (no WFA2-lib counterpart; there is no reference interface
 * this replaces). For callers that may not allocate device memory themselves or let a
 * library do it — code inside a framework that owns every device allocation, or code
 * that must not allocate while latency-critical work runs. The caller passes device
 * pointers to its inputs (sequence bytes, per-pair offsets and lengths) and to its
 * outputs (scores, statuses, run offsets and lengths, and a runs buffer of runs_cap
 * entries) and a cudaStream_t (or NULL); everything else lives in a fixed 30.7 MiB
 * __device__ array inside the library, held by every GPU that loads it until exit.
 * No cudaMalloc, cudaFree or other allocating call is made.
 *   - The first call on a device looks up that array's address (with that device
 *     current); make that first call before any stream capture.
 *   - Calls share the array: calls that overlap on the GPU race. Serialize them.
 *   - Limits per call: at most WFG_NOALLOC_MAX_PAIRS pairs (else WF_STATUS_UNSUPPORTED
 *     is returned and nothing runs); pairs with plen + tlen above
 *     WFG_NOALLOC_MAX_PAIR_LEN get status WF_STATUS_UNSUPPORTED; penalties whose score
 *     scope max(o+e, x)+1 exceeds 16 are refused; a pair that outgrows the fixed arena
 *     gets WF_STATUS_OOM: the arenas are sized like wfg_run's first pass, so a pair that
 *     wfg_run finishes only in a retry pass (a unidirectional leaf of more than 131,072
 *     offsets, e.g. a wide end-reached recovery leaf) comes back WF_STATUS_OOM here, never
 *     with a different score or CIGAR.
 *   - Throughput: one launch of 16 resident warps (one pair per warp at a time), so a call
 *     suits modest batches; it is far below wfg_run's occupancy on large ones.
 * Returns WF_STATUS_ALG_COMPLETED once the work is enqueued on the stream; per-pair
 * results (the same as wfg_run's, up to the OOM case above) are valid after the stream
 * completes. */
#define WFG_NOALLOC_MAX_PAIRS 4096
#define WFG_NOALLOC_MAX_PAIR_LEN 1024
int wfg_align_noalloc(const wfg_config_t* cfg, int num_pairs, const char* d_seq,
                      const int64_t* d_p_off, const int* d_plen, const int64_t* d_t_off, const int* d_tlen,
                      int* d_scores, int* d_status, int64_t* d_run_off, int* d_run_len,
                      uint32_t* d_runs, int64_t runs_cap, void* stream);

/* Seeded synthetic pair generator (host; deterministic on every platform).
 * workload: 1 = 1 kbp / 5 % (sub/ins/del 1/3 each, single-base indels),
 *           2 = 150 bp / 2 %, 3 = uneven: log-uniform 100..10000 bp, 1..10 % error,
 *           geometric indel length mean 2, 4 = long noisy: 50..100 kbp, 12 % error,
 *           50/25/25 sub/ins/del, geometric indel length mean 3, 5 = equal mixture of 1..3.
 * Two-phase: call with seq == NULL to get *seq_len_out (bytes needed), then again. */
int wfg_generate(int workload, int num_pairs, uint64_t seed, char* seq, int64_t* seq_len_out,
                 int64_t* p_off, int* plen, int64_t* t_off, int* tlen);

#ifdef __cplusplus
}
#endif
#endif /* WFA_GPU_H_ */
