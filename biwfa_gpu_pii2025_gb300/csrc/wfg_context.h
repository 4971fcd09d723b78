// Private host-side definitions shared by the runtime translation units (not installed).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/wfa_gpu.h"
#include "wfg_internal.h"

namespace wfg {

template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;  // elements
  cudaError_t reserve(size_t n) {
    if (n <= cap && ptr != nullptr) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc((void**)&ptr, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

template <typename T>
struct PinBuf {
  T* ptr = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t n) {
    if (n <= cap && ptr != nullptr) return cudaSuccess;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n, 1);
    cudaError_t e = cudaMallocHost((void**)&ptr, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

constexpr int kNumPasses = 3;
constexpr uint32_t kPlainRingCap = 4096;
constexpr int kDirectWideSum = 32768;         // sorted schedule: plen + tlen above this takes the multi-warp launch
constexpr int kSmemRingW = 1024;              // widest ring of the shared-memory ring shape
constexpr int64_t kSmemRingBytes = 200 << 10;  // dynamic shared memory budget for both rings
constexpr int kCountersPerPass = 4;  // [queue head, retry count, -, -]
constexpr int kOutHeadIndex = kNumPasses * kCountersPerPass;
constexpr int kNumCounters = kOutHeadIndex + 4;

// Kernel launchers (biwfa_kernel.cu, mlp_kernel.cu).
cudaError_t launch_biwfa(const KernelParams& p, int grid, cudaStream_t stream);
cudaError_t biwfa_occupancy(int* blocks_per_sm);
cudaError_t biwfa_occupancy_shape(int group_warps, int ring_in_smem, size_t dyn_smem, int* blocks_per_sm,
                                  int kind);
int biwfa_kernel_kind(int metric, int scope);
int biwfa_warps_per_block();
int biwfa_groups_per_block(int group_warps, int ring_in_smem);
cudaError_t launch_pack(int n, const uint8_t* ascii, PairDesc* pairs, uint32_t* words, int num_sms,
                        cudaStream_t stream);
int mlp_param_count();
cudaError_t launch_kmer_features(int n, const uint8_t* ascii, const PairDesc* pairs, void* feats_bf16, int num_sms,
                                 cudaStream_t stream);
cudaError_t launch_mlp_forward(int n, const void* feats_bf16, const float* master, const void* w1t, const void* w2t,
                               float* y_out, float* score_out, int num_sms, cudaStream_t stream);
cudaError_t launch_mlp_train_step(const void* feats_bf16, const float* target, const int* rows_idx, int rows,
                                  const float* master, const void* w1t, const void* w2t, float* grad, float* loss_sum,
                                  int num_sms, cudaStream_t stream);
cudaError_t launch_mlp_adam(float* master, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                            float eps, const int* step, void* w1t, void* w2t, cudaStream_t stream);
int sched_bin_words();
cudaError_t launch_bin_order(int n, const float* pred, float wide_threshold, int wide_cap, int* work, int* stats,
                             int* order, int num_sms, cudaStream_t stream, int base = 0);
cudaError_t launch_mlp_sync_bf16(const float* master, void* w1t, void* w2t, cudaStream_t stream);

}  // namespace wfg

struct wfg_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // batch
  int n = 0;
  int64_t seq_len = 0;
  int max_plen = 0, max_tlen = 0, max_sum = 0;
  std::vector<int> h_plen, h_tlen;
  std::vector<wfg::PairDesc> h_pairs;
  std::vector<int> h_order;
  std::vector<float> h_pred;
  bool have_order = false, have_pred = false;
  int64_t total_words = 0;
  int64_t out_cap = 0;
  wfg::DevBuf<uint8_t> d_seq;
  wfg::DevBuf<wfg::PairDesc> d_pairs;
  wfg::DevBuf<uint32_t> d_words;
  wfg::DevBuf<int> d_order;
  wfg::DevBuf<int> d_retry;  // kNumPasses-1 lists of n
  wfg::DevBuf<int> d_scores, d_status, d_runlen;
  wfg::DevBuf<int64_t> d_runoff;
  wfg::DevBuf<uint32_t> d_runs;
  wfg::DevBuf<unsigned long long> d_counters;
  wfg::DevBuf<unsigned long long> d_batch_heads;  // work-queue cursors of the plain path's launches
  wfg::DevBuf<uint8_t> d_arena;
  wfg::DevBuf<uint8_t> d_flush;
  wfg::PinBuf<unsigned long long> h_counters;
  wfg::PinBuf<wfg::PairDesc> h_pairs_pinned;
  cudaEvent_t ev[8] = {};
  wfg_stats_t stats{};
  bool ran = false;
  int last_score_only = 0;
  int limit_ring_w = 0, limit_leaf_words = 0;
  // learned scheduling
  wfg::DevBuf<uint16_t> d_feats;   // num_pairs x 32 bf16
  wfg::DevBuf<float> d_pred;       // predicted scores
  wfg::DevBuf<int> d_bin_work;     // device binning scratch (histogram, cursors, stats)
  wfg::PinBuf<int> h_bin_stats;    // bin sizes and maxima read back by the learned schedule
  bool feats_valid = false;
  bool pred_valid = false;
  wfg_model* model = nullptr;
  // execution shape of the plain/given first pass (tests and the autotuner)
  int force_gw = 1, force_smem = 0;
  // learned-schedule policy (wfg_set_learned_policy)
  struct {
    float wide_threshold = 1200.f;  // predicted score from which a pair may take the wide shape
                                    // (the heaviest ones, at most one resident wave; FLT_MAX: none)
    int wide_warps = 8;
    int wide_smem = 1;
    float ring_margin = 1.4f;       // ring width = margin * predicted score / e + 64
    int retry_warps = 8;            // warps per pair in the retry passes (their pairs are wide)
  } tune;
  cudaStream_t aux_stream = nullptr;
  // end-to-end pipeline (wfg_align_host): input copies on their own stream, per-chunk events
  cudaStream_t copy_stream = nullptr;
  cudaStream_t alt_stream = nullptr;  // odd chunks' first passes
  int pipeline = 1;  // wfg_set_pipeline
  std::vector<cudaEvent_t> chunk_ev;
  // wfg_run's device work as a CUDA graph (wfg_set_graph)
  int use_graph = 1;
  // timing of the last upload (wfg_get_stats)
  double upload_host_ms = 0.0;
  bool uploaded = false;
  cudaGraphExec_t graph_exec = nullptr;
  wfg::PinBuf<int> h_order_pin;  // the processing order, copied by the graph's first node
};

int wfg_fail(wfg_context* c, cudaError_t e, const char* where);
int wfg_stage_pairs(wfg_context* c, int n, int64_t seq_len, const int64_t* p_off, const int* plen, const int64_t* t_off,
                    const int* tlen);
// Predicted scores of pairs [first, first + count) of the resident batch, features and MLP
// forward on `stream` (wfg_model.cpp).
int wfg_model_predict_range(wfg_model* m, wfg_context* c, int first, int count, cudaStream_t stream);
#define WFG_CHECK(c, call)                                  \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return wfg_fail((c), _e, #call); \
  } while (0)
