// Host runtime of the GB300 BiWFA aligner: the wfg_* batch API and the WFA2-lib
// compatible single-pair API of include/wfa_gpu.h.
//
// One wfg_context owns a CUDA stream and grow-only device buffers. wfg_run enqueues,
// without any host synchronisation:
//   1. pack_pairs_kernel            ASCII -> 2-bit (or 8-bit) words, forward and reversed
//   2. biwfa_persistent_kernel x3   main pass + two retry passes with larger arenas; each
//                                   pass reads the previous pass's overflow count from HBM,
//                                   so an empty retry pass costs one launch and exits.
// Results stay in HBM until wfg_fetch.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/wfa_gpu.h"
#include "wfg_internal.h"

namespace wfg {
cudaError_t launch_biwfa(const KernelParams& p, int grid, cudaStream_t stream);
cudaError_t biwfa_occupancy(int* blocks_per_sm);
int biwfa_warps_per_block();
cudaError_t launch_pack(int n, const uint8_t* ascii, PairDesc* pairs, uint32_t* words, int num_sms,
                        cudaStream_t stream);
}  // namespace wfg

using namespace wfg;

namespace {

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

uint32_t next_pow2(uint64_t v) {
  uint64_t p = 1;
  while (p < v) p <<= 1;
  return (uint32_t)std::min<uint64_t>(p, 1u << 30);
}

constexpr int kNumPasses = 3;
constexpr int kCountersPerPass = 4;  // [queue head, retry count, -, -]
constexpr int kOutHeadIndex = kNumPasses * kCountersPerPass;
constexpr int kNumCounters = kOutHeadIndex + 4;

}  // namespace

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
  std::vector<PairDesc> h_pairs;
  std::vector<int> h_order;
  std::vector<float> h_pred;
  bool have_order = false, have_pred = false;
  int64_t total_words = 0;
  int64_t out_cap = 0;
  DevBuf<uint8_t> d_seq;
  DevBuf<PairDesc> d_pairs;
  DevBuf<uint32_t> d_words;
  DevBuf<int> d_order;
  DevBuf<int> d_retry;  // kNumPasses-1 lists of n
  DevBuf<int> d_scores, d_status, d_runlen;
  DevBuf<int64_t> d_runoff;
  DevBuf<uint32_t> d_runs;
  DevBuf<unsigned long long> d_counters;
  DevBuf<uint8_t> d_arena;
  DevBuf<uint8_t> d_flush;
  PinBuf<unsigned long long> h_counters;
  PinBuf<PairDesc> h_pairs_pinned;
  cudaEvent_t ev[8] = {};
  wfg_stats_t stats{};
  bool ran = false;
  int last_score_only = 0;
  int limit_ring_w = 0, limit_leaf_words = 0;
};

static int fail(wfg_context* c, cudaError_t e, const char* where) {
  if (c) {
    c->err = std::string(where) + ": " + cudaGetErrorString(e);
  }
  return WF_STATUS_DEVICE_ERROR;
}
#define WFG_CHECK(c, call)                                 \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return fail((c), _e, #call);    \
  } while (0)

extern "C" {

wfg_context_t* wfg_context_create(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  wfg_context* c = new wfg_context();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return nullptr;
  }
  for (auto& e : c->ev) cudaEventCreate(&e);
  if (c->d_counters.reserve(kNumCounters) != cudaSuccess || c->h_counters.reserve(kNumCounters) != cudaSuccess) {
    delete c;
    return nullptr;
  }
  return c;
}

void wfg_context_destroy(wfg_context_t* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->d_seq.release(); c->d_pairs.release(); c->d_words.release(); c->d_order.release();
  c->d_retry.release(); c->d_scores.release(); c->d_status.release(); c->d_runlen.release();
  c->d_runoff.release(); c->d_runs.release(); c->d_counters.release(); c->d_arena.release();
  c->d_flush.release(); c->h_counters.release(); c->h_pairs_pinned.release();
  for (auto& e : c->ev) if (e) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
}

const char* wfg_last_error(wfg_context_t* c) { return c ? c->err.c_str() : "null context"; }

int wfg_upload(wfg_context_t* c, int n, const char* seq, int64_t seq_len, const int64_t* p_off,
               const int* plen, const int64_t* t_off, const int* tlen) {
  if (!c || n < 0 || (n > 0 && (!seq || !p_off || !plen || !t_off || !tlen))) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  c->n = n;
  c->seq_len = seq_len;
  c->h_plen.assign(plen, plen + n);
  c->h_tlen.assign(tlen, tlen + n);
  c->have_order = c->have_pred = false;
  c->max_plen = c->max_tlen = c->max_sum = 0;
  int64_t words = 0, out_cap = 0;
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));  // host staging buffers are reused below
  WFG_CHECK(c, c->h_pairs_pinned.reserve((size_t)std::max(n, 1)));
  PairDesc* hp = c->h_pairs_pinned.ptr;
  for (int i = 0; i < n; ++i) {
    if (plen[i] < 0 || tlen[i] < 0 || p_off[i] < 0 || t_off[i] < 0 || p_off[i] + plen[i] > seq_len ||
        t_off[i] + tlen[i] > seq_len) {
      c->err = "pair " + std::to_string(i) + " lies outside the sequence buffer";
      return WF_STATUS_UNSUPPORTED;
    }
    PairDesc d;
    d.word_off = words;
    d.p_off = p_off[i];
    d.t_off = t_off[i];
    d.plen = plen[i];
    d.tlen = tlen[i];
    d.pw_len = (plen[i] + 3) / 4 + 2;  // sized for 8 bits per char; 2-bit pairs use the front
    d.tw_len = (tlen[i] + 3) / 4 + 2;
    d.bits = 8;
    d.pad = 0;
    hp[i] = d;
    words += 2 * (int64_t)d.pw_len + 2 * (int64_t)d.tw_len;
    out_cap += (int64_t)plen[i] + tlen[i] + 1;
    c->max_plen = std::max(c->max_plen, plen[i]);
    c->max_tlen = std::max(c->max_tlen, tlen[i]);
    c->max_sum = std::max(c->max_sum, plen[i] + tlen[i]);
  }
  c->total_words = words;
  c->out_cap = out_cap;
  WFG_CHECK(c, c->d_seq.reserve((size_t)std::max<int64_t>(seq_len, 1)));
  WFG_CHECK(c, c->d_pairs.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, c->d_words.reserve((size_t)std::max<int64_t>(words, 1)));
  WFG_CHECK(c, c->d_order.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, c->d_retry.reserve((size_t)std::max(n, 1) * (kNumPasses - 1)));
  WFG_CHECK(c, c->d_scores.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, c->d_status.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, c->d_runlen.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, c->d_runoff.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, c->d_runs.reserve((size_t)std::max<int64_t>(out_cap, 1)));
  if (seq_len > 0) WFG_CHECK(c, cudaMemcpyAsync(c->d_seq.ptr, seq, (size_t)seq_len, cudaMemcpyHostToDevice, c->stream));
  if (n > 0) WFG_CHECK(c, cudaMemcpyAsync(c->d_pairs.ptr, hp, sizeof(PairDesc) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  c->stats.h2d_bytes = seq_len + (int64_t)sizeof(PairDesc) * n;
  c->ran = false;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_order(wfg_context_t* c, const int* order) {
  if (!c || !order) return WF_STATUS_UNSUPPORTED;
  std::vector<char> seen((size_t)c->n, 0);
  for (int i = 0; i < c->n; ++i) {
    if (order[i] < 0 || order[i] >= c->n || seen[(size_t)order[i]]) {
      c->err = "order is not a permutation";
      return WF_STATUS_UNSUPPORTED;
    }
    seen[(size_t)order[i]] = 1;
  }
  c->h_order.assign(order, order + c->n);
  c->have_order = true;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_predictions(wfg_context_t* c, const float* pred) {
  if (!c || !pred) return WF_STATUS_UNSUPPORTED;
  c->h_pred.assign(pred, pred + c->n);
  c->have_pred = true;
  return WF_STATUS_ALG_COMPLETED;
}

}  // extern "C"

namespace {

struct PassShape {
  int ring_w, leaf_words, leaf_max_score, run_cap, leaf_run_cap, stack_cap;
  int64_t warps;
  ArenaLayout L;
};

// Internal penalties (WFA2-lib wavefront_penalties_set_affine, wavefront_penalties.c:95-130).
struct IntPen { int x, o, e, scope; };
IntPen internal_penalties(const wfg_config_t* cfg) {
  IntPen p;
  if (cfg->match < 0) {
    p.x = 2 * cfg->mismatch - 2 * cfg->match;
    p.o = 2 * cfg->gap_opening;
    p.e = 2 * cfg->gap_extension - cfg->match;
  } else {
    p.x = cfg->mismatch; p.o = cfg->gap_opening; p.e = cfg->gap_extension;
  }
  p.scope = std::max(p.o + p.e, p.x) + 1;
  return p;
}

// Largest score a unidirectional leaf can reach: 500 (END_REACHED recovery) or the
// optimal score of a whole pair of <= 100 bp (the short-pair fallback).
int leaf_score_bound(const IntPen& p) {
  const int short_pair = p.x * 100 + p.o + p.e * 100 + p.scope;
  return std::max(520, short_pair) + 8;
}

PassShape shape_pass(const wfg_context* c, const IntPen& p, int pass, int ring_w_hint) {
  if (pass == 0 && c->limit_ring_w > 0) ring_w_hint = c->limit_ring_w;
  PassShape s;
  const int maxsum = std::max(c->max_sum, 1);
  const uint32_t ring_full = next_pow2((uint64_t)maxsum + 8);
  s.leaf_max_score = leaf_score_bound(p);
  s.run_cap = maxsum + 2;
  s.leaf_run_cap = maxsum + 2;
  s.stack_cap = 64;
  // Leaf store bound: every non-null step of a leaf of score <= leaf_max_score allocates at
  // most 3 * min(window + 8, 2*s/e + 8) offsets.
  int64_t leaf_full = 0;
  for (int sc = 0; sc <= s.leaf_max_score; ++sc)
    leaf_full += 3LL * std::min<int64_t>(maxsum + 8, 2LL * sc / std::max(p.e, 1) + 8);
  leaf_full = std::min<int64_t>(leaf_full, (int64_t)1 << 28);
  if (pass == 0) {
    s.ring_w = ring_w_hint > 0 ? (int)std::min<uint32_t>(next_pow2((uint64_t)ring_w_hint), ring_full) : (int)ring_full;
    s.leaf_words = (int)std::min<int64_t>(leaf_full, 1 << 16);
    if (c->limit_leaf_words > 0) s.leaf_words = std::max(c->limit_leaf_words, 16);
  } else if (pass == 1) {
    s.ring_w = (int)ring_full;
    s.leaf_words = (int)std::min<int64_t>(leaf_full, 1 << 18);
  } else {
    s.ring_w = (int)ring_full;
    s.leaf_words = (int)leaf_full;
    s.stack_cap = 256;
  }
  s.L = wfg_arena_layout(p.scope, s.ring_w, s.leaf_max_score, s.leaf_words, s.run_cap, s.leaf_run_cap, s.stack_cap);
  s.warps = 0;
  return s;
}

}  // namespace

extern "C" {

int wfg_run(wfg_context_t* c, const wfg_config_t* cfg, wfg_sched_t sched) {
  if (!c || !cfg) return WF_STATUS_UNSUPPORTED;
  if (cfg->match > 0 || cfg->mismatch <= 0 || cfg->gap_opening < 0 || cfg->gap_extension <= 0) {
    c->err = "penalties must satisfy match <= 0, mismatch > 0, gap_opening >= 0, gap_extension > 0";
    return WF_STATUS_UNSUPPORTED;
  }
  const IntPen p = internal_penalties(cfg);
  if (p.scope > 32) {
    c->err = "max_score_scope above 32 is not supported";
    return WF_STATUS_UNSUPPORTED;
  }
  cudaSetDevice(c->device);
  const int n = c->n;
  const int64_t h2d_upload = c->stats.h2d_bytes;
  c->stats = wfg_stats_t{};
  c->stats.h2d_bytes = h2d_upload + (int64_t)sizeof(int) * n;  // upload + processing order
  c->last_score_only = cfg->score_only;
  // ---- order
  std::vector<int> order((size_t)n);
  int ring_hint = 0;
  if (sched == WFG_SCHED_GIVEN && c->have_order) {
    order = c->h_order;
  } else if (sched == WFG_SCHED_LEARNED && c->have_pred) {
    // Longest predicted work first; the ring is sized for the largest predicted score
    // (with margin); mispredicted pairs overflow into the next pass.
    std::iota(order.begin(), order.end(), 0);
    std::vector<double> cost((size_t)n);
    float maxpred = 0.f;
    for (int i = 0; i < n; ++i) {
      const double s = std::max(1.0f, c->h_pred[(size_t)i]);
      cost[(size_t)i] = s * s + (double)(c->h_plen[(size_t)i] + c->h_tlen[(size_t)i]);
      maxpred = std::max(maxpred, c->h_pred[(size_t)i]);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[(size_t)a] > cost[(size_t)b]; });
    ring_hint = (int)(2.0 * (1.25 * maxpred + 64) / std::max(p.e, 1) + 16);
  } else {
    // Plain path: longest pairs first, a stable counting sort on plen + tlen (O(n)).
    std::vector<int> cnt((size_t)c->max_sum + 2, 0);
    for (int i = 0; i < n; ++i) cnt[(size_t)(c->max_sum - (c->h_plen[(size_t)i] + c->h_tlen[(size_t)i])) + 1]++;
    for (size_t v = 1; v < cnt.size(); ++v) cnt[v] += cnt[v - 1];
    for (int i = 0; i < n; ++i)
      order[(size_t)cnt[(size_t)(c->max_sum - (c->h_plen[(size_t)i] + c->h_tlen[(size_t)i]))]++] = i;
  }
  // ---- pass shapes and arena
  int bps = 0;
  WFG_CHECK(c, biwfa_occupancy(&bps));
  const int wpb = biwfa_warps_per_block();
  const int64_t max_warps = (int64_t)std::max(bps, 1) * c->num_sms * wpb;
  const int64_t arena_budget = (int64_t)24 << 30;  // bytes of HBM for per-warp arenas
  PassShape shapes[kNumPasses];
  int64_t arena_need = 0;
  for (int ps = 0; ps < kNumPasses; ++ps) {
    shapes[ps] = shape_pass(c, p, ps, ring_hint);
    int64_t w = std::min<int64_t>(max_warps, std::max<int64_t>(wpb, (int64_t)n));
    if (ps == 1) w = std::min<int64_t>(w, (int64_t)c->num_sms * wpb * 2);
    if (ps == 2) w = std::min<int64_t>(w, (int64_t)c->num_sms * wpb);
    const int64_t fit = arena_budget / std::max<int64_t>(shapes[ps].L.total, 1);
    w = std::max<int64_t>(wpb, std::min<int64_t>(w, fit));
    w = (w / wpb) * wpb;
    shapes[ps].warps = w;
    arena_need = std::max(arena_need, w * shapes[ps].L.total);
  }
  WFG_CHECK(c, c->d_arena.reserve((size_t)arena_need));
  if (n > 0) WFG_CHECK(c, cudaMemcpyAsync(c->d_order.ptr, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  WFG_CHECK(c, cudaEventRecord(c->ev[0], c->stream));
  WFG_CHECK(c, cudaMemsetAsync(c->d_counters.ptr, 0, sizeof(unsigned long long) * kNumCounters, c->stream));
  WFG_CHECK(c, launch_pack(n, c->d_seq.ptr, c->d_pairs.ptr, c->d_words.ptr, c->num_sms, c->stream));
  WFG_CHECK(c, cudaEventRecord(c->ev[1], c->stream));
  int launches = 1;
  for (int ps = 0; ps < kNumPasses; ++ps) {
    const PassShape& s = shapes[ps];
    KernelParams kp{};
    kp.x = p.x; kp.o = p.o; kp.e = p.e; kp.scope = p.scope;
    kp.match_o = cfg->match; kp.x_o = cfg->mismatch; kp.o_o = cfg->gap_opening; kp.e_o = cfg->gap_extension;
    kp.score_only = cfg->score_only;
    kp.max_steps = cfg->max_alignment_steps > 0 ? cfg->max_alignment_steps : INT_MAX;
    kp.num_pairs = n;
    kp.num_pairs_ptr = (ps == 0) ? nullptr : c->d_counters.ptr + (ps - 1) * kCountersPerPass + 1;
    kp.pairs = c->d_pairs.ptr;
    kp.order = (ps == 0) ? c->d_order.ptr : c->d_retry.ptr + (size_t)(ps - 1) * n;
    kp.retry_out = (ps + 1 < kNumPasses) ? c->d_retry.ptr + (size_t)ps * n : nullptr;
    kp.retry_count = c->d_counters.ptr + ps * kCountersPerPass + 1;
    kp.queue_head = c->d_counters.ptr + ps * kCountersPerPass + 0;
    kp.words = c->d_words.ptr;
    kp.arena = c->d_arena.ptr;
    kp.arena_bytes = s.L.total;
    kp.ring_w = s.ring_w;
    kp.leaf_words = s.leaf_words;
    kp.leaf_max_score = s.leaf_max_score;
    kp.run_cap = s.run_cap;
    kp.leaf_run_cap = s.leaf_run_cap;
    kp.stack_cap = s.stack_cap;
    kp.scores = c->d_scores.ptr;
    kp.status = c->d_status.ptr;
    kp.run_off = c->d_runoff.ptr;
    kp.run_len = c->d_runlen.ptr;
    kp.out_runs = c->d_runs.ptr;
    kp.out_cap = c->out_cap;
    kp.out_head = c->d_counters.ptr + kOutHeadIndex;
    kp.stats = nullptr;
    if (n > 0) {
      WFG_CHECK(c, launch_biwfa(kp, (int)(s.warps / wpb), c->stream));
      ++launches;
    }
    if (ps == 0) WFG_CHECK(c, cudaEventRecord(c->ev[2], c->stream));
  }
  WFG_CHECK(c, cudaEventRecord(c->ev[3], c->stream));
  WFG_CHECK(c, cudaMemcpyAsync(c->h_counters.ptr, c->d_counters.ptr, sizeof(unsigned long long) * kNumCounters,
                               cudaMemcpyDeviceToHost, c->stream));
  c->stats.launches = launches;
  c->stats.num_warps = (int)shapes[0].warps;
  c->stats.ring_w = shapes[0].ring_w;
  c->stats.arena_bytes = shapes[0].L.total;
  c->ran = true;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_synchronize(wfg_context_t* c) {
  if (!c) return WF_STATUS_UNSUPPORTED;
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_get_stats(wfg_context_t* c, wfg_stats_t* out) {
  if (!c || !out) return WF_STATUS_UNSUPPORTED;
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  if (c->ran) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[1], c->ev[3]) == cudaSuccess) c->stats.kernel_ms = ms;
    if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]) == cudaSuccess) c->stats.pack_ms = ms;
    if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[3]) == cudaSuccess) c->stats.total_ms = ms;
    c->stats.retried_pairs = (int)c->h_counters.ptr[1];
    c->stats.total_runs = (int64_t)c->h_counters.ptr[kOutHeadIndex];
  }
  *out = c->stats;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_fetch(wfg_context_t* c, int* scores, int* statuses, int64_t* run_off, int* run_len, uint32_t* runs,
              int64_t runs_cap, int64_t* total_runs) {
  if (!c || !c->ran) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));  // counters are in pinned memory now
  const int n = c->n;
  const int64_t nruns = c->last_score_only ? 0 : (int64_t)c->h_counters.ptr[kOutHeadIndex];
  int64_t d2h = 0;
  if (scores && n) { WFG_CHECK(c, cudaMemcpyAsync(scores, c->d_scores.ptr, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream)); d2h += 4LL * n; }
  if (statuses && n) { WFG_CHECK(c, cudaMemcpyAsync(statuses, c->d_status.ptr, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream)); d2h += 4LL * n; }
  if (run_off && n) { WFG_CHECK(c, cudaMemcpyAsync(run_off, c->d_runoff.ptr, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream)); d2h += 8LL * n; }
  if (run_len && n) { WFG_CHECK(c, cudaMemcpyAsync(run_len, c->d_runlen.ptr, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream)); d2h += 4LL * n; }
  if (runs && nruns > 0) {
    if (nruns > runs_cap) {
      c->err = "runs buffer too small: need " + std::to_string(nruns);
      return WF_STATUS_OOM;
    }
    WFG_CHECK(c, cudaMemcpyAsync(runs, c->d_runs.ptr, sizeof(uint32_t) * (size_t)nruns, cudaMemcpyDeviceToHost, c->stream));
    d2h += 4LL * nruns;
  }
  if (total_runs) *total_runs = nruns;
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  c->stats.d2h_bytes = d2h;
  // Map internal statuses onto WFA2-lib's public codes.
  if (statuses) {
    for (int i = 0; i < n; ++i) {
      if (statuses[i] == WFG_ST_SCRATCH_OVERFLOW || statuses[i] == WFG_ST_OUTPUT_OVERFLOW) statuses[i] = WF_STATUS_OOM;
    }
  }
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_align_host(wfg_context_t* c, const wfg_config_t* cfg, wfg_sched_t sched, int n, const char* seq,
                   int64_t seq_len, const int64_t* p_off, const int* plen, const int64_t* t_off, const int* tlen,
                   int* scores, int* statuses, int64_t* run_off, int* run_len, uint32_t* runs, int64_t runs_cap,
                   int64_t* total_runs) {
  int st = wfg_upload(c, n, seq, seq_len, p_off, plen, t_off, tlen);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  st = wfg_run(c, cfg, sched);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  return wfg_fetch(c, scores, statuses, run_off, run_len, runs, runs_cap, total_runs);
}

void* wfg_host_alloc(int64_t bytes) {
  void* p = nullptr;
  if (bytes <= 0 || cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) return nullptr;
  return p;
}

void wfg_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int wfg_set_arena_limits(wfg_context_t* c, int ring_w, int leaf_words) {
  if (!c || ring_w < 0 || leaf_words < 0) return WF_STATUS_UNSUPPORTED;
  c->limit_ring_w = ring_w;
  c->limit_leaf_words = leaf_words;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_flush_l2(wfg_context_t* c, int64_t bytes) {
  if (!c) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  WFG_CHECK(c, c->d_flush.reserve((size_t)bytes));
  WFG_CHECK(c, cudaMemsetAsync(c->d_flush.ptr, 0x5a, (size_t)bytes, c->stream));
  return WF_STATUS_ALG_COMPLETED;
}

}  // extern "C"
