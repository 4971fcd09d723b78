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
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/wfa_gpu.h"
#include "wfg_context.h"
#include "wfg_internal.h"

using namespace wfg;

namespace {

uint32_t next_pow2(uint64_t v) {
  uint64_t p = 1;
  while (p < v) p <<= 1;
  return (uint32_t)std::min<uint64_t>(p, 1u << 30);
}

}  // namespace

int wfg_fail(wfg_context* c, cudaError_t e, const char* where) {
  if (c) {
    c->err = std::string(where) + ": " + cudaGetErrorString(e);
  }
  return WF_STATUS_DEVICE_ERROR;
}

// The host half of an upload: validates the pairs, builds their descriptors in the pinned
// staging buffer and sizes the device buffers (no copy). The staging buffers are reused, so
// every copy still reading them must be done first.
int wfg_stage_pairs(wfg_context* c, int n, int64_t seq_len, const int64_t* p_off, const int* plen, const int64_t* t_off,
                    const int* tlen) {
  const auto host_t0 = std::chrono::steady_clock::now();
  c->n = n;
  c->seq_len = seq_len;
  c->h_plen.assign(plen, plen + n);
  c->h_tlen.assign(tlen, tlen + n);
  c->have_order = c->have_pred = false;
  c->feats_valid = c->pred_valid = false;
  c->max_plen = c->max_tlen = c->max_sum = 0;
  int64_t words = 0, out_cap = 0;
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  if (c->copy_stream) WFG_CHECK(c, cudaStreamSynchronize(c->copy_stream));
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
  c->upload_host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host_t0).count();
  return WF_STATUS_ALG_COMPLETED;
}

extern "C" {

wfg_context_t* wfg_context_create(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  wfg_context* c = new wfg_context();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking) != cudaSuccess) {
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
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  c->h_order_pin.release();
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  if (c->alt_stream) {
    cudaStreamSynchronize(c->alt_stream);
    cudaStreamDestroy(c->alt_stream);
  }
  for (auto& e : c->chunk_ev) cudaEventDestroy(e);
  c->d_feats.release(); c->d_pred.release(); c->d_bin_work.release(); c->h_bin_stats.release();
  c->d_batch_heads.release();
  cudaStreamDestroy(c->stream);
  cudaStreamDestroy(c->aux_stream);
  delete c;
}

const char* wfg_last_error(wfg_context_t* c) { return c ? c->err.c_str() : "null context"; }

int wfg_upload(wfg_context_t* c, int n, const char* seq, int64_t seq_len, const int64_t* p_off,
               const int* plen, const int64_t* t_off, const int* tlen) {
  if (!c || n < 0 || (n > 0 && (!seq || !p_off || !plen || !t_off || !tlen))) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  const int st = wfg_stage_pairs(c, n, seq_len, p_off, plen, t_off, tlen);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  WFG_CHECK(c, cudaEventRecord(c->ev[6], c->stream));
  if (seq_len > 0) WFG_CHECK(c, cudaMemcpyAsync(c->d_seq.ptr, seq, (size_t)seq_len, cudaMemcpyHostToDevice, c->stream));
  if (n > 0)
    WFG_CHECK(c, cudaMemcpyAsync(c->d_pairs.ptr, c->h_pairs_pinned.ptr, sizeof(PairDesc) * (size_t)n,
                                 cudaMemcpyHostToDevice, c->stream));
  WFG_CHECK(c, cudaEventRecord(c->ev[7], c->stream));
  c->uploaded = true;
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

// Internal penalties (WFA2-lib wavefront_penalties_set_affine, wavefront_penalties.c:95-130).
// nc: stored components (3, or 5 for two gap pieces); emin: the cheapest gap base (bounds how
// fast a wavefront widens with the score); g: the spacing of the scores that can hold a
// wavefront (the gcd of the step costs).
struct IntPen {
  int x, o, e, scope, nphys;
  int o2 = 0, e2 = 0, nc = 3, emin = 1, g = 1;
};
IntPen internal_penalties(const wfg_config_t* cfg) {
  IntPen p;
  if (cfg->metric == WFG_METRIC_GAP_AFFINE_2P) {
    // wavefront_penalties_set_affine2p (wavefront_penalties.c:132-173);
    // wavefront_components_dimensions_affine2p: scope max(x, o1+e1, o2+e2) + 1
    if (cfg->match < 0) {
      p.x = 2 * cfg->mismatch - 2 * cfg->match;
      p.o = 2 * cfg->gap_opening; p.e = 2 * cfg->gap_extension - cfg->match;
      p.o2 = 2 * cfg->gap_opening2; p.e2 = 2 * cfg->gap_extension2 - cfg->match;
    } else {
      p.x = cfg->mismatch; p.o = cfg->gap_opening; p.e = cfg->gap_extension;
      p.o2 = cfg->gap_opening2; p.e2 = cfg->gap_extension2;
    }
    p.scope = std::max(std::max(p.o + p.e, p.o2 + p.e2), p.x) + 1;
    p.nphys = wfg_ring_buffers_2p(p.x, p.o, p.e, p.o2, p.e2);
    p.nc = 5;
    p.emin = std::max(std::min(p.e, p.e2), 1);
    p.g = wfg_gcd(wfg_gcd(wfg_gcd(p.x, p.o + p.e), wfg_gcd(p.e, p.o2 + p.e2)), p.e2);
    return p;
  }
  if (cfg->metric == WFG_METRIC_EDIT || cfg->metric == WFG_METRIC_INDEL) {
    // wavefront_penalties_set_edit / _indel: one component, a wavefront at every score,
    // max_score_scope 2 (wavefront_components.c:45-60). x bounds the score guard only
    // (an indel-distance mismatch is two indels).
    p.x = (cfg->metric == WFG_METRIC_EDIT) ? 1 : 2; p.o = 1; p.e = 1;
    p.scope = 2; p.nphys = 2;
    p.emin = 1; p.g = 1;
    return p;
  }
  if (cfg->metric == WFG_METRIC_GAP_LINEAR) {
    // wavefront_penalties_set_linear (wavefront_penalties.c:63-94), indel from gap_opening;
    // wavefront_components_dimensions_linear: scope max(x, indel) + 1
    if (cfg->match < 0) { p.x = 2 * cfg->mismatch - 2 * cfg->match; p.o = 2 * cfg->gap_opening - cfg->match; }
    else { p.x = cfg->mismatch; p.o = cfg->gap_opening; }
    p.e = 0;
    p.scope = std::max(p.x, p.o) + 1;
    p.nphys = wfg_ring_buffers(p.x, p.o, 0);
    p.emin = std::max(p.o, 1);  // one diagonal per indel on each side
    p.g = wfg_gcd(p.x, p.o);
    return p;
  }
  if (cfg->match < 0) {
    p.x = 2 * cfg->mismatch - 2 * cfg->match;
    p.o = 2 * cfg->gap_opening;
    p.e = 2 * cfg->gap_extension - cfg->match;
  } else {
    p.x = cfg->mismatch; p.o = cfg->gap_opening; p.e = cfg->gap_extension;
  }
  p.scope = std::max(p.o + p.e, p.x) + 1;
  p.nphys = wfg_ring_buffers(p.x, p.o, p.e);
  p.emin = std::max(p.e, 1);
  p.g = wfg_gcd(wfg_gcd(p.x, p.o + p.e), p.e);
  return p;
}

// Largest score a unidirectional leaf can reach: 500 (END_REACHED recovery) or the
// optimal score of a whole pair of <= 100 bp (the short-pair fallback).
int leaf_score_bound(const IntPen& p) {
  const int short_pair = p.x * 100 + p.o + std::max(p.e, p.o) * 100 + p.scope;
  return std::max(520, short_pair) + 8;
}

// One persistent launch: execution shape, arena carving and the pairs it drains.
struct Launch {
  int gw = 1;            // warps per pair
  int smem = 0;          // rings in shared memory
  int ring_w = 0, leaf_words = 0, leaf_max_score = 0, run_cap = 0, leaf_run_cap = 0, stack_cap = 0;
  int64_t groups = 0;    // pairs in flight
  bool batched = false;  // consecutive launches of `groups` pairs each instead of one persistent launch
  ArenaLayout L{};
  int64_t arena_off = 0; // byte offset of this launch's arenas
  int order_off = 0, count = 0;
};

// Scratch sizes of a pass: pass 0 is bounded by the ring hint (predicted width or the plain
// cap) and a small leaf store; the retry passes size rings from the longest pair.
void size_launch(const wfg_context* c, const IntPen& p, int pass, int ring_w_hint, Launch& s) {
  const int maxsum = std::max(c->max_sum, 1);
  const uint32_t ring_full = next_pow2((uint64_t)maxsum + 8);
  s.leaf_max_score = leaf_score_bound(p);
  s.run_cap = maxsum + 2;
  s.leaf_run_cap = maxsum + 2;
  s.stack_cap = 64;
  // Leaf store bound: a leaf's wavefronts sit at scores that are multiples of g, and the step
  // at score s allocates at most nc * min(window + 8, 2*s/emin + 8) offsets. Pass 0 holds a
  // leaf that starts at the BiWFA fallback score (250) with room to spare, pass 1 four times
  // that, pass 2 the full bound (recovery leaves up to score 500, whole short pairs).
  auto leaf_words_upto = [&](int smax) {
    int64_t w = 0;
    for (int sc = 0; sc <= smax; sc += p.g) w += (int64_t)p.nc * std::min<int64_t>(maxsum + 8, 2LL * sc / p.emin + 8);
    return w;
  };
  const int64_t leaf_full = std::min<int64_t>(leaf_words_upto(s.leaf_max_score), (int64_t)1 << 28);
  const int64_t leaf_typical = leaf_words_upto(250) * 5 / 4;
  if (pass == 0) {
    const uint32_t plain_cap = std::min<uint32_t>(ring_full, kPlainRingCap);
    s.ring_w = ring_w_hint > 0 ? (int)std::min<uint32_t>(next_pow2((uint64_t)ring_w_hint), ring_full) : (int)plain_cap;
    s.leaf_words = (int)std::min<int64_t>(leaf_full, std::max<int64_t>(1 << 16, leaf_typical));
    if (c->limit_leaf_words > 0) s.leaf_words = std::max(c->limit_leaf_words, 16);
  } else if (pass == 1) {
    s.ring_w = (int)ring_full;
    s.leaf_words = (int)std::min<int64_t>(leaf_full, std::max<int64_t>(1 << 18, 4 * leaf_typical));
  } else {
    s.ring_w = (int)ring_full;
    s.leaf_words = (int)leaf_full;
    s.stack_cap = 256;
  }
  if (s.smem) {
    // Both rings of the group in dynamic shared memory: the widest power of two that keeps
    // them within kSmemRingBytes; penalties with many live buffers fall back to HBM rings.
    int w = kSmemRingW;
    while (w >= 64 && (int64_t)2 * p.nphys * p.nc * w * 4 > kSmemRingBytes) w >>= 1;
    if (w < 64) s.smem = 0;
    else s.ring_w = std::min(s.ring_w, w);
  }
  s.L = wfg_arena_layout(s.smem ? 0 : p.nphys, s.ring_w, s.leaf_max_score, s.leaf_words, s.run_cap, s.leaf_run_cap,
                         s.stack_cap, p.nc);
}

// Groups that fit the device at once for a shape (persistent grid).
int64_t max_groups(const wfg_context* c, const IntPen& p, const Launch& l) {
  const size_t dyn = l.smem ? (size_t)2 * p.nphys * p.nc * (size_t)l.ring_w * sizeof(int32_t) : 0;
  int bps = 0;
  if (biwfa_occupancy_shape(l.gw, l.smem, dyn, &bps, biwfa_kernel_kind(p.nc == 5 ? 4 : 0, p.scope)) != cudaSuccess ||
      bps < 1) {
    (void)cudaGetLastError();
    bps = 1;
  }
  return (int64_t)bps * c->num_sms * biwfa_groups_per_block(l.gw, l.smem);
}

// Kernel parameters of one launch of pass ps (0: first pass; the retry passes read the
// previous pass's overflow list); the work queue (order, count, head) is set by the caller.
KernelParams launch_params(const wfg_context* c, const wfg_config_t* cfg, const IntPen& p, const Launch& l, int ps) {
  const int n = c->n;
  KernelParams kp{};
  kp.x = p.x; kp.o = p.o; kp.e = p.e; kp.scope = p.scope; kp.o2 = p.o2; kp.e2 = p.e2;
  kp.match_o = cfg->match; kp.x_o = cfg->mismatch; kp.o_o = cfg->gap_opening; kp.e_o = cfg->gap_extension;
  if (p.nc == 5) { kp.o2_o = cfg->gap_opening2; kp.e2_o = cfg->gap_extension2; }
  kp.metric = cfg->metric;
  kp.score_only = cfg->score_only;
  kp.max_steps = cfg->max_alignment_steps > 0 ? cfg->max_alignment_steps : INT_MAX;
  kp.pairs = c->d_pairs.ptr;
  kp.words = c->d_words.ptr;
  kp.arena = c->d_arena.ptr + l.arena_off;
  kp.arena_bytes = l.L.total;
  kp.ring_w = l.ring_w;
  kp.leaf_words = l.leaf_words;
  kp.leaf_max_score = l.leaf_max_score;
  kp.run_cap = l.run_cap;
  kp.leaf_run_cap = l.leaf_run_cap;
  kp.stack_cap = l.stack_cap;
  kp.scores = c->d_scores.ptr;
  kp.status = c->d_status.ptr;
  kp.run_off = c->d_runoff.ptr;
  kp.run_len = c->d_runlen.ptr;
  kp.out_runs = c->d_runs.ptr;
  kp.out_cap = c->out_cap;
  kp.out_head = c->d_counters.ptr + kOutHeadIndex;
  kp.stats = nullptr;
  kp.group_warps = l.gw;
  kp.ring_in_smem = l.smem;
  kp.ring_nphys = p.nphys;
  kp.retry_out = (ps + 1 < kNumPasses) ? c->d_retry.ptr + (size_t)ps * n : nullptr;
  kp.retry_count = c->d_counters.ptr + ps * kCountersPerPass + 1;
  return kp;
}

// Shapes and arenas of the retry passes (1 .. kNumPasses-1), which realign the pairs that
// overflowed the previous pass; returns the arena bytes the largest of them needs.
int64_t plan_retry_passes(const wfg_context* c, const IntPen& p, int64_t arena_budget, Launch* retry) {
  int64_t need = 0;
  for (int ps = 1; ps < kNumPasses; ++ps) {
    Launch& l = retry[ps];
    l.gw = c->tune.retry_warps;  // pairs that overflowed the first pass are wide
    size_launch(c, p, ps, 0, l);
    const int gpb = biwfa_groups_per_block(l.gw, l.smem);
    int64_t gmax = std::min<int64_t>(max_groups(c, p, l), std::max<int64_t>(gpb, (int64_t)c->n));
    if (l.gw == 1) gmax = std::min<int64_t>(gmax, ps == 1 ? (int64_t)c->num_sms * 4 : (int64_t)c->num_sms * 2);
    const int64_t fit = arena_budget / std::max<int64_t>(l.L.total, 1);
    l.groups = std::max<int64_t>(gpb, (std::min(gmax, fit) / gpb) * gpb);
    need = std::max(need, l.groups * l.L.total);
  }
  return need;
}

// Launch sizes of the first pass over `count` pairs with ring hint `hint` (0: the plain cap):
// groups in flight within the device's residency and the arena budget.
void plan_first_pass(const wfg_context* c, const IntPen& p, int hint, int64_t arena_budget, Launch& l) {
  if (l.gw < 1) l.gw = 1;
  if (l.gw != 1 && l.gw != 4 && l.gw != 8) l.gw = 8;
  size_launch(c, p, 0, hint, l);
  const int64_t gmax = std::min<int64_t>(max_groups(c, p, l), std::max<int64_t>(1, l.count));
  const int64_t fit = arena_budget / std::max<int64_t>(l.L.total, 1);
  l.groups = std::max<int64_t>(1, std::min(gmax, fit));
  const int gpb = biwfa_groups_per_block(l.gw, l.smem);
  l.groups = std::max<int64_t>(gpb, (l.groups / gpb) * gpb);
}

// The arena budget of a run: half of the device memory that is free or already held by the
// arena, within [4 GiB, 96 GiB] (one GB300 has 288 GB of HBM).
int64_t arena_budget_of(const wfg_context* c) {
  int64_t budget = (int64_t)24 << 30;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    const int64_t avail = (int64_t)free_b + (int64_t)c->d_arena.cap;
    budget = std::min<int64_t>((int64_t)96 << 30, std::max<int64_t>((int64_t)4 << 30, avail / 2));
  } else {
    (void)cudaGetLastError();
  }
  return budget;
}

// The distance and penalties of a run, checked against the resident batch; *p receives the
// internal penalties. Configuration errors are statuses with a message, never exits.
int validate_config(wfg_context* c, const wfg_config_t* cfg, IntPen* p) {
  if (cfg->metric != WFG_METRIC_GAP_AFFINE && cfg->metric != WFG_METRIC_EDIT && cfg->metric != WFG_METRIC_INDEL &&
      cfg->metric != WFG_METRIC_GAP_LINEAR && cfg->metric != WFG_METRIC_GAP_AFFINE_2P) {
    c->err = "unknown distance metric";
    return WF_STATUS_UNSUPPORTED;
  }
  if (cfg->metric == WFG_METRIC_GAP_LINEAR && (cfg->match > 0 || cfg->mismatch <= 0 || cfg->gap_opening <= 0)) {
    c->err = "gap-linear penalties must satisfy match <= 0, mismatch > 0, indel (gap_opening) > 0";
    return WF_STATUS_UNSUPPORTED;
  }
  if (cfg->metric == WFG_METRIC_GAP_AFFINE &&
      (cfg->match > 0 || cfg->mismatch <= 0 || cfg->gap_opening < 0 || cfg->gap_extension <= 0)) {
    c->err = "penalties must satisfy match <= 0, mismatch > 0, gap_opening >= 0, gap_extension > 0";
    return WF_STATUS_UNSUPPORTED;
  }
  if (cfg->metric == WFG_METRIC_GAP_AFFINE_2P &&
      (cfg->match > 0 || cfg->mismatch <= 0 || cfg->gap_opening < 0 || cfg->gap_extension <= 0 ||
       cfg->gap_opening2 < 0 || cfg->gap_extension2 <= 0)) {
    c->err = "two-piece penalties must satisfy match <= 0, mismatch > 0, o1 >= 0, e1 > 0, o2 >= 0, e2 > 0";
    return WF_STATUS_UNSUPPORTED;
  }
  *p = internal_penalties(cfg);
  if (p->scope > WFG_MAX_SCOPE_2P) {
    c->err = "max_score_scope above 64 is not supported";
    return WF_STATUS_UNSUPPORTED;
  }
  if ((int64_t)(c->max_sum + 16) * (int64_t)std::max(p->x, std::max(p->o + p->e, p->o2 + p->e2)) >= ((int64_t)1 << 26)) {
    c->err = "pair too long for 27-bit scores";
    return WF_STATUS_UNSUPPORTED;
  }
  return WF_STATUS_ALG_COMPLETED;
}

}  // namespace

extern "C" {

int wfg_run(wfg_context_t* c, const wfg_config_t* cfg, wfg_sched_t sched) {
  if (!c || !cfg) return WF_STATUS_UNSUPPORTED;
  IntPen p;
  const int vst = validate_config(c, cfg, &p);
  if (vst != WF_STATUS_ALG_COMPLETED) return vst;
  cudaSetDevice(c->device);
  const int n = c->n;
  const int64_t h2d_upload = c->stats.h2d_bytes;
  c->stats = wfg_stats_t{};
  c->stats.h2d_bytes = h2d_upload + (int64_t)sizeof(int) * n;  // upload + processing order
  c->last_score_only = cfg->score_only;
  // ---- order and pass-0 launches
  std::vector<int> order((size_t)n);
  bool order_on_device = false;  // the learned schedule writes the order on the device
  int predict_launches = 0;      // features, MLP forward and binning kernels of the learned schedule
  std::vector<Launch> first;  // concurrent pass-0 launches
  if (sched == WFG_SCHED_GIVEN && c->have_order) {
    order = c->h_order;
    Launch l; l.gw = c->force_gw; l.smem = c->force_smem; l.count = n;
    first.push_back(l);
  } else if (sched == WFG_SCHED_LEARNED && (c->have_pred || c->model != nullptr)) {
    // Predictions on the device: the model's (4-mer features + MLP forward, recomputed every
    // run) or the caller's. Binning and ordering also run on the device (launch_bin_order):
    // one order by predicted score, largest first; its head — the pairs predicted at or above
    // the wide threshold, at most one resident wave of the multi-warp shape — forms the
    // multi-warp launch (aux stream), the rest the single-warp launch. Rings are sized from
    // each launch's largest prediction (a mispredicted pair overflows into the retry passes).
    // Only the two launch sizes and prediction bounds come back to the host.
    WFG_CHECK(c, c->d_pred.reserve((size_t)std::max(n, 1)));
    if (c->model != nullptr) {
      c->feats_valid = false;
      const int st = wfg_model_predict(c->model, c, nullptr);
      if (st != WF_STATUS_ALG_COMPLETED) return st;
    } else if (n > 0) {
      WFG_CHECK(c, cudaMemcpyAsync(c->d_pred.ptr, c->h_pred.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice,
                                   c->stream));
    }
    const bool use_wide = c->tune.wide_warps > 1 && c->tune.wide_threshold < 3.0e38f;  // FLT_MAX: no wide launch
    int64_t wide_cap = 0;
    if (use_wide) {
      Launch lw; lw.gw = c->tune.wide_warps; lw.smem = c->tune.wide_smem; lw.ring_w = kSmemRingW;
      wide_cap = max_groups(c, p, lw);
    }
    WFG_CHECK(c, c->d_bin_work.reserve((size_t)sched_bin_words()));
    WFG_CHECK(c, c->h_bin_stats.reserve(4));
    WFG_CHECK(c, launch_bin_order(n, c->d_pred.ptr, use_wide ? c->tune.wide_threshold : INFINITY, (int)wide_cap,
                                  c->d_bin_work.ptr, c->d_bin_work.ptr + sched_bin_words() - 4, c->d_order.ptr,
                                  c->num_sms, c->stream));
    WFG_CHECK(c, cudaMemcpyAsync(c->h_bin_stats.ptr, c->d_bin_work.ptr + sched_bin_words() - 4, sizeof(int) * 4,
                                 cudaMemcpyDeviceToHost, c->stream));
    WFG_CHECK(c, cudaStreamSynchronize(c->stream));
    order_on_device = true;
    predict_launches = (c->model != nullptr ? 2 : 0) + (n > 0 ? 3 : 0);
    const int n_wide = c->h_bin_stats.ptr[0], n_narrow = c->h_bin_stats.ptr[1];
    float max_wide, max_narrow;
    memcpy(&max_wide, &c->h_bin_stats.ptr[2], sizeof(float));
    memcpy(&max_narrow, &c->h_bin_stats.ptr[n_wide > 0 ? 3 : 2], sizeof(float));
    const double m = c->tune.ring_margin;
    if (n_wide > 0) {
      Launch l; l.gw = c->tune.wide_warps; l.order_off = 0; l.count = n_wide;
      const int w_need = (int)(m * max_wide / p.emin) + 64;
      l.smem = (c->tune.wide_smem && next_pow2((uint64_t)w_need) <= (uint32_t)kSmemRingW) ? 1 : 0;
      l.ring_w = w_need;
      first.push_back(l);
    }
    if (n_narrow > 0) {
      Launch l; l.gw = 1; l.order_off = n_wide; l.count = n_narrow;
      l.ring_w = (int)(m * max_narrow / p.emin) + 64;
      first.push_back(l);
    }
  } else {
    // Plain and sorted paths: longest pairs first, a stable counting sort on plen + tlen (O(n)).
    // The plain path then runs them in consecutive launches of one resident set each.
    std::vector<int> cnt((size_t)c->max_sum + 2, 0);
    for (int i = 0; i < n; ++i) cnt[(size_t)(c->max_sum - (c->h_plen[(size_t)i] + c->h_tlen[(size_t)i])) + 1]++;
    for (size_t v = 1; v < cnt.size(); ++v) cnt[v] += cnt[v - 1];
    for (int i = 0; i < n; ++i)
      order[(size_t)cnt[(size_t)(c->max_sum - (c->h_plen[(size_t)i] + c->h_tlen[(size_t)i]))]++] = i;
    // The sorted schedule sends pairs longer than kDirectWideSum (a prefix of this order)
    // straight to a multi-warp launch with rings as wide as the batch's longest pair, on the aux
    // stream beside the single-warp launch: a single warp would take the longest of them far
    // beyond the rest of the batch, and their wavefronts outgrow the first pass's ring cap.
    int n_long = 0;
    if (sched == WFG_SCHED_SORTED && c->force_gw == 1 && !c->force_smem && c->limit_ring_w == 0)
      while (n_long < n && c->h_plen[(size_t)order[(size_t)n_long]] + c->h_tlen[(size_t)order[(size_t)n_long]] >
                               kDirectWideSum)
        ++n_long;
    if (n_long > 0) {
      Launch lw; lw.gw = c->tune.retry_warps; lw.count = n_long; lw.order_off = 0;
      lw.ring_w = (int)next_pow2((uint64_t)c->max_sum + 8);
      first.push_back(lw);
    }
    if (n - n_long > 0 || first.empty()) {
      Launch l; l.gw = c->force_gw; l.smem = c->force_smem; l.count = n - n_long; l.order_off = n_long;
      l.batched = (sched == WFG_SCHED_PLAIN);
      first.push_back(l);
    }
  }
  if (first.empty()) { Launch l; l.count = 0; first.push_back(l); }
  // ---- shapes and arena (pass-0 launches run concurrently; retry passes reuse the arena)
  const int64_t arena_budget = arena_budget_of(c);
  int64_t pass0_bytes = 0;
  for (Launch& l : first) {
    const int hint = l.ring_w > 0 ? l.ring_w : c->limit_ring_w;
    plan_first_pass(c, p, hint, arena_budget / (int64_t)first.size(), l);
    l.arena_off = pass0_bytes;
    pass0_bytes += l.groups * l.L.total;
  }
  Launch retry[kNumPasses];
  const int64_t arena_need = std::max(pass0_bytes, plan_retry_passes(c, p, arena_budget, retry));
  WFG_CHECK(c, c->d_arena.reserve((size_t)arena_need));
  int64_t num_batches = 0;
  for (const Launch& l : first)
    if (l.batched) num_batches += (l.count + l.groups - 1) / l.groups;
  WFG_CHECK(c, c->d_batch_heads.reserve((size_t)std::max<int64_t>(num_batches, 1)));
  // The order goes through a pinned buffer (a graph's copy node reads it when the graph
  // runs): wait until the previous run's copy of it is done before overwriting it.
  if (c->ran) WFG_CHECK(c, cudaEventSynchronize(c->ev[0]));
  WFG_CHECK(c, c->h_order_pin.reserve((size_t)std::max(n, 1)));
  if (n > 0 && !order_on_device) std::copy(order.begin(), order.end(), c->h_order_pin.ptr);
  auto params = [&](const Launch& l, int ps) { return launch_params(c, cfg, p, l, ps); };
  int launches = 0;
  // The device work of one run. Timing events are external record nodes when captured;
  // ev[5] / ev[4] fork the aux stream off and join it back (capture dependencies).
  auto enqueue = [&](bool capturing) -> cudaError_t {
    auto mark = [&](cudaEvent_t ev) {
      return capturing ? cudaEventRecordWithFlags(ev, c->stream, cudaEventRecordExternal) : cudaEventRecord(ev, c->stream);
    };
    cudaError_t e = cudaSuccess;
    launches = 1;
    if (n > 0 && !order_on_device &&
        (e = cudaMemcpyAsync(c->d_order.ptr, c->h_order_pin.ptr, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                             c->stream)) != cudaSuccess)
      return e;
    if ((e = mark(c->ev[0])) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->d_counters.ptr, 0, sizeof(unsigned long long) * kNumCounters, c->stream)) != cudaSuccess)
      return e;
    if (num_batches > 0 && (e = cudaMemsetAsync(c->d_batch_heads.ptr, 0, sizeof(unsigned long long) * (size_t)num_batches,
                                                c->stream)) != cudaSuccess)
      return e;
    if ((e = launch_pack(n, c->d_seq.ptr, c->d_pairs.ptr, c->d_words.ptr, c->num_sms, c->stream)) != cudaSuccess) return e;
    if ((e = mark(c->ev[1])) != cudaSuccess) return e;
    // pass 0: the first launch on the context's stream, a second one on the aux stream,
    // forked before the first so that the two run concurrently, joined before the retry passes
    int64_t batch_index = 0;
    const bool fork = first.size() > 1 && first[1].count > 0 && first[0].count > 0;
    if (fork) {
      if ((e = cudaEventRecord(c->ev[5], c->stream)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(c->aux_stream, c->ev[5], 0)) != cudaSuccess) return e;
    }
    for (size_t li = 0; li < first.size(); ++li) {
      const Launch& l = first[li];
      if (l.count <= 0) continue;
      if (l.batched) {
        // one launch per resident set of pairs, each waiting for its slowest pair
        const int gpb = biwfa_groups_per_block(l.gw, l.smem);
        for (int64_t b0 = 0; b0 < l.count; b0 += l.groups, ++batch_index) {
          KernelParams kp = params(l, 0);
          kp.num_pairs = (int)std::min<int64_t>(l.groups, l.count - b0);
          kp.num_pairs_ptr = nullptr;
          kp.order = c->d_order.ptr + l.order_off + b0;
          kp.queue_head = c->d_batch_heads.ptr + batch_index;
          const int blocks = (int)((kp.num_pairs + gpb - 1) / gpb);
          if ((e = launch_biwfa(kp, blocks, c->stream)) != cudaSuccess) return e;
          ++launches;
        }
        continue;
      }
      KernelParams kp = params(l, 0);
      kp.num_pairs = l.count;
      kp.num_pairs_ptr = nullptr;
      kp.order = c->d_order.ptr + l.order_off;
      kp.queue_head = c->d_counters.ptr + (li == 0 ? 0 : 2);
      const cudaStream_t st = (fork && li > 0) ? c->aux_stream : c->stream;
      if ((e = launch_biwfa(kp, (int)(l.groups / biwfa_groups_per_block(l.gw, l.smem)), st)) != cudaSuccess) return e;
      ++launches;
    }
    if (fork) {
      if ((e = cudaEventRecord(c->ev[4], c->aux_stream)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(c->stream, c->ev[4], 0)) != cudaSuccess) return e;
    }
    if ((e = mark(c->ev[2])) != cudaSuccess) return e;
    for (int ps = 1; ps < kNumPasses; ++ps) {
      const Launch& l = retry[ps];
      if (n <= 0) break;
      KernelParams kp = params(l, ps);
      kp.num_pairs = n;
      kp.num_pairs_ptr = c->d_counters.ptr + (ps - 1) * kCountersPerPass + 1;
      kp.order = c->d_retry.ptr + (size_t)(ps - 1) * n;
      kp.queue_head = c->d_counters.ptr + ps * kCountersPerPass + 0;
      if ((e = launch_biwfa(kp, (int)(l.groups / biwfa_groups_per_block(l.gw, l.smem)), c->stream)) != cudaSuccess)
        return e;
      ++launches;
    }
    if ((e = mark(c->ev[3])) != cudaSuccess) return e;
    return cudaMemcpyAsync(c->h_counters.ptr, c->d_counters.ptr, sizeof(unsigned long long) * kNumCounters,
                           cudaMemcpyDeviceToHost, c->stream);
  };
  c->stats.used_graph = 0;
  if (c->use_graph) {
    WFG_CHECK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const cudaError_t e = enqueue(true);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess || ec != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return wfg_fail(c, e != cudaSuccess ? e : ec, "wfg_run graph capture");
    }
    if (c->graph_exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(c->graph_exec, graph, &info) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(c->graph_exec);
        c->graph_exec = nullptr;
      }
    }
    cudaError_t ei = cudaSuccess;
    if (!c->graph_exec) ei = cudaGraphInstantiate(&c->graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    WFG_CHECK(c, ei);
    WFG_CHECK(c, cudaGraphLaunch(c->graph_exec, c->stream));
    c->stats.used_graph = 1;
  } else {
    WFG_CHECK(c, enqueue(false));
  }
  c->stats.launches = launches + predict_launches;
  c->stats.num_warps = (int)(first[0].groups * first[0].gw);
  c->stats.ring_w = first[0].ring_w;
  c->stats.arena_bytes = first[0].L.total;
  c->ran = true;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_retry_shape(wfg_context_t* c, int group_warps) {
  if (!c || (group_warps != 1 && group_warps != 4 && group_warps != 8)) return WF_STATUS_UNSUPPORTED;
  c->tune.retry_warps = group_warps;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_pipeline(wfg_context_t* c, int enable) {
  if (!c) return WF_STATUS_UNSUPPORTED;
  c->pipeline = enable ? 1 : 0;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_graph(wfg_context_t* c, int enable) {
  if (!c) return WF_STATUS_UNSUPPORTED;
  c->use_graph = enable ? 1 : 0;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_exec_shape(wfg_context_t* c, int group_warps, int ring_in_smem) {
  if (!c || (group_warps != 1 && group_warps != 4 && group_warps != 8)) return WF_STATUS_UNSUPPORTED;
  c->force_gw = group_warps;
  c->force_smem = (group_warps > 1 && ring_in_smem) ? 1 : 0;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_learned_policy(wfg_context_t* c, float wide_threshold, int wide_warps, int wide_smem, float ring_margin) {
  if (!c || (wide_warps != 1 && wide_warps != 4 && wide_warps != 8) || ring_margin < 1.0f) return WF_STATUS_UNSUPPORTED;
  c->tune.wide_threshold = wide_threshold;
  c->tune.wide_warps = wide_warps;
  c->tune.wide_smem = wide_smem ? 1 : 0;
  c->tune.ring_margin = ring_margin;
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
  c->stats.upload_host_ms = c->upload_host_ms;
  if (c->uploaded) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]) == cudaSuccess) c->stats.upload_copy_ms = ms;
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

}  // extern "C"

namespace {

constexpr int kPipelineMinPairs = 131072;  // batches from which wfg_align_host overlaps its input copy
constexpr int kPipelineHeadDiv = 8;        // the head chunk: the first 1/8 of the pairs

// End-to-end alignment with the input copy overlapped with the alignment. The pairs are cut
// into chunks by index: a head of 1/8 of the pairs, then the rest (K = 2; the code takes any
// K, the head fixed). The copy stream uploads the descriptors, then the sequence bytes up to
// each chunk's last byte, chunk by chunk. As soon as chunk k's bytes are in, the aux stream
// packs it and (learned schedule) computes its features, predictions and binned order; chunk
// k's first pass then runs on the main stream (even k) or the alternate stream (odd k), in its
// own arena region, so that it takes over the SMs as chunk k-1's persistent warps retire. The
// head's alignment outlasts the copy of everything else, and the rest then runs in one
// launch, heaviest first: with many equal chunks, each chunk's heaviest pairs (about 0.3 s for
// one warp) started only when the chunk did, and the last chunk's ones ended after the rest
// (measured: 8 equal chunks cost 190 ms of device time, as much as the copy they hid). The
// retry passes run once, over the overflows of every chunk. Scheduling only: every pair's
// result is the one wfg_run gives.
int align_host_pipelined(wfg_context* c, const wfg_config_t* cfg, wfg_sched_t sched, int n, const char* seq,
                         int64_t seq_len, const int64_t* p_off, const int* plen, const int64_t* t_off, const int* tlen,
                         int K) {
  int st = wfg_stage_pairs(c, n, seq_len, p_off, plen, t_off, tlen);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  IntPen p;
  st = validate_config(c, cfg, &p);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  const bool learned = sched == WFG_SCHED_LEARNED;
  if (!c->copy_stream) WFG_CHECK(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  while ((int)c->chunk_ev.size() < 2 * K) {
    cudaEvent_t e;
    WFG_CHECK(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->chunk_ev.push_back(e);
  }
  // chunk k = pairs [cb[k], cb[k+1]); its bytes all lie below hi[k]
  std::vector<int> cb((size_t)K + 1);
  std::vector<int64_t> hi((size_t)K);
  int64_t end = 0;
  const int head = n / kPipelineHeadDiv;
  for (int k = 0; k < K; ++k) {
    cb[(size_t)k] = k == 0 ? 0 : head + (int)((int64_t)(n - head) * (k - 1) / (K - 1));
    cb[(size_t)k + 1] = head + (int)((int64_t)(n - head) * k / (K - 1));
    for (int i = cb[(size_t)k]; i < cb[(size_t)k + 1]; ++i)
      end = std::max(end, std::max(p_off[i] + plen[i], t_off[i] + tlen[i]));
    hi[(size_t)k] = end;
  }
  c->stats = wfg_stats_t{};
  c->last_score_only = cfg->score_only;
  c->stats.h2d_bytes = seq_len + (int64_t)sizeof(PairDesc) * n + (learned ? 0 : (int64_t)sizeof(int) * n);
  // ---- host-side order of the sorted schedule: longest pairs first within each chunk
  if (!learned) {
    WFG_CHECK(c, c->h_order_pin.reserve((size_t)n));
    std::vector<int> cnt((size_t)c->max_sum + 2);
    for (int k = 0; k < K; ++k) {
      std::fill(cnt.begin(), cnt.end(), 0);
      const int a = cb[(size_t)k], b = cb[(size_t)k + 1];
      for (int i = a; i < b; ++i) cnt[(size_t)(c->max_sum - (plen[i] + tlen[i])) + 1]++;
      for (size_t v = 1; v < cnt.size(); ++v) cnt[v] += cnt[v - 1];
      for (int i = a; i < b; ++i) c->h_order_pin.ptr[a + cnt[(size_t)(c->max_sum - (plen[i] + tlen[i]))]++] = i;
    }
  } else {
    WFG_CHECK(c, c->d_pred.reserve((size_t)n));
    WFG_CHECK(c, c->d_feats.reserve((size_t)n * WFG_MODEL_FEATURES));
    WFG_CHECK(c, c->d_bin_work.reserve((size_t)sched_bin_words()));
    WFG_CHECK(c, c->h_bin_stats.reserve((size_t)4 * K));
  }
  // ---- arena: two regions, for consecutive chunks' first passes that overlap (even chunks on
  // the main stream, odd ones on the alternate stream), each sized for a first pass at the plain
  // ring cap; the retry passes use the whole arena after both streams join. A chunk whose
  // predictions need wider rings grows the regions between chunks.
  const int64_t budget = arena_budget_of(c) / 2;
  Launch retry[kNumPasses];
  const int64_t retry_need = plan_retry_passes(c, p, 2 * budget, retry);
  int64_t region = 0;
  {
    Launch l;
    l.count = cb[1] - cb[0];
    plan_first_pass(c, p, c->limit_ring_w, budget, l);
    region = wfg_align256(l.groups * l.L.total);
  }
  WFG_CHECK(c, c->d_arena.reserve((size_t)std::max(2 * region, retry_need)));
  WFG_CHECK(c, c->d_batch_heads.reserve((size_t)K));
  if (!c->alt_stream) WFG_CHECK(c, cudaStreamCreateWithFlags(&c->alt_stream, cudaStreamNonBlocking));
  // ---- copies
  cudaStream_t cs = c->copy_stream, ms = c->stream, as = c->aux_stream;
  WFG_CHECK(c, cudaEventRecord(c->ev[6], cs));
  WFG_CHECK(c, cudaMemcpyAsync(c->d_pairs.ptr, c->h_pairs_pinned.ptr, sizeof(PairDesc) * (size_t)n,
                               cudaMemcpyHostToDevice, cs));
  if (!learned)
    WFG_CHECK(c, cudaMemcpyAsync(c->d_order.ptr, c->h_order_pin.ptr, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                                 cs));
  int64_t lo = 0;
  for (int k = 0; k < K; ++k) {
    if (hi[(size_t)k] > lo)
      WFG_CHECK(c, cudaMemcpyAsync(c->d_seq.ptr + lo, seq + lo, (size_t)(hi[(size_t)k] - lo), cudaMemcpyHostToDevice,
                                   cs));
    lo = std::max(lo, hi[(size_t)k]);
    WFG_CHECK(c, cudaEventRecord(c->chunk_ev[(size_t)k], cs));
  }
  WFG_CHECK(c, cudaEventRecord(c->ev[7], cs));
  // ---- main stream prologue
  WFG_CHECK(c, cudaEventRecord(c->ev[0], ms));
  WFG_CHECK(c, cudaEventRecord(c->ev[1], ms));
  WFG_CHECK(c, cudaMemsetAsync(c->d_counters.ptr, 0, sizeof(unsigned long long) * kNumCounters, ms));
  WFG_CHECK(c, cudaMemsetAsync(c->d_batch_heads.ptr, 0, sizeof(unsigned long long) * (size_t)K, ms));
  WFG_CHECK(c, cudaEventRecord(c->ev[5], ms));
  WFG_CHECK(c, cudaStreamWaitEvent(as, c->ev[5], 0));  // the aux and alternate streams follow this run's start
  WFG_CHECK(c, cudaStreamWaitEvent(c->alt_stream, c->ev[5], 0));
  int launches = 0;
  int64_t first_warps = 0;
  int first_ring = 0;
  int64_t first_arena = 0;
  for (int k = 0; k < K; ++k) {
    const int a = cb[(size_t)k], m = cb[(size_t)k + 1] - a;
    cudaEvent_t ready = c->chunk_ev[(size_t)K + k];
    // aux: pack, and for the learned schedule features, predictions and the chunk's order
    WFG_CHECK(c, cudaStreamWaitEvent(as, c->chunk_ev[(size_t)k], 0));
    WFG_CHECK(c, launch_pack(m, c->d_seq.ptr, c->d_pairs.ptr + a, c->d_words.ptr, c->num_sms, as));
    ++launches;
    if (learned) {
      st = wfg_model_predict_range(c->model, c, a, m, as);
      if (st != WF_STATUS_ALG_COMPLETED) return st;
      int* stats = c->d_bin_work.ptr + sched_bin_words() - 4;
      WFG_CHECK(c, launch_bin_order(m, c->d_pred.ptr + a, INFINITY, 0, c->d_bin_work.ptr, stats, c->d_order.ptr + a,
                                    c->num_sms, as, a));
      WFG_CHECK(c, cudaMemcpyAsync(c->h_bin_stats.ptr + 4 * k, stats, sizeof(int) * 4, cudaMemcpyDeviceToHost, as));
      launches += 5;
    }
    WFG_CHECK(c, cudaEventRecord(ready, as));
    // host: the chunk's ring width from its largest prediction (learned), then its first pass
    Launch l;
    l.count = m;
    l.order_off = a;
    int hint = c->limit_ring_w;
    if (learned) {
      WFG_CHECK(c, cudaEventSynchronize(ready));
      float max_pred;
      memcpy(&max_pred, &c->h_bin_stats.ptr[4 * k + 2], sizeof(float));
      hint = (int)(c->tune.ring_margin * max_pred / p.emin) + 64;
    }
    plan_first_pass(c, p, hint, budget, l);
    if (l.groups * l.L.total > region) {
      // the earlier chunks' launches use the arena: wait for them, then grow both regions
      WFG_CHECK(c, cudaStreamSynchronize(ms));
      WFG_CHECK(c, cudaStreamSynchronize(c->alt_stream));
      region = wfg_align256(l.groups * l.L.total);
      WFG_CHECK(c, c->d_arena.reserve((size_t)std::max(2 * region, retry_need)));
    }
    l.arena_off = (k & 1) * region;
    const cudaStream_t ks = (k & 1) ? c->alt_stream : ms;
    WFG_CHECK(c, cudaStreamWaitEvent(ks, ready, 0));
    KernelParams kp = launch_params(c, cfg, p, l, 0);
    kp.num_pairs = m;
    kp.num_pairs_ptr = nullptr;
    kp.order = c->d_order.ptr + a;
    kp.queue_head = c->d_batch_heads.ptr + k;
    WFG_CHECK(c, launch_biwfa(kp, (int)(l.groups / biwfa_groups_per_block(l.gw, l.smem)), ks));
    ++launches;
    if (k == 0) { first_warps = l.groups * l.gw; first_ring = l.ring_w; first_arena = l.L.total; }
  }
  WFG_CHECK(c, cudaEventRecord(c->ev[4], c->alt_stream));
  WFG_CHECK(c, cudaStreamWaitEvent(ms, c->ev[4], 0));
  WFG_CHECK(c, cudaEventRecord(c->ev[2], ms));
  for (int ps = 1; ps < kNumPasses; ++ps) {
    const Launch& l = retry[ps];
    KernelParams kp = launch_params(c, cfg, p, l, ps);
    kp.num_pairs = n;
    kp.num_pairs_ptr = c->d_counters.ptr + (ps - 1) * kCountersPerPass + 1;
    kp.order = c->d_retry.ptr + (size_t)(ps - 1) * n;
    kp.queue_head = c->d_counters.ptr + ps * kCountersPerPass + 0;
    WFG_CHECK(c, launch_biwfa(kp, (int)(l.groups / biwfa_groups_per_block(l.gw, l.smem)), ms));
    ++launches;
  }
  WFG_CHECK(c, cudaEventRecord(c->ev[3], ms));
  WFG_CHECK(c, cudaMemcpyAsync(c->h_counters.ptr, c->d_counters.ptr, sizeof(unsigned long long) * kNumCounters,
                               cudaMemcpyDeviceToHost, ms));
  c->stats.used_graph = 0;
  c->stats.launches = launches;
  c->stats.num_warps = (int)first_warps;
  c->stats.ring_w = first_ring;
  c->stats.arena_bytes = first_arena;
  c->stats.pipeline_chunks = K;
  c->uploaded = true;
  c->ran = true;
  return WF_STATUS_ALG_COMPLETED;
}

}  // namespace

extern "C" {

int wfg_align_host(wfg_context_t* c, const wfg_config_t* cfg, wfg_sched_t sched, int n, const char* seq,
                   int64_t seq_len, const int64_t* p_off, const int* plen, const int64_t* t_off, const int* tlen,
                   int* scores, int* statuses, int64_t* run_off, int* run_len, uint32_t* runs, int64_t runs_cap,
                   int64_t* total_runs) {
  if (!c || !cfg || n < 0 || (n > 0 && (!seq || !p_off || !plen || !t_off || !tlen))) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  // Large batches on the persistent schedules overlap the input copy with the alignment (the
  // learned schedule with the context's model and a single-warp policy); the rest upload first.
  const bool single_warp_policy = c->tune.wide_warps <= 1 || c->tune.wide_threshold >= 3.0e38f;
  const bool pipelined = c->pipeline && n >= kPipelineMinPairs && c->force_gw == 1 && !c->force_smem &&
                         (sched == WFG_SCHED_SORTED || (sched == WFG_SCHED_LEARNED && c->model != nullptr &&
                                                        single_warp_policy));
  if (pipelined) {
    const int K = 2;
    const int st = align_host_pipelined(c, cfg, sched, n, seq, seq_len, p_off, plen, t_off, tlen, K);
    if (st != WF_STATUS_ALG_COMPLETED) return st;
    return wfg_fetch(c, scores, statuses, run_off, run_len, runs, runs_cap, total_runs);
  }
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
