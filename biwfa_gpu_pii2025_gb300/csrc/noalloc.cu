// wfg_align_noalloc: the batch aligner for callers that cannot allocate device memory.
//
// Some callers may not call cudaMalloc at all: code running inside a host framework
// that owns every device allocation (a memory pool or arena it must account for), or
// code that must not allocate while the framework runs latency-critical work. They own
// the inputs and outputs already; what they cannot provide is this library's scratch.
// This entry point therefore keeps all of its scratch — per-pair descriptors, packed
// sequences, the work queue and the per-warp BiWFA arenas — in one file-scope
// __device__ array of fixed size (kScratchBytes below, at most 32 MiB). Every GPU that loads
// the library holds that array until the process exits.
//
// Host code cannot use the array's name as a device address (it is a host-side
// stand-in), so the first call on each device, with that device current, looks the
// address up with cudaGetSymbolAddress and caches it. That first call should come
// before any stream capture. All calls share the one array and it keeps the last
// call's contents: the work-queue counters are cleared at the start of every call, and
// calls that overlap on the GPU (two streams, or two host threads) race on the array.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/wfa_gpu.h"
#include "wfg_internal.h"

namespace wfg {
cudaError_t launch_biwfa(const KernelParams& p, int grid, cudaStream_t stream);
int biwfa_warps_per_block();
cudaError_t launch_pack(int n, const uint8_t* ascii, PairDesc* pairs, uint32_t* words, int num_sms,
                        cudaStream_t stream);
}  // namespace wfg

using namespace wfg;

namespace {

// Limits of one call (also stated in include/wfa_gpu.h).
constexpr int kMaxPairs = WFG_NOALLOC_MAX_PAIRS;        // 4096
constexpr int kMaxPairLen = WFG_NOALLOC_MAX_PAIR_LEN;   // plen + tlen <= 1024
constexpr int kMaxScope = 16;                           // max(o+e, x) + 1 after the match transform
constexpr int kWarps = 16;                              // resident warps of the aligner launch
constexpr int kRingW = 2048;                            // >= kMaxPairLen + 8, power of two
constexpr int kLeafWords = 1 << 17;                     // leaf offsets per warp (512 KiB)
// Leaf descriptors for every score a unidirectional leaf can reach under any accepted
// penalties (the batch path's bound, max(520, 100 x + o + 100 max(o, e) + scope) + 8, at its
// largest for scope <= 16: x = 15, o = 14, e = 1). A leaf whose offsets outgrow kLeafWords
// ends its pair with WF_STATUS_OOM (the batch path would finish it in a retry pass).
constexpr int kLeafMaxScore = 15 * 100 + 14 + 14 * 100 + kMaxScope + 8;
constexpr int kRunCap = kMaxPairLen + 2;
constexpr int kStackCap = 64;
// One fixed slot of packed words per pair: 2 x ((plen+3)/4 + 2) + 2 x ((tlen+3)/4 + 2).
constexpr int64_t kWordsPerPair = 2 * ((kMaxPairLen + 3) / 4 + 2) + 8;

constexpr int64_t kHeaderBytes = 256;                                  // counters
constexpr int64_t kDescBytes = wfg_align256((int64_t)kMaxPairs * (int64_t)sizeof(PairDesc));
constexpr int64_t kOrderBytes = wfg_align256((int64_t)kMaxPairs * 4);
constexpr int64_t kWordBytes = wfg_align256((int64_t)kMaxPairs * kWordsPerPair * 4);
constexpr int64_t kArenaBytes =
    wfg_arena_layout(kMaxScope, kRingW, kLeafMaxScore, kLeafWords, kRunCap, kRunCap, kStackCap).total;
constexpr int64_t kScratchBytes = kHeaderBytes + kDescBytes + kOrderBytes + kWordBytes + kWarps * kArenaBytes;
static_assert(kScratchBytes <= (int64_t)32 << 20, "no-alloc scratch above its stated 32 MiB");

// The scratch. Device code may name it; host code must use its looked-up address.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint8_t* g_scratch_addr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Per-pair descriptors in fixed word slots; pairs outside the limits are answered with
// WF_STATUS_UNSUPPORTED here and kept out of the work queue.
__global__ void noalloc_setup_kernel(int n, const int64_t* __restrict__ p_off, const int* __restrict__ plen,
                                     const int64_t* __restrict__ t_off, const int* __restrict__ tlen,
                                     PairDesc* __restrict__ descs, int* __restrict__ order,
                                     unsigned long long* __restrict__ queue_len, int* __restrict__ scores,
                                     int* __restrict__ status, int64_t* __restrict__ run_off,
                                     int* __restrict__ run_len) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int pl = plen[i], tl = tlen[i];
    if (pl < 0 || tl < 0 || (int64_t)pl + tl > kMaxPairLen || p_off[i] < 0 || t_off[i] < 0) {
      // An empty descriptor, so packing reads no bytes for this pair.
      PairDesc z;
      z.word_off = (int64_t)i * kWordsPerPair;
      z.p_off = 0; z.t_off = 0; z.plen = 0; z.tlen = 0; z.pw_len = 2; z.tw_len = 2; z.bits = 8; z.pad = 0;
      descs[i] = z;
      scores[i] = 0;
      status[i] = WF_STATUS_UNSUPPORTED;
      run_off[i] = 0;
      run_len[i] = 0;
      continue;
    }
    PairDesc d;
    d.word_off = (int64_t)i * kWordsPerPair;
    d.p_off = p_off[i];
    d.t_off = t_off[i];
    d.plen = pl;
    d.tlen = tl;
    d.pw_len = (pl + 3) / 4 + 2;
    d.tw_len = (tl + 3) / 4 + 2;
    d.bits = 8;
    d.pad = 0;
    descs[i] = d;
    const unsigned long long slot = atomicAdd(queue_len, 1ull);
    order[slot] = i;
  }
}

// Scratch exhaustion inside the fixed arenas is reported as WF_STATUS_OOM, like the
// batch path does for pairs that outgrow every arena it tries.
__global__ void noalloc_finish_kernel(int n, int* __restrict__ status) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = status[i];
    if (s == WFG_ST_SCRATCH_OVERFLOW || s == WFG_ST_OUTPUT_OVERFLOW) status[i] = WF_STATUS_OOM;
  }
}

int setup_device(int device) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (device < 0 || device >= kMaxDevices) return WF_STATUS_DEVICE_ERROR;
  if (g_scratch_addr[device] != nullptr) return WF_STATUS_ALG_COMPLETED;
  void* addr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
  if (e != cudaSuccess || addr == nullptr) {
    fprintf(stderr, "[WFA-GB300] wfg_align_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
    return WF_STATUS_DEVICE_ERROR;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  g_num_sms[device] = sms > 0 ? sms : 1;
  g_scratch_addr[device] = (uint8_t*)addr;
  return WF_STATUS_ALG_COMPLETED;
}

}  // namespace

extern "C" int wfg_align_noalloc(const wfg_config_t* cfg, int num_pairs, const char* d_seq,
                                 const int64_t* d_p_off, const int* d_plen, const int64_t* d_t_off,
                                 const int* d_tlen, int* d_scores, int* d_status, int64_t* d_run_off,
                                 int* d_run_len, uint32_t* d_runs, int64_t runs_cap, void* stream_handle) {
  if (cfg == nullptr || num_pairs < 0) return WF_STATUS_UNSUPPORTED;
  if (num_pairs > kMaxPairs) {
    fprintf(stderr, "[WFA-GB300] wfg_align_noalloc: %d pairs exceed the limit of %d per call\n", num_pairs,
            kMaxPairs);
    return WF_STATUS_UNSUPPORTED;
  }
  if (cfg->metric != WFG_METRIC_GAP_AFFINE || cfg->match > 0 || cfg->mismatch <= 0 || cfg->gap_opening < 0 ||
      cfg->gap_extension <= 0) {
    fprintf(stderr, "[WFA-GB300] wfg_align_noalloc: gap-affine penalties with match <= 0 only\n");
    return WF_STATUS_UNSUPPORTED;
  }
  int x, o, e;
  if (cfg->match < 0) {
    x = 2 * cfg->mismatch - 2 * cfg->match; o = 2 * cfg->gap_opening; e = 2 * cfg->gap_extension - cfg->match;
  } else {
    x = cfg->mismatch; o = cfg->gap_opening; e = cfg->gap_extension;
  }
  const int scope = (o + e > x ? o + e : x) + 1;
  if (scope > kMaxScope) {
    fprintf(stderr, "[WFA-GB300] wfg_align_noalloc: penalties give a score scope of %d (limit %d)\n", scope,
            kMaxScope);
    return WF_STATUS_UNSUPPORTED;
  }
  if (num_pairs == 0) return WF_STATUS_ALG_COMPLETED;
  if (!d_seq || !d_p_off || !d_plen || !d_t_off || !d_tlen || !d_scores || !d_status || !d_run_off ||
      !d_run_len || (!cfg->score_only && !d_runs))
    return WF_STATUS_UNSUPPORTED;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return WF_STATUS_DEVICE_ERROR;
  const int st = setup_device(device);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  cudaStream_t stream = (cudaStream_t)stream_handle;

  uint8_t* base = g_scratch_addr[device];
  unsigned long long* counters = (unsigned long long*)base;  // [0] queue length, [1] queue head, [2] output head
  PairDesc* descs = (PairDesc*)(base + kHeaderBytes);
  int* order = (int*)(base + kHeaderBytes + kDescBytes);
  uint32_t* words = (uint32_t*)(base + kHeaderBytes + kDescBytes + kOrderBytes);
  uint8_t* arenas = base + kHeaderBytes + kDescBytes + kOrderBytes + kWordBytes;

  if (cudaMemsetAsync(counters, 0, kHeaderBytes, stream) != cudaSuccess) return WF_STATUS_DEVICE_ERROR;
  const int threads = 256;
  const int blocks = (num_pairs + threads - 1) / threads;
  noalloc_setup_kernel<<<blocks, threads, 0, stream>>>(num_pairs, d_p_off, d_plen, d_t_off, d_tlen, descs, order,
                                                        &counters[0], d_scores, d_status, d_run_off, d_run_len);
  if (cudaGetLastError() != cudaSuccess) return WF_STATUS_DEVICE_ERROR;
  // Refused pairs carry empty descriptors and stay out of the work queue.
  if (launch_pack(num_pairs, (const uint8_t*)d_seq, descs, words, g_num_sms[device], stream) != cudaSuccess)
    return WF_STATUS_DEVICE_ERROR;

  KernelParams kp{};
  kp.x = x; kp.o = o; kp.e = e; kp.scope = scope;
  kp.match_o = cfg->match; kp.x_o = cfg->mismatch; kp.o_o = cfg->gap_opening; kp.e_o = cfg->gap_extension;
  kp.score_only = cfg->score_only;
  kp.max_steps = cfg->max_alignment_steps > 0 ? cfg->max_alignment_steps : INT_MAX;
  kp.num_pairs = num_pairs;
  kp.num_pairs_ptr = &counters[0];
  kp.pairs = descs;
  kp.order = order;
  kp.retry_out = nullptr;
  kp.retry_count = nullptr;
  kp.queue_head = &counters[1];
  kp.words = words;
  kp.arena = arenas;
  kp.arena_bytes = kArenaBytes;
  kp.ring_w = kRingW;
  kp.leaf_words = kLeafWords;
  kp.leaf_max_score = kLeafMaxScore;
  kp.run_cap = kRunCap;
  kp.leaf_run_cap = kRunCap;
  kp.stack_cap = kStackCap;
  kp.scores = d_scores;
  kp.status = d_status;
  kp.run_off = d_run_off;
  kp.run_len = d_run_len;
  kp.out_runs = d_runs;
  kp.out_cap = cfg->score_only ? 0 : runs_cap;
  kp.out_head = &counters[2];
  kp.stats = nullptr;
  if (launch_biwfa(kp, kWarps / biwfa_warps_per_block(), stream) != cudaSuccess) return WF_STATUS_DEVICE_ERROR;
  noalloc_finish_kernel<<<blocks, threads, 0, stream>>>(num_pairs, d_status);
  if (cudaGetLastError() != cudaSuccess) return WF_STATUS_DEVICE_ERROR;
  return WF_STATUS_ALG_COMPLETED;
}
