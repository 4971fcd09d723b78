// Autotuner of the learned schedule: whether the heaviest predicted pairs (at most one
// resident wave of the multi-warp shape, from a predicted-score threshold up) run with several
// warps per pair, and with their rings in shared memory, trades per-pair latency against pairs
// in flight and depends on the batch, so it is measured rather than modelled. Each candidate
// policy runs the resident batch twice; the time of the second run decides.
#include <cuda_runtime.h>

#include <cfloat>
#include <vector>

#include "../../include/wfa_gpu.h"
#include "wfg_context.h"

extern "C" int wfg_autotune_learned_policy(wfg_context_t* c, const wfg_config_t* cfg, float* best_ms,
                                           float* best_threshold, int* best_warps, int* best_smem) {
  if (!c || !cfg || !c->model) return WF_STATUS_UNSUPPORTED;
  struct Cand { float thr; int gw; int smem; };
  std::vector<Cand> cands;
  cands.push_back({FLT_MAX, 8, 0});  // no wide launch
  for (float thr : {1200.f, 2400.f, 4800.f}) {
    cands.push_back({thr, 8, 1});
    cands.push_back({thr, 8, 0});
    cands.push_back({thr, 4, 0});
  }
  const auto saved = c->tune;
  float best = FLT_MAX;
  Cand pick = cands[0];
  cudaEvent_t e0, e1;
  WFG_CHECK(c, cudaEventCreate(&e0));
  WFG_CHECK(c, cudaEventCreate(&e1));
  int st = WF_STATUS_ALG_COMPLETED;
  for (size_t i = 0; i < cands.size() && st == WF_STATUS_ALG_COMPLETED; ++i) {
    c->tune.wide_threshold = cands[i].thr;
    c->tune.wide_warps = cands[i].gw;
    c->tune.wide_smem = cands[i].smem;
    float ms = 0.f;
    for (int rep = 0; rep < 2 && st == WF_STATUS_ALG_COMPLETED; ++rep) {
      if (cudaEventRecord(e0, c->stream) != cudaSuccess) { st = WF_STATUS_DEVICE_ERROR; break; }
      st = wfg_run(c, cfg, WFG_SCHED_LEARNED);
      if (st != WF_STATUS_ALG_COMPLETED) break;
      if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        st = WF_STATUS_DEVICE_ERROR;
      }
    }
    if (st == WF_STATUS_ALG_COMPLETED && ms < best) {
      best = ms;
      pick = cands[i];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != WF_STATUS_ALG_COMPLETED) {
    c->tune = saved;
    return st;
  }
  c->tune = saved;
  c->tune.wide_threshold = pick.thr;
  c->tune.wide_warps = pick.gw;
  c->tune.wide_smem = pick.smem;
  if (best_ms) *best_ms = best;
  if (best_threshold) *best_threshold = pick.thr;
  if (best_warps) *best_warps = pick.gw;
  if (best_smem) *best_smem = pick.smem;
  return WF_STATUS_ALG_COMPLETED;
}
