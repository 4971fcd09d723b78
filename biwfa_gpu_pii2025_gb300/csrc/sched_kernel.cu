// Device-side binning of the learned schedule: from the predicted scores to the processing
// order, without a host round trip for the per-pair predictions.
//
// Pairs are ordered by predicted score, largest first (longest-processing-time-first for the
// persistent work queues), in buckets of 1/128 octave: bucket = floor(128 * log2(1 + score)).
// The first n_wide pairs of that order — at most wide_cap (one resident wave of the
// multi-warp shape), and only pairs whose bucket reaches the wide threshold's — form the
// multi-warp launch; the rest the single-warp launch. Order within a bucket is whatever the
// atomics give; the alignment results never depend on the order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "wfg_context.h"

namespace wfg {
namespace {

constexpr int kBuckets = 4096;
constexpr int kBinThreads = 256;

__device__ __forceinline__ int bucket_of(float pred) {
  const float s = fmaxf(pred, 0.f);  // NaN becomes 0
  const int b = (int)(__log2f(1.f + s) * 128.f);
  return b < 0 ? 0 : (b >= kBuckets ? kBuckets - 1 : b);
}

// Per-block histogram in shared memory, flushed to the global one; maximum prediction.
__global__ void __launch_bounds__(kBinThreads) bin_hist_kernel(int n, const float* __restrict__ pred,
                                                               int* __restrict__ hist, int* __restrict__ stats) {
  __shared__ int sh[kBuckets];
  __shared__ int smax;
  for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) sh[i] = 0;
  if (threadIdx.x == 0) smax = 0;
  __syncthreads();
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    atomicAdd(&sh[bucket_of(pred[i])], 1);
    m = max(m, __float_as_int(fmaxf(pred[i], 0.f)));  // non-negative floats order like their bits
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(&smax, m);
  __syncthreads();
  for (int i = threadIdx.x; i < kBuckets; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
  if (threadIdx.x == 0) atomicMax(&stats[2], smax);
}

// Exclusive scan from the top bucket down (write cursors), then the wide/narrow split:
// stats = {n_wide, n_narrow, max prediction (float bits), upper bound of the narrow
// launch's predictions (float bits)}.
__global__ void __launch_bounds__(1024) bin_scan_kernel(const int* __restrict__ hist, int* __restrict__ cursor,
                                                        int* __restrict__ stats, int n, int wide_cap,
                                                        int wide_bucket) {
  constexpr int kPer = kBuckets / 1024;  // 4 buckets per thread
  __shared__ int warp_sums[32];
  __shared__ int wide_avail;
  const int t = threadIdx.x;
  if (t == 0) wide_avail = 0;
  int local[kPer];
  int sum = 0;
  #pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int b = kBuckets - 1 - (t * kPer + j);  // rank order: top bucket first
    local[j] = hist[b];
    sum += local[j];
  }
  const int lane = t & 31, w = t >> 5;
  int incl = sum;
  #pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += v;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    int ws = warp_sums[lane];
    #pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, ws, d);
      if (lane >= d) ws += v;
    }
    warp_sums[lane] = ws;
  }
  __syncthreads();
  int run = incl - sum + (w > 0 ? warp_sums[w - 1] : 0);
  #pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int b = kBuckets - 1 - (t * kPer + j);
    cursor[b] = run;
    if (b == wide_bucket) wide_avail = run + local[j];  // pairs in buckets >= the threshold's
    run += local[j];
  }
  __syncthreads();
  if (t == 0) {
    const int avail = wide_bucket < kBuckets ? wide_avail : 0;
    const int nw = min(avail, wide_cap);
    stats[0] = nw;
    stats[1] = n - nw;
    // upper bound of the narrow predictions: the top of the bucket holding rank nw
    int ub_bucket = 0;
    for (int b = kBuckets - 1; b >= 0; --b) {
      if (hist[b] > 0 && cursor[b] + hist[b] > nw) { ub_bucket = b; break; }
    }
    stats[3] = __float_as_int(exp2f((ub_bucket + 1) / 128.f) - 1.f);
  }
}

__global__ void __launch_bounds__(kBinThreads) bin_scatter_kernel(int n, const float* __restrict__ pred,
                                                                  int* __restrict__ cursor, int* __restrict__ order,
                                                                  int base) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    order[atomicAdd(&cursor[bucket_of(pred[i])], 1)] = base + i;
}

}  // namespace

int sched_bin_words() { return 2 * kBuckets + 4; }

// work: sched_bin_words() ints of scratch; stats (device, 4 ints) as bin_scan_kernel writes
// them. wide_threshold: predicted score from which a pair may take the multi-warp launch;
// wide_cap: at most that many pairs do (0 disables the wide launch). order receives base + i
// for the n pairs pred[0..n) (base: the index of pred[0] in the batch).
cudaError_t launch_bin_order(int n, const float* pred, float wide_threshold, int wide_cap, int* work, int* stats,
                             int* order, int num_sms, cudaStream_t stream, int base) {
  int* hist = work;
  int* cursor = work + kBuckets;
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(int) * kBuckets, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(stats, 0, sizeof(int) * 4, stream);
  if (e != cudaSuccess) return e;
  if (n <= 0) return cudaSuccess;
  // the threshold's bucket, computed as the device computes buckets (kBuckets = none)
  int wide_bucket = kBuckets;
  if (wide_cap > 0 && wide_threshold < 3.0e38f) {
    const double b = std::log2(1.0 + (double)std::max(wide_threshold, 0.f)) * 128.0;
    wide_bucket = b >= kBuckets - 1 ? kBuckets - 1 : (int)b;
  }
  int blocks = (n + kBinThreads - 1) / kBinThreads;
  if (blocks > num_sms * 4) blocks = num_sms * 4;
  bin_hist_kernel<<<blocks, kBinThreads, 0, stream>>>(n, pred, hist, stats);
  bin_scan_kernel<<<1, 1024, 0, stream>>>(hist, cursor, stats, n, wide_cap, wide_bucket);
  bin_scatter_kernel<<<blocks, kBinThreads, 0, stream>>>(n, pred, cursor, order, base);
  return cudaGetLastError();
}

}  // namespace wfg
