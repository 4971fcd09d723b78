// Learned scheduling: per-pair sketch features and a small MLP that predicts each pair's
// alignment score. The prediction only orders and bins pairs and sizes scratch; it never
// changes a result (a mispredicted pair overflows into a larger-arena pass).
//
// Features (32 per pair, bf16):
//   f0  log2(|P|+1)/16          f1  log2(|T|+1)/16        f2  (|P|-|T|)/(|P|+|T|+1)
//   f3..f30  histogram of the 256 per-4-mer count differences |cP[k]-cT[k]| in 28 bins
//            (d = 0..15 one bin each, then one bin per power of two up to 2^15), / 256
//   f31 the 4-mer count L1 distance sum_k |cP[k]-cT[k]| / (|P|+|T|+1)
// Network: 32 -> 64 -> 64 -> 1, ReLU, bf16 weights and activations between layers, fp32
// accumulation (mma.sync m16n8k16 bf16 -> f32), target log(1 + |score|).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "wfg_internal.h"

namespace wfg {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kIn = 32, kHid = 64;

__device__ __forceinline__ int kmer_bin(int d) {
  if (d < 16) return d;
  const int lg = 31 - __clz(d);  // >= 4
  return min(27, 16 + (lg - 4));
}

// One warp per pair: 4-mer counts of both sequences in shared memory, then the features.
template <int WPB>
__global__ void __launch_bounds__(WPB * 32) kmer_features_kernel(int n, const uint8_t* __restrict__ ascii,
                                                                const PairDesc* __restrict__ pairs,
                                                                __nv_bfloat16* __restrict__ feats) {
  __shared__ int s_cnt[WPB][2][256];
  __shared__ int s_hist[WPB][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  for (long long i = (long long)blockIdx.x * WPB + wib; i < n; i += (long long)gridDim.x * WPB) {
    const PairDesc pd = pairs[i];
    for (int k = lane; k < 512; k += 32) (&s_cnt[wib][0][0])[k] = 0;
    s_hist[wib][lane] = 0;
    __syncwarp();
    for (int side = 0; side < 2; ++side) {
      const uint8_t* s = ascii + (side ? pd.t_off : pd.p_off);
      const int len = side ? pd.tlen : pd.plen;
      for (int j = lane; j + 3 < len; j += 32) {
        const int code = (((s[j] >> 1) & 3) << 6) | (((s[j + 1] >> 1) & 3) << 4) | (((s[j + 2] >> 1) & 3) << 2) |
                         ((s[j + 3] >> 1) & 3);
        atomicAdd(&s_cnt[wib][side][code], 1);
      }
    }
    __syncwarp();
    int l1 = 0;
    for (int k = lane; k < 256; k += 32) {
      const int d = abs(s_cnt[wib][0][k] - s_cnt[wib][1][k]);
      l1 += d;
      atomicAdd(&s_hist[wib][kmer_bin(d)], 1);
    }
    l1 = __reduce_add_sync(kFull, l1);
    __syncwarp();
    const float tot = (float)(pd.plen + pd.tlen + 1);
    float f;
    if (lane == 0) f = log2f((float)pd.plen + 1.f) * (1.f / 16.f);
    else if (lane == 1) f = log2f((float)pd.tlen + 1.f) * (1.f / 16.f);
    else if (lane == 2) f = (float)(pd.plen - pd.tlen) / tot;
    else if (lane < 31) f = (float)s_hist[wib][lane - 3] * (1.f / 256.f);
    else f = (float)l1 / tot;
    feats[i * kIn + lane] = __float2bfloat16(f);
    __syncwarp();
  }
}

// Parameters: fp32 master copy in one block {W1[32][64] (in-major), b1[64], W2[64][64], b2[64],
// w3[64], b3}; bf16 copies of the weight matrices transposed to [out][in] (mma B operands).
struct MlpParams {
  const float* master;            // kParamCount floats
  const __nv_bfloat16* w1t;       // [64][32]
  const __nv_bfloat16* w2t;       // [64][64]
};
constexpr int kOffW1 = 0, kOffB1 = kIn * kHid, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid, kParamCount = kOffB3 + 1;
// Per-warp staging floats of the train step: h1, dh2 (16 x 64 each), x (16 x 32), dy (16),
// the bf16 input tile (16 x 32 bf16 = 256 floats).
constexpr int kTrainWarpFloats = 32 * kHid + 16 * kIn + 16 + (16 * kIn) / 2;
constexpr int kTrainWpb = 4;
constexpr size_t kTrainSmemBytes =
    sizeof(float) * ((size_t)kHid * kHid + ((kParamCount + 3) & ~3) + (size_t)kTrainWpb * kTrainWarpFloats);

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Forward of one 16-row tile by one warp. Fragment layouts of m16n8k16 (g = lane/4, t = lane%4):
// A rows g / g+8, columns 2t..2t+1 and 2t+8..2t+9; B (col) rows 2t..2t+1 and 2t+8..2t+9 of
// column g; C rows g / g+8, columns 2t..2t+1. Layer outputs in C layout are re-packed in
// registers as the next layer's A fragments (two 8-column tiles form one 16-column k-step).
struct TileAct {
  float h1[8][4];   // layer-1 outputs after ReLU, as bf16-rounded floats (8 n-tiles)
  float h2[8][4];   // layer-2 outputs after ReLU
  float y[2];       // rows g and g+8 (valid in every lane of the group)
};

__device__ __forceinline__ void mlp_tile_forward(const __nv_bfloat16* __restrict__ x, int row0, int n,
                                                 const __nv_bfloat16* s_w1t, const __nv_bfloat16* s_w2t,
                                                 const float* s_b1, const float* s_b2, const float* s_w3,
                                                 float b3, int lane, TileAct& act) {
  const int g = lane >> 2, t = lane & 3;
  const int r0 = row0 + g, r1 = row0 + g + 8;
  // A fragments of the input tile (2 k-steps of 16 features)
  uint32_t a[2][4];
  for (int ks = 0; ks < 2; ++ks) {
    const int c0 = ks * 16 + 2 * t;
    auto ld = [&](int r, int c) -> uint32_t {
      if (r >= n) return 0u;
      return *reinterpret_cast<const uint32_t*>(x + (size_t)r * kIn + c);
    };
    a[ks][0] = ld(r0, c0);
    a[ks][1] = ld(r1, c0);
    a[ks][2] = ld(r0, c0 + 8);
    a[ks][3] = ld(r1, c0 + 8);
  }
  // Layer 1: 8 n-tiles of 8 outputs
  for (int j = 0; j < 8; ++j) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const int col = j * 8 + g;  // B column held by this lane
    for (int ks = 0; ks < 2; ++ks) {
      const __nv_bfloat16* wrow = s_w1t + col * kIn + ks * 16 + 2 * t;
      mma_bf16(d, a[ks], *reinterpret_cast<const uint32_t*>(wrow), *reinterpret_cast<const uint32_t*>(wrow + 8));
    }
    const int c = j * 8 + 2 * t;
    act.h1[j][0] = __bfloat162float(__float2bfloat16(fmaxf(d[0] + s_b1[c], 0.f)));
    act.h1[j][1] = __bfloat162float(__float2bfloat16(fmaxf(d[1] + s_b1[c + 1], 0.f)));
    act.h1[j][2] = __bfloat162float(__float2bfloat16(fmaxf(d[2] + s_b1[c], 0.f)));
    act.h1[j][3] = __bfloat162float(__float2bfloat16(fmaxf(d[3] + s_b1[c + 1], 0.f)));
  }
  // Layer 2: A from layer-1 tiles (2j, 2j+1) per k-step
  uint32_t a2[4][4];
  for (int ks = 0; ks < 4; ++ks) {
    a2[ks][0] = pack_bf16x2(act.h1[2 * ks][0], act.h1[2 * ks][1]);
    a2[ks][1] = pack_bf16x2(act.h1[2 * ks][2], act.h1[2 * ks][3]);
    a2[ks][2] = pack_bf16x2(act.h1[2 * ks + 1][0], act.h1[2 * ks + 1][1]);
    a2[ks][3] = pack_bf16x2(act.h1[2 * ks + 1][2], act.h1[2 * ks + 1][3]);
  }
  float y0 = 0.f, y1 = 0.f;
  for (int j = 0; j < 8; ++j) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const int col = j * 8 + g;
    for (int ks = 0; ks < 4; ++ks) {
      const __nv_bfloat16* wrow = s_w2t + col * kHid + ks * 16 + 2 * t;
      mma_bf16(d, a2[ks], *reinterpret_cast<const uint32_t*>(wrow), *reinterpret_cast<const uint32_t*>(wrow + 8));
    }
    const int c = j * 8 + 2 * t;
    act.h2[j][0] = fmaxf(d[0] + s_b2[c], 0.f);
    act.h2[j][1] = fmaxf(d[1] + s_b2[c + 1], 0.f);
    act.h2[j][2] = fmaxf(d[2] + s_b2[c], 0.f);
    act.h2[j][3] = fmaxf(d[3] + s_b2[c + 1], 0.f);
    y0 += act.h2[j][0] * s_w3[c] + act.h2[j][1] * s_w3[c + 1];
    y1 += act.h2[j][2] * s_w3[c] + act.h2[j][3] * s_w3[c + 1];
  }
  // Layer 3: reduce the 4 lanes of a group (columns 2t..2t+1 of every tile)
  y0 += __shfl_xor_sync(kFull, y0, 1); y0 += __shfl_xor_sync(kFull, y0, 2);
  y1 += __shfl_xor_sync(kFull, y1, 1); y1 += __shfl_xor_sync(kFull, y1, 2);
  act.y[0] = y0 + b3;
  act.y[1] = y1 + b3;
}

template <int WPB>
__device__ __forceinline__ void load_params_smem(const MlpParams& prm, __nv_bfloat16* s_w1t, __nv_bfloat16* s_w2t,
                                                 float* s_b1, float* s_b2, float* s_w3) {
  for (int i = threadIdx.x; i < kHid * kIn; i += WPB * 32) s_w1t[i] = prm.w1t[i];
  for (int i = threadIdx.x; i < kHid * kHid; i += WPB * 32) s_w2t[i] = prm.w2t[i];
  for (int i = threadIdx.x; i < kHid; i += WPB * 32) {
    s_b1[i] = prm.master[kOffB1 + i];
    s_b2[i] = prm.master[kOffB2 + i];
    s_w3[i] = prm.master[kOffW3 + i];
  }
  __syncthreads();
}

// Inference: y[i] = MLP(features[i]) (log-score), and the predicted score expm1(y) >= 0.
template <int WPB>
__global__ void __launch_bounds__(WPB * 32) mlp_forward_kernel(int n, const __nv_bfloat16* __restrict__ x,
                                                              MlpParams prm, float* __restrict__ y_out,
                                                              float* __restrict__ score_out) {
  __shared__ __align__(16) __nv_bfloat16 s_w1t[kHid * kIn];
  __shared__ __align__(16) __nv_bfloat16 s_w2t[kHid * kHid];
  __shared__ float s_b1[kHid], s_b2[kHid], s_w3[kHid];
  load_params_smem<WPB>(prm, s_w1t, s_w2t, s_b1, s_b2, s_w3);
  const float b3 = prm.master[kOffB3];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int tiles = (n + 15) / 16;
  for (int tile = blockIdx.x * WPB + wib; tile < tiles; tile += gridDim.x * WPB) {
    TileAct act;
    mlp_tile_forward(x, tile * 16, n, s_w1t, s_w2t, s_b1, s_b2, s_w3, b3, lane, act);
    if (t == 0) {
      const int r0 = tile * 16 + g, r1 = r0 + 8;
      if (r0 < n) { if (y_out) y_out[r0] = act.y[0]; if (score_out) score_out[r0] = fmaxf(expm1f(act.y[0]), 0.f); }
      if (r1 < n) { if (y_out) y_out[r1] = act.y[1]; if (score_out) score_out[r1] = fmaxf(expm1f(act.y[1]), 0.f); }
    }
  }
}

// Training step: forward (tensor cores) + backward (fp32) of the mean-squared error on a
// minibatch of rows [row_begin, row_begin + rows); gradients are summed into grad (zeroed by
// the caller). Per warp: one 16-row tile at a time, activations staged in shared memory.
template <int WPB>
__global__ void __launch_bounds__(WPB * 32) mlp_train_step_kernel(const __nv_bfloat16* __restrict__ x,
                                                                 const float* __restrict__ target,
                                                                 const int* __restrict__ rows_idx, int rows,
                                                                 MlpParams prm, float* __restrict__ grad,
                                                                 float* __restrict__ loss_sum) {
  __shared__ __align__(16) __nv_bfloat16 s_w1t[kHid * kIn];
  __shared__ __align__(16) __nv_bfloat16 s_w2t[kHid * kHid];
  __shared__ float s_b1[kHid], s_b2[kHid], s_w3[kHid];
  // Dynamic shared memory (train_step_smem_bytes): fp32 W2 [in][out] for dH1, the block's
  // gradient accumulator, and per-warp staging of one 16-row tile.
  extern __shared__ __align__(16) float s_dyn[];
  float* s_w2 = s_dyn;                                       // kHid*kHid
  float* s_g = s_w2 + kHid * kHid;                           // kParamCount (padded to 4)
  float* s_warp = s_g + ((kParamCount + 3) & ~3);
  const int wib0 = threadIdx.x >> 5;
  float (*s_h1_w)[kHid] = reinterpret_cast<float (*)[kHid]>(s_warp + wib0 * kTrainWarpFloats);
  float (*s_dh2_w)[kHid] = reinterpret_cast<float (*)[kHid]>(s_warp + wib0 * kTrainWarpFloats + 16 * kHid);
  float (*s_xin_w)[kIn] = reinterpret_cast<float (*)[kIn]>(s_warp + wib0 * kTrainWarpFloats + 32 * kHid);
  float* s_dy_w = s_warp + wib0 * kTrainWarpFloats + 32 * kHid + 16 * kIn;
  __nv_bfloat16* s_xt_w = reinterpret_cast<__nv_bfloat16*>(s_warp + wib0 * kTrainWarpFloats + 32 * kHid + 16 * kIn + 16);
  load_params_smem<WPB>(prm, s_w1t, s_w2t, s_b1, s_b2, s_w3);
  for (int i = threadIdx.x; i < kHid * kHid; i += WPB * 32) s_w2[i] = prm.master[kOffW2 + i];
  for (int i = threadIdx.x; i < kParamCount; i += WPB * 32) s_g[i] = 0.f;
  __syncthreads();
  const float b3 = prm.master[kOffB3];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const float inv_rows = 1.f / (float)rows;
  float lsum = 0.f;
  const int tiles = (rows + 15) / 16;
  for (int tile = blockIdx.x * WPB + wib; tile < tiles; tile += gridDim.x * WPB) {
    // gather the tile's rows
    for (int e = lane; e < 16 * kIn; e += 32) {
      const int r = e / kIn, c = e % kIn;
      const int rr = tile * 16 + r;
      __nv_bfloat16 v = __float2bfloat16(0.f);
      if (rr < rows) v = x[(size_t)rows_idx[rr] * kIn + c];
      s_xt_w[e] = v;
      s_xin_w[r][c] = __bfloat162float(v);
    }
    __syncwarp();
    const int valid = min(16, rows - tile * 16);
    TileAct act;
    mlp_tile_forward(s_xt_w, 0, valid, s_w1t, s_w2t, s_b1, s_b2, s_w3, b3, lane, act);
    // dL/dy = 2 (y - target) / rows
    float dy0 = 0.f, dy1 = 0.f;
    if (g < valid) { const float e0 = act.y[0] - target[rows_idx[tile * 16 + g]]; dy0 = 2.f * e0 * inv_rows; if (t == 0) lsum += e0 * e0; }
    if (g + 8 < valid) { const float e1 = act.y[1] - target[rows_idx[tile * 16 + g + 8]]; dy1 = 2.f * e1 * inv_rows; if (t == 0) lsum += e1 * e1; }
    if (t == 0) { s_dy_w[g] = dy0; s_dy_w[g + 8] = dy1; }
    // stage h1 and dh2 = dy * w3 * (h2 > 0); accumulate dW3, db3
    for (int j = 0; j < 8; ++j) {
      const int c = j * 8 + 2 * t;
      s_h1_w[g][c] = act.h1[j][0]; s_h1_w[g][c + 1] = act.h1[j][1];
      s_h1_w[g + 8][c] = act.h1[j][2]; s_h1_w[g + 8][c + 1] = act.h1[j][3];
      s_dh2_w[g][c] = act.h2[j][0] > 0.f ? dy0 * s_w3[c] : 0.f;
      s_dh2_w[g][c + 1] = act.h2[j][1] > 0.f ? dy0 * s_w3[c + 1] : 0.f;
      s_dh2_w[g + 8][c] = act.h2[j][2] > 0.f ? dy1 * s_w3[c] : 0.f;
      s_dh2_w[g + 8][c + 1] = act.h2[j][3] > 0.f ? dy1 * s_w3[c + 1] : 0.f;
      float gw0 = act.h2[j][0] * dy0 + act.h2[j][2] * dy1;
      float gw1 = act.h2[j][1] * dy0 + act.h2[j][3] * dy1;
      // sum over the 8 row-groups (lanes with equal t)
      for (int off = 4; off < 32; off <<= 1) {
        gw0 += __shfl_xor_sync(kFull, gw0, off);
        gw1 += __shfl_xor_sync(kFull, gw1, off);
      }
      if (g == 0) { atomicAdd(&s_g[kOffW3 + c], gw0); atomicAdd(&s_g[kOffW3 + c + 1], gw1); }
    }
    if (lane == 0) {
      float db3 = 0.f;
      for (int r = 0; r < 16; ++r) db3 += s_dy_w[r];
      atomicAdd(&s_g[kOffB3], db3);
    }
    __syncwarp();
    // dW2[i][j] = sum_r h1[r][i] dh2[r][j]; db2[j] = sum_r dh2[r][j]; lane owns 2 columns j
    for (int jj = 0; jj < 2; ++jj) {
      const int j = lane * 2 + jj;
      float db2 = 0.f;
      for (int r = 0; r < 16; ++r) db2 += s_dh2_w[r][j];
      atomicAdd(&s_g[kOffB2 + j], db2);
      for (int i = 0; i < kHid; ++i) {
        float acc = 0.f;
        for (int r = 0; r < 16; ++r) acc += s_h1_w[r][i] * s_dh2_w[r][j];
        atomicAdd(&s_g[kOffW2 + i * kHid + j], acc);
      }
    }
    // dh1[r][i] = (h1 > 0) * sum_j dh2[r][j] W2[i][j]; dW1[f][i] = sum_r x[r][f] dh1[r][i]
    for (int ii = 0; ii < 2; ++ii) {
      const int i = lane * 2 + ii;
      float dh1[16];
      for (int r = 0; r < 16; ++r) {
        float acc = 0.f;
        for (int j = 0; j < kHid; ++j) acc += s_dh2_w[r][j] * s_w2[i * kHid + j];
        dh1[r] = s_h1_w[r][i] > 0.f ? acc : 0.f;
      }
      float db1 = 0.f;
      for (int r = 0; r < 16; ++r) db1 += dh1[r];
      atomicAdd(&s_g[kOffB1 + i], db1);
      for (int f = 0; f < kIn; ++f) {
        float acc = 0.f;
        for (int r = 0; r < 16; ++r) acc += s_xin_w[r][f] * dh1[r];
        atomicAdd(&s_g[kOffW1 + f * kHid + i], acc);
      }
    }
    __syncwarp();
  }
  lsum = __reduce_add_sync(kFull, (int)0) + lsum;  // keep warps converged
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(kFull, lsum, off);
  if (lane == 0 && loss_sum) atomicAdd(loss_sum, lsum);
  __syncthreads();
  for (int i = threadIdx.x; i < kParamCount; i += WPB * 32) atomicAdd(&grad[i], s_g[i]);
}

// Adam update of the fp32 master parameters, then the bf16 transposed weight copies.
// step points at the 1-based Adam step count in device memory, so a captured training
// epoch replays with fresh bias corrections; the last block advances it.
__global__ void mlp_adam_kernel(float* __restrict__ master, const float* __restrict__ grad, float* __restrict__ m,
                                float* __restrict__ v, float lr, float beta1, float beta2, float eps,
                                const int* __restrict__ step, __nv_bfloat16* __restrict__ w1t,
                                __nv_bfloat16* __restrict__ w2t) {
  const float t = (float)(*step);
  const float bc1 = 1.f - powf(beta1, t), bc2 = 1.f - powf(beta2, t);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParamCount; i += gridDim.x * blockDim.x) {
    const float gi = grad[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float p = master[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    master[i] = p;
    if (i < kOffB1) { const int f = i / kHid, o = i % kHid; w1t[o * kIn + f] = __float2bfloat16(p); }
    else if (i >= kOffW2 && i < kOffB2) { const int a = (i - kOffW2) / kHid, o = (i - kOffW2) % kHid; w2t[o * kHid + a] = __float2bfloat16(p); }
  }
}

// bf16 transposed copies of the weight matrices from the fp32 master (after init or load).
__global__ void mlp_sync_bf16_kernel(const float* __restrict__ master, __nv_bfloat16* __restrict__ w1t,
                                     __nv_bfloat16* __restrict__ w2t) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kIn * kHid + kHid * kHid; i += gridDim.x * blockDim.x) {
    if (i < kIn * kHid) { const int f = i / kHid, o = i % kHid; w1t[o * kIn + f] = __float2bfloat16(master[kOffW1 + i]); }
    else { const int k = i - kIn * kHid; const int a = k / kHid, o = k % kHid; w2t[o * kHid + a] = __float2bfloat16(master[kOffW2 + k]); }
  }
}

}  // namespace

int mlp_param_count() { return kParamCount; }

cudaError_t launch_kmer_features(int n, const uint8_t* ascii, const PairDesc* pairs, void* feats_bf16, int num_sms,
                                 cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  constexpr int WPB = 8;
  long long blocks = ((long long)n + WPB - 1) / WPB;
  if (blocks > (long long)num_sms * 8) blocks = (long long)num_sms * 8;
  kmer_features_kernel<WPB><<<(int)blocks, WPB * 32, 0, stream>>>(n, ascii, pairs, (__nv_bfloat16*)feats_bf16);
  return cudaGetLastError();
}

cudaError_t launch_mlp_forward(int n, const void* feats_bf16, const float* master, const void* w1t, const void* w2t,
                               float* y_out, float* score_out, int num_sms, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  constexpr int WPB = 4;
  MlpParams prm{master, (const __nv_bfloat16*)w1t, (const __nv_bfloat16*)w2t};
  const int tiles = (n + 15) / 16;
  long long blocks = ((long long)tiles + WPB - 1) / WPB;
  if (blocks > (long long)num_sms * 8) blocks = (long long)num_sms * 8;
  mlp_forward_kernel<WPB><<<(int)blocks, WPB * 32, 0, stream>>>(n, (const __nv_bfloat16*)feats_bf16, prm, y_out,
                                                                score_out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_train_step(const void* feats_bf16, const float* target, const int* rows_idx, int rows,
                                  const float* master, const void* w1t, const void* w2t, float* grad, float* loss_sum,
                                  int num_sms, cudaStream_t stream) {
  if (rows <= 0) return cudaSuccess;
  constexpr int WPB = kTrainWpb;
  static bool attr_set = false;
  if (!attr_set) {
    const cudaError_t e = cudaFuncSetAttribute(mlp_train_step_kernel<WPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kTrainSmemBytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  MlpParams prm{master, (const __nv_bfloat16*)w1t, (const __nv_bfloat16*)w2t};
  const int tiles = (rows + 15) / 16;
  long long blocks = ((long long)tiles + WPB - 1) / WPB;
  if (blocks > (long long)num_sms * 2) blocks = (long long)num_sms * 2;
  mlp_train_step_kernel<WPB><<<(int)blocks, WPB * 32, kTrainSmemBytes, stream>>>((const __nv_bfloat16*)feats_bf16, target,
                                                                   rows_idx, rows, prm, grad, loss_sum);
  return cudaGetLastError();
}

__global__ void mlp_step_advance_kernel(int* step) { *step += 1; }

cudaError_t launch_mlp_adam(float* master, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                            float eps, const int* step, void* w1t, void* w2t, cudaStream_t stream) {
  mlp_adam_kernel<<<(kParamCount + 255) / 256, 256, 0, stream>>>(master, grad, m, v, lr, beta1, beta2, eps, step,
                                                                 (__nv_bfloat16*)w1t, (__nv_bfloat16*)w2t);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mlp_step_advance_kernel<<<1, 1, 0, stream>>>(const_cast<int*>(step));
  return cudaGetLastError();
}

cudaError_t launch_mlp_sync_bf16(const float* master, void* w1t, void* w2t, cudaStream_t stream) {
  mlp_sync_bf16_kernel<<<(kIn * kHid + kHid * kHid + 255) / 256, 256, 0, stream>>>(master, (__nv_bfloat16*)w1t,
                                                                                    (__nv_bfloat16*)w2t);
  return cudaGetLastError();
}

}  // namespace wfg
