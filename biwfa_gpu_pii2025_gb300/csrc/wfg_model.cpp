// Learned scheduling, host side: the score-predictor model (wfg_model_*), feature extraction
// and prediction on a context's resident batch, and GPU training with the library's own
// kernels (mlp_kernel.cu). One training epoch is captured once as a CUDA graph and
// replayed (the minibatch loop is launch-bound otherwise).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/wfa_gpu.h"
#include "wfg_context.h"

using namespace wfg;

struct wfg_model {
  int device = 0;
  int nparams = 0;
  DevBuf<float> d_master, d_grad, d_m, d_v, d_loss, d_targets;
  DevBuf<uint16_t> d_w1t, d_w2t;  // bf16 bit patterns
  DevBuf<int> d_rows, d_step;
  // captured epoch
  cudaGraphExec_t epoch_exec = nullptr;
  int graph_rows = -1, graph_batch = -1;
  float graph_lr = -1.f;
  const void* graph_feats = nullptr;
};

namespace {

// splitmix64 stream for initialisation and shuffling (deterministic on every platform)
struct Mix {
  uint64_t x;
  uint64_t next() {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
};

constexpr int kIn = WFG_MODEL_FEATURES, kHid = 64;

int ensure_features(wfg_context* c) {
  if (c->feats_valid) return WF_STATUS_ALG_COMPLETED;
  WFG_CHECK(c, c->d_feats.reserve((size_t)std::max(c->n, 1) * kIn));
  WFG_CHECK(c, launch_kmer_features(c->n, c->d_seq.ptr, c->d_pairs.ptr, c->d_feats.ptr, c->num_sms, c->stream));
  c->feats_valid = true;
  return WF_STATUS_ALG_COMPLETED;
}

}  // namespace

extern "C" {

int wfg_model_param_count(void) { return mlp_param_count(); }

wfg_model_t* wfg_model_create(wfg_context_t* c, uint64_t seed) {
  if (!c) return nullptr;
  cudaSetDevice(c->device);
  wfg_model* m = new wfg_model();
  m->device = c->device;
  m->nparams = mlp_param_count();
  if (m->d_master.reserve(m->nparams) != cudaSuccess || m->d_grad.reserve(m->nparams) != cudaSuccess ||
      m->d_m.reserve(m->nparams) != cudaSuccess || m->d_v.reserve(m->nparams) != cudaSuccess ||
      m->d_loss.reserve(4) != cudaSuccess || m->d_w1t.reserve(kIn * kHid) != cudaSuccess ||
      m->d_w2t.reserve(kHid * kHid) != cudaSuccess || m->d_step.reserve(1) != cudaSuccess) {
    delete m;
    return nullptr;
  }
  // He-uniform weights, zero biases
  std::vector<float> p((size_t)m->nparams, 0.f);
  Mix mix{seed};
  const int offb1 = kIn * kHid, offw2 = offb1 + kHid, offb2 = offw2 + kHid * kHid, offw3 = offb2 + kHid;
  const double a1 = std::sqrt(6.0 / kIn), a2 = std::sqrt(6.0 / kHid);
  for (int i = 0; i < kIn * kHid; ++i) p[(size_t)i] = (float)((2 * mix.uniform() - 1) * a1);
  for (int i = 0; i < kHid * kHid; ++i) p[(size_t)(offw2 + i)] = (float)((2 * mix.uniform() - 1) * a2);
  for (int i = 0; i < kHid; ++i) p[(size_t)(offw3 + i)] = (float)((2 * mix.uniform() - 1) * a2 * 0.5);
  if (wfg_model_set_params(m, p.data()) != WF_STATUS_ALG_COMPLETED) {
    wfg_model_destroy(m);
    return nullptr;
  }
  return m;
}

void wfg_model_destroy(wfg_model_t* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->epoch_exec) cudaGraphExecDestroy(m->epoch_exec);
  m->d_master.release(); m->d_grad.release(); m->d_m.release(); m->d_v.release(); m->d_loss.release();
  m->d_targets.release(); m->d_w1t.release(); m->d_w2t.release(); m->d_rows.release(); m->d_step.release();
  delete m;
}

int wfg_model_get_params(wfg_model_t* m, float* params) {
  if (!m || !params) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(m->device);
  if (cudaMemcpy(params, m->d_master.ptr, sizeof(float) * (size_t)m->nparams, cudaMemcpyDeviceToHost) != cudaSuccess)
    return WF_STATUS_DEVICE_ERROR;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_model_set_params(wfg_model_t* m, const float* params) {
  if (!m || !params) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(m->device);
  const size_t bytes = sizeof(float) * (size_t)m->nparams;
  if (cudaMemcpy(m->d_master.ptr, params, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(m->d_m.ptr, 0, bytes) != cudaSuccess || cudaMemset(m->d_v.ptr, 0, bytes) != cudaSuccess)
    return WF_STATUS_DEVICE_ERROR;
  const int one = 1;
  if (cudaMemcpy(m->d_step.ptr, &one, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return WF_STATUS_DEVICE_ERROR;
  if (launch_mlp_sync_bf16(m->d_master.ptr, m->d_w1t.ptr, m->d_w2t.ptr, 0) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess)
    return WF_STATUS_DEVICE_ERROR;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_features(wfg_context_t* c, uint16_t* host_features) {
  if (!c) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  const int st = ensure_features(c);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  if (host_features && c->n > 0) {
    WFG_CHECK(c, cudaMemcpyAsync(host_features, c->d_feats.ptr, sizeof(uint16_t) * (size_t)c->n * kIn,
                                 cudaMemcpyDeviceToHost, c->stream));
    WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  }
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_model_gradient(wfg_model_t* m, wfg_context_t* c, const float* log_targets, float* grad, float* loss) {
  if (!m || !c || !log_targets || !grad) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  const int n = c->n;
  int st = ensure_features(c);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  WFG_CHECK(c, m->d_targets.reserve((size_t)std::max(n, 1)));
  WFG_CHECK(c, m->d_rows.reserve((size_t)std::max(n, 1)));
  std::vector<int> rows((size_t)n);
  std::iota(rows.begin(), rows.end(), 0);
  WFG_CHECK(c, cudaMemcpyAsync(m->d_targets.ptr, log_targets, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  WFG_CHECK(c, cudaMemcpyAsync(m->d_rows.ptr, rows.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  WFG_CHECK(c, cudaMemsetAsync(m->d_grad.ptr, 0, sizeof(float) * (size_t)m->nparams, c->stream));
  WFG_CHECK(c, cudaMemsetAsync(m->d_loss.ptr, 0, sizeof(float), c->stream));
  WFG_CHECK(c, launch_mlp_train_step(c->d_feats.ptr, m->d_targets.ptr, m->d_rows.ptr, n, m->d_master.ptr, m->d_w1t.ptr,
                                     m->d_w2t.ptr, m->d_grad.ptr, m->d_loss.ptr, c->num_sms, c->stream));
  WFG_CHECK(c, cudaMemcpyAsync(grad, m->d_grad.ptr, sizeof(float) * (size_t)m->nparams, cudaMemcpyDeviceToHost, c->stream));
  float lsum = 0.f;
  WFG_CHECK(c, cudaMemcpyAsync(&lsum, m->d_loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  if (loss) *loss = n > 0 ? lsum / (float)n : 0.f;
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_model_train(wfg_model_t* m, wfg_context_t* c, const int* target_scores, int epochs, int batch_rows, float lr,
                    uint64_t seed, float* epoch_loss) {
  if (!m || !c || !target_scores || epochs < 0 || batch_rows <= 0) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  const int n = c->n;
  if (n == 0) return WF_STATUS_ALG_COMPLETED;
  int st = ensure_features(c);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  std::vector<float> tgt((size_t)n);
  for (int i = 0; i < n; ++i) tgt[(size_t)i] = (float)std::log1p((double)std::abs((double)target_scores[i]));
  WFG_CHECK(c, m->d_targets.reserve((size_t)n));
  WFG_CHECK(c, m->d_rows.reserve((size_t)n));
  WFG_CHECK(c, cudaMemcpyAsync(m->d_targets.ptr, tgt.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  // Capture one epoch (all minibatches) once; replays read the shuffled row order from d_rows.
  if (!m->epoch_exec || m->graph_rows != n || m->graph_batch != batch_rows || m->graph_lr != lr ||
      m->graph_feats != c->d_feats.ptr) {
    if (m->epoch_exec) { cudaGraphExecDestroy(m->epoch_exec); m->epoch_exec = nullptr; }
    cudaGraph_t graph;
    WFG_CHECK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    for (int b0 = 0; b0 < n && err == cudaSuccess; b0 += batch_rows) {
      const int rows = std::min(batch_rows, n - b0);
      err = cudaMemsetAsync(m->d_grad.ptr, 0, sizeof(float) * (size_t)m->nparams, c->stream);
      if (err == cudaSuccess)
        err = launch_mlp_train_step(c->d_feats.ptr, m->d_targets.ptr, m->d_rows.ptr + b0, rows, m->d_master.ptr,
                                    m->d_w1t.ptr, m->d_w2t.ptr, m->d_grad.ptr, m->d_loss.ptr, c->num_sms, c->stream);
      if (err == cudaSuccess)
        err = launch_mlp_adam(m->d_master.ptr, m->d_grad.ptr, m->d_m.ptr, m->d_v.ptr, lr, beta1, beta2, eps,
                              m->d_step.ptr, m->d_w1t.ptr, m->d_w2t.ptr, c->stream);
    }
    const cudaError_t end = cudaStreamEndCapture(c->stream, &graph);
    if (err != cudaSuccess) return wfg_fail(c, err, "capture of the training epoch");
    if (end != cudaSuccess) return wfg_fail(c, end, "cudaStreamEndCapture");
    const cudaError_t inst = cudaGraphInstantiate(&m->epoch_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (inst != cudaSuccess) return wfg_fail(c, inst, "cudaGraphInstantiate");
    m->graph_rows = n; m->graph_batch = batch_rows; m->graph_lr = lr; m->graph_feats = c->d_feats.ptr;
  }
  std::vector<int> rows((size_t)n);
  std::iota(rows.begin(), rows.end(), 0);
  Mix mix{seed};
  PinBuf<int> h_rows;
  WFG_CHECK(c, h_rows.reserve((size_t)n));
  for (int ep = 0; ep < epochs; ++ep) {
    for (int i = n - 1; i > 0; --i) std::swap(rows[(size_t)i], rows[(size_t)mix.below((uint64_t)i + 1)]);
    memcpy(h_rows.ptr, rows.data(), sizeof(int) * (size_t)n);
    WFG_CHECK(c, cudaMemcpyAsync(m->d_rows.ptr, h_rows.ptr, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    WFG_CHECK(c, cudaMemsetAsync(m->d_loss.ptr, 0, sizeof(float), c->stream));
    WFG_CHECK(c, cudaGraphLaunch(m->epoch_exec, c->stream));
    float lsum = 0.f;
    WFG_CHECK(c, cudaMemcpyAsync(&lsum, m->d_loss.ptr, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    WFG_CHECK(c, cudaStreamSynchronize(c->stream));
    if (epoch_loss) epoch_loss[ep] = lsum / (float)n;
  }
  h_rows.release();
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_model_predict(wfg_model_t* m, wfg_context_t* c, float* host_pred) {
  if (!m || !c) return WF_STATUS_UNSUPPORTED;
  cudaSetDevice(c->device);
  int st = ensure_features(c);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  WFG_CHECK(c, c->d_pred.reserve((size_t)std::max(c->n, 1)));
  WFG_CHECK(c, launch_mlp_forward(c->n, c->d_feats.ptr, m->d_master.ptr, m->d_w1t.ptr, m->d_w2t.ptr, nullptr,
                                  c->d_pred.ptr, c->num_sms, c->stream));
  c->pred_valid = true;
  if (host_pred && c->n > 0) {
    WFG_CHECK(c, cudaMemcpyAsync(host_pred, c->d_pred.ptr, sizeof(float) * (size_t)c->n, cudaMemcpyDeviceToHost, c->stream));
    WFG_CHECK(c, cudaStreamSynchronize(c->stream));
  }
  return WF_STATUS_ALG_COMPLETED;
}

int wfg_set_model(wfg_context_t* c, wfg_model_t* m) {
  if (!c) return WF_STATUS_UNSUPPORTED;
  c->model = m;
  return WF_STATUS_ALG_COMPLETED;
}

}  // extern "C"

int wfg_model_predict_range(wfg_model* m, wfg_context* c, int first, int count, cudaStream_t stream) {
  if (!m || !c || first < 0 || count < 0 || first + count > c->n) return WF_STATUS_UNSUPPORTED;
  if (count == 0) return WF_STATUS_ALG_COMPLETED;
  WFG_CHECK(c, c->d_feats.reserve((size_t)std::max(c->n, 1) * kIn));
  WFG_CHECK(c, c->d_pred.reserve((size_t)std::max(c->n, 1)));
  uint16_t* feats = c->d_feats.ptr + (size_t)first * kIn;
  WFG_CHECK(c, launch_kmer_features(count, c->d_seq.ptr, c->d_pairs.ptr + first, feats, c->num_sms, stream));
  WFG_CHECK(c, launch_mlp_forward(count, feats, m->d_master.ptr, m->d_w1t.ptr, m->d_w2t.ptr, nullptr,
                                  c->d_pred.ptr + first, c->num_sms, stream));
  return WF_STATUS_ALG_COMPLETED;
}
