// Phase profiler and pipe-peak probes.
//
// With profiling on, the hot path brackets each phase of work it enqueues (a Jacobi
// sweep graph, a GEMM launch, a QR factorisation) by a pair of CUDA events on the
// context's stream and records the phase's class, launch count and algorithmic flops and
// bytes.  tn_profile_read drains the stream, resolves the event pairs and returns the
// totals per class, so a caller can time the kernels of a step as they run inside it.
// The pipe-peak probe measures the FP32 / FP64 fused multiply-add rate of the CUDA cores
// with a register-resident FMA loop (the roofline denominator for CUDA-core kernels).
#include <algorithm>

#include "tn_internal.cuh"

namespace {

cudaEvent_t prof_event(tn_ctx* ctx) {
  if (!ctx->prof_pool.empty()) {
    cudaEvent_t e = ctx->prof_pool.back();
    ctx->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// resolve every recorded pair (the stream is drained first)
tn_status_t prof_collect(tn_ctx* ctx) {
  if (ctx->prof_recs.empty()) return TN_OK;
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto& r : ctx->prof_recs) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess && r.cls >= 0 && r.cls < TN_PROF_NCLASS) {
      ctx->prof_ms[r.cls] += ms;
      ctx->prof_launches[r.cls] += r.launches;
      ctx->prof_flops[r.cls] += r.flops;
      ctx->prof_bytes[r.cls] += r.bytes;
    }
    ctx->prof_pool.push_back(r.a);
    ctx->prof_pool.push_back(r.b);
  }
  ctx->prof_recs.clear();
  return TN_OK;
}

template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(int iters, T seed, T* out) {
  T a0 = seed + (T)threadIdx.x, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
  const T b = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
      a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
  }
  const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == (T)-1) out[blockIdx.x] = s;  // keeps the chains live
}

template <typename T>
tn_status_t fma_peak(tn_ctx* ctx, double* tflops) {
  const int blocks = ctx->num_sms * 8, threads = 256, iters = sizeof(T) == 8 ? 256 : 4096;
  T* sink = nullptr;
  TN_RETURN_IF(tn_dev_alloc(ctx, sizeof(T) * (size_t)blocks, (void**)&sink));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  TN_CHECK_CUDA(ctx, cudaEventCreate(&e0));
  TN_CHECK_CUDA(ctx, cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, ctx->stream);
    k_fma_probe<T><<<blocks, threads, 0, ctx->stream>>>(iters, (T)0.5, sink);
    cudaEventRecord(e1, ctx->stream);
    TN_CHECK_CUDA(ctx, cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = std::min(best, ms);  // the first launch warms the clocks
  }
  TN_LAUNCHED(ctx);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  tn_dev_free(ctx, sink);
  const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return TN_OK;
}

}  // namespace

int prof_begin(tn_ctx* ctx) {
  if (!ctx->prof_on) return -1;
  if (ctx->prof_recs.size() >= 8192 && prof_collect(ctx) != TN_OK) return -1;
  cudaEvent_t a = prof_event(ctx), b = prof_event(ctx);
  if (!a || !b) return -1;
  cudaEventRecord(a, ctx->stream);
  tn_ctx::prof_rec r;
  r.cls = -1;
  r.a = a;
  r.b = b;
  r.launches = 0;
  r.flops = r.bytes = 0.0;
  ctx->prof_recs.push_back(r);
  return (int)ctx->prof_recs.size() - 1;
}

void prof_end(tn_ctx* ctx, int slot, int cls, int64_t launches, double flops, double bytes) {
  if (slot < 0 || slot >= (int)ctx->prof_recs.size()) return;
  auto& r = ctx->prof_recs[slot];
  cudaEventRecord(r.b, ctx->stream);
  r.cls = cls;
  r.launches = launches;
  r.flops = flops;
  r.bytes = bytes;
}

extern "C" tn_status_t tn_profile_enable(tn_ctx* ctx, int32_t enable) {
  if (!ctx) return TN_EINVAL;
  TN_RETURN_IF(prof_collect(ctx));
  ctx->prof_on = enable != 0;
  for (int c = 0; c < 16; ++c) {
    ctx->prof_launches[c] = 0;
    ctx->prof_ms[c] = ctx->prof_flops[c] = ctx->prof_bytes[c] = 0.0;
  }
  return TN_OK;
}

extern "C" tn_status_t tn_profile_read(tn_ctx* ctx, int32_t cls, int64_t* launches, double* ms, double* flops,
                                       double* bytes) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, cls >= 0 && cls < TN_PROF_NCLASS, "tn_profile_read: unknown class");
  TN_RETURN_IF(prof_collect(ctx));
  if (launches) *launches = ctx->prof_launches[cls];
  if (ms) *ms = ctx->prof_ms[cls];
  if (flops) *flops = ctx->prof_flops[cls];
  if (bytes) *bytes = ctx->prof_bytes[cls];
  return TN_OK;
}

extern "C" tn_status_t tn_pipe_peak(tn_ctx* ctx, int32_t which, double* tflops) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, tflops && (which == 0 || which == 1), "tn_pipe_peak: which must be 0 (FP32) or 1 (FP64)");
  return which == 0 ? fma_peak<float>(ctx, tflops) : fma_peak<double>(ctx, tflops);
}
