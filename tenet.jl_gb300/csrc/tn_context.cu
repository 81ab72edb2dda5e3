// Context, device memory accounting, workspace arena, errors.
#include <cstdarg>
#include <cstdlib>
#include <cstring>

#include "tn_internal.cuh"

static thread_local std::string g_create_error;

tn_status_t tn_set_error(tn_ctx* ctx, tn_status_t st, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx)
    ctx->last_error = buf;
  else
    g_create_error = buf;
  return st;
}

tn_status_t tn_dev_alloc(tn_ctx* ctx, size_t bytes, void** p) {
  if (bytes == 0) bytes = 256;
  if (ctx->budget && ctx->in_use + bytes > ctx->budget)
    return tn_set_error(ctx, TN_ENOMEM, "HBM budget exceeded: %zu in use + %zu > %zu",
                        ctx->in_use, bytes, ctx->budget);
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return tn_set_error(ctx, TN_ENOMEM, "cudaMalloc(%zu) failed: %s", bytes,
                        cudaGetErrorString(e));
  }
  ctx->allocs[*p] = bytes;
  ctx->in_use += bytes;
  return TN_OK;
}

tn_status_t tn_dev_free(tn_ctx* ctx, void* p) {
  if (!p) return TN_OK;
  auto it = ctx->allocs.find(p);
  if (it == ctx->allocs.end())
    return tn_set_error(ctx, TN_EINVAL, "tn_free: pointer %p not allocated by this context", p);
  ctx->in_use -= it->second;
  ctx->allocs.erase(it);
  TN_CHECK_CUDA(ctx, cudaFree(p));
  return TN_OK;
}

void ws_overflow(tn_ctx* ctx, size_t need) {
  cudaStreamSynchronize(ctx->stream);
  fprintf(stderr, "tenetgb: workspace overflow: %zu bytes taken, %zu reserved (a missing ws_reserve)\n", need,
          ctx->ws_cap);
  fflush(stderr);
  std::abort();
}

tn_status_t ws_reserve(tn_ctx* ctx, size_t bytes) {
  ctx->ws_top = 0;
  if (bytes <= ctx->ws_cap) return TN_OK;
  // growth: the stream must be idle before the old arena is released
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  // (the cached graphs point into the arena; the profiler's events do not and stay)
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
  ctx->graphs.clear();
  if (ctx->ws) TN_RETURN_IF(tn_dev_free(ctx, ctx->ws));
  ctx->ws = nullptr;
  ctx->ws_cap = 0;
  size_t cap = bytes + bytes / 4 + (1 << 20);
  void* p = nullptr;
  TN_RETURN_IF(tn_dev_alloc(ctx, cap, &p));
  ctx->ws = (char*)p;
  ctx->ws_cap = cap;
  return TN_OK;
}

tn_status_t ctx_flags(tn_ctx* ctx, size_t n, int** out) {
  if (n > ctx->flags_cap) {
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->d_flags) TN_RETURN_IF(tn_dev_free(ctx, ctx->d_flags));
    ctx->d_flags = nullptr;
    size_t cap = n < 1024 ? 1024 : n * 2;
    void* p = nullptr;
    TN_RETURN_IF(tn_dev_alloc(ctx, cap * sizeof(int), &p));
    ctx->d_flags = (int*)p;
    ctx->flags_cap = cap;
  }
  *out = ctx->d_flags;
  return TN_OK;
}

extern "C" {

const char* tn_version(void) { return "tenetgb 0.1.0 (sm_103a)"; }

tn_status_t tn_create(tn_ctx** out, int device) {
  if (!out) return tn_set_error(nullptr, TN_EINVAL, "tn_create: null output");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return tn_set_error(nullptr, TN_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (device < 0 || device >= n)
    return tn_set_error(nullptr, TN_EINVAL, "device %d out of range (%d devices)", device, n);
  tn_ctx* ctx = new tn_ctx();
  ctx->device = device;
  cudaSetDevice(device);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  ctx->num_sms = prop.multiProcessorCount;
  if (prop.major < 10) {
    delete ctx;
    return tn_set_error(nullptr, TN_EUNSUPPORTED,
                        "device %d is sm_%d%d; libtenetgb is built for sm_103a", device,
                        prop.major, prop.minor);
  }
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    return tn_set_error(nullptr, TN_ECUDA, "stream create: %s", cudaGetErrorString(e));
  }
  ctx->stream = ctx->own_stream;
  e = cudaMallocHost(&ctx->pinned, 1 << 16);
  if (e != cudaSuccess) {
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return tn_set_error(nullptr, TN_ECUDA, "pinned alloc: %s", cudaGetErrorString(e));
  }
  *out = ctx;
  return TN_OK;
}

}  // extern "C"

void ctx_release(tn_ctx* ctx) {
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
  ctx->graphs.clear();
  for (auto& r : ctx->prof_recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (cudaEvent_t e : ctx->prof_pool) cudaEventDestroy(e);
  for (auto& kv : ctx->allocs) cudaFree(kv.first);
  ctx->allocs.clear();
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

extern "C" {

tn_status_t tn_destroy(tn_ctx* ctx) {
  if (!ctx) return TN_OK;
  if (ctx->refs > 0) {
    ctx->destroy_requested = true;  // released by the last tn_mps_destroy
    return TN_OK;
  }
  ctx_release(ctx);
  return TN_OK;
}

tn_status_t tn_set_stream(tn_ctx* ctx, void* stream) {
  if (!ctx) return TN_EINVAL;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return TN_OK;
}

void* tn_get_stream(tn_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

tn_status_t tn_sync(tn_ctx* ctx) {
  if (!ctx) return TN_EINVAL;
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_alloc(tn_ctx* ctx, size_t bytes, void** dptr) {
  if (!ctx || !dptr) return TN_EINVAL;
  return tn_dev_alloc(ctx, bytes, dptr);
}

tn_status_t tn_free(tn_ctx* ctx, void* dptr) {
  if (!ctx) return TN_EINVAL;
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return tn_dev_free(ctx, dptr);
}

tn_status_t tn_memcpy_h2d(tn_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, dst && src, "tn_memcpy_h2d: null pointer");
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_memcpy_d2h(tn_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, dst && src, "tn_memcpy_d2h: null pointer");
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_memcpy_d2d(tn_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, dst && src, "tn_memcpy_d2d: null pointer");
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  return TN_OK;
}

tn_status_t tn_set_hbm_budget(tn_ctx* ctx, size_t bytes) {
  if (!ctx) return TN_EINVAL;
  ctx->budget = bytes;
  return TN_OK;
}

tn_status_t tn_hbm_in_use(tn_ctx* ctx, size_t* bytes) {
  if (!ctx || !bytes) return TN_EINVAL;
  *bytes = ctx->in_use;
  return TN_OK;
}

tn_status_t tn_kernel_launches(tn_ctx* ctx, int64_t* count) {
  if (!ctx || !count) return TN_EINVAL;
  *count = ctx->launches;
  return TN_OK;
}

tn_status_t tn_set_autotune(tn_ctx* ctx, int32_t enable) {
  if (!ctx) return TN_EINVAL;
  ctx->autotune = enable != 0;
  return TN_OK;
}

// text form: one "key value1 value2" line per tuned shape
tn_status_t tn_tuning_dump(tn_ctx* ctx, char* buf, size_t len, size_t* needed) {
  if (!ctx) return TN_EINVAL;
  std::string out;
  for (auto& kv : ctx->tuning)
    out += kv.first + " " + std::to_string(kv.second.first) + " " + std::to_string(kv.second.second) + "\n";
  if (needed) *needed = out.size() + 1;
  if (buf && len > 0) {
    size_t c = out.size() < len - 1 ? out.size() : len - 1;
    memcpy(buf, out.data(), c);
    buf[c] = 0;
  }
  return TN_OK;
}

tn_status_t tn_tuning_load(tn_ctx* ctx, const char* text) {
  if (!ctx || !text) return TN_EINVAL;
  const char* p = text;
  while (*p) {
    char key[128];
    int a = 0, b = 0, used = 0;
    if (sscanf(p, "%127s %d %d%n", key, &a, &b, &used) != 3) break;
    // the autotuner's candidate set: panel widths 1…32 and slab widths 1, 2, 4 (powers of two)
    const bool pow2 = (a & (a - 1)) == 0 && (b & (b - 1)) == 0;
    if (a < 1 || a > 32 || b < 1 || b > 4 || !pow2)
      return tn_set_error(ctx, TN_EINVAL, "tn_tuning_load: bad entry %s %d %d", key, a, b);
    ctx->tuning[key] = {a, b};
    p += used;
    while (*p == '\n' || *p == ' ') ++p;
  }
  return TN_OK;
}

const char* tn_last_error_string(tn_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : g_create_error.c_str();
}

}  // extern "C"
