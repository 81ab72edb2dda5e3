// Internal definitions shared by the translation units of libtenetgb.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include "tenet_gb300.h"

// ---------------------------------------------------------------------------------
// complex scalars: interleaved (re, im) == Julia Complex{T} == cuDoubleComplex layout
// ---------------------------------------------------------------------------------
template <typename T>
struct alignas(2 * sizeof(T)) cx {
  T x, y;
};
using cxd = cx<double>;
using cxf = cx<float>;

template <typename T>
__host__ __device__ __forceinline__ cx<T> mkcx(T a, T b) {
  cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) {
  return mkcx<T>(a.x + b.x, a.y + b.y);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) {
  return mkcx<T>(a.x - b.x, a.y - b.y);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) {
  return mkcx<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(T s, cx<T> a) {
  return mkcx<T>(s * a.x, s * a.y);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> conjg(cx<T> a) {
  return mkcx<T>(a.x, -a.y);
}
template <typename T>
__host__ __device__ __forceinline__ T abs2(cx<T> a) {
  return a.x * a.x + a.y * a.y;
}
// acc += a * b
template <typename T>
__host__ __device__ __forceinline__ void cfma(cx<T>& acc, cx<T> a, cx<T> b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ void cfma_cj(cx<T>& acc, cx<T> a, cx<T> b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Orthonormal completion of columns [first, ncols) of U (m × ncols, ld m, m ≥ ncols)
// against all earlier columns, as a Householder SVD's U has for numerically zero σ: unit
// vectors e_k taken in turn, orthogonalised twice, accepted once ≥ 0.5/√m of them remains
// (the complement's projector has trace m − j ≥ 1, so some e_k keeps ≥ 1/√m).  Called by
// a whole block (blockDim.x a multiple of 32, ≤ 1024); c: shared scratch of ncols
// elements, red: 32 shared doubles, next_k: a shared counter.
template <typename T>
__device__ void complete_columns(int64_t m, int64_t ncols, int64_t first, cx<T>* U0, cx<T>* c, double* red,
                                 int64_t* next_k) {
  if (threadIdx.x == 0) *next_k = 0;
  __syncthreads();
  const double accept = 0.5 / sqrt((double)m);
  for (int64_t j = first; j < ncols; ++j) {
    cx<T>* u = U0 + j * m;
    for (int64_t attempt = 0; attempt < m; ++attempt) {
      const int64_t k = *next_k;
      for (int64_t t = threadIdx.x; t < m; t += blockDim.x) u[t] = mkcx<T>(t == k ? T(1) : T(0), T(0));
      __syncthreads();
      for (int pass = 0; pass < 2; ++pass) {
        for (int64_t q = threadIdx.x; q < j; q += blockDim.x) {
          cx<T> acc = mkcx<T>(0, 0);
          const cx<T>* uq = U0 + q * m;
          for (int64_t t = 0; t < m; ++t) cfma_cj(acc, uq[t], u[t]);
          c[q] = acc;
        }
        __syncthreads();
        for (int64_t t = threadIdx.x; t < m; t += blockDim.x) {
          cx<T> v = u[t];
          for (int64_t q = 0; q < j; ++q) v = v - U0[q * m + t] * c[q];
          u[t] = v;
        }
        __syncthreads();
      }
      double ss = 0.0;
      for (int64_t t = threadIdx.x; t < m; t += blockDim.x) ss += (double)abs2(u[t]);
      ss = warp_sum(ss);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
      __syncthreads();
      double nrm = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) nrm += red[w];
      nrm = sqrt(nrm);
      __syncthreads();
      if (threadIdx.x == 0) *next_k = (k + 1) % m;
      if (nrm >= accept) {
        const T inv = T(1.0 / nrm);
        for (int64_t t = threadIdx.x; t < m; t += blockDim.x) u[t] = inv * u[t];
        __syncthreads();
        break;
      }
      __syncthreads();
    }
  }
}

// first index of the trailing σ (sorted descending, n values) with σ² ≤ 2·max(negl_rel·Σσ²,
// floor_abs): the columns one-sided Jacobi leaves as numerically zero
__device__ inline int64_t negligible_start(const double* s, int64_t n, double negl_rel, double floor_abs) {
  double f = 0.0;
  for (int64_t j = 0; j < n; ++j) f += s[j] * s[j];
  const double thr2 = 2.0 * (negl_rel * f > floor_abs ? negl_rel * f : floor_abs);
  int64_t r = n;
  while (r > 0 && !(s[r - 1] * s[r - 1] > thr2)) --r;
  return r;
}

// ---------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------
struct tn_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  std::string last_error;
  // workspace arena: reserved per top-level call, carved with ws_take
  char* ws = nullptr;
  size_t ws_cap = 0;
  size_t ws_top = 0;
  // small pinned host buffer for scalar read-backs
  void* pinned = nullptr;
  int* d_flags = nullptr;  // device status / convergence words
  size_t flags_cap = 0;
  // accounting
  size_t budget = 0;  // 0 = unlimited
  size_t in_use = 0;
  std::unordered_map<void*, size_t> allocs;
  int64_t launches = 0;
  // instantiated CUDA graphs (e.g. one Jacobi sweep), keyed by shape + buffer addresses
  std::unordered_map<std::string, cudaGraphExec_t> graphs;
  // live objects (MPS handles) that refer to this context; tn_destroy defers the
  // release until the last of them is destroyed
  int refs = 0;
  bool destroy_requested = false;
  // diagnostics of the last Jacobi SVD: sweeps per precision, rotations per sweep of
  // the worst active matrix of the large-matrix path (-1: shared-memory path)
  int last_sweeps_fp32 = 0, last_sweeps_fp64 = 0;
  int last_refine_iters = 0;     // refinement iterations of the last truncated mixed SVD
  int last_refine_clusters = 0;  // its near-degenerate pairs left to the FP64 check
  // cumulative over the context: truncated mixed SVD calls, refinement iterations, marked
  // pairs, calls finished by the full FP64 sweeps
  int64_t refine_totals[4] = {0, 0, 0, 0};
  // the last truncated mixed SVD: per iteration the largest step, the largest |R_ij|, the
  // largest ‖E‖_F and the marked pairs; outcome 0 converged, 1 diverged (FP64 sweeps from
  // the pre-pass basis), 2 out of iterations (FP64 sweeps from the refined basis)
  float refine_trace[8][4] = {};
  int refine_outcome = 0;
  int sweep_rotations[64] = {0};
  float sweep_ratio[64] = {0};  // largest off-diagonal ratio of each sweep (worst active matrix)
  // time of the last DMRG run per phase (ms): gauge moves, environments, eigensolves,
  // pair splits; and its local updates
  double dmrg_ms[4] = {0, 0, 0, 0};
  int64_t dmrg_updates = 0;
  int64_t dmrg_svd_sweeps = 0;  // Jacobi sweeps summed over the pair splits
  // phase profiler (tn_profile_*): event pairs around hot-path phases, resolved on read
  bool prof_on = false;
  struct prof_rec {
    int cls;
    cudaEvent_t a, b;
    int64_t launches;
    double flops, bytes;
  };
  std::vector<prof_rec> prof_recs;
  std::vector<cudaEvent_t> prof_pool;
  int64_t prof_launches[16] = {0};
  double prof_ms[16] = {0}, prof_flops[16] = {0}, prof_bytes[16] = {0};
  // split-BF16 GEMM: digit planes per operand, its operand-plane scratch and error word
  int split_slices = 8;
  char* oz_ws = nullptr;
  size_t oz_cap = 0;
  int* oz_err = nullptr;
  // autotuned launch parameters, keyed by kernel family + shape bucket
  bool autotune = false;
  std::unordered_map<std::string, std::pair<int, int>> tuning;
};
void ctx_release(tn_ctx* ctx);  // frees the context (called when refs drop to 0)

// ---------------------------------------------------------------------------------
// phase profiler: classes of hot-path work timed by CUDA events on the context stream
// (tn_profile_enable / tn_profile_read).  prof_begin returns a slot (-1 when profiling
// is off); prof_end records the closing event with the work done in between.
// ---------------------------------------------------------------------------------
enum {
  TN_PROF_JACOBI_F32 = 0,   // one-sided Jacobi sweeps, FP32 (k_jacobi_step_reg<float>)
  TN_PROF_JACOBI_F64 = 1,   // one-sided Jacobi sweeps, FP64 (k_jacobi_step_reg<double>)
  TN_PROF_GEMM_F64 = 2,     // complex FP64 CUDA-core GEMM (k_gemm_cx<double>)
  TN_PROF_GEMM_SPLIT = 3,   // split-BF16 tensor-core GEMM kernel (k_gemm_oz)
  TN_PROF_SPLIT_PREP = 4,   // its digit-plane preparation
  TN_PROF_QR = 5,           // blocked Householder QR (panel + block reflector)
  TN_PROF_JACOBI_COOP = 6,  // cooperative small-matrix Jacobi (whole iteration)
  TN_PROF_NCLASS = 7
};
int prof_begin(tn_ctx* ctx);
void prof_end(tn_ctx* ctx, int slot, int cls, int64_t launches, double flops, double bytes);

tn_status_t tn_set_error(tn_ctx* ctx, tn_status_t st, const char* fmt, ...);

#define TN_CHECK_CUDA(ctx, call)                                                    \
  do {                                                                              \
    cudaError_t _e = (call);                                                        \
    if (_e != cudaSuccess)                                                          \
      return tn_set_error((ctx), TN_ECUDA, "%s failed: %s (%s:%d)", #call,          \
                          cudaGetErrorString(_e), __FILE__, __LINE__);              \
  } while (0)

#define TN_RETURN_IF(st)           \
  do {                             \
    tn_status_t _s = (st);         \
    if (_s != TN_OK) return _s;    \
  } while (0)

#define TN_ARG(ctx, cond, msg)                                   \
  do {                                                           \
    if (!(cond)) return tn_set_error((ctx), TN_EINVAL, "%s", msg); \
  } while (0)

// after every launch: count it and surface launch errors
#define TN_LAUNCHED(ctx)                                                               \
  do {                                                                                 \
    (ctx)->launches++;                                                                 \
    cudaError_t _e = cudaGetLastError();                                               \
    if (_e != cudaSuccess)                                                             \
      return tn_set_error((ctx), TN_ECUDA, "kernel launch failed: %s (%s:%d)",         \
                          cudaGetErrorString(_e), __FILE__, __LINE__);                 \
  } while (0)

// device allocation with accounting against the HBM budget
tn_status_t tn_dev_alloc(tn_ctx* ctx, size_t bytes, void** p);
tn_status_t tn_dev_free(tn_ctx* ctx, void* p);

// workspace: reserve (may reallocate: only between operations), then take
tn_status_t ws_reserve(tn_ctx* ctx, size_t bytes);
inline size_t ws_round(size_t b) { return (b + 255) & ~size_t(255); }
// a take beyond the reserved arena is a bug in the caller's size computation: stop the
// process on the host (after the stream has drained, so no kernel is left in flight)
// rather than hand a kernel memory outside the arena
[[noreturn]] void ws_overflow(tn_ctx* ctx, size_t need);
template <typename T>
T* ws_take(tn_ctx* ctx, size_t count) {
  size_t b = ws_round(count * sizeof(T));
  if (ctx->ws_top + b > ctx->ws_cap) ws_overflow(ctx, ctx->ws_top + b);
  char* p = ctx->ws + ctx->ws_top;
  ctx->ws_top += b;
  return reinterpret_cast<T*>(p);
}
inline void ws_reset(tn_ctx* ctx) { ctx->ws_top = 0; }

// flag words (device ints), at least n, zeroed by caller when needed
tn_status_t ctx_flags(tn_ctx* ctx, size_t n, int** out);

inline size_t dtype_size(tn_dtype_t t) {
  switch (t) {
    case TN_F32: return 4;
    case TN_F64: return 8;
    case TN_C32: return 8;
    case TN_C64: return 16;
  }
  return 0;
}
inline bool dtype_complex(tn_dtype_t t) { return t == TN_C32 || t == TN_C64; }

inline unsigned cdiv(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// ---------------------------------------------------------------------------------
// internal entry points shared across translation units (typed, no validation)
// ---------------------------------------------------------------------------------
template <typename T>
tn_status_t gemm_cx(tn_ctx* ctx, char opa, char opb, int64_t m, int64_t n, int64_t k,
                    cx<T> alpha, const cx<T>* A, int64_t lda, int64_t sA, const cx<T>* B,
                    int64_t ldb, int64_t sB, cx<T> beta, cx<T>* C, int64_t ldc, int64_t sC,
                    int64_t batch);

// C = Aᴴ A (A k × n, C n × n Hermitian), batched
template <typename T>
tn_status_t herk_cx(tn_ctx* ctx, int64_t n, int64_t k, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* C, int64_t ldc,
                    int64_t sC, int64_t batch);

template <typename T>
tn_status_t permute_t(tn_ctx* ctx, int rank, const int64_t* dims, const int64_t* in_strides,
                      const int32_t* perm, const T* in, T* out, bool conj);

// (conjugate) transpose of a batch of column-major m×n matrices: out (n×m)
template <typename T>
tn_status_t transpose_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* in, int64_t lda,
                         int64_t sIn, cx<T>* out, int64_t ldo, int64_t sOut, int64_t batch,
                         bool conj);

// workspace bytes needed by qr_cx / svd_cx
template <typename T>
size_t qr_workspace(int64_t m, int64_t n, int64_t batch);
template <typename T>
tn_status_t qr_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA,
                  cx<T>* Q, int64_t sQ, cx<T>* R, int64_t sR, int64_t batch);

template <typename T>
size_t svd_workspace(int64_t m, int64_t n, int64_t batch);
// one-sided Jacobi SVD, m >= n required here; U m×n, S n (FP64), V n×n (not Vh)
template <typename T>
tn_status_t svd_tall_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* A, int64_t lda,
                        int64_t sA, cx<T>* U, int64_t sU, double* S, int64_t sS, cx<T>* V,
                        int64_t sV, int64_t batch, int* sweeps_out);

// mixed precision SVD (C64 data): FP32 Jacobi pre-pass + FP64 polish.  keep > 0 (V null
// only): only the `keep` largest triplets are wanted; the rest of U and S is approximate.
size_t svd_mixed_workspace(int64_t m, int64_t n, int64_t batch);
tn_status_t svd_tall_mixed(tn_ctx* ctx, int64_t m, int64_t n, const cxd* A, int64_t lda,
                           int64_t sA, cxd* U, int64_t sU, double* S, int64_t sS, cxd* V,
                           int64_t sV, int64_t batch, int64_t keep);

// left vectors + values only (m >= n): U m×n, S n (no V accumulation on large matrices).
// keep > 0: a truncation to at most `keep` values follows (the mixed path then skips the
// work that only the discarded tail would need; plain FP64 ignores it).
size_t svd_left_workspace(tn_precision_t prec, int64_t m, int64_t n, int64_t batch);
tn_status_t svd_left(tn_ctx* ctx, tn_precision_t prec, int64_t m, int64_t n, const cxd* A, int64_t lda, int64_t sA,
                     cxd* U, int64_t sU, double* S, int64_t sS, int64_t batch, int64_t keep = 0);

// full thin SVD for any m, n: U m×k, S k, Vh k×n (reserves its own workspace when
// ws_managed is false)
size_t svd_any_workspace(tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n,
                         int64_t batch);
tn_status_t svd_any(tn_ctx* ctx, tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n,
                    const void* A, int64_t lda, int64_t sA, void* U, int64_t sU, double* S,
                    int64_t sS, void* Vh, int64_t sVh, int64_t batch);

// any-dtype GEMM (no workspace reservation: the caller reserves gemm_any_workspace)
size_t gemm_any_workspace(tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n, int64_t k);
tn_status_t gemm_any(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, char opa, char opb, int64_t m, int64_t n,
                     int64_t k, const double* alpha, const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb,
                     int64_t sB, const double* beta, void* C, int64_t ldc, int64_t sC, int64_t batch);
// the driver's cuTensorMapEncodeTiled (resolved once through the runtime; null with the
// context's error set when unavailable).  Needs <cuda.h> for the CUtensorMap types.
#ifdef CUDA_VERSION
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tn_encode_tiled_fn(tn_ctx* ctx);
#endif
// Ozaki-style split-BF16 complex FP64 GEMM on the tcgen05 tensor pipe (tn_gemm_oz.cu):
// C = alpha op(A) op(B) + beta C with every operand cut into `slices` exact BF16 digit
// planes; FP64-grade (the error is set by the slice count).  Its operand planes live in
// a context scratch of their own (grown between calls), so callers reserve nothing.
constexpr int kSplitSlicesDefault = 8;
tn_status_t gemm_c64_split(tn_ctx* ctx, int slices, char opa, char opb, int64_t m, int64_t n, int64_t k, cxd alpha,
                           const cxd* A, int64_t lda, int64_t sA, const cxd* B, int64_t ldb, int64_t sB, cxd beta,
                           cxd* C, int64_t ldc, int64_t sC, int64_t batch);
// reads (and clears) the split GEMMs' error word after draining the stream: TN_ETIMEOUT
// when a pipeline wait ran out since the last check
tn_status_t split_gemm_check(tn_ctx* ctx);
// ComplexF64 GEMM in the arithmetic `prec` asks for: the split-BF16 tensor path for
// TN_PREC_MIXED / TN_PREC_SPLIT_BF16 on shapes large enough to pay for it, else the FP64
// CUDA-core kernel
tn_status_t gemm_c64(tn_ctx* ctx, tn_precision_t prec, char opa, char opb, int64_t m, int64_t n, int64_t k, cxd alpha,
                     const cxd* A, int64_t lda, int64_t sA, const cxd* B, int64_t ldb, int64_t sB, cxd beta, cxd* C,
                     int64_t ldc, int64_t sC, int64_t batch);
// tcgen05 TF32 GEMM (tn_gemm_tc.cu)
size_t tc_gemm_workspace(bool complex_in, int passes, int64_t m, int64_t n, int64_t k);
tn_status_t tc_gemm(tn_ctx* ctx, bool complex_in, int passes, char opa, char opb, int64_t m, int64_t n, int64_t k,
                    float alpha, const void* A, int64_t lda, const void* B, int64_t ldb, float beta, void* C,
                    int64_t ldc);

// K5 helpers
tn_status_t rank_select(tn_ctx* ctx, const double* S, int64_t k, int64_t maxdim,
                        double threshold, int64_t* rank);
// per-instance ranks; returns the max and zeroes S_b beyond rank_b up to the max so that
// a common (padded) bond dimension carries exactly each instance's truncated state
tn_status_t rank_select_batched(tn_ctx* ctx, double* S, int64_t k, int64_t sS, int64_t batch,
                                int64_t maxdim, double threshold, int64_t* rank_max,
                                int64_t* ranks);
template <typename T>
tn_status_t scale_cols_sqrt(tn_ctx* ctx, cx<T>* X, int64_t rows, int64_t cols, int64_t ld,
                            const double* S, int64_t sX = 0, int64_t sS = 0, int64_t batch = 1);
template <typename T>
tn_status_t scale_rows_sqrt(tn_ctx* ctx, cx<T>* X, int64_t rows, int64_t cols, int64_t ld,
                            const double* S, int64_t sX = 0, int64_t sS = 0, int64_t batch = 1);
// X_b(r, c) *= 1/sqrt(S_b[r]) (0 where S_b[r] == 0)
tn_status_t scale_rows_invsqrt(tn_ctx* ctx, cxd* X, int64_t rows, int64_t cols, int64_t ld,
                               const double* S, int64_t sX, int64_t sS, int64_t batch);
// X_b(r, c) *= S_b[r] (mode 1), or zeroed where S_b[r] == 0 (mode 0)
tn_status_t scale_rows_mode(tn_ctx* ctx, cxd* X, int64_t rows, int64_t cols, int64_t ld, const double* S, int64_t sX,
                            int64_t sS, int64_t batch, int mode);
// how a two-site update splits S between the two sites (simple_update_core)
constexpr int kAbsorbEqually = 0, kAbsorbRight = 1, kAbsorbLeft = 2;
// X_b(r, c) *= S_b[c] (mode 1), or zeroed where S_b[c] == 0 (mode 0)
tn_status_t scale_cols_mode(tn_ctx* ctx, cxd* X, int64_t rows, int64_t cols, int64_t ld, const double* S, int64_t sX,
                            int64_t sS, int64_t batch, int mode);
// out[l, p, blk] = Σ_q G[p, q] in[l, q, blk] over nblk contiguous rows × D blocks (in ≠ out)
tn_status_t apply_phys(tn_ctx* ctx, int64_t rows, int64_t D, int64_t nblk, const cxd* in, cxd* out, const cxd* G);
// dst_b (cols × rows) = src_b (rows × cols)ᴴ
tn_status_t adjoint_cxd(tn_ctx* ctx, int64_t rows, int64_t cols, const cxd* src, int64_t lds, int64_t sSrc, cxd* dst,
                        int64_t ldd, int64_t sDst, int64_t batch);
tn_status_t norm2_cxd(tn_ctx* ctx, int64_t n, const cxd* x, double* h_out);
tn_status_t copy_matrix_cxd(tn_ctx* ctx, int64_t rows, int64_t cols, const cxd* src,
                            int64_t lds, cxd* dst, int64_t ldd, int64_t sSrc = 0,
                            int64_t sDst = 0, int64_t batch = 1);
tn_status_t norms_batched(tn_ctx* ctx, bool complex_data, int64_t n, const void* x, int64_t sx,
                          int64_t batch, double* h_out);
tn_status_t zdotc_batched(tn_ctx* ctx, int64_t n, const cxd* x, int64_t sx, const cxd* y,
                          int64_t sy, int64_t batch, double* h_out);
