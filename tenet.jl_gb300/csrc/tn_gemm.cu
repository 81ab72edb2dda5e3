// K2 (native arithmetic) — batched strided complex GEMM on the CUDA cores.
//
//   C = alpha · op(A) · op(B) + beta · C,  op ∈ {N, T, C}, column-major.
//
// This is the plain-form contraction GEMM (ComplexF64 in FP64, ComplexF32 in FP32).  It
// replaces the BLAS zgemm/cgemm inside Muscle.binary_einsum.  On GB300 the FP64 pipe is
// the bound for this kernel, so the design goal is to keep every SM's DFMA units fed:
// register tiles of 4×4 (or 2×2 for small grids) complex accumulators per thread,
// A/B tiles staged through shared memory, and a tile size chosen so the grid covers
// all 152 SMs even for the small bond-dimension GEMMs of an MPS sweep.
#include "tn_internal.cuh"

namespace {

template <typename T>
__device__ __forceinline__ cx<T> load_op(const cx<T>* __restrict__ X, int64_t ld, char op,
                                         int64_t r, int64_t c) {
  // element (r, c) of op(X)
  if (op == 'N') return X[r + c * ld];
  cx<T> v = X[c + r * ld];
  if (op == 'C') v.y = -v.y;
  return v;
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm_cx(char opa, char opb, int64_t m, int64_t n, int64_t k, cx<T> alpha,
              const cx<T>* __restrict__ A, int64_t lda, int64_t sA, const cx<T>* __restrict__ B,
              int64_t ldb, int64_t sB, cx<T> beta, cx<T>* __restrict__ C, int64_t ldc, int64_t sC,
              int64_t batch, bool upper) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int RX = BN / TN;  // threads along n
  constexpr int RY = BM / TM;  // threads along m
  __shared__ cx<T> As[BK][BM + 1];
  __shared__ cx<T> Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % RX, ty = tid / RX;
  const int64_t i0 = (int64_t)blockIdx.x * BM;
  const int64_t j0 = (int64_t)blockIdx.y * BN;
  if (upper && i0 >= j0 + BN) return;  // Hermitian product: tiles below the diagonal are mirrored
  for (int64_t bz = blockIdx.z; bz < batch; bz += gridDim.z) {
    const cx<T>* Ab = A + bz * sA;
    const cx<T>* Bb = B + bz * sB;
    cx<T>* Cb = C + bz * sC;
    cx<T> acc[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
      for (int b = 0; b < TN; ++b) acc[a][b] = mkcx<T>(0, 0);

    for (int64_t p0 = 0; p0 < k; p0 += BK) {
      // stage A tile (BM × BK)
      for (int t = tid; t < BM * BK; t += NT) {
        int ii, pp;
        if (opa == 'N') {
          ii = t % BM;
          pp = t / BM;
        } else {
          pp = t % BK;
          ii = t / BK;
        }
        int64_t gi = i0 + ii, gp = p0 + pp;
        As[pp][ii] = (gi < m && gp < k) ? load_op(Ab, lda, opa, gi, gp) : mkcx<T>(0, 0);
      }
      // stage B tile (BK × BN)
      for (int t = tid; t < BK * BN; t += NT) {
        int pp, jj;
        if (opb == 'N') {
          pp = t % BK;
          jj = t / BK;
        } else {
          jj = t % BN;
          pp = t / BN;
        }
        int64_t gp = p0 + pp, gj = j0 + jj;
        Bs[pp][jj] = (gp < k && gj < n) ? load_op(Bb, ldb, opb, gp, gj) : mkcx<T>(0, 0);
      }
      __syncthreads();
#pragma unroll
      for (int pp = 0; pp < BK; ++pp) {
        cx<T> a[TM], b[TN];
#pragma unroll
        for (int r = 0; r < TM; ++r) a[r] = As[pp][ty + r * RY];
#pragma unroll
        for (int c = 0; c < TN; ++c) b[c] = Bs[pp][tx + c * RX];
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
          for (int c = 0; c < TN; ++c) cfma(acc[r][c], a[r], b[c]);
      }
      __syncthreads();
    }
    const bool beta0 = beta.x == T(0) && beta.y == T(0);
#pragma unroll
    for (int r = 0; r < TM; ++r) {
      int64_t gi = i0 + ty + r * RY;
      if (gi >= m) continue;
#pragma unroll
      for (int c = 0; c < TN; ++c) {
        int64_t gj = j0 + tx + c * RX;
        if (gj >= n) continue;
        cx<T> v = alpha * acc[r][c];
        if (!beta0) v = v + beta * Cb[gi + gj * ldc];
        Cb[gi + gj * ldc] = v;
      }
    }
  }
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
tn_status_t launch(tn_ctx* ctx, char opa, char opb, int64_t m, int64_t n, int64_t k, cx<T> alpha,
                   const cx<T>* A, int64_t lda, int64_t sA, const cx<T>* B, int64_t ldb, int64_t sB,
                   cx<T> beta, cx<T>* C, int64_t ldc, int64_t sC, int64_t batch, bool upper = false) {
  dim3 grid(cdiv(m, BM), cdiv(n, BN), (unsigned)(batch < 65535 ? batch : 65535));
  if (grid.x > 0x7fffffffu || grid.y > 65535u) return tn_set_error(ctx, TN_EINVAL, "gemm: grid too large");
  const int slot = sizeof(T) == 8 ? prof_begin(ctx) : -1;
  k_gemm_cx<T, BM, BN, BK, TM, TN><<<grid, (BM / TM) * (BN / TN), 0, ctx->stream>>>(
      opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, upper);
  TN_LAUNCHED(ctx);
  if (slot >= 0) {
    const bool b0 = beta.x == T(0) && beta.y == T(0);
    prof_end(ctx, slot, TN_PROF_GEMM_F64, 1, 8.0 * m * n * k * batch,
             sizeof(cx<T>) * ((double)m * k + (double)k * n + (double)m * n * (b0 ? 1 : 2)) * batch);
  }
  return TN_OK;
}

// C(i, j) = conj(C(j, i)) for i > j (n × n, batched)
template <typename T>
__global__ void k_mirror_lower(int64_t n, cx<T>* C, int64_t ldc, int64_t sC, int64_t batch) {
  const int64_t total = n * n;
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
      const int64_t i = t % n, j = t / n;
      if (i > j) C[b * sC + i + j * ldc] = conjg(C[b * sC + j + i * ldc]);
    }
}

}  // namespace

template <typename T>
tn_status_t gemm_cx(tn_ctx* ctx, char opa, char opb, int64_t m, int64_t n, int64_t k, cx<T> alpha,
                    const cx<T>* A, int64_t lda, int64_t sA, const cx<T>* B, int64_t ldb,
                    int64_t sB, cx<T> beta, cx<T>* C, int64_t ldc, int64_t sC, int64_t batch) {
  if (m == 0 || n == 0 || batch == 0) return TN_OK;
  if (k == 0) {
    // C = beta C: run the kernel with an empty reduction
  }
  // a few rows against wide operands (batched amplitudes, environment rows): row tiles
  // of 8 / 16 so the DFMA work is not spent on padding
  if (m <= 8 && n >= 64)
    return launch<T, 8, 32, 8, 1, 1>(ctx, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
  if (m <= 16 && n >= 64)
    return launch<T, 16, 32, 8, 2, 1>(ctx, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
  int64_t tiles64 = (int64_t)cdiv(m, 64) * cdiv(n, 64) * batch;
  if (tiles64 >= ctx->num_sms)
    return launch<T, 64, 64, 8, 4, 4>(ctx, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C,
                                      ldc, sC, batch);
  return launch<T, 32, 32, 8, 2, 2>(ctx, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C,
                                    ldc, sC, batch);
}

// C = Aᴴ A (k × n input, n × n Hermitian output, batched): the tiles on and above the
// diagonal by the GEMM kernel, the rest mirrored
template <typename T>
tn_status_t herk_cx(tn_ctx* ctx, int64_t n, int64_t k, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* C, int64_t ldc,
                    int64_t sC, int64_t batch) {
  if (n == 0 || batch == 0) return TN_OK;
  const cx<T> one = mkcx<T>(1, 0), zero = mkcx<T>(0, 0);
  const int64_t tiles64 = (int64_t)cdiv(n, 64) * cdiv(n, 64) * batch;
  if (tiles64 >= 2 * ctx->num_sms)
    TN_RETURN_IF((launch<T, 64, 64, 8, 4, 4>(ctx, 'C', 'N', n, n, k, one, A, lda, sA, A, lda, sA, zero, C, ldc, sC,
                                              batch, true)));
  else
    TN_RETURN_IF((launch<T, 32, 32, 8, 2, 2>(ctx, 'C', 'N', n, n, k, one, A, lda, sA, A, lda, sA, zero, C, ldc, sC,
                                              batch, true)));
  const int64_t blocks = std::min<int64_t>((n * n + 255) / 256, 2048);
  k_mirror_lower<T><<<dim3((unsigned)blocks, (unsigned)(batch < 65535 ? batch : 65535)), 256, 0, ctx->stream>>>(
      n, C, ldc, sC, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}
template tn_status_t herk_cx<double>(tn_ctx*, int64_t, int64_t, const cxd*, int64_t, int64_t, cxd*, int64_t, int64_t,
                                     int64_t);

template tn_status_t gemm_cx<double>(tn_ctx*, char, char, int64_t, int64_t, int64_t, cxd,
                                     const cxd*, int64_t, int64_t, const cxd*, int64_t, int64_t,
                                     cxd, cxd*, int64_t, int64_t, int64_t);
template tn_status_t gemm_cx<float>(tn_ctx*, char, char, int64_t, int64_t, int64_t, cxf,
                                    const cxf*, int64_t, int64_t, const cxf*, int64_t, int64_t,
                                    cxf, cxf*, int64_t, int64_t, int64_t);

// real GEMMs reuse the complex kernel through a zero-imaginary copy would waste half the
// work; they go through a dedicated real kernel below.
namespace {
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm_re(char opa, char opb, int64_t m, int64_t n, int64_t k, T alpha, const T* __restrict__ A,
              int64_t lda, int64_t sA, const T* __restrict__ B, int64_t ldb, int64_t sB, T beta,
              T* __restrict__ C, int64_t ldc, int64_t sC, int64_t batch) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int RX = BN / TN, RY = BM / TM;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x, tx = tid % RX, ty = tid / RX;
  const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
  for (int64_t bz = blockIdx.z; bz < batch; bz += gridDim.z) {
    const T* Ab = A + bz * sA;
    const T* Bb = B + bz * sB;
    T* Cb = C + bz * sC;
    T acc[TM][TN] = {};
    for (int64_t p0 = 0; p0 < k; p0 += BK) {
      for (int t = tid; t < BM * BK; t += NT) {
        int ii = opa == 'N' ? t % BM : t / BK, pp = opa == 'N' ? t / BM : t % BK;
        int64_t gi = i0 + ii, gp = p0 + pp;
        As[pp][ii] = (gi < m && gp < k) ? (opa == 'N' ? Ab[gi + gp * lda] : Ab[gp + gi * lda]) : T(0);
      }
      for (int t = tid; t < BK * BN; t += NT) {
        int pp = opb == 'N' ? t % BK : t / BN, jj = opb == 'N' ? t / BK : t % BN;
        int64_t gp = p0 + pp, gj = j0 + jj;
        Bs[pp][jj] = (gp < k && gj < n) ? (opb == 'N' ? Bb[gp + gj * ldb] : Bb[gj + gp * ldb]) : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int pp = 0; pp < BK; ++pp)
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
          for (int c = 0; c < TN; ++c) acc[r][c] = fma(As[pp][ty + r * RY], Bs[pp][tx + c * RX], acc[r][c]);
      __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < TM; ++r) {
      int64_t gi = i0 + ty + r * RY;
      if (gi >= m) continue;
#pragma unroll
      for (int c = 0; c < TN; ++c) {
        int64_t gj = j0 + tx + c * RX;
        if (gj >= n) continue;
        T v = alpha * acc[r][c];
        if (beta != T(0)) v += beta * Cb[gi + gj * ldc];
        Cb[gi + gj * ldc] = v;
      }
    }
  }
}
}  // namespace

template <typename T>
static tn_status_t gemm_re(tn_ctx* ctx, char opa, char opb, int64_t m, int64_t n, int64_t k, T alpha,
                           const T* A, int64_t lda, int64_t sA, const T* B, int64_t ldb, int64_t sB,
                           T beta, T* C, int64_t ldc, int64_t sC, int64_t batch) {
  if (m == 0 || n == 0 || batch == 0) return TN_OK;
  dim3 grid(cdiv(m, 64), cdiv(n, 64), (unsigned)(batch < 65535 ? batch : 65535));
  k_gemm_re<T, 64, 64, 16, 4, 4><<<grid, 256, 0, ctx->stream>>>(opa, opb, m, n, k, alpha, A, lda, sA, B,
                                                                ldb, sB, beta, C, ldc, sC, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

static bool valid_op(char c) { return c == 'N' || c == 'T' || c == 'C'; }

// The tensor path pays an operand-preparation pass (split + 4M expansion) and 128×128
// tiles; skinny GEMMs (any of m, n < 64 or k < 32) are HBM-bound and stay on the FP32
// CUDA cores, which are also the more accurate choice.
static bool use_tensor_path(tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n, int64_t k) {
  return (dt == TN_C32 || dt == TN_F32) && prec != TN_PREC_NATIVE && m >= 64 && n >= 64 && k >= 32;
}

size_t gemm_any_workspace(tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n, int64_t k) {
  if (use_tensor_path(dt, prec, m, n, k)) return tc_gemm_workspace(dt == TN_C32, prec == TN_PREC_TF32 ? 1 : 3, m, n, k);
  return 0;
}

tn_status_t gemm_any(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, char opa, char opb, int64_t m, int64_t n,
                     int64_t k, const double* alpha, const void* A, int64_t lda, int64_t strideA, const void* B,
                     int64_t ldb, int64_t strideB, const double* beta, void* C, int64_t ldc, int64_t strideC,
                     int64_t batch) {
  const bool tc = use_tensor_path(dtype, prec, m, n, k);
  if (tc) {
    if (dtype == TN_C32 && (alpha[1] != 0.0 || beta[1] != 0.0))
      return tn_set_error(ctx, TN_EUNSUPPORTED, "tensor-core GEMM: complex alpha/beta not supported");
    const int passes = prec == TN_PREC_TF32 ? 1 : 3;
    const size_t es = dtype == TN_C32 ? 8 : 4;
    const size_t top = ctx->ws_top;
    for (int64_t b = 0; b < batch; ++b) {
      ctx->ws_top = top;
      TN_RETURN_IF(tc_gemm(ctx, dtype == TN_C32, passes, opa, opb, m, n, k, (float)alpha[0],
                           (const char*)A + es * b * strideA, lda, (const char*)B + es * b * strideB, ldb, (float)beta[0],
                           (char*)C + es * b * strideC, ldc));
    }
    ctx->ws_top = top;
    return TN_OK;
  }
  switch (dtype) {
    case TN_C64: {
      cxd a = mkcx(alpha[0], alpha[1]), b = mkcx(beta[0], beta[1]);
      return gemm_c64(ctx, prec, opa, opb, m, n, k, a, (const cxd*)A, lda, strideA, (const cxd*)B, ldb, strideB, b,
                      (cxd*)C, ldc, strideC, batch);
    }
    case TN_C32: {
      cxf a = mkcx((float)alpha[0], (float)alpha[1]), b = mkcx((float)beta[0], (float)beta[1]);
      return gemm_cx<float>(ctx, opa, opb, m, n, k, a, (const cxf*)A, lda, strideA, (const cxf*)B, ldb, strideB, b,
                            (cxf*)C, ldc, strideC, batch);
    }
    case TN_F64:
      return gemm_re<double>(ctx, opa, opb, m, n, k, alpha[0], (const double*)A, lda, strideA, (const double*)B, ldb,
                             strideB, beta[0], (double*)C, ldc, strideC, batch);
    case TN_F32:
      return gemm_re<float>(ctx, opa, opb, m, n, k, (float)alpha[0], (const float*)A, lda, strideA, (const float*)B,
                            ldb, strideB, (float)beta[0], (float*)C, ldc, strideC, batch);
  }
  return tn_set_error(ctx, TN_EINVAL, "gemm: bad dtype");
}

extern "C" tn_status_t tn_gemm(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, char opa, char opb,
                               int64_t m, int64_t n, int64_t k, const double* alpha, const void* A,
                               int64_t lda, int64_t strideA, const void* B, int64_t ldb,
                               int64_t strideB, const double* beta, void* C, int64_t ldc,
                               int64_t strideC, int64_t batch) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, valid_op(opa) && valid_op(opb), "tn_gemm: op must be 'N', 'T' or 'C'");
  TN_ARG(ctx, m >= 0 && n >= 0 && k >= 0 && batch >= 0, "tn_gemm: negative size");
  TN_ARG(ctx, alpha && beta, "tn_gemm: null alpha/beta");
  TN_ARG(ctx, (m == 0 || n == 0 || batch == 0) || (A && B && C), "tn_gemm: null matrix");
  TN_ARG(ctx, dtype_complex(dtype) || (opa != 'C' && opb != 'C'), "tn_gemm: 'C' needs a complex dtype");
  int64_t ra = opa == 'N' ? m : k, rb = opb == 'N' ? k : n;
  TN_ARG(ctx, lda >= (ra > 1 ? ra : 1) && ldb >= (rb > 1 ? rb : 1) && ldc >= (m > 1 ? m : 1),
         "tn_gemm: leading dimension too small");
  TN_RETURN_IF(ws_reserve(ctx, gemm_any_workspace(dtype, prec, m, n, k)));
  TN_RETURN_IF(gemm_any(ctx, dtype, prec, opa, opb, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C, ldc,
                        strideC, batch));
  return split_gemm_check(ctx);
}
