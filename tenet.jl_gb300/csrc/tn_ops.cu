// K5 — small fused ops: Hadamard (Λ absorption), √S absorption into U / Vh, the
// truncation-rank decision on the singular-value spectrum, FP64 norms.
#include <algorithm>

#include "tn_internal.cuh"

namespace {

template <typename E, typename R>
__global__ void k_hadamard(int64_t total, int64_t inner, int64_t ext, const E* __restrict__ t,
                           const double* __restrict__ s, E* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t a = (i / inner) % ext;
    out[i] = R::mul(t[i], s[a]);
  }
}
struct MulR64 {
  __device__ static double mul(double x, double s) { return x * s; }
};
struct MulR32 {
  __device__ static float mul(float x, double s) { return (float)(x * s); }
};
struct MulC64 {
  __device__ static double2 mul(double2 x, double s) { return make_double2(x.x * s, x.y * s); }
};
struct MulC32 {
  __device__ static float2 mul(float2 x, double s) { return make_float2((float)(x.x * s), (float)(x.y * s)); }
};

// X_b(r, c) *= sqrt(S_b[c])   (rows × cols, ld; batch strides sX, sS)
template <typename T>
__global__ void k_scale_cols_sqrt(cx<T>* X, int64_t rows, int64_t cols, int64_t ld, int64_t sX, const double* S,
                                  int64_t sS, int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % rows, c = t / rows;
      X[b * sX + r + c * ld] = T(sqrt(S[b * sS + c])) * X[b * sX + r + c * ld];
    }
}
// X_b(r, c) *= sqrt(S_b[r])
template <typename T>
__global__ void k_scale_rows_sqrt(cx<T>* X, int64_t rows, int64_t cols, int64_t ld, int64_t sX, const double* S,
                                  int64_t sS, int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % rows, c = t / rows;
      X[b * sX + r + c * ld] = T(sqrt(S[b * sS + r])) * X[b * sX + r + c * ld];
    }
}

__global__ void k_scale_rows_invsqrt(cxd* X, int64_t rows, int64_t cols, int64_t ld, int64_t sX, const double* S,
                                     int64_t sS, int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % rows, c = t / rows;
      const double s = S[b * sS + r];
      const double f = s > 0.0 ? 1.0 / sqrt(s) : 0.0;
      X[b * sX + r + c * ld] = f * X[b * sX + r + c * ld];
    }
}

// X_b(r, c) *= S_b[r] (mode 1) or keeps its value where S_b[r] > 0 and becomes 0 elsewhere
// (mode 0: the rows beyond an instance's kept rank of a zero-padded batch)
__global__ void k_scale_rows_mode(cxd* X, int64_t rows, int64_t cols, int64_t ld, int64_t sX, const double* S,
                                  int64_t sS, int64_t batch, int mode) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % rows, c = t / rows;
      const double s = S[b * sS + r];
      const double f = mode == 1 ? s : (s > 0.0 ? 1.0 : 0.0);
      X[b * sX + r + c * ld] = f * X[b * sX + r + c * ld];
    }
}

// rank_b = #{ j < min(maxdim, k) : |S_b[j]| > threshold }, at least 1 (S descending);
// one block per instance
__global__ void k_rank_select(const double* S, int64_t k, int64_t sS, int64_t maxdim, double threshold, int* out) {
  __shared__ int cnt;
  const double* Sb = S + blockIdx.x * sS;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int64_t kk = (maxdim > 0 && maxdim < k) ? maxdim : k;
  int local = 0;
  for (int64_t j = threadIdx.x; j < kk; j += blockDim.x) local += (threshold <= 0.0 || fabs(Sb[j]) > threshold) ? 1 : 0;
  atomicAdd(&cnt, local);
  __syncthreads();
  if (threadIdx.x == 0) out[blockIdx.x] = cnt > 0 ? cnt : 1;
}
// S_b[j] = 0 for rank_b <= j < r (padding of a common bond dimension)
__global__ void k_zero_tail(double* S, int64_t sS, const int* rank, int64_t r, int64_t batch) {
  const int64_t b = blockIdx.x;
  if (b >= batch) return;
  for (int64_t j = rank[b] + threadIdx.x; j < r; j += blockDim.x) S[b * sS + j] = 0.0;
}

template <typename E>
__device__ __forceinline__ double nrm2_elem(E v);
template <>
__device__ __forceinline__ double nrm2_elem<double>(double v) {
  return v * v;
}
template <>
__device__ __forceinline__ double nrm2_elem<float>(float v) {
  return (double)v * v;
}
template <>
__device__ __forceinline__ double nrm2_elem<double2>(double2 v) {
  return v.x * v.x + v.y * v.y;
}
template <>
__device__ __forceinline__ double nrm2_elem<float2>(float2 v) {
  return (double)v.x * v.x + (double)v.y * v.y;
}

// two-level deterministic reduction: fixed grid, per-block partials, then one block
template <typename E>
__global__ void k_sumsq_partial(int64_t n, const E* __restrict__ x, double* partial) {
  __shared__ double red[32];
  double s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += nrm2_elem<E>(x[i]);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}
__global__ void k_sum_final(int n, const double* partial, double* out) {
  __shared__ double red[32];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) out[0] = v;
  }
}

template <typename E>
__global__ void k_scale(int64_t n, E* x, double s);
template <>
__global__ void k_scale<double>(int64_t n, double* x, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= s;
}
template <>
__global__ void k_scale<float>(int64_t n, float* x, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (float)(x[i] * s);
}
template <>
__global__ void k_scale<double2>(int64_t n, double2* x, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i].x *= s;
    x[i].y *= s;
  }
}
template <>
__global__ void k_scale<float2>(int64_t n, float2* x, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i].x = (float)(x[i].x * s);
    x[i].y = (float)(x[i].y * s);
  }
}

__global__ void k_copy_matrix(int64_t rows, int64_t cols, const cxd* src, int64_t lds, int64_t sSrc, cxd* dst,
                              int64_t ldd, int64_t sDst, int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % rows, c = t / rows;
      dst[b * sDst + r + c * ldd] = src[b * sSrc + r + c * lds];
    }
}

unsigned blocks_for(tn_ctx* ctx, int64_t n) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)ctx->num_sms * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

template <typename E>
tn_status_t sumsq(tn_ctx* ctx, int64_t n, const E* x, double* h_out) {
  int* flags = nullptr;
  const int nb = 256;
  TN_RETURN_IF(ctx_flags(ctx, 2 * (nb + 2), &flags));
  double* partial = reinterpret_cast<double*>(flags);
  k_sumsq_partial<E><<<nb, 256, 0, ctx->stream>>>(n, x, partial);
  TN_LAUNCHED(ctx);
  k_sum_final<<<1, 256, 0, ctx->stream>>>(nb, partial, partial + nb);
  TN_LAUNCHED(ctx);
  double* hp = reinterpret_cast<double*>(ctx->pinned);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(hp, partial + nb, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *h_out = hp[0];
  return TN_OK;
}

}  // namespace

tn_status_t rank_select_batched(tn_ctx* ctx, double* S, int64_t k, int64_t sS, int64_t batch, int64_t maxdim,
                                double threshold, int64_t* rank_max, int64_t* ranks) {
  int* flags = nullptr;
  TN_RETURN_IF(ctx_flags(ctx, (size_t)batch + 4, &flags));
  if (batch > 8192) return tn_set_error(ctx, TN_EUNSUPPORTED, "rank select: batch > 8192");
  k_rank_select<<<(unsigned)batch, 256, 0, ctx->stream>>>(S, k, sS, maxdim, threshold, flags);
  TN_LAUNCHED(ctx);
  int* hp = reinterpret_cast<int*>(ctx->pinned);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(hp, flags, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t r = 0;
  bool uneven = false;
  for (int64_t b = 0; b < batch; ++b) {
    if (ranks) ranks[b] = hp[b];
    r = hp[b] > r ? hp[b] : r;
  }
  for (int64_t b = 0; b < batch; ++b) uneven |= hp[b] != r;
  if (uneven) {
    k_zero_tail<<<(unsigned)batch, 128, 0, ctx->stream>>>(S, sS, flags, r, batch);
    TN_LAUNCHED(ctx);
  }
  *rank_max = r;
  return TN_OK;
}

tn_status_t rank_select(tn_ctx* ctx, const double* S, int64_t k, int64_t maxdim, double threshold, int64_t* rank) {
  return rank_select_batched(ctx, const_cast<double*>(S), k, k, 1, maxdim, threshold, rank, nullptr);
}

template <typename T>
tn_status_t scale_cols_sqrt(tn_ctx* ctx, cx<T>* X, int64_t rows, int64_t cols, int64_t ld, const double* S,
                            int64_t sX, int64_t sS, int64_t batch) {
  if (rows * cols * batch == 0) return TN_OK;
  dim3 g(blocks_for(ctx, rows * cols), (unsigned)(batch < 65535 ? batch : 65535));
  k_scale_cols_sqrt<T><<<g, 256, 0, ctx->stream>>>(X, rows, cols, ld, sX, S, sS, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}
template <typename T>
tn_status_t scale_rows_sqrt(tn_ctx* ctx, cx<T>* X, int64_t rows, int64_t cols, int64_t ld, const double* S,
                            int64_t sX, int64_t sS, int64_t batch) {
  if (rows * cols * batch == 0) return TN_OK;
  dim3 g(blocks_for(ctx, rows * cols), (unsigned)(batch < 65535 ? batch : 65535));
  k_scale_rows_sqrt<T><<<g, 256, 0, ctx->stream>>>(X, rows, cols, ld, sX, S, sS, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}
template tn_status_t scale_cols_sqrt<double>(tn_ctx*, cxd*, int64_t, int64_t, int64_t, const double*, int64_t, int64_t, int64_t);
template tn_status_t scale_cols_sqrt<float>(tn_ctx*, cxf*, int64_t, int64_t, int64_t, const double*, int64_t, int64_t, int64_t);
template tn_status_t scale_rows_sqrt<double>(tn_ctx*, cxd*, int64_t, int64_t, int64_t, const double*, int64_t, int64_t, int64_t);
template tn_status_t scale_rows_sqrt<float>(tn_ctx*, cxf*, int64_t, int64_t, int64_t, const double*, int64_t, int64_t, int64_t);

tn_status_t norm2_cxd(tn_ctx* ctx, int64_t n, const cxd* x, double* h_out) {
  double ss = 0;
  TN_RETURN_IF(sumsq<double2>(ctx, n, reinterpret_cast<const double2*>(x), &ss));
  *h_out = sqrt(ss);
  return TN_OK;
}

tn_status_t scale_rows_mode(tn_ctx* ctx, cxd* X, int64_t rows, int64_t cols, int64_t ld, const double* S, int64_t sX,
                            int64_t sS, int64_t batch, int mode) {
  if (rows * cols * batch == 0) return TN_OK;
  dim3 g(blocks_for(ctx, rows * cols), (unsigned)(batch < 65535 ? batch : 65535));
  k_scale_rows_mode<<<g, 256, 0, ctx->stream>>>(X, rows, cols, ld, sX, S, sS, batch, mode);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// X_b(r, c) *= S_b[c] (mode 1), or zeroed where S_b[c] == 0 (mode 0)
__global__ void k_scale_cols_mode(cxd* X, int64_t rows, int64_t cols, int64_t ld, int64_t sX, const double* S,
                                  int64_t sS, int64_t batch, int mode) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols; t += (int64_t)gridDim.x * blockDim.x) {
      const int64_t r = t % rows, c = t / rows;
      const double s = S[b * sS + c];
      const double f = mode == 1 ? s : (s > 0.0 ? 1.0 : 0.0);
      X[b * sX + r + c * ld] = f * X[b * sX + r + c * ld];
    }
}

tn_status_t scale_cols_mode(tn_ctx* ctx, cxd* X, int64_t rows, int64_t cols, int64_t ld, const double* S, int64_t sX,
                            int64_t sS, int64_t batch, int mode) {
  if (rows * cols * batch == 0) return TN_OK;
  dim3 g(blocks_for(ctx, rows * cols), (unsigned)(batch < 65535 ? batch : 65535));
  k_scale_cols_mode<<<g, 256, 0, ctx->stream>>>(X, rows, cols, ld, sX, S, sS, batch, mode);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// out[l, p, blk] = Σ_q G[p, q] · in[l, q, blk] for blocks of rows × D (column-major,
// contiguous, D ≤ 16): one thread per (l, blk) holds the D inputs and writes the D
// outputs; G (D × D, column-major) sits in shared memory.  Reads and writes each element
// once, coalesced along l (a physical-index operator on an MPS site or a two-site θ).
template <int D>
__global__ void __launch_bounds__(256) k_apply_phys(int64_t rows, int64_t nblk, const cxd* __restrict__ in,
                                                     cxd* __restrict__ out, const cxd* __restrict__ G) {
  __shared__ cxd g[D * D];
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) g[t] = G[t];
  __syncthreads();
  const int64_t total = rows * nblk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = t % rows, blk = t / rows;
    const cxd* src = in + blk * rows * D + l;
    cxd x[D];
#pragma unroll
    for (int q = 0; q < D; ++q) x[q] = src[q * rows];
    cxd* dst = out + blk * rows * D + l;
#pragma unroll
    for (int p2 = 0; p2 < D; ++p2) {
      cxd acc = mkcx(0.0, 0.0);
#pragma unroll
      for (int q = 0; q < D; ++q) cfma(acc, g[p2 + q * D], x[q]);
      dst[p2 * rows] = acc;
    }
  }
}

tn_status_t apply_phys(tn_ctx* ctx, int64_t rows, int64_t D, int64_t nblk, const cxd* in, cxd* out, const cxd* G) {
  if (rows * nblk == 0) return TN_OK;
  const unsigned g = (unsigned)std::min<int64_t>((rows * nblk + 255) / 256, (int64_t)ctx->num_sms * 16);
  switch (D) {
    case 2: k_apply_phys<2><<<g, 256, 0, ctx->stream>>>(rows, nblk, in, out, G); break;
    case 3: k_apply_phys<3><<<g, 256, 0, ctx->stream>>>(rows, nblk, in, out, G); break;
    case 4: k_apply_phys<4><<<g, 256, 0, ctx->stream>>>(rows, nblk, in, out, G); break;
    case 9: k_apply_phys<9><<<g, 256, 0, ctx->stream>>>(rows, nblk, in, out, G); break;
    case 16: k_apply_phys<16><<<g, 256, 0, ctx->stream>>>(rows, nblk, in, out, G); break;
    default:
      return gemm_cx<double>(ctx, 'N', 'T', rows, D, D, mkcx(1.0, 0.0), in, rows, rows * D, G, D, 0, mkcx(0.0, 0.0), out,
                             rows, rows * D, nblk);
  }
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// dst_b (cols × rows, ld ldd) = src_b (rows × cols, ld lds)ᴴ through 32×32 shared-memory
// tiles (both sides coalesced); grid (tiles, batch)
__global__ void __launch_bounds__(256) k_adjoint_cxd(int64_t rows, int64_t cols, const cxd* __restrict__ src,
                                                     int64_t lds, int64_t sSrc, cxd* __restrict__ dst, int64_t ldd,
                                                     int64_t sDst, int64_t batch) {
  __shared__ cxd tile[32][33];
  const int64_t tr = (rows + 31) / 32, tcn = (cols + 31) / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 × 8
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x; t < tr * tcn; t += gridDim.x) {
      const int64_t r0 = (t % tr) * 32, c0 = (t / tr) * 32;
      for (int q = ty; q < 32; q += 8) {
        const int64_t r = r0 + tx, c = c0 + q;
        if (r < rows && c < cols) tile[q][tx] = src[b * sSrc + r + c * lds];
      }
      __syncthreads();
      for (int q = ty; q < 32; q += 8) {
        const int64_t c = c0 + tx, r = r0 + q;  // dst(c, r) = conj(src(r, c))
        if (r < rows && c < cols) {
          const cxd v = tile[tx][q];
          dst[b * sDst + c + r * ldd] = mkcx(v.x, -v.y);
        }
      }
      __syncthreads();
    }
}

tn_status_t adjoint_cxd(tn_ctx* ctx, int64_t rows, int64_t cols, const cxd* src, int64_t lds, int64_t sSrc, cxd* dst,
                        int64_t ldd, int64_t sDst, int64_t batch) {
  if (rows * cols * batch == 0) return TN_OK;
  const int64_t tiles = ((rows + 31) / 32) * ((cols + 31) / 32);
  dim3 g((unsigned)std::min<int64_t>(tiles, 4096), (unsigned)(batch < 65535 ? batch : 65535));
  k_adjoint_cxd<<<g, 256, 0, ctx->stream>>>(rows, cols, src, lds, sSrc, dst, ldd, sDst, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

tn_status_t scale_rows_invsqrt(tn_ctx* ctx, cxd* X, int64_t rows, int64_t cols, int64_t ld, const double* S,
                               int64_t sX, int64_t sS, int64_t batch) {
  if (rows * cols * batch == 0) return TN_OK;
  dim3 g(blocks_for(ctx, rows * cols), (unsigned)(batch < 65535 ? batch : 65535));
  k_scale_rows_invsqrt<<<g, 256, 0, ctx->stream>>>(X, rows, cols, ld, sX, S, sS, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

tn_status_t copy_matrix_cxd(tn_ctx* ctx, int64_t rows, int64_t cols, const cxd* src, int64_t lds, cxd* dst,
                            int64_t ldd, int64_t sSrc, int64_t sDst, int64_t batch) {
  if (rows * cols * batch == 0) return TN_OK;
  dim3 g(blocks_for(ctx, rows * cols), (unsigned)(batch < 65535 ? batch : 65535));
  k_copy_matrix<<<g, 256, 0, ctx->stream>>>(rows, cols, src, lds, sSrc, dst, ldd, sDst, batch);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// per-instance Σ|x|² for a batch of equal-length vectors at stride sx (FP64), to host
__global__ void k_sumsq_batched(int64_t n, const double2* x, int64_t sx, double* out) {
  __shared__ double red[32];
  const double2* xb = x + blockIdx.x * sx;
  double s = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += xb[i].x * xb[i].x + xb[i].y * xb[i].y;
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) out[blockIdx.x] = v;
  }
}
__global__ void k_sumsq_real_batched(int64_t n, const double* x, int64_t sx, double* out) {
  __shared__ double red[32];
  const double* xb = x + blockIdx.x * sx;
  double s = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += xb[i] * xb[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) out[blockIdx.x] = v;
  }
}
tn_status_t norms_batched(tn_ctx* ctx, bool complex_data, int64_t n, const void* x, int64_t sx, int64_t batch,
                          double* h_out) {
  int* flags = nullptr;
  TN_RETURN_IF(ctx_flags(ctx, 2 * (size_t)batch + 8, &flags));
  double* d = reinterpret_cast<double*>(flags);
  if (complex_data)
    k_sumsq_batched<<<(unsigned)batch, 512, 0, ctx->stream>>>(n, (const double2*)x, sx, d);
  else
    k_sumsq_real_batched<<<(unsigned)batch, 512, 0, ctx->stream>>>(n, (const double*)x, sx, d);
  TN_LAUNCHED(ctx);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_out, d, sizeof(double) * batch, cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int64_t b = 0; b < batch; ++b) h_out[b] = sqrt(h_out[b]);
  return TN_OK;
}

// batched zdotc: out_b = Σ conj(x_b)·y_b (FP64, fixed order), to host
__global__ void k_zdotc_batched(int64_t n, const double2* x, int64_t sx, const double2* y, int64_t sy, double* out) {
  __shared__ double rx[32], ry[32];
  const double2* xb = x + blockIdx.x * sx;
  const double2* yb = y + blockIdx.x * sy;
  double sr = 0, si = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double2 a = xb[i], c = yb[i];
    sr = fma(a.x, c.x, sr);
    sr = fma(a.y, c.y, sr);
    si = fma(a.x, c.y, si);
    si = fma(-a.y, c.x, si);
  }
  sr = warp_sum(sr);
  si = warp_sum(si);
  if ((threadIdx.x & 31) == 0) {
    rx[threadIdx.x >> 5] = sr;
    ry[threadIdx.x >> 5] = si;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double vx = threadIdx.x < (blockDim.x >> 5) ? rx[threadIdx.x] : 0.0;
    double vy = threadIdx.x < (blockDim.x >> 5) ? ry[threadIdx.x] : 0.0;
    vx = warp_sum(vx);
    vy = warp_sum(vy);
    if (threadIdx.x == 0) {
      out[2 * blockIdx.x] = vx;
      out[2 * blockIdx.x + 1] = vy;
    }
  }
}
tn_status_t zdotc_batched(tn_ctx* ctx, int64_t n, const cxd* x, int64_t sx, const cxd* y, int64_t sy, int64_t batch,
                          double* h_out) {
  int* flags = nullptr;
  TN_RETURN_IF(ctx_flags(ctx, 4 * (size_t)batch + 8, &flags));
  double* d = reinterpret_cast<double*>(flags);
  k_zdotc_batched<<<(unsigned)batch, 512, 0, ctx->stream>>>(n, (const double2*)x, sx, (const double2*)y, sy, d);
  TN_LAUNCHED(ctx);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_out, d, 2 * sizeof(double) * batch, cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

namespace {
// y += a x (complex a)
__global__ void k_axpy_cx(int64_t n, double ar, double ai, const double2* __restrict__ x, double2* __restrict__ y) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = x[t];
    double2 w = y[t];
    w.x = fma(ar, v.x, fma(-ai, v.y, w.x));
    w.y = fma(ar, v.y, fma(ai, v.x, w.y));
    y[t] = w;
  }
}
}  // namespace

extern "C" {

tn_status_t tn_truncation_rank(tn_ctx* ctx, const double* S, int64_t k, int64_t maxdim, double threshold,
                               int64_t* rank) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, S && rank && k > 0, "tn_truncation_rank: bad arguments");
  return rank_select(ctx, S, k, maxdim, threshold, rank);
}

tn_status_t tn_hadamard(tn_ctx* ctx, tn_dtype_t dtype, int32_t rank, const int64_t* dims, int32_t axis,
                        const void* t, const double* s, void* out) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, rank >= 1 && rank <= TN_MAX_RANK && axis >= 0 && axis < rank, "tn_hadamard: bad rank/axis");
  TN_ARG(ctx, dims && t && s && out, "tn_hadamard: null pointer");
  int64_t inner = 1, total = 1;
  for (int i = 0; i < rank; ++i) {
    TN_ARG(ctx, dims[i] >= 0, "tn_hadamard: negative extent");
    if (i < axis) inner *= dims[i];
    total *= dims[i];
  }
  if (total == 0) return TN_OK;
  unsigned nb = blocks_for(ctx, total);
  switch (dtype) {
    case TN_F64: k_hadamard<double, MulR64><<<nb, 256, 0, ctx->stream>>>(total, inner, dims[axis], (const double*)t, s, (double*)out); break;
    case TN_F32: k_hadamard<float, MulR32><<<nb, 256, 0, ctx->stream>>>(total, inner, dims[axis], (const float*)t, s, (float*)out); break;
    case TN_C64: k_hadamard<double2, MulC64><<<nb, 256, 0, ctx->stream>>>(total, inner, dims[axis], (const double2*)t, s, (double2*)out); break;
    case TN_C32: k_hadamard<float2, MulC32><<<nb, 256, 0, ctx->stream>>>(total, inner, dims[axis], (const float2*)t, s, (float2*)out); break;
    default: return tn_set_error(ctx, TN_EINVAL, "tn_hadamard: bad dtype");
  }
  TN_LAUNCHED(ctx);
  return TN_OK;
}

tn_status_t tn_norm2(tn_ctx* ctx, tn_dtype_t dtype, int64_t n, const void* x, double* h_out) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, n >= 0 && h_out && (n == 0 || x), "tn_norm2: bad arguments");
  if (n == 0) {
    *h_out = 0;
    return TN_OK;
  }
  double ss = 0;
  switch (dtype) {
    case TN_F64: TN_RETURN_IF(sumsq<double>(ctx, n, (const double*)x, &ss)); break;
    case TN_F32: TN_RETURN_IF(sumsq<float>(ctx, n, (const float*)x, &ss)); break;
    case TN_C64: TN_RETURN_IF(sumsq<double2>(ctx, n, (const double2*)x, &ss)); break;
    case TN_C32: TN_RETURN_IF(sumsq<float2>(ctx, n, (const float2*)x, &ss)); break;
    default: return tn_set_error(ctx, TN_EINVAL, "tn_norm2: bad dtype");
  }
  *h_out = sqrt(ss);
  return TN_OK;
}

tn_status_t tn_scale(tn_ctx* ctx, tn_dtype_t dtype, int64_t n, void* x, double s) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, n >= 0 && (n == 0 || x), "tn_scale: bad arguments");
  if (n == 0) return TN_OK;
  unsigned nb = blocks_for(ctx, n);
  switch (dtype) {
    case TN_F64: k_scale<double><<<nb, 256, 0, ctx->stream>>>(n, (double*)x, s); break;
    case TN_F32: k_scale<float><<<nb, 256, 0, ctx->stream>>>(n, (float*)x, s); break;
    case TN_C64: k_scale<double2><<<nb, 256, 0, ctx->stream>>>(n, (double2*)x, s); break;
    case TN_C32: k_scale<float2><<<nb, 256, 0, ctx->stream>>>(n, (float2*)x, s); break;
    default: return tn_set_error(ctx, TN_EINVAL, "tn_scale: bad dtype");
  }
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// ⟨x, y⟩ = Σ conj(x_i) y_i for ComplexF64 vectors (h_out = re, im): the Krylov solver's dot
tn_status_t tn_dotc(tn_ctx* ctx, int64_t n, const void* x, const void* y, double* h_out) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, n >= 0 && h_out && (n == 0 || (x && y)), "tn_dotc: bad arguments");
  if (n == 0) {
    h_out[0] = h_out[1] = 0;
    return TN_OK;
  }
  return zdotc_batched(ctx, n, (const cxd*)x, 0, (const cxd*)y, 0, 1, h_out);
}

// y += a x for ComplexF64 vectors, a = (ar, ai)
tn_status_t tn_axpy(tn_ctx* ctx, int64_t n, double ar, double ai, const void* x, void* y) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, n >= 0 && (n == 0 || (x && y)), "tn_axpy: bad arguments");
  if (n == 0) return TN_OK;
  k_axpy_cx<<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(n, ar, ai, (const double2*)x, (double2*)y);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

}  // extern "C"
