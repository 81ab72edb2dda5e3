// K3 — batched blocked Householder QR (thin), complex FP64 / FP32.
//
// Replaces LAPACK geqrf + ungqr behind Muscle.tensor_qr_thin, which Tenet calls once per
// gauge move (src/Operations/canonize.jl:58): A (m×n) = Q (m×k) · R (k×n), k = min(m,n).
//
// Algorithm: right-looking blocked Householder with the compact-WY form
//   H_1 … H_jb = I − V T Vᴴ  (Schreiber & Van Loan 1989),
// LAPACK's reflector convention (H = I − τ v vᴴ, v_1 = 1, R_ii real).
//  * panel kernel (one CTA per matrix): the m×jb panel lives in shared memory; warp 0
//    forms each reflector (norm by warp-shuffle reduction), all warps apply it to the
//    remaining panel columns (one warp per column, shuffle-reduced dot products), then
//    the jb×jb T factor is built from the panel's Gram matrix.
//  * block-reflector kernel (a grid of column slabs × matrices): W = Vᴴ A_slab,
//    Y = Tᴴ W (or T W when forming Q), A_slab −= V Y.  Every SM works on the trailing
//    update, which holds O(m n²) of the O(m n²) flops.
//  * Q is formed by applying the panels in reverse to [I_k; 0] (LAPACK ungqr order).
#include "tn_internal.cuh"

namespace {

constexpr int kPanelThreads = 256;
constexpr int kSlabCols = 4;
constexpr size_t kPanelSmemMax = 180 * 1024;  // + 34 KB static (Gram, T) <= 227 KB

template <typename T>
int panel_width(int64_t m) {
  int64_t cap = (int64_t)(kPanelSmemMax / (sizeof(cx<T>) * (size_t)(m > 0 ? m : 1)));
  int nb = 32;
  while (nb > 1 && nb > cap) nb >>= 1;
  return nb;
}

// V[r, a] of the panel stored in W (rows j0.., columns j0+a) with unit diagonal
template <typename T>
__device__ __forceinline__ cx<T> vget(const cx<T>* P, int64_t ld, int64_t r, int a) {
  if (r < a) return mkcx<T>(0, 0);
  if (r == a) return mkcx<T>(1, 0);
  return P[r + (int64_t)a * ld];
}

// Factor the panel W[j0:m, j0:j0+jb] of each matrix; write tau and T (ldT = nb).
template <typename T>
__global__ void __launch_bounds__(kPanelThreads)
    k_qr_panel(int64_t m, int64_t j0, int jb, int nb, cx<T>* W, int64_t ldw, int64_t sW, cx<T>* tau,
               int64_t sTau, cx<T>* Tm, int64_t sT) {
  extern __shared__ unsigned char smem_raw[];
  cx<T>* P = reinterpret_cast<cx<T>*>(smem_raw);
  __shared__ cx<T> s_tau[32];
  __shared__ cx<T> s_G[32][33];
  const int64_t mr = m - j0;
  const int64_t b = blockIdx.x;
  cx<T>* Wb = W + b * sW + j0 + j0 * ldw;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  // load panel (column-major, ld = mr)
  for (int64_t t = tid; t < mr * jb; t += blockDim.x) {
    int64_t r = t % mr, c = t / mr;
    P[t] = Wb[r + c * ldw];
  }
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    cx<T>* col = P + (int64_t)c * mr;
    if (warp == 0) {
      T s2 = 0;
      for (int64_t r = c + 1 + lane; r < mr; r += 32) s2 += abs2(col[r]);
      s2 = warp_sum(s2);
      cx<T> alpha = col[c];
      cx<T> tc;
      cx<T> scale;
      T beta;
      if (s2 == T(0) && alpha.y == T(0)) {
        tc = mkcx<T>(0, 0);
        scale = mkcx<T>(0, 0);
        beta = alpha.x;
      } else {
        T nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + s2);
        beta = alpha.x >= T(0) ? -nrm : nrm;
        tc = mkcx<T>((beta - alpha.x) / beta, -alpha.y / beta);
        // scale = 1 / (alpha - beta)
        cx<T> d = mkcx<T>(alpha.x - beta, alpha.y);
        T dd = abs2(d);
        scale = mkcx<T>(d.x / dd, -d.y / dd);
      }
      for (int64_t r = c + 1 + lane; r < mr; r += 32) col[r] = col[r] * scale;
      __syncwarp();
      if (lane == 0) {
        col[c] = mkcx<T>(beta, 0);
        s_tau[c] = tc;
      }
    }
    __syncthreads();
    // apply Hᴴ = I − conj(τ) v vᴴ to the remaining panel columns
    const cx<T> ctau = conjg(s_tau[c]);
    for (int j = c + 1 + warp; j < jb; j += nwarps) {
      cx<T>* cj = P + (int64_t)j * mr;
      cx<T> w = mkcx<T>(0, 0);
      for (int64_t r = c + lane; r < mr; r += 32) {
        cx<T> v = r == c ? mkcx<T>(1, 0) : col[r];
        cfma_cj(w, v, cj[r]);
      }
      w.x = warp_sum(w.x);
      w.y = warp_sum(w.y);
      cx<T> f = ctau * w;
      for (int64_t r = c + lane; r < mr; r += 32) {
        cx<T> v = r == c ? mkcx<T>(1, 0) : col[r];
        cj[r] = cj[r] - v * f;
      }
    }
    __syncthreads();
  }
  // Gram of V: G[a][i] = V(:,a)ᴴ V(:,i) for a < i
  for (int pair = warp; pair < jb * jb; pair += nwarps) {
    int a = pair % jb, i = pair / jb;
    if (a >= i) continue;
    cx<T> g = mkcx<T>(0, 0);
    for (int64_t r = i + lane; r < mr; r += 32) {
      cx<T> vi = r == i ? mkcx<T>(1, 0) : P[r + (int64_t)i * mr];
      cfma_cj(g, P[r + (int64_t)a * mr], vi);  // r >= i > a: V(r,a) stored
    }
    g.x = warp_sum(g.x);
    g.y = warp_sum(g.y);
    if (lane == 0) s_G[a][i] = g;
  }
  __syncthreads();
  // T(i,i) = τ_i; T(0:i, i) = −τ_i T(0:i,0:i) G(0:i, i): column by column, rows of a
  // column in parallel (warp 0), T kept in shared memory (reuses s_G's lower part is
  // not possible: G is read for all a < i), written out at the end
  __shared__ cx<T> s_T[32][33];
  if (warp == 0) {
    for (int i = 0; i < jb; ++i) {
      cx<T> s = mkcx<T>(0, 0);
      const int a = lane;
      if (a < i)
        for (int q = a; q < i; ++q) cfma(s, s_T[a][q], s_G[q][i]);
      __syncwarp();
      if (a < i) s_T[a][i] = mkcx<T>(0, 0) - s_tau[i] * s;
      if (a == i) s_T[i][i] = s_tau[i];
      if (a > i && a < jb) s_T[a][i] = mkcx<T>(0, 0);
      __syncwarp();
    }
  }
  __syncthreads();
  cx<T>* Tb = Tm + b * sT;
  for (int t = tid; t < jb * jb; t += blockDim.x) {
    int a = t % jb, i = t / jb;
    Tb[a + i * nb] = s_T[a][i];
  }
  if (tid < jb) tau[b * sTau + j0 + tid] = s_tau[tid];
  // store panel back
  for (int64_t t = tid; t < mr * jb; t += blockDim.x) {
    int64_t r = t % mr, c = t / mr;
    Wb[r + c * ldw] = P[t];
  }
}

// X[j0:m, c0:c1] ← (I − V T Vᴴ)^{op} X  where op = ᴴ (conjT = true, trailing update of
// the factorisation) or identity (conjT = false, forming Q).  V is the panel stored in
// W[j0:m, j0:j0+jb].
template <typename T>
__global__ void __launch_bounds__(256)
    k_apply_block_reflector(int64_t m, int64_t j0, int jb, int nb, const cx<T>* W, int64_t ldw, int64_t sW,
                            const cx<T>* Tm, int64_t sT, cx<T>* X, int64_t ldx, int64_t sX, int64_t c0,
                            int64_t c1, bool conjT) {
  __shared__ cx<T> sW_[32][kSlabCols];
  __shared__ cx<T> sY[32][kSlabCols];
  const int64_t b = blockIdx.y;
  const int64_t mr = m - j0;
  const cx<T>* V = W + b * sW + j0 + j0 * ldw;
  const cx<T>* Tb = Tm + b * sT;
  const int64_t cs = c0 + (int64_t)blockIdx.x * kSlabCols;
  const int ncol = (int)(c1 - cs < kSlabCols ? c1 - cs : kSlabCols);
  cx<T>* Xb = X + b * sX + j0 + cs * ldx;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  // W = Vᴴ X_slab  (jb × ncol)
  for (int pair = warp; pair < jb * ncol; pair += nwarps) {
    int a = pair % jb, c = pair / jb;
    cx<T> w = mkcx<T>(0, 0);
    const cx<T>* xc = Xb + (int64_t)c * ldx;
    for (int64_t r = a + lane; r < mr; r += 32) cfma_cj(w, vget(V, ldw, r, a), xc[r]);
    w.x = warp_sum(w.x);
    w.y = warp_sum(w.y);
    if (lane == 0) sW_[a][c] = w;
  }
  __syncthreads();
  // Y = op(T) W
  if (tid < jb * ncol) {
    int a = tid % jb, c = tid / jb;
    cx<T> y = mkcx<T>(0, 0);
    if (conjT) {  // (Tᴴ)[a][q] = conj(T[q][a]), T upper: q <= a
      for (int q = 0; q <= a; ++q) cfma_cj(y, Tb[q + a * nb], sW_[q][c]);
    } else {  // T[a][q], q >= a
      for (int q = a; q < jb; ++q) cfma(y, Tb[a + q * nb], sW_[q][c]);
    }
    sY[a][c] = y;
  }
  __syncthreads();
  // X_slab −= V Y
  for (int64_t t = tid; t < mr * ncol; t += blockDim.x) {
    int64_t r = t % mr;
    int c = (int)(t / mr);
    cx<T> acc = mkcx<T>(0, 0);
    int amax = (int)(r < jb - 1 ? r : jb - 1);
    for (int a = 0; a <= amax; ++a) cfma(acc, vget(V, ldw, r, a), sY[a][c]);
    Xb[r + (int64_t)c * ldx] = Xb[r + (int64_t)c * ldx] - acc;
  }
}

template <typename T>
__global__ void k_copy_in(int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* W,
                          int64_t sW, int64_t batch) {
  int64_t total = m * n;
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % m, c = t / m;
      W[b * sW + t] = A[b * sA + r + c * lda];
    }
}

// R (k×n) = upper triangle of W's first k rows; Q = [I_k; 0]
template <typename T>
__global__ void k_extract_r_init_q(int64_t m, int64_t n, int64_t k, const cx<T>* W, int64_t sW, cx<T>* R,
                                   int64_t sR, cx<T>* Q, int64_t sQ, int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < k * n; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % k, c = t / k;
      R[b * sR + t] = r <= c ? W[b * sW + r + c * m] : mkcx<T>(0, 0);
    }
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * k; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % m, c = t / m;
      Q[b * sQ + t] = mkcx<T>(r == c ? T(1) : T(0), 0);
    }
  }
}

}  // namespace

template <typename T>
size_t qr_workspace(int64_t m, int64_t n, int64_t batch) {
  int64_t k = m < n ? m : n;
  int nb = panel_width<T>(m);
  int64_t npan = (k + nb - 1) / nb;
  size_t w = ws_round(sizeof(cx<T>) * (size_t)(m * n * batch));
  size_t tau = ws_round(sizeof(cx<T>) * (size_t)(k * batch + 1));
  size_t tm = ws_round(sizeof(cx<T>) * (size_t)(npan * nb * nb * batch + 1));
  return w + tau + tm;
}
template size_t qr_workspace<double>(int64_t, int64_t, int64_t);
template size_t qr_workspace<float>(int64_t, int64_t, int64_t);

template <typename T>
tn_status_t qr_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* Q,
                  int64_t sQ, cx<T>* R, int64_t sR, int64_t batch) {
  // workspace must have been reserved by the caller (qr_workspace) and is taken here
  const int64_t k = m < n ? m : n;
  if (m == 0 || n == 0 || batch == 0) return TN_OK;
  const int nb = panel_width<T>(m);
  const int64_t npan = (k + nb - 1) / nb;
  cx<T>* W = ws_take<cx<T>>(ctx, (size_t)(m * n * batch));
  cx<T>* tau = ws_take<cx<T>>(ctx, (size_t)(k * batch + 1));
  cx<T>* Tm = ws_take<cx<T>>(ctx, (size_t)(npan * nb * nb * batch + 1));
  const int64_t sW = m * n, sTau = k, sT = npan * nb * nb;
  const unsigned gy = (unsigned)(batch < 65535 ? batch : 65535);
  {
    int64_t blocks = ((m * n) + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_copy_in<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(m, n, A, lda, sA, W, sW, batch);
    TN_LAUNCHED(ctx);
  }
  const size_t smem = sizeof(cx<T>) * (size_t)m * nb;
  if (smem > kPanelSmemMax) return tn_set_error(ctx, TN_EUNSUPPORTED, "qr: m=%lld too large for the panel kernel", (long long)m);
  TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_qr_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemMax));
  if (batch > 2147483647) return tn_set_error(ctx, TN_EINVAL, "qr: batch too large");
  for (int64_t p = 0; p < npan; ++p) {
    const int64_t j0 = p * nb;
    const int jb = (int)(k - j0 < nb ? k - j0 : nb);
    k_qr_panel<T><<<(unsigned)batch, kPanelThreads, sizeof(cx<T>) * (size_t)(m - j0) * jb, ctx->stream>>>(
        m, j0, jb, nb, W, m, sW, tau, sTau, Tm + p * nb * nb, sT);
    TN_LAUNCHED(ctx);
    const int64_t c0 = j0 + jb;
    if (c0 < n) {
      dim3 grid(cdiv(n - c0, kSlabCols), gy);
      k_apply_block_reflector<T><<<grid, 256, 0, ctx->stream>>>(m, j0, jb, nb, W, m, sW, Tm + p * nb * nb, sT, W,
                                                                 m, sW, c0, n, true);
      TN_LAUNCHED(ctx);
    }
  }
  {
    int64_t blocks = ((m * k) + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_extract_r_init_q<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(m, n, k, W, sW, R, sR, Q, sQ,
                                                                                batch);
    TN_LAUNCHED(ctx);
  }
  for (int64_t p = npan - 1; p >= 0; --p) {
    const int64_t j0 = p * nb;
    const int jb = (int)(k - j0 < nb ? k - j0 : nb);
    dim3 grid(cdiv(k - j0, kSlabCols), gy);
    k_apply_block_reflector<T><<<grid, 256, 0, ctx->stream>>>(m, j0, jb, nb, W, m, sW, Tm + p * nb * nb, sT, Q, m,
                                                               sQ, j0, k, false);
    TN_LAUNCHED(ctx);
  }
  return TN_OK;
}
template tn_status_t qr_cx<double>(tn_ctx*, int64_t, int64_t, const cxd*, int64_t, int64_t, cxd*, int64_t,
                                   cxd*, int64_t, int64_t);
template tn_status_t qr_cx<float>(tn_ctx*, int64_t, int64_t, const cxf*, int64_t, int64_t, cxf*, int64_t,
                                  cxf*, int64_t, int64_t);

extern "C" tn_status_t tn_qr_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, int64_t m, int64_t n,
                                  const void* A, int64_t lda, int64_t strideA, void* Q, int64_t strideQ,
                                  void* R, int64_t strideR, int64_t batch) {
  (void)prec;
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, m >= 0 && n >= 0 && batch >= 0, "tn_qr_thin: negative size");
  TN_ARG(ctx, lda >= (m > 1 ? m : 1), "tn_qr_thin: lda < m");
  TN_ARG(ctx, (m == 0 || n == 0 || batch == 0) || (A && Q && R), "tn_qr_thin: null pointer");
  if (dtype == TN_C64) {
    TN_RETURN_IF(ws_reserve(ctx, qr_workspace<double>(m, n, batch)));
    return qr_cx<double>(ctx, m, n, (const cxd*)A, lda, strideA, (cxd*)Q, strideQ, (cxd*)R, strideR, batch);
  }
  if (dtype == TN_C32) {
    TN_RETURN_IF(ws_reserve(ctx, qr_workspace<float>(m, n, batch)));
    return qr_cx<float>(ctx, m, n, (const cxf*)A, lda, strideA, (cxf*)Q, strideQ, (cxf*)R, strideR, batch);
  }
  return tn_set_error(ctx, TN_EUNSUPPORTED, "tn_qr_thin: only C64 and C32 are implemented");
}
