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
#include <algorithm>

#include "tn_internal.cuh"

namespace {

constexpr int kPanelThreads = 256;
constexpr int kMaxPanel = 32;
constexpr size_t kPanelSmemMax = 180 * 1024;  // + 34 KB static (Gram, T) <= 227 KB

// widest panel whose m×nb block fits the panel kernel's shared memory
template <typename T>
int panel_width_max(int64_t m) {
  int64_t cap = (int64_t)(kPanelSmemMax / (sizeof(cx<T>) * (size_t)(m > 0 ? m : 1)));
  int nb = kMaxPanel;
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
template <typename T, int kSlabCols>
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
  const int64_t k = m < n ? m : n;
  const int nb = panel_width_max<T>(m);
  const int64_t npan = (k + nb - 1) / nb;
  size_t w = ws_round(sizeof(cx<T>) * (size_t)(m * n * batch));
  size_t tau = ws_round(sizeof(cx<T>) * (size_t)(k * batch + 1));
  // T factors: npan·nb² per matrix at the widest panel bounds every narrower choice
  size_t tm = ws_round(sizeof(cx<T>) * (size_t)((npan + 1) * nb * nb * batch + 1));
  // the autotuner's private copy of A (Q may alias A)
  size_t a0 = ws_round(sizeof(cx<T>) * (size_t)(m * n * batch));
  return w + tau + tm + a0;
}
template size_t qr_workspace<double>(int64_t, int64_t, int64_t);
template size_t qr_workspace<float>(int64_t, int64_t, int64_t);

namespace {

template <typename T>
tn_status_t launch_reflector(tn_ctx* ctx, int slab, dim3 grid, int64_t m, int64_t j0, int jb, int nb, const cx<T>* W,
                             int64_t sW, const cx<T>* Tm, int64_t sT, cx<T>* X, int64_t sX, int64_t c0, int64_t c1,
                             bool conjT) {
  switch (slab) {
    case 1:
      k_apply_block_reflector<T, 1><<<grid, 256, 0, ctx->stream>>>(m, j0, jb, nb, W, m, sW, Tm, sT, X, m, sX, c0, c1, conjT);
      break;
    case 2:
      k_apply_block_reflector<T, 2><<<grid, 256, 0, ctx->stream>>>(m, j0, jb, nb, W, m, sW, Tm, sT, X, m, sX, c0, c1, conjT);
      break;
    default:
      k_apply_block_reflector<T, 4><<<grid, 256, 0, ctx->stream>>>(m, j0, jb, nb, W, m, sW, Tm, sT, X, m, sX, c0, c1, conjT);
      break;
  }
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// one factorisation with panel width nb and block-reflector slab width `slab`
template <typename T>
tn_status_t qr_run(tn_ctx* ctx, int nb, int slab, int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA,
                   cx<T>* Q, int64_t sQ, cx<T>* R, int64_t sR, int64_t batch, cx<T>* W, cx<T>* tau, cx<T>* Tm) {
  const int64_t k = m < n ? m : n;
  const int64_t npan = (k + nb - 1) / nb;
  const int64_t sW = m * n, sTau = k, sT = npan * nb * nb;
  const unsigned gy = (unsigned)(batch < 65535 ? batch : 65535);
  {
    int64_t blocks = ((m * n) + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_copy_in<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(m, n, A, lda, sA, W, sW, batch);
    TN_LAUNCHED(ctx);
  }
  for (int64_t p = 0; p < npan; ++p) {
    const int64_t j0 = p * nb;
    const int jb = (int)(k - j0 < nb ? k - j0 : nb);
    k_qr_panel<T><<<(unsigned)batch, kPanelThreads, sizeof(cx<T>) * (size_t)(m - j0) * jb, ctx->stream>>>(
        m, j0, jb, nb, W, m, sW, tau, sTau, Tm + p * nb * nb, sT);
    TN_LAUNCHED(ctx);
    const int64_t c0 = j0 + jb;
    if (c0 < n)
      TN_RETURN_IF(launch_reflector<T>(ctx, slab, dim3(cdiv(n - c0, slab), gy), m, j0, jb, nb, W, sW, Tm + p * nb * nb,
                                       sT, W, sW, c0, n, true));
  }
  {
    int64_t blocks = ((m * k) + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_extract_r_init_q<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(m, n, k, W, sW, R, sR, Q, sQ, batch);
    TN_LAUNCHED(ctx);
  }
  for (int64_t p = npan - 1; p >= 0; --p) {
    const int64_t j0 = p * nb;
    const int jb = (int)(k - j0 < nb ? k - j0 : nb);
    TN_RETURN_IF(launch_reflector<T>(ctx, slab, dim3(cdiv(k - j0, slab), gy), m, j0, jb, nb, W, sW, Tm + p * nb * nb,
                                     sT, Q, sQ, j0, k, false));
  }
  return TN_OK;
}

}  // namespace

// Panel width and slab width come from the context's tuning table, keyed by the shape
// (m, n and a batch bucket).  With autotuning on, the first call of an unseen shape
// times every candidate (panel 4/8/16/32 that fits shared memory × slab 1/2/4) with
// CUDA events and records the fastest; otherwise the default is panel 8, slab 2.
template <typename T>
tn_status_t qr_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* Q, int64_t sQ,
                  cx<T>* R, int64_t sR, int64_t batch) {
  const int64_t k = m < n ? m : n;
  if (m == 0 || n == 0 || batch == 0) return TN_OK;
  if (batch > 2147483647) return tn_set_error(ctx, TN_EINVAL, "qr: batch too large");
  const int nb_max = panel_width_max<T>(m);
  if (sizeof(cx<T>) * (size_t)m * 1 > kPanelSmemMax)
    return tn_set_error(ctx, TN_EUNSUPPORTED, "qr: m=%lld too large for the panel kernel", (long long)m);
  const int64_t npan_max = (k + nb_max - 1) / nb_max;
  cx<T>* W = ws_take<cx<T>>(ctx, (size_t)(m * n * batch));
  cx<T>* tau = ws_take<cx<T>>(ctx, (size_t)(k * batch + 1));
  cx<T>* Tm = ws_take<cx<T>>(ctx, (size_t)((npan_max + 1) * nb_max * nb_max * batch + 1));
  TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_qr_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemMax));
  const int bb = batch <= 1 ? 1 : batch <= 4 ? 4 : batch <= 16 ? 16 : 64;
  char key[96];
  snprintf(key, sizeof(key), "qr%zu:%lld:%lld:%d", sizeof(T), (long long)m, (long long)n, bb);
  auto it = ctx->tuning.find(key);
  int nb = std::min(8, nb_max), slab = 2;
  if (it != ctx->tuning.end()) {
    nb = std::min(it->second.first, nb_max);
    slab = it->second.second;
  } else if (ctx->autotune) {
    // Every candidate factorises the same input, and Q may alias A (the in-place gauge
    // move): the candidates and the final run read a private copy of A.
    cx<T>* A0 = ws_take<cx<T>>(ctx, (size_t)(m * n * batch));
    {
      int64_t blocks = ((m * n) + 255) / 256;
      if (blocks > 4096) blocks = 4096;
      k_copy_in<T><<<dim3((unsigned)blocks, (unsigned)(batch < 65535 ? batch : 65535)), 256, 0, ctx->stream>>>(
          m, n, A, lda, sA, A0, m * n, batch);
      TN_LAUNCHED(ctx);
    }
    A = A0;
    lda = m;
    sA = m * n;
    float best = 1e30f;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto sweep = [&]() -> tn_status_t {
      TN_CHECK_CUDA(ctx, cudaEventCreate(&e0));
      TN_CHECK_CUDA(ctx, cudaEventCreate(&e1));
      for (int cand_nb = 4; cand_nb <= nb_max; cand_nb *= 2)
        for (int cand_slab = 1; cand_slab <= 4; cand_slab *= 2) {
          TN_CHECK_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
          TN_RETURN_IF(qr_run<T>(ctx, cand_nb, cand_slab, m, n, A, lda, sA, Q, sQ, R, sR, batch, W, tau, Tm));
          TN_CHECK_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
          TN_CHECK_CUDA(ctx, cudaEventSynchronize(e1));
          float ms = 0;
          TN_CHECK_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
          if (ms < best) {
            best = ms;
            nb = cand_nb;
            slab = cand_slab;
          }
        }
      return TN_OK;
    };
    const tn_status_t st = sweep();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    TN_RETURN_IF(st);
    ctx->tuning[key] = {nb, slab};
  }
  const int slot = prof_begin(ctx);
  const int64_t l0 = ctx->launches;
  TN_RETURN_IF(qr_run<T>(ctx, nb, slab, m, n, A, lda, sA, Q, sQ, R, sR, batch, W, tau, Tm));
  if (slot >= 0) {
    // geqrf + forming Q: 2 × 4·(2mk² − ⅔k³)·… (LAWN 41, ×4 complex); A read, Q and R written
    const double kk = (double)k, f = 4.0 * (2.0 * m * kk * kk - 2.0 / 3.0 * kk * kk * kk);
    prof_end(ctx, slot, TN_PROF_QR, ctx->launches - l0, 2.0 * f * batch,
             sizeof(cx<T>) * ((double)m * n + (double)m * k + (double)k * n) * batch);
  }
  return TN_OK;
}
template tn_status_t qr_cx<double>(tn_ctx*, int64_t, int64_t, const cxd*, int64_t, int64_t, cxd*, int64_t, cxd*,
                                   int64_t, int64_t);
template tn_status_t qr_cx<float>(tn_ctx*, int64_t, int64_t, const cxf*, int64_t, int64_t, cxf*, int64_t, cxf*,
                                  int64_t, int64_t);

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
