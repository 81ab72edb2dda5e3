// DMRG ground-state search on a device MPS (Tenet.jl v0.10.3 src/Algorithms/DMRG.jl):
// Dmrg1 (DMRG.jl:45-210) and Dmrg2 (DMRG.jl:212-459) with KrylovKit's restarted Lanczos
// (eigsolve(x0, 1, :LM; ishermitian = true, krylovdim, maxiter), KrylovKit 0.9.5–0.10,
// src/eigsolve/lanczos.jl) as the local eigensolver.  All B instances of the MPS advance in
// lockstep (their bond dimensions never differ: Dmrg2 keeps min(maxdim, k) values without
// a threshold), each with its own Hamiltonian if B MPOs are given.
//
// Layouts (column-major, per instance):
//   left environment  Lc_k [a, a', w]   (ket, bra, MPO bond) stored CONJUGATED
//   right environment R_k  [w, b, b']   (MPO bond, ket, bra)
//   MPO site          Wp_i [w_l, s, o, w_r]  (s = input, o = output index)
//                     Ws_i [s, w_l, o, w_r]  (for the right environment update)
// With these, every contraction of the effective Hamiltonian is a GEMM or a "fiber"
// product (a small MPO matrix applied along strided fibres of a tensor) without any
// permutation:
//   1-site  y = Heff x:  T1 = Lcᴴ x  →  T2 = fiber(T1, Wp_i)  →  y = T2 · R_i
//   2-site  y = Heff θ:  T1 = Lcᴴ θ  →  fiber(Wp_j)  →  fiber(Wp_{j+1})  →  y = T3 · R_{j+1}
//
// The Lanczos scalars stay on the device: one block per instance orthogonalises the new
// vector (two Gram–Schmidt passes against the basis), one thread per instance
// diagonalises the tridiagonal matrix (cyclic Jacobi) and decides convergence / restart,
// and an element-wise kernel forms the Ritz vector.  An eigensolve is therefore a fixed
// sequence of launches with no host round trip.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tn_mps_internal.cuh"

namespace {

constexpr int kLzMax = 16;   // Krylov basis + residual slot
constexpr int kFiberP = 16;  // fiber kernel: inputs per output kept in registers
const cxd kOne = {1.0, 0.0};
const cxd kZero = {0.0, 0.0};

struct LzState {
  double alpha[kLzMax];
  double beta[kLzMax];
  double coef[kLzMax];
  double theta;  // leading Ritz value
  double f;      // its residual norm estimate β_K·u_K
  double rsign;  // sign that makes the restart residual coefficient positive
  int K;         // basis vectors with a known α
  int ncoef;     // Ritz coefficients held in coef (the basis size when they were formed)
  int frozen;    // invariant subspace reached (β ≤ tol)
  int done;      // converged or out of iterations
  int action;    // 0 none, 1 finish (Ritz vector → slot 0), 2 restart
  int it;        // Lanczos iteration (1-based)
};

template <int NT>
__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < NT / 32 ? red[threadIdx.x] : 0.0;
    r = warp_sum(r);
    if (threadIdx.x == 0) red[0] = r;
  }
  __syncthreads();
  r = red[0];
  return r;
}

constexpr int kLzThreads = 1024;

// v0 = x0 / ‖x0‖; state reset
__global__ void __launch_bounds__(kLzThreads) k_lz_start(int64_t N, const double2* __restrict__ x0, int64_t sx0,
                                                          double2* __restrict__ V, int64_t sV, LzState* st) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  const double2* x = x0 + b * sx0;
  double2* v = V + b * sV;
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < N; t += kLzThreads) s += x[t].x * x[t].x + x[t].y * x[t].y;
  s = block_sum<kLzThreads>(s, red);
  const double nrm = sqrt(s);
  const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
  for (int64_t t = threadIdx.x; t < N; t += kLzThreads) v[t] = make_double2(x[t].x * inv, x[t].y * inv);
  if (threadIdx.x == 0) {
    LzState& S = st[b];
    for (int j = 0; j < kLzMax; ++j) S.alpha[j] = S.beta[j] = S.coef[j] = 0.0;
    S.theta = S.f = 0.0;
    S.rsign = 1.0;
    S.K = 0;
    S.ncoef = 0;
    S.frozen = 0;
    S.done = nrm > 0.0 ? 0 : 1;  // a zero start vector has no Krylov space
    S.action = 0;
    S.it = 1;
  }
}

// Lanczos step k: w = H v_k has been formed in W.  α_k, β_k, v_{k+1} = r / β_k with r = w
// orthogonalised against v_0..v_k (two classical Gram–Schmidt passes).
// KM ≥ k+1 dot products are accumulated in registers; NT threads per block
template <int KM, int NT>
__global__ void __launch_bounds__(NT) k_lz_orth(int64_t N, int k, double2* __restrict__ V, int64_t sV, int64_t slot,
                                                double2* __restrict__ W, int64_t sW, LzState* st, double tol) {
  __shared__ double red[32];
  __shared__ double cs[2 * KM];
  const int b = blockIdx.x;
  if (st[b].done || st[b].frozen || st[b].K != k) return;
  double2* v = V + b * sV;
  double2* w = W + b * sW;
  double alpha = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    double cr[KM], ci[KM];
#pragma unroll
    for (int j = 0; j < KM; ++j) cr[j] = ci[j] = 0.0;
    for (int64_t t = threadIdx.x; t < N; t += NT) {
      const double2 y = w[t];
#pragma unroll
      for (int j = 0; j < KM; ++j)
        if (j <= k) {
          const double2 q = v[j * slot + t];
          cr[j] = fma(q.x, y.x, fma(q.y, y.y, cr[j]));
          ci[j] = fma(q.x, y.y, fma(-q.y, y.x, ci[j]));
        }
    }
#pragma unroll
    for (int j = 0; j < KM; ++j)
      if (j <= k) {
        const double r = block_sum<NT>(cr[j], red);
        const double i = block_sum<NT>(ci[j], red);
        if (threadIdx.x == 0) {
          cs[2 * j] = r;
          cs[2 * j + 1] = i;
        }
      }
    __syncthreads();
    alpha += cs[2 * k];
    for (int64_t t = threadIdx.x; t < N; t += NT) {
      double2 y = w[t];
      for (int j = 0; j <= k; ++j) {
        const double2 q = v[j * slot + t];
        const double a = cs[2 * j], c = cs[2 * j + 1];
        y.x -= a * q.x - c * q.y;
        y.y -= a * q.y + c * q.x;
      }
      w[t] = y;
    }
    __syncthreads();
  }
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < N; t += NT) s += w[t].x * w[t].x + w[t].y * w[t].y;
  s = block_sum<NT>(s, red);
  const double beta = sqrt(s);
  if (beta > tol) {
    const double inv = 1.0 / beta;
    for (int64_t t = threadIdx.x; t < N; t += NT)
      v[(k + 1) * slot + t] = make_double2(w[t].x * inv, w[t].y * inv);
  }
  if (threadIdx.x == 0) {
    LzState& S = st[b];
    S.alpha[k] = alpha;
    S.beta[k] = beta;
    S.K = k + 1;
    if (!(beta > tol)) S.frozen = 1;
  }
}

// eigen-decomposition of a small real symmetric matrix (cyclic Jacobi), A overwritten by
// its eigenvalues on the diagonal, Z by the eigenvectors (columns)
__device__ void sym_eig(int n, double (*A)[kLzMax], double (*Z)[kLzMax]) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Z[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i) {
      diag += A[i][i] * A[i][i];
      for (int j = i + 1; j < n; ++j) off += A[i][j] * A[i][j];
    }
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p][q];
        if (apq == 0.0) continue;
        const double tau = (A[q][q] - A[p][p]) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double zkp = Z[k][p], zkq = Z[k][q];
          Z[k][p] = c * zkp - s * zkq;
          Z[k][q] = s * zkp + c * zkq;
        }
      }
  }
}

// Rayleigh–Ritz on the tridiagonal matrix, KrylovKit's convergence test and restart rule
// (keep = ⌊(3·krylovdim + 2·converged)/5⌋ = 1 Ritz vector while nothing converged)
__global__ void k_lz_ritz(int B, int kdim, int maxiter, double tol, LzState* st) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  LzState& S = st[b];
  S.action = 0;
  if (S.done) return;
  const int K = S.K;
  if (K < 1) {
    S.done = 1;
    return;
  }
  double A[kLzMax][kLzMax], Z[kLzMax][kLzMax];
  for (int i = 0; i < K; ++i)
    for (int j = 0; j < K; ++j) A[i][j] = 0.0;
  for (int i = 0; i < K; ++i) A[i][i] = S.alpha[i];
  for (int i = 0; i + 1 < K; ++i) A[i][i + 1] = A[i + 1][i] = S.beta[i];
  sym_eig(K, A, Z);
  // ascending order, then a stable sort by descending |θ| (which = :LM)
  int idx[kLzMax];
  for (int i = 0; i < K; ++i) idx[i] = i;
  for (int i = 1; i < K; ++i)
    for (int j = i; j > 0 && A[idx[j]][idx[j]] < A[idx[j - 1]][idx[j - 1]]; --j) {
      const int t = idx[j];
      idx[j] = idx[j - 1];
      idx[j - 1] = t;
    }
  int best = idx[0];
  for (int i = 1; i < K; ++i)
    if (fabs(A[idx[i]][idx[i]]) > fabs(A[best][best])) best = idx[i];
  const double theta = A[best][best];
  const double f = S.beta[K - 1] * Z[K - 1][best];
  for (int i = 0; i < K; ++i) S.coef[i] = Z[i][best];
  S.ncoef = K;
  S.theta = theta;
  S.f = f;
  const bool converged = fabs(f) <= tol || S.frozen;
  if (converged || K < kdim || S.it >= maxiter) {
    S.done = 1;
    S.action = 1;
    return;
  }
  S.action = 2;
  S.rsign = f >= 0.0 ? 1.0 : -1.0;
  for (int j = 0; j < kLzMax; ++j) S.alpha[j] = S.beta[j] = 0.0;
  S.alpha[0] = theta;
  S.beta[0] = fabs(f);
  S.K = 1;
  S.it += 1;
}

// Ritz vector u = Σ_j coef_j v_j into slot 0; on a restart also slot 1 = ±(residual slot)
__global__ void k_lz_combine(int64_t N, double2* __restrict__ V, int64_t sV, int64_t slot, const LzState* st) {
  const int b = blockIdx.y;
  const LzState& S = st[b];
  const int act = S.action;
  if (act == 0) return;
  const int K = S.ncoef;
  double2* v = V + b * sV;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N; t += (int64_t)gridDim.x * blockDim.x) {
    double ux = 0.0, uy = 0.0;
    for (int j = 0; j < K; ++j) {
      const double2 q = v[j * slot + t];
      ux = fma(S.coef[j], q.x, ux);
      uy = fma(S.coef[j], q.y, uy);
    }
    double2 r = make_double2(0.0, 0.0);
    if (act == 2) r = v[K * slot + t];
    v[t] = make_double2(ux, uy);
    if (act == 2) v[slot + t] = make_double2(S.rsign * r.x, S.rsign * r.y);
  }
}

// out[b][x + X(q + Q j)] = Σ_p in[b][x + X(p + P j)] · M[b][p + P q]
__global__ void k_fiber(int64_t X, int P, int Q, int64_t J, const cxd* __restrict__ in, int64_t sIn,
                        const cxd* __restrict__ M, int64_t sM, cxd* __restrict__ out, int64_t sOut) {
  extern __shared__ cxd Ms[];
  const int b = blockIdx.y;
  for (int t = threadIdx.x; t < P * Q; t += blockDim.x) Ms[t] = M[b * sM + t];
  __syncthreads();
  const cxd* ib = in + b * sIn;
  cxd* ob = out + b * sOut;
  const int64_t total = X * J;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = t % X, j = t / X;
    cxd v[kFiberP];
#pragma unroll
    for (int p = 0; p < kFiberP; ++p)
      if (p < P) v[p] = ib[x + X * (p + (int64_t)P * j)];
    for (int q = 0; q < Q; ++q) {
      cxd acc = mkcx(0.0, 0.0);
#pragma unroll
      for (int p = 0; p < kFiberP; ++p)
        if (p < P) cfma(acc, v[p], Ms[p + P * q]);
      ob[x + X * (q + (int64_t)Q * j)] = acc;
    }
  }
}

// out[b][y + Y(x + X z)] = in[b][x + X(y + Y z)]
__global__ void k_swap01(int64_t X, int64_t Y, int64_t Z, const cxd* __restrict__ in, int64_t sIn,
                         cxd* __restrict__ out, int64_t sOut) {
  const int b = blockIdx.y;
  const int64_t total = X * Y * Z;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = t % X, y = (t / X) % Y, z = t / (X * Y);
    out[b * sOut + y + Y * (x + X * z)] = in[b * sIn + t];
  }
}

// 1 / ‖S_b[0:keep]‖ per instance
__global__ void k_inv_norm(int keep, const double* __restrict__ S, int64_t sS, double* __restrict__ out) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  double s = 0.0;
  for (int t = threadIdx.x; t < keep; t += 256) s += S[b * sS + t] * S[b * sS + t];
  s = block_sum<256>(s, red);
  if (threadIdx.x == 0) out[b] = s > 0.0 ? 1.0 / sqrt(s) : 0.0;
}

// rows: out(r, c) = S(r)/‖S‖ · Vh(r, c) for r < keep (Vh ld k, out ld keep)
__global__ void k_absorb_rows(int64_t keep, int64_t n, const cxd* __restrict__ Vh, int64_t ldv, int64_t sV,
                              const double* __restrict__ S, int64_t sS, const double* __restrict__ inv,
                              cxd* __restrict__ out, int64_t sOut) {
  const int b = blockIdx.y;
  const double g = inv[b];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < keep * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % keep, c = t / keep;
    const double s = S[b * sS + r] * g;
    const cxd v = Vh[b * sV + r + ldv * c];
    out[b * sOut + t] = mkcx(s * v.x, s * v.y);
  }
}

// cols: out(r, c) = U(r, c) · S(c)/‖S‖ for c < keep (U and out ld m)
__global__ void k_absorb_cols(int64_t m, int64_t keep, const cxd* __restrict__ U, int64_t sU,
                              const double* __restrict__ S, int64_t sS, const double* __restrict__ inv,
                              cxd* __restrict__ out, int64_t sOut) {
  const int b = blockIdx.y;
  const double g = inv[b];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * keep; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / m;
    const double s = S[b * sS + c] * g;
    const cxd v = U[b * sU + t];
    out[b * sOut + t] = mkcx(s * v.x, s * v.y);
  }
}

__global__ void k_fill_one(cxd* x, int64_t stride) { x[blockIdx.x * stride] = mkcx(1.0, 0.0); }

unsigned grid_for(tn_ctx* ctx, int64_t work, int threads) {
  const int64_t cap = (int64_t)std::max(ctx->num_sms, 1) * 8;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cap, (work + threads - 1) / threads));
}

struct Dmrg {
  tn_mps* p = nullptr;
  tn_ctx* ctx = nullptr;
  int L = 0, d = 0, B = 1, kdim = 3, maxiter = 2, method = 1;
  double tol = 1e-12;
  int64_t maxdim = 128;
  std::vector<int64_t> w, cap;  // MPO bonds and bond capacities, 0..L
  std::vector<cxd*> Wp, Ws;     // 1..L
  std::vector<int64_t> sW;      // MPO instance stride per site (0: shared)
  std::vector<cxd*> eL, eR;     // 0..L
  std::vector<int64_t> eS;      // environment instance stride per bond
  cxd *V = nullptr, *Wv = nullptr, *x0 = nullptr, *TA = nullptr, *TB = nullptr, *U = nullptr, *Vh = nullptr;
  double *S = nullptr, *inv = nullptr;
  LzState* st = nullptr;
  int64_t Nmax = 0, sV = 0, sTA = 0, sTB = 0;
  std::vector<void*> owned;
  // phase timing: an event before each phase of each local update; the elapsed times are
  // summed once at the end (no synchronisation inside the sweep)
  std::vector<cudaEvent_t> ev;
  std::vector<int> ev_phase;  // phase that starts at ev[k] (-1: end marker)
  tn_status_t mark(int phase) {
    cudaEvent_t e;
    TN_CHECK_CUDA(ctx, cudaEventCreate(&e));
    TN_CHECK_CUDA(ctx, cudaEventRecord(e, ctx->stream));
    ev.push_back(e);
    ev_phase.push_back(phase);
    return TN_OK;
  }

  ~Dmrg() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    if (ctx) {
      cudaStreamSynchronize(ctx->stream);
      for (void* q : owned) tn_dev_free(ctx, q);
    }
  }
  template <typename T>
  tn_status_t alloc(size_t count, T** out) {
    void* q = nullptr;
    TN_RETURN_IF(tn_dev_alloc(ctx, std::max<size_t>(count, 1) * sizeof(T), &q));
    owned.push_back(q);
    *out = (T*)q;
    return TN_OK;
  }
};

// out = fiber(in; X, P, Q, J; M) for all instances
tn_status_t fiber(Dmrg& D, int64_t X, int64_t P, int64_t Q, int64_t J, const cxd* in, int64_t sIn, const cxd* M,
                  int64_t sM, cxd* out, int64_t sOut) {
  tn_ctx* ctx = D.ctx;
  if (P <= kFiberP && P * Q <= 3072) {
    dim3 grid(grid_for(ctx, X * J, 256), (unsigned)D.B);
    k_fiber<<<grid, 256, sizeof(cxd) * P * Q, ctx->stream>>>(X, (int)P, (int)Q, J, in, sIn, M, sM, out, sOut);
    TN_LAUNCHED(ctx);
    return TN_OK;
  }
  // wide MPO bonds: one batched GEMM per instance over the fibres j
  for (int b = 0; b < D.B; ++b)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', X, Q, P, kOne, in + b * sIn, X, X * P, M + b * sM, P, 0, kZero,
                                 out + b * sOut, X, X * Q, J));
  return TN_OK;
}

// Lc_i (bond i) from Lc_{i-1}, site i and W_i
tn_status_t update_left(Dmrg& D, int i) {
  tn_mps* p = D.p;
  tn_ctx* ctx = D.ctx;
  const int64_t chl = p->bond[i - 1], chr = p->bond[i], d = D.d, wl = D.w[i - 1], wr = D.w[i];
  const cxd* A = p->site[i];
  const int64_t sA = (int64_t)p->cap[i];
  TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', chl * wl, d * chr, chl, kOne, D.eL[i - 1], chl, D.eS[i - 1], A, chl, sA,
                               kZero, D.TA, chl * wl, D.sTA, D.B));
  TN_RETURN_IF(fiber(D, chl, wl * d, d * wr, chr, D.TA, D.sTA, D.Wp[i], D.sW[i], D.TB, D.sTB));
  for (int64_t v = 0; v < wr; ++v)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', chr, chr, chl * d, kOne, D.TB + v * chl * d, chl * d * wr, D.sTB, A,
                                 chl * d, sA, kZero, D.eL[i] + v * chr * chr, chr, D.eS[i], D.B));
  return TN_OK;
}

// R_{i-1} (bond i-1) from R_i, site i and W_i
tn_status_t update_right(Dmrg& D, int i) {
  tn_mps* p = D.p;
  tn_ctx* ctx = D.ctx;
  const int64_t chl = p->bond[i - 1], chr = p->bond[i], d = D.d, wl = D.w[i - 1], wr = D.w[i];
  const cxd* A = p->site[i];
  const int64_t sA = (int64_t)p->cap[i];
  // TA [a, (w o v), b] = A[a, s, b] · Ws[s, (w o v)]
  TN_RETURN_IF(fiber(D, chl, d, wl * d * wr, chr, A, sA, D.Ws[i], D.sW[i], D.TA, D.sTA));
  // TB [(a w o), b'] = TA [(a w o), (v b)] · R_i [(v b), b']
  TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', chl * wl * d, chr, wr * chr, kOne, D.TA, chl * wl * d, D.sTA, D.eR[i],
                               wr * chr, D.eS[i], kZero, D.TB, chl * wl * d, D.sTB, D.B));
  // TA [(a w), a'] = TB [(a w), (o b')] · Aᴴ
  TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'C', chl * wl, chl, d * chr, kOne, D.TB, chl * wl, D.sTB, A, chl, sA, kZero,
                               D.TA, chl * wl, D.sTA, D.B));
  dim3 grid(grid_for(ctx, chl * wl * chl, 256), (unsigned)D.B);
  k_swap01<<<grid, 256, 0, ctx->stream>>>(chl, wl, chl, D.TA, D.sTA, D.eR[i - 1], D.eS[i - 1]);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// y (D.Wv) = Heff · (slot k of D.V) for the single site i (nsite 1) or the pair (i, i+1)
tn_status_t matvec(Dmrg& D, int nsite, int i, int k) {
  tn_mps* p = D.p;
  tn_ctx* ctx = D.ctx;
  const int64_t d = D.d;
  const cxd* x = D.V + (int64_t)k * D.Nmax;
  if (nsite == 1) {
    const int64_t chl = p->bond[i - 1], chr = p->bond[i], wl = D.w[i - 1], wr = D.w[i];
    TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', chl * wl, d * chr, chl, kOne, D.eL[i - 1], chl, D.eS[i - 1], x, chl,
                                 D.sV, kZero, D.TA, chl * wl, D.sTA, D.B));
    TN_RETURN_IF(fiber(D, chl, wl * d, d * wr, chr, D.TA, D.sTA, D.Wp[i], D.sW[i], D.TB, D.sTB));
    return gemm_cx<double>(ctx, 'N', 'N', chl * d, chr, wr * chr, kOne, D.TB, chl * d, D.sTB, D.eR[i], wr * chr,
                           D.eS[i], kZero, D.Wv, chl * d, D.Nmax, D.B);
  }
  const int64_t chl = p->bond[i - 1], chr = p->bond[i + 1], wl = D.w[i - 1], wm = D.w[i], wr = D.w[i + 1];
  TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', chl * wl, d * d * chr, chl, kOne, D.eL[i - 1], chl, D.eS[i - 1], x, chl,
                               D.sV, kZero, D.TA, chl * wl, D.sTA, D.B));
  TN_RETURN_IF(fiber(D, chl, wl * d, d * wm, d * chr, D.TA, D.sTA, D.Wp[i], D.sW[i], D.TB, D.sTB));
  TN_RETURN_IF(fiber(D, chl * d, wm * d, d * wr, chr, D.TB, D.sTB, D.Wp[i + 1], D.sW[i + 1], D.TA, D.sTA));
  return gemm_cx<double>(ctx, 'N', 'N', chl * d * d, chr, wr * chr, kOne, D.TA, chl * d * d, D.sTA, D.eR[i + 1],
                         wr * chr, D.eS[i + 1], kZero, D.Wv, chl * d * d, D.Nmax, D.B);
}

// restarted Lanczos from x0 (instance stride sx0, N elements); the Ritz vector ends in slot 0
tn_status_t eigsolve(Dmrg& D, int nsite, int i, int64_t N, const cxd* x0, int64_t sx0) {
  tn_ctx* ctx = D.ctx;
  k_lz_start<<<D.B, kLzThreads, 0, ctx->stream>>>(N, (const double2*)x0, sx0, (double2*)D.V, D.sV, D.st);
  TN_LAUNCHED(ctx);
  for (int it = 1; it <= D.maxiter; ++it) {
    for (int k = it == 1 ? 0 : 1; k < D.kdim; ++k) {
      TN_RETURN_IF(matvec(D, nsite, i, k));
      if (k < 4)
        k_lz_orth<4, 1024><<<D.B, 1024, 0, ctx->stream>>>(N, k, (double2*)D.V, D.sV, D.Nmax, (double2*)D.Wv, D.Nmax,
                                                           D.st, D.tol);
      else if (k < 8)
        k_lz_orth<8, 512><<<D.B, 512, 0, ctx->stream>>>(N, k, (double2*)D.V, D.sV, D.Nmax, (double2*)D.Wv, D.Nmax,
                                                         D.st, D.tol);
      else
        k_lz_orth<kLzMax, 256><<<D.B, 256, 0, ctx->stream>>>(N, k, (double2*)D.V, D.sV, D.Nmax, (double2*)D.Wv,
                                                              D.Nmax, D.st, D.tol);
      TN_LAUNCHED(ctx);
    }
    k_lz_ritz<<<cdiv(D.B, 32), 32, 0, ctx->stream>>>(D.B, D.kdim, D.maxiter, D.tol, D.st);
    TN_LAUNCHED(ctx);
    dim3 grid(grid_for(ctx, N, 256), (unsigned)D.B);
    k_lz_combine<<<grid, 256, 0, ctx->stream>>>(N, (double2*)D.V, D.sV, D.Nmax, D.st);
    TN_LAUNCHED(ctx);
  }
  return TN_OK;
}

tn_status_t copy_out(tn_ctx* ctx, cxd* dst, size_t sDst, const cxd* src, size_t sSrc, size_t elems, int B) {
  TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(dst, sDst * sizeof(cxd), src, sSrc * sizeof(cxd), elems * sizeof(cxd), B,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
  return TN_OK;
}

// X_b ← inv_b · X_b (elems elements per instance)
__global__ void k_scale_inst(int64_t elems, cxd* __restrict__ X, int64_t sX, const double* __restrict__ inv) {
  const int b = blockIdx.y;
  const double g = inv[b];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < elems; t += (int64_t)gridDim.x * blockDim.x) {
    cxd v = X[b * sX + t];
    X[b * sX + t] = mkcx(g * v.x, g * v.y);
  }
}

tn_status_t scale_inst(Dmrg& D, cxd* X, int64_t sX, int64_t elems) {
  dim3 grid(grid_for(D.ctx, elems, 256), (unsigned)D.B);
  k_scale_inst<<<grid, 256, 0, D.ctx->stream>>>(elems, X, sX, D.inv);
  TN_LAUNCHED(D.ctx);
  return TN_OK;
}

// split the optimised pair (j, j+1) held in slot 0 (θ, m × n with m = χ_{j-1} d and
// n = d χ_{j+1}): thin SVD, keep min(maxdim, k) values, normalise them and absorb them
// into site j+1 (absorb_right) or site j (DMRG.jl:338-349, 437-448).  Only the singular
// vectors on the side that stays an isometry are computed; the other side is the
// projection of θ onto them, which equals S·Vᴴ (or U·S) without dividing by S:
//   absorb right, m ≥ n:  U S = svd_left(θ);   site j = U_keep,   site j+1 = U_keepᴴ θ / ‖S_keep‖
//   absorb left,  n ≥ m:  V S = svd_left(θᴴ);  site j+1 = V_keepᴴ, site j = θ V_keep / ‖S_keep‖
// Near the chain ends (the other shapes) the full thin SVD is used.
tn_status_t split_pair_impl(Dmrg& D, int j, bool absorb_right) {
  tn_mps* p = D.p;
  tn_ctx* ctx = D.ctx;
  const int64_t d = D.d, m = p->bond[j - 1] * d, n = d * p->bond[j + 1], k = std::min(m, n);
  const int64_t keep = std::min(D.maxdim, k);
  const cxd* theta = D.V;
  if (absorb_right && m >= n) {
    TN_RETURN_IF(ws_reserve(ctx, svd_left_workspace(p->prec, m, n, D.B)));
    TN_RETURN_IF(svd_left(ctx, p->prec, m, n, theta, m, D.sV, D.U, D.Nmax, D.S, D.Nmax, D.B, keep));
    k_inv_norm<<<D.B, 256, 0, ctx->stream>>>((int)keep, D.S, D.Nmax, D.inv);
    TN_LAUNCHED(ctx);
    TN_RETURN_IF(mps_ensure_site(p, j, (size_t)(m * keep)));
    TN_RETURN_IF(mps_ensure_site(p, j + 1, (size_t)(keep * n)));
    TN_RETURN_IF(copy_out(ctx, p->site[j], p->cap[j], D.U, D.Nmax, (size_t)(m * keep), D.B));
    TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', keep, n, m, kOne, D.U, m, D.Nmax, theta, m, D.sV, kZero,
                                 p->site[j + 1], keep, (int64_t)p->cap[j + 1], D.B));
    TN_RETURN_IF(scale_inst(D, p->site[j + 1], (int64_t)p->cap[j + 1], keep * n));
  } else if (!absorb_right && n >= m) {
    // θᴴ (n × m) into the x0 buffer (θ itself stays in slot 0)
    TN_RETURN_IF(transpose_cx<double>(ctx, m, n, theta, m, D.sV, D.x0, n, D.Nmax, D.B, true));
    TN_RETURN_IF(ws_reserve(ctx, svd_left_workspace(p->prec, n, m, D.B)));
    TN_RETURN_IF(svd_left(ctx, p->prec, n, m, D.x0, n, D.Nmax, D.U, D.Nmax, D.S, D.Nmax, D.B, keep));
    k_inv_norm<<<D.B, 256, 0, ctx->stream>>>((int)keep, D.S, D.Nmax, D.inv);
    TN_LAUNCHED(ctx);
    TN_RETURN_IF(mps_ensure_site(p, j, (size_t)(m * keep)));
    TN_RETURN_IF(mps_ensure_site(p, j + 1, (size_t)(keep * n)));
    TN_RETURN_IF(transpose_cx<double>(ctx, n, keep, D.U, n, D.Nmax, p->site[j + 1], keep, (int64_t)p->cap[j + 1], D.B,
                                      true));
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', m, keep, n, kOne, theta, m, D.sV, D.U, n, D.Nmax, kZero, p->site[j], m,
                                 (int64_t)p->cap[j], D.B));
    TN_RETURN_IF(scale_inst(D, p->site[j], (int64_t)p->cap[j], m * keep));
  } else {
    TN_RETURN_IF(ws_reserve(ctx, svd_any_workspace(TN_C64, p->prec, m, n, D.B)));
    TN_RETURN_IF(svd_any(ctx, TN_C64, p->prec, m, n, theta, m, D.sV, D.U, D.Nmax, D.S, D.Nmax, D.Vh, D.Nmax, D.B));
    k_inv_norm<<<D.B, 256, 0, ctx->stream>>>((int)keep, D.S, D.Nmax, D.inv);
    TN_LAUNCHED(ctx);
    TN_RETURN_IF(mps_ensure_site(p, j, (size_t)(m * keep)));
    TN_RETURN_IF(mps_ensure_site(p, j + 1, (size_t)(keep * n)));
    dim3 gU(grid_for(ctx, m * keep, 256), (unsigned)D.B), gV(grid_for(ctx, keep * n, 256), (unsigned)D.B);
    if (absorb_right) {
      TN_RETURN_IF(copy_out(ctx, p->site[j], p->cap[j], D.U, D.Nmax, (size_t)(m * keep), D.B));
      k_absorb_rows<<<gV, 256, 0, ctx->stream>>>(keep, n, D.Vh, k, D.Nmax, D.S, D.Nmax, D.inv, p->site[j + 1],
                                                 (int64_t)p->cap[j + 1]);
      TN_LAUNCHED(ctx);
    } else {
      k_absorb_cols<<<gU, 256, 0, ctx->stream>>>(m, keep, D.U, D.Nmax, D.S, D.Nmax, D.inv, p->site[j],
                                                 (int64_t)p->cap[j]);
      TN_LAUNCHED(ctx);
      TN_RETURN_IF(copy_matrix_cxd(ctx, keep, n, D.Vh, k, p->site[j + 1], keep, D.Nmax, (int64_t)p->cap[j + 1], D.B));
    }
  }
  p->bond[j] = keep;
  p->cap_bond[j] = std::max(p->cap_bond[j], keep);
  p->lam_len = 0;
  return TN_OK;
}

// A split whose SVD does not converge leaves the pair matrix (instance 0) in
// $TENETGB_DUMP_DIR/dmrg_pair_<j>.bin when that variable is set: int64 m, n, then the
// column-major ComplexF64 data — the input a bug report needs.
tn_status_t split_pair(Dmrg& D, int j, bool absorb_right) {
  const tn_status_t st = split_pair_impl(D, j, absorb_right);
  D.ctx->dmrg_svd_sweeps += std::max(0, D.ctx->last_sweeps_fp64) + std::max(0, D.ctx->last_sweeps_fp32);
  const char* dir = getenv("TENETGB_DUMP_DIR");
  if (st != TN_ENOCONV || !dir) return st;
  tn_mps* p = D.p;
  const int64_t m = p->bond[j - 1] * D.d, n = D.d * p->bond[j + 1];
  std::vector<cxd> h((size_t)(m * n));
  if (cudaMemcpy(h.data(), D.V, sizeof(cxd) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return st;
  char path[1024];
  snprintf(path, sizeof(path), "%s/dmrg_pair_%d.bin", dir, j);
  if (FILE* f = fopen(path, "wb")) {
    fwrite(&m, sizeof(m), 1, f);
    fwrite(&n, sizeof(n), 1, f);
    fwrite(h.data(), sizeof(cxd), h.size(), f);
    fclose(f);
  }
  return st;
}

// θ = site j · site j+1 over their shared bond, into D.x0 (instance stride Nmax)
tn_status_t form_pair(Dmrg& D, int j) {
  tn_mps* p = D.p;
  const int64_t d = D.d, m = p->bond[j - 1] * d, c = p->bond[j], n = d * p->bond[j + 1];
  return gemm_cx<double>(D.ctx, 'N', 'N', m, n, c, kOne, p->site[j], m, (int64_t)p->cap[j], p->site[j + 1], c,
                         (int64_t)p->cap[j + 1], kZero, D.x0, m, D.Nmax, D.B);
}

tn_status_t read_energies(Dmrg& D, double* h) {
  std::vector<LzState> hs(D.B);
  TN_CHECK_CUDA(D.ctx, cudaMemcpyAsync(hs.data(), D.st, sizeof(LzState) * D.B, cudaMemcpyDeviceToHost, D.ctx->stream));
  TN_CHECK_CUDA(D.ctx, cudaStreamSynchronize(D.ctx->stream));
  for (int b = 0; b < D.B; ++b) h[b] = hs[b].theta;
  return TN_OK;
}

int64_t pow_sat(int64_t d, int64_t e, int64_t cap) {
  int64_t r = 1;
  for (int64_t i = 0; i < e && r < cap; ++i) r *= d;
  return std::min(r, cap);
}

tn_status_t run(Dmrg& D, const void* const* h_mpo, int mpo_count, int nsweeps, double* h_energy, double* h_hist) {
  tn_mps* p = D.p;
  tn_ctx* ctx = D.ctx;
  const int L = D.L, B = D.B;
  const int64_t d = D.d;
  // bond capacities: Dmrg1 never grows a bond (QR gauge moves keep k = min(m, n) ≤ n);
  // Dmrg2 bonds reach at most min(maxdim, d^k, d^(L-k))
  ctx->dmrg_svd_sweeps = 0;
  D.cap.assign(L + 1, 1);
  for (int k = 1; k < L; ++k) {
    D.cap[k] = p->bond[k];
    if (D.method == 2)
      D.cap[k] = std::max(D.cap[k], std::min(pow_sat(d, k, D.maxdim), pow_sat(d, L - k, D.maxdim)));
  }
  int64_t wmax = 1, n1 = 1, n2 = 1;
  for (int k = 0; k <= L; ++k) wmax = std::max(wmax, D.w[k]);
  for (int i = 1; i <= L; ++i) n1 = std::max(n1, D.cap[i - 1] * d * D.cap[i]);
  for (int j = 1; j < L; ++j) n2 = std::max(n2, D.cap[j - 1] * d * d * D.cap[j + 1]);
  D.Nmax = D.method == 1 ? n1 : std::max(n1, n2);
  D.sV = (int64_t)(D.kdim + 1) * D.Nmax;
  D.sTA = std::max(wmax * wmax * n1, wmax * D.Nmax);
  for (int k = 1; k < L; ++k) D.sTA = std::max(D.sTA, D.cap[k] * D.cap[k] * wmax);
  D.sTB = wmax * D.Nmax;
  TN_RETURN_IF(D.alloc((size_t)(D.sV * B), &D.V));
  TN_RETURN_IF(D.alloc((size_t)(D.Nmax * B), &D.Wv));
  TN_RETURN_IF(D.alloc((size_t)(D.sTA * B), &D.TA));
  TN_RETURN_IF(D.alloc((size_t)(D.sTB * B), &D.TB));
  TN_RETURN_IF(D.alloc((size_t)B, &D.st));
  TN_RETURN_IF(D.alloc((size_t)B, &D.inv));
  TN_CHECK_CUDA(ctx, cudaMemsetAsync(D.V, 0, sizeof(cxd) * (size_t)(D.sV * B), ctx->stream));
  if (D.method == 2) {
    TN_RETURN_IF(D.alloc((size_t)(D.Nmax * B), &D.x0));
    TN_RETURN_IF(D.alloc((size_t)(D.Nmax * B), &D.U));
    TN_RETURN_IF(D.alloc((size_t)(D.Nmax * B), &D.Vh));
    TN_RETURN_IF(D.alloc((size_t)(D.Nmax * B), &D.S));
  }
  // environments
  D.eL.assign(L + 1, nullptr);
  D.eR.assign(L + 1, nullptr);
  D.eS.assign(L + 1, 1);
  for (int k = 0; k <= L; ++k) {
    D.eS[k] = D.cap[k] * D.cap[k] * D.w[k];
    TN_RETURN_IF(D.alloc((size_t)(D.eS[k] * B), &D.eL[k]));
    TN_RETURN_IF(D.alloc((size_t)(D.eS[k] * B), &D.eR[k]));
  }
  k_fill_one<<<B, 1, 0, ctx->stream>>>(D.eL[0], D.eS[0]);
  TN_LAUNCHED(ctx);
  k_fill_one<<<B, 1, 0, ctx->stream>>>(D.eR[L], D.eS[L]);
  TN_LAUNCHED(ctx);
  // MPO sites in the two working layouts
  D.Wp.assign(L + 1, nullptr);
  D.Ws.assign(L + 1, nullptr);
  D.sW.assign(L + 1, 0);
  for (int i = 1; i <= L; ++i) {
    const int64_t wl = D.w[i - 1], wr = D.w[i], sz = wl * d * d * wr;
    std::vector<cxd> hp((size_t)(sz * mpo_count)), hsw((size_t)(sz * mpo_count));
    for (int c = 0; c < mpo_count; ++c) {
      const cxd* W = (const cxd*)h_mpo[(size_t)c * L + (i - 1)];
      for (int64_t v = 0; v < wr; ++v)
        for (int64_t s = 0; s < d; ++s)
          for (int64_t o = 0; o < d; ++o)
            for (int64_t a = 0; a < wl; ++a) {
              const cxd val = W[a + wl * (o + d * (s + d * v))];
              hp[(size_t)(c * sz + a + wl * (s + d * (o + d * v)))] = val;
              hsw[(size_t)(c * sz + s + d * (a + wl * (o + d * v)))] = val;
            }
    }
    TN_RETURN_IF(D.alloc((size_t)(sz * mpo_count), &D.Wp[i]));
    TN_RETURN_IF(D.alloc((size_t)(sz * mpo_count), &D.Ws[i]));
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(D.Wp[i], hp.data(), sizeof(cxd) * hp.size(), cudaMemcpyHostToDevice,
                                       ctx->stream));
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(D.Ws[i], hsw.data(), sizeof(cxd) * hsw.size(), cudaMemcpyHostToDevice,
                                       ctx->stream));
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // pageable sources
    D.sW[i] = mpo_count == 1 ? 0 : sz;
  }
  // right environments from canonize!(ψ, i), i = L-1 … 1 (DMRG.jl:63-83)
  for (int i = L - 1; i >= 1; --i) {
    TN_RETURN_IF(tn_mps_canonize_mixed(p, i, i));
    TN_RETURN_IF(update_right(D, i + 1));
  }
  int hist = 0;
  for (int sweep = 0; sweep < nsweeps; ++sweep) {
    if (D.method == 1) {
      for (int i = 2; i <= L; ++i) {  // DMRG.jl:88-146
        TN_RETURN_IF(D.mark(0));
        TN_RETURN_IF(tn_mps_canonize_mixed(p, i, i));
        TN_RETURN_IF(D.mark(1));
        TN_RETURN_IF(update_left(D, i - 1));
        const int64_t N = p->bond[i - 1] * d * p->bond[i];
        TN_RETURN_IF(D.mark(2));
        TN_RETURN_IF(eigsolve(D, 1, i, N, p->site[i], (int64_t)p->cap[i]));
        TN_RETURN_IF(copy_out(ctx, p->site[i], p->cap[i], D.V, D.sV, (size_t)N, B));
      }
      if (h_hist) TN_RETURN_IF(read_energies(D, h_hist + (size_t)(hist++) * B));
      for (int i = L - 1; i >= 1; --i) {  // DMRG.jl:150-206
        TN_RETURN_IF(D.mark(0));
        TN_RETURN_IF(tn_mps_canonize_mixed(p, i, i));
        TN_RETURN_IF(D.mark(1));
        TN_RETURN_IF(update_right(D, i + 1));
        const int64_t N = p->bond[i - 1] * d * p->bond[i];
        TN_RETURN_IF(D.mark(2));
        TN_RETURN_IF(eigsolve(D, 1, i, N, p->site[i], (int64_t)p->cap[i]));
        TN_RETURN_IF(copy_out(ctx, p->site[i], p->cap[i], D.V, D.sV, (size_t)N, B));
      }
      if (h_hist) TN_RETURN_IF(read_energies(D, h_hist + (size_t)(hist++) * B));
    } else {
      for (int i = 2; i <= L; ++i) {  // DMRG.jl:258-357
        TN_RETURN_IF(D.mark(0));
        TN_RETURN_IF(tn_mps_canonize_mixed(p, i, i));
        TN_RETURN_IF(D.mark(1));
        if (i > 2) TN_RETURN_IF(update_left(D, i - 2));
        TN_RETURN_IF(D.mark(2));
        TN_RETURN_IF(form_pair(D, i - 1));
        const int64_t N = p->bond[i - 2] * d * d * p->bond[i];
        TN_RETURN_IF(eigsolve(D, 2, i - 1, N, D.x0, D.Nmax));
        TN_RETURN_IF(D.mark(3));
        TN_RETURN_IF(split_pair(D, i - 1, true));
        p->kind = TN_FORM_MIXED;
        p->lo = p->hi = i;
      }
      if (h_hist) TN_RETURN_IF(read_energies(D, h_hist + (size_t)(hist++) * B));
      for (int i = L - 1; i >= 1; --i) {  // DMRG.jl:361-455
        TN_RETURN_IF(D.mark(0));
        TN_RETURN_IF(tn_mps_canonize_mixed(p, i, i));
        TN_RETURN_IF(D.mark(1));
        if (i < L - 1) TN_RETURN_IF(update_right(D, i + 2));
        TN_RETURN_IF(D.mark(2));
        TN_RETURN_IF(form_pair(D, i));
        const int64_t N = p->bond[i - 1] * d * d * p->bond[i + 1];
        TN_RETURN_IF(eigsolve(D, 2, i, N, D.x0, D.Nmax));
        TN_RETURN_IF(D.mark(3));
        TN_RETURN_IF(split_pair(D, i, false));
        p->kind = TN_FORM_MIXED;
        p->lo = p->hi = i;
      }
      if (h_hist) TN_RETURN_IF(read_energies(D, h_hist + (size_t)(hist++) * B));
    }
  }
  TN_RETURN_IF(D.mark(-1));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 4; ++k) ctx->dmrg_ms[k] = 0.0;
  ctx->dmrg_updates = 0;
  for (size_t k = 0; k + 1 < D.ev.size(); ++k) {
    float ms = 0.f;
    if (D.ev_phase[k] < 0 || cudaEventElapsedTime(&ms, D.ev[k], D.ev[k + 1]) != cudaSuccess) continue;
    ctx->dmrg_ms[D.ev_phase[k]] += ms;
    ctx->dmrg_updates += D.ev_phase[k] == 0;
  }
  if (h_energy) {
    if (nsweeps == 0)
      for (int b = 0; b < B; ++b) h_energy[b] = 0.0;
    else
      TN_RETURN_IF(read_energies(D, h_energy));
  }
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

}  // namespace

extern "C" {

tn_status_t tn_mps_dmrg(tn_mps* p, const void* const* h_mpo_sites, const int64_t* mpo_bonds, int32_t mpo_count,
                        int32_t method, int32_t nsweeps, int64_t maxdim, int32_t krylovdim, int32_t maxiter, double tol,
                        double* h_energy, double* h_history) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, h_mpo_sites != nullptr, "dmrg: null MPO");
  TN_ARG(ctx, method == 1 || method == 2, "dmrg: method must be 1 (Dmrg1) or 2 (Dmrg2)");
  TN_ARG(ctx, mpo_count == 1 || mpo_count == p->B, "dmrg: give one MPO or one per instance");
  TN_ARG(ctx, nsweeps >= 0, "dmrg: nsweeps must be non-negative");
  TN_ARG(ctx, krylovdim >= 2 && krylovdim < kLzMax, "dmrg: krylovdim must be in [2, 15]");
  TN_ARG(ctx, maxiter >= 1, "dmrg: maxiter must be positive");
  const int L = p->L;
  for (int c = 0; c < mpo_count; ++c)
    for (int i = 0; i < L; ++i) TN_ARG(ctx, h_mpo_sites[(size_t)c * L + i] != nullptr, "dmrg: null MPO site");
  Dmrg D;
  D.p = p;
  D.ctx = ctx;
  D.L = L;
  D.d = p->d;
  D.B = p->B;
  D.kdim = krylovdim;
  D.maxiter = maxiter;
  D.method = method;
  D.tol = tol > 0 ? tol : 1e-12;
  D.maxdim = maxdim > 0 ? maxdim : 128;
  D.w.assign(L + 1, 1);
  for (int i = 1; i < L; ++i) {
    TN_ARG(ctx, mpo_bonds && mpo_bonds[i - 1] >= 1, "dmrg: MPO bond dimensions must be positive");
    D.w[i] = mpo_bonds[i - 1];
  }
  return run(D, h_mpo_sites, mpo_count, nsweeps, h_energy, h_history);
}

tn_status_t tn_dmrg_last_stats(tn_ctx* ctx, double* h_ms, int64_t* h_updates) {
  if (!ctx) return TN_EINVAL;
  for (int k = 0; h_ms && k < 4; ++k) h_ms[k] = ctx->dmrg_ms[k];
  if (h_updates) {
    h_updates[0] = ctx->dmrg_updates;
    h_updates[1] = ctx->dmrg_svd_sweeps;
  }
  return TN_OK;
}

}  // extern "C"
