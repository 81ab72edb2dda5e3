// Grouped (ragged) MPS batches: B independent MPS of different lengths and bond
// dimensions, advanced in lockstep by grouped launches.
//
// One call runs, for every instance b, the reference's
//   canonize!(ψ_b, MixedCanonical(L_b))        src/Operations/canonize.jl:121-150
//   compress!(ψ_b; maxdim = maxdim_b)           src/Operations/compress.jl:21-69
//   norm(ψ_b)   (= ‖Λ_{L_b−1}‖ in the final bond-canonical form)   src/Operations/norm.jl:31-34
// as three sweeps whose step k is ONE launch per kernel over all instances that still have
// a site k (a descriptor table gives each instance's shapes and pointers):
//   A  QR sweep left→right: A_k = Q R, A_k ← Q, A_{k+1} ← R A_{k+1}
//   B  LQ sweep right→left (the centre moves back to site 1): A_i = L Q via the QR of A_iᴴ,
//      A_i ← Q, A_{i−1} ← A_{i−1} L
//   C  SVD sweep left→right with truncation: M_k = U Σ Vᴴ (one-sided Jacobi on M_k, U and Σ
//      only), keep r = min(maxdim, rows, χ_k) columns, A_k ← U_r, A_{k+1} ← (U_rᴴ M_k) A_{k+1}
//      (= Σ_r V_rᴴ A_{k+1}: the next bond's centre with Λ already absorbed).
// Sweep B + C is compress!'s sequence of bond canonisations with the gauge moves done by
// QR (Tenet moves the centre by QR and bond-canonizes by SVD, canonize.jl:158-232); the
// final state and every Λ_k are the reference's up to rounding (gauge-invariant).  At the
// end site L_b holds Λ Vᴴ A_L (the state with Λ absorbed) and Λ_{L−1} is kept apart.
// All arithmetic is FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "tn_internal.cuh"

namespace {

// ---------------------------------------------------------------------------------
// descriptors (device-resident tables, one entry per instance in a step)
// ---------------------------------------------------------------------------------
struct CopyD {
  const cxd* src;
  cxd* dst;
  int64_t lds, ldd, rows, cols;  // of src
  int conjT;                     // 0: dst(r, c) = src(r, c); 1: dst(c, r) = conj(src(r, c))
};
struct GemmD {
  const cxd* A;
  const cxd* B;
  cxd* C;
  int64_t m, n, k, lda, ldb, ldc;
  int opa, opb;  // 'N' / 'C'
};
struct QrD {
  cxd* W;  // m × n work (ld m), factored in place
  cxd* tau;
  cxd* T;  // npan · nb · nb
  cxd* Q;  // m × n (ld m)
  cxd* R;  // n × n (ld n)
  int64_t m, n;
};
struct JacD {
  cxd* W;  // m × n (ld m)
  double* nrm;
  double* S;
  int* order;
  cxd* U;  // m × r (ld m): the r leading left vectors
  int64_t m, n, r;
  int N;
};

// ---------------------------------------------------------------------------------
// grouped copy
// ---------------------------------------------------------------------------------
__global__ void k_g_copy(const CopyD* __restrict__ D) {
  const CopyD d = D[blockIdx.y];
  const int64_t total = d.rows * d.cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % d.rows, c = t / d.rows;
    const cxd v = d.src[r + c * d.lds];
    if (d.conjT)
      d.dst[c + r * d.ldd] = conjg(v);
    else
      d.dst[r + c * d.ldd] = v;
  }
}

// ---------------------------------------------------------------------------------
// grouped GEMM: C_b = op(A_b) op(B_b); CTA → (instance, tile) through a prefix table
// ---------------------------------------------------------------------------------
__device__ __forceinline__ cxd g_load(const cxd* X, int64_t ld, int op, int64_t r, int64_t c) {
  if (op == 'N') return X[r + c * ld];
  const cxd v = X[c + r * ld];
  return mkcx(v.x, -v.y);  // 'C'
}

template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_g_gemm(const GemmD* __restrict__ D, const int64_t* __restrict__ tile_start, int nprob) {
  constexpr int NT = (BM / TM) * (BN / TN), RX = BN / TN, RY = BM / TM;
  __shared__ cxd As[BK][BM + 1];
  __shared__ cxd Bs[BK][BN + 1];
  // instance: the last b with tile_start[b] <= blockIdx.x
  int lo = 0, hi = nprob - 1;
  const int64_t tile = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tile_start[mid] <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  const GemmD d = D[lo];
  const int64_t t = tile - tile_start[lo];
  const int64_t tiles_m = (d.m + BM - 1) / BM;
  const int64_t i0 = (t % tiles_m) * BM, j0 = (t / tiles_m) * BN;
  const int tid = threadIdx.x, tx = tid % RX, ty = tid / RX;
  cxd acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = mkcx(0.0, 0.0);
  for (int64_t p0 = 0; p0 < d.k; p0 += BK) {
    for (int u = tid; u < BM * BK; u += NT) {
      int ii, pp;
      if (d.opa == 'N') {
        ii = u % BM;
        pp = u / BM;
      } else {
        pp = u % BK;
        ii = u / BK;
      }
      const int64_t gi = i0 + ii, gp = p0 + pp;
      As[pp][ii] = (gi < d.m && gp < d.k) ? g_load(d.A, d.lda, d.opa, gi, gp) : mkcx(0.0, 0.0);
    }
    for (int u = tid; u < BK * BN; u += NT) {
      int pp, jj;
      if (d.opb == 'N') {
        pp = u % BK;
        jj = u / BK;
      } else {
        jj = u % BN;
        pp = u / BN;
      }
      const int64_t gp = p0 + pp, gj = j0 + jj;
      Bs[pp][jj] = (gp < d.k && gj < d.n) ? g_load(d.B, d.ldb, d.opb, gp, gj) : mkcx(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int pp = 0; pp < BK; ++pp) {
      cxd a[TM], b[TN];
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
#pragma unroll
  for (int r = 0; r < TM; ++r) {
    const int64_t gi = i0 + ty + r * RY;
    if (gi >= d.m) continue;
#pragma unroll
    for (int c = 0; c < TN; ++c) {
      const int64_t gj = j0 + tx + c * RX;
      if (gj < d.n) d.C[gi + gj * d.ldc] = acc[r][c];
    }
  }
}

// ---------------------------------------------------------------------------------
// grouped Householder QR (m ≥ n), compact WY with panel width kNb (LAPACK convention
// H = I − τ v vᴴ, v_1 = 1), as the uniform-batch kernels: panel in shared memory, block
// reflector over column slabs, Q formed by applying the panels in reverse to [I; 0]
// ---------------------------------------------------------------------------------
constexpr int kNb = 8;
constexpr int kSlab = 2;

__device__ __forceinline__ cxd vget(const cxd* P, int64_t ld, int64_t r, int a) {
  if (r < a) return mkcx(0.0, 0.0);
  if (r == a) return mkcx(1.0, 0.0);
  return P[r + (int64_t)a * ld];
}

__global__ void __launch_bounds__(256) k_g_qr_panel(const QrD* __restrict__ D, int64_t j0) {
  extern __shared__ unsigned char smem_raw[];
  cxd* P = reinterpret_cast<cxd*>(smem_raw);
  __shared__ cxd s_tau[kNb];
  __shared__ cxd s_G[kNb][kNb + 1];
  __shared__ cxd s_T[kNb][kNb + 1];
  const QrD d = D[blockIdx.x];
  if (j0 >= d.n) return;
  const int jb = (int)(d.n - j0 < kNb ? d.n - j0 : kNb);
  const int64_t mr = d.m - j0, ldw = d.m;
  cxd* Wb = d.W + j0 + j0 * ldw;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  for (int64_t t = tid; t < mr * jb; t += blockDim.x) P[t] = Wb[(t % mr) + (t / mr) * ldw];
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    cxd* col = P + (int64_t)c * mr;
    if (warp == 0) {
      double s2 = 0;
      for (int64_t r = c + 1 + lane; r < mr; r += 32) s2 += abs2(col[r]);
      s2 = warp_sum(s2);
      const cxd alpha = col[c];
      cxd tc, scale;
      double beta;
      if (s2 == 0.0 && alpha.y == 0.0) {
        tc = mkcx(0.0, 0.0);
        scale = mkcx(0.0, 0.0);
        beta = alpha.x;
      } else {
        const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + s2);
        beta = alpha.x >= 0.0 ? -nrm : nrm;
        tc = mkcx((beta - alpha.x) / beta, -alpha.y / beta);
        const cxd dd = mkcx(alpha.x - beta, alpha.y);
        const double q = abs2(dd);
        scale = mkcx(dd.x / q, -dd.y / q);  // 1 / (α − β)
      }
      for (int64_t r = c + 1 + lane; r < mr; r += 32) col[r] = col[r] * scale;
      __syncwarp();
      if (lane == 0) {
        col[c] = mkcx(beta, 0.0);
        s_tau[c] = tc;
      }
    }
    __syncthreads();
    const cxd ctau = conjg(s_tau[c]);
    for (int j = c + 1 + warp; j < jb; j += nwarps) {
      cxd* cj = P + (int64_t)j * mr;
      cxd w = mkcx(0.0, 0.0);
      for (int64_t r = c + lane; r < mr; r += 32) cfma_cj(w, r == c ? mkcx(1.0, 0.0) : col[r], cj[r]);
      w.x = warp_sum(w.x);
      w.y = warp_sum(w.y);
      const cxd f = ctau * w;
      for (int64_t r = c + lane; r < mr; r += 32) cj[r] = cj[r] - (r == c ? mkcx(1.0, 0.0) : col[r]) * f;
    }
    __syncthreads();
  }
  for (int pair = warp; pair < jb * jb; pair += nwarps) {
    const int a = pair % jb, i = pair / jb;
    if (a >= i) continue;
    cxd g = mkcx(0.0, 0.0);
    for (int64_t r = i + lane; r < mr; r += 32) cfma_cj(g, P[r + (int64_t)a * mr], r == i ? mkcx(1.0, 0.0) : P[r + (int64_t)i * mr]);
    g.x = warp_sum(g.x);
    g.y = warp_sum(g.y);
    if (lane == 0) s_G[a][i] = g;
  }
  __syncthreads();
  // T(i,i) = τ_i; T(0:i, i) = −τ_i T(0:i, 0:i) G(0:i, i)
  if (warp == 0) {
    for (int i = 0; i < jb; ++i) {
      cxd s = mkcx(0.0, 0.0);
      const int a = lane;
      if (a < i)
        for (int q = a; q < i; ++q) cfma(s, s_T[a][q], s_G[q][i]);
      __syncwarp();
      if (a < i) s_T[a][i] = mkcx(0.0, 0.0) - s_tau[i] * s;
      if (a == i) s_T[i][i] = s_tau[i];
      if (a > i && a < jb) s_T[a][i] = mkcx(0.0, 0.0);
      __syncwarp();
    }
  }
  __syncthreads();
  cxd* Tb = d.T + (j0 / kNb) * kNb * kNb;
  for (int t = tid; t < jb * jb; t += blockDim.x) Tb[(t % jb) + (t / jb) * kNb] = s_T[t % jb][t / jb];
  if (tid < jb) d.tau[j0 + tid] = s_tau[tid];
  for (int64_t t = tid; t < mr * jb; t += blockDim.x) Wb[(t % mr) + (t / mr) * ldw] = P[t];
}

// X[j0:m, cols] ← (I − V T Vᴴ)^{op} X: trailing update (onQ = false: X = W, columns
// j0+jb..n, op = ᴴ) or Q formation (onQ = true: X = Q, columns j0..n, op = identity)
__global__ void __launch_bounds__(256) k_g_qr_apply(const QrD* __restrict__ D, int64_t j0, bool onQ) {
  __shared__ cxd sW_[kNb][kSlab];
  __shared__ cxd sY[kNb][kSlab];
  const QrD d = D[blockIdx.y];
  if (j0 >= d.n) return;
  const int jb = (int)(d.n - j0 < kNb ? d.n - j0 : kNb);
  const int64_t c0 = onQ ? j0 : j0 + jb, c1 = d.n;
  const int64_t cs = c0 + (int64_t)blockIdx.x * kSlab;
  if (cs >= c1) return;
  const int ncol = (int)(c1 - cs < kSlab ? c1 - cs : kSlab);
  const int64_t mr = d.m - j0, ld = d.m;
  const cxd* V = d.W + j0 + j0 * ld;
  const cxd* Tb = d.T + (j0 / kNb) * kNb * kNb;
  cxd* Xb = (onQ ? d.Q : d.W) + j0 + cs * ld;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  for (int pair = warp; pair < jb * ncol; pair += nwarps) {
    const int a = pair % jb, c = pair / jb;
    cxd w = mkcx(0.0, 0.0);
    const cxd* xc = Xb + (int64_t)c * ld;
    for (int64_t r = a + lane; r < mr; r += 32) cfma_cj(w, vget(V, ld, r, a), xc[r]);
    w.x = warp_sum(w.x);
    w.y = warp_sum(w.y);
    if (lane == 0) sW_[a][c] = w;
  }
  __syncthreads();
  if (tid < jb * ncol) {
    const int a = tid % jb, c = tid / jb;
    cxd y = mkcx(0.0, 0.0);
    if (!onQ) {
      for (int q = 0; q <= a; ++q) cfma_cj(y, Tb[q + a * kNb], sW_[q][c]);  // Tᴴ
    } else {
      for (int q = a; q < jb; ++q) cfma(y, Tb[a + q * kNb], sW_[q][c]);  // T
    }
    sY[a][c] = y;
  }
  __syncthreads();
  for (int64_t t = tid; t < mr * ncol; t += blockDim.x) {
    const int64_t r = t % mr;
    const int c = (int)(t / mr);
    cxd acc = mkcx(0.0, 0.0);
    const int amax = (int)(r < jb - 1 ? r : jb - 1);
    for (int a = 0; a <= amax; ++a) cfma(acc, vget(V, ld, r, a), sY[a][c]);
    Xb[r + (int64_t)c * ld] = Xb[r + (int64_t)c * ld] - acc;
  }
}

// R = upper triangle of W's first n rows; Q = [I_n; 0]
__global__ void k_g_qr_extract(const QrD* __restrict__ D) {
  const QrD d = D[blockIdx.y];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < d.n * d.n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % d.n, c = t / d.n;
    d.R[t] = r <= c ? d.W[r + c * d.m] : mkcx(0.0, 0.0);
  }
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < d.m * d.n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % d.m, c = t / d.m;
    d.Q[t] = mkcx(r == c ? 1.0 : 0.0, 0.0);
  }
}

// ---------------------------------------------------------------------------------
// grouped one-sided Jacobi (FP64): columns of W_b orthogonalised in place
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void rr_pair(int N, int r, int k, int& i, int& j) {
  if (k == 0) {
    i = r % (N - 1);
    j = N - 1;
  } else {
    i = (r + k) % (N - 1);
    j = (r - k + (N - 1)) % (N - 1);
  }
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
}

__global__ void k_g_colnorms(const JacD* __restrict__ D, const int* __restrict__ active) {
  const JacD d = D[blockIdx.y];
  if (!active[blockIdx.y]) return;
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = gw; c < d.n; c += nw) {
    const cxd* w = d.W + c * d.m;
    double s = 0;
    for (int64_t t = lane; t < d.m; t += 32) s += abs2(w[t]);
    s = warp_sum(s);
    if (lane == 0) d.nrm[c] = s;
  }
}

// d.nrm[d.n] = ‖W‖²_F (fixed summation order), for the negligible-column threshold
__global__ void __launch_bounds__(256) k_g_fro(const JacD* __restrict__ D, const int* __restrict__ active) {
  __shared__ double red[8];
  const JacD d = D[blockIdx.x];
  if (!active[blockIdx.x]) return;
  double f = 0.0;
  for (int64_t c = threadIdx.x; c < d.n; c += 256) f += d.nrm[c];
  f = warp_sum(f);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = f;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < 8; ++w) a += red[w];
    d.nrm[d.n] = a;
  }
}

// one round of the circle ordering: CTA (pair, instance), the pair's columns held in
// registers (m ≤ NT·R); rotation formed by one thread (see the uniform-batch kernel)
template <int NT, int R>
__global__ void __launch_bounds__(NT)
    k_g_jacobi_step(const JacD* __restrict__ D, int r, const int* __restrict__ active, int* __restrict__ rotated,
                    int nprob) {
  const int b = blockIdx.y;
  if (!active[b]) return;
  const JacD d = D[b];
  if (r >= d.N - 1 || (int)blockIdx.x >= d.N / 2) return;
  int i, j;
  rr_pair(d.N, r, blockIdx.x, i, j);
  if (j >= d.n) return;
  const double tol = 4.0 * sqrt((double)(d.m > 1 ? d.m : 1)) * 2.220446049250313e-16;
  cxd* wi = d.W + (int64_t)i * d.m;
  cxd* wj = d.W + (int64_t)j * d.m;
  constexpr int NW = NT / 32;
  __shared__ double red[NW][2];
  __shared__ double s_rot[3];
  __shared__ int s_apply;
  cxd x[R], y[R];
  cxd g = mkcx(0.0, 0.0);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int64_t t = threadIdx.x + (int64_t)q * NT;
    if (t < d.m) {
      x[q] = wi[t];
      y[q] = wj[t];
      cfma_cj(g, x[q], y[q]);
    }
  }
  g.x = warp_sum(g.x);
  g.y = warp_sum(g.y);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[warp][0] = g.x;
    red[warp][1] = g.y;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    g = mkcx(0.0, 0.0);
    for (int w = 0; w < NW; ++w) {
      g.x += red[w][0];
      g.y += red[w][1];
    }
    const double al = d.nrm[i], be = d.nrm[j];
    // columns at or below ε²·‖W‖²_F are numerically zero and left alone (the uniform
    // batch kernel's rule: a graded matrix's near-null columns otherwise keep nearly every
    // pair rotating for tens of sweeps); |γ| and √α√β without squaring small numbers
    const double negl = 4.930380657631324e-32 * d.nrm[d.n];
    const double fl = negl > 1e-290 ? negl : 1e-290;
    double ag = 0.0;
    int apply = 0;
    if (al > fl && be > fl) {
      const double ab = al * be;
      if (ab > 1e-290) {
        const double ag2 = abs2(g);
        apply = ag2 > tol * tol * ab && ag2 > 0.0;
        atomicMax(&rotated[nprob + b], __float_as_int(sqrtf((float)(ag2 / ab))));
        ag = sqrt(ag2);
      } else {
        ag = hypot(g.x, g.y);
        const double sab = sqrt(al) * sqrt(be);
        apply = ag > tol * sab && ag > 0.0;
        atomicMax(&rotated[nprob + b], __float_as_int((float)(ag / sab)));
      }
    }
    double c = 1.0, sx = 0.0, sy = 0.0;
    if (apply) {
      const double zeta = (be - al) / (2.0 * ag);
      const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      if (t == 0.0) {
        apply = 0;
      } else {
        c = 1.0 / sqrt(1.0 + t * t);
        const double s = c * t;
        sx = s * (g.x / ag);
        sy = s * (g.y / ag);
        atomicAdd(&rotated[b], 1);
        d.nrm[i] = al - t * ag;
        d.nrm[j] = be + t * ag;
      }
    }
    s_apply = apply;
    s_rot[0] = c;
    s_rot[1] = sx;
    s_rot[2] = sy;
  }
  __syncthreads();
  if (!s_apply) return;
  const double c = s_rot[0];
  const cxd se = mkcx(s_rot[1], s_rot[2]);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int64_t t = threadIdx.x + (int64_t)q * NT;
    if (t < d.m) {
      // wi' = c wi − conj(se) wj ; wj' = se wi + c wj
      const cxd a = c * x[q] - conjg(se) * y[q];
      const cxd bb = se * x[q] + c * y[q];
      wi[t] = a;
      wj[t] = bb;
    }
  }
}

// σ_c = ‖w_c‖ sorted descending (bitonic in shared memory), then U's r leading columns
__global__ void __launch_bounds__(512) k_g_svd_finish(const JacD* __restrict__ D, int P2max) {
  extern __shared__ unsigned char smem_raw[];
  double* key = reinterpret_cast<double*>(smem_raw);
  int* idx = reinterpret_cast<int*>(key + P2max);
  const JacD d = D[blockIdx.x];
  int P2 = 1;
  while (P2 < d.n) P2 <<= 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int c = warp; c < P2; c += nwarps) {
    double s = 0;
    if (c < d.n) {
      const cxd* w = d.W + (int64_t)c * d.m;
      for (int64_t t = lane; t < d.m; t += 32) s += abs2(w[t]);
      s = warp_sum(s);
    }
    if (lane == 0) {
      key[c] = c < d.n ? sqrt(s) : -1.0;
      idx[c] = c;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P2; k <<= 1)
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = threadIdx.x; t < P2; t += blockDim.x) {
        const int u = t ^ jj;
        if (u > t) {
          const bool desc = (t & k) == 0;
          const double a = key[t], b = key[u];
          if (desc ? (a < b) : (a > b)) {
            key[t] = b;
            key[u] = a;
            const int q = idx[t];
            idx[t] = idx[u];
            idx[u] = q;
          }
        }
      }
      __syncthreads();
    }
  for (int c = threadIdx.x; c < d.n; c += blockDim.x) {
    d.S[c] = key[c];
    d.order[c] = idx[c];
  }
  for (int64_t t = threadIdx.x; t < d.m * d.r; t += blockDim.x) {
    const int64_t row = t % d.m, c = t / d.m;
    const double s = key[c];
    const cxd w = d.W[row + (int64_t)idx[c] * d.m];
    d.U[t] = s > 0.0 ? mkcx(w.x / s, w.y / s) : mkcx(0.0, 0.0);
  }
}

// orthonormal completion of the kept U columns whose σ is numerically zero (the columns
// the sweeps left alone), as for the uniform batch
__global__ void __launch_bounds__(256) k_g_complete(const JacD* __restrict__ D) {
  extern __shared__ unsigned char smem_raw[];
  cxd* c = reinterpret_cast<cxd*>(smem_raw);
  __shared__ double red[32];
  __shared__ int64_t first, next_k;
  const JacD d = D[blockIdx.x];
  if (threadIdx.x == 0) first = negligible_start(d.S, d.n, 4.930380657631324e-32, 1e-290);  // ε² of FP64
  __syncthreads();
  if (first >= d.r) return;
  complete_columns<double>(d.m, d.r, first, d.U, c, red, &next_k);
}

// Gaussian fill (counter-based hash → Box–Muller) with per-site variance 1/(d χ_{i-1})
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_g_fill(cxd* x, int64_t n, uint64_t seed, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed ^ mix64(2 * (uint64_t)i));
    const uint64_t h2 = mix64(seed ^ mix64(2 * (uint64_t)i + 1));
    const double u1 = ((h1 >> 11) + 1) * (1.0 / 9007199254740992.0);
    const double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);
    const double rad = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    x[i] = mkcx(rad * cs * scale * 0.70710678118654752, rad * sn * scale * 0.70710678118654752);
  }
}

unsigned blk(int64_t n, int64_t cap = 1024) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, cap)); }

}  // namespace

struct tn_group {
  tn_ctx* ctx = nullptr;
  int B = 0, d = 2;
  std::vector<int> L;
  std::vector<std::vector<int64_t>> bond;   // [b][0..L] current
  std::vector<std::vector<int64_t>> bond0;  // [b][0..L] at creation (the site capacities)
  std::vector<std::vector<int64_t>> cap;   // [b][1..L] elements
  std::vector<std::vector<cxd*>> site;     // [b][1..L]
  std::vector<std::vector<double>> lambda;  // Λ_{L−1} after compress
  void* block = nullptr;
  bool compressed = false;
  int64_t steps_launched = 0;
};

namespace {

// upload a host table into workspace (pageable copy: the host vector may be reused at once)
// the workspace reserved for a step must hold everything taken from it
tn_status_t ws_check(tn_ctx* ctx) {
  if (ctx->ws_top > ctx->ws_cap)
    return tn_set_error(ctx, TN_ECUDA, "group: workspace overrun (%zu > %zu)", ctx->ws_top, ctx->ws_cap);
  return TN_OK;
}

template <typename D>
tn_status_t upload(tn_ctx* ctx, const std::vector<D>& h, D** out) {
  *out = ws_take<D>(ctx, std::max<size_t>(h.size(), 1));
  TN_RETURN_IF(ws_check(ctx));
  if (!h.empty())
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(*out, h.data(), sizeof(D) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
  return TN_OK;
}

tn_status_t g_copy(tn_ctx* ctx, const std::vector<CopyD>& h) {
  if (h.empty()) return TN_OK;
  CopyD* d = nullptr;
  TN_RETURN_IF(upload(ctx, h, &d));
  int64_t mx = 1;
  for (auto& c : h) mx = std::max(mx, c.rows * c.cols);
  k_g_copy<<<dim3(blk(mx, 512), (unsigned)h.size()), 256, 0, ctx->stream>>>(d);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

tn_status_t g_gemm(tn_ctx* ctx, const std::vector<GemmD>& h) {
  if (h.empty()) return TN_OK;
  // 64×64 tiles when the group fills the GPU twice over with them, else 32×32
  int64_t t64 = 0;
  for (auto& g : h) t64 += ((g.m + 63) / 64) * ((g.n + 63) / 64);
  const bool big = t64 >= 2 * (int64_t)ctx->num_sms;
  const int BM = big ? 64 : 32;
  std::vector<int64_t> start(h.size() + 1, 0);
  for (size_t b = 0; b < h.size(); ++b) start[b + 1] = start[b] + ((h[b].m + BM - 1) / BM) * ((h[b].n + BM - 1) / BM);
  GemmD* d = nullptr;
  int64_t* st = nullptr;
  TN_RETURN_IF(upload(ctx, h, &d));
  TN_RETURN_IF(upload(ctx, start, &st));
  const int64_t tiles = start.back();
  if (tiles <= 0) return TN_OK;
  if (tiles > 0x7fffffffll) return tn_set_error(ctx, TN_EUNSUPPORTED, "group gemm: too many tiles");
  if (big)
    k_g_gemm<64, 64, 8, 4, 4><<<(unsigned)tiles, 256, 0, ctx->stream>>>(d, st, (int)h.size());
  else
    k_g_gemm<32, 32, 8, 2, 2><<<(unsigned)tiles, 256, 0, ctx->stream>>>(d, st, (int)h.size());
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// QR of every W (m ≥ n), Q and R written to the descriptor's buffers
tn_status_t g_qr(tn_ctx* ctx, const std::vector<QrD>& h) {
  if (h.empty()) return TN_OK;
  QrD* d = nullptr;
  TN_RETURN_IF(upload(ctx, h, &d));
  int64_t mmax = 1, nmax = 1;
  for (auto& q : h) {
    mmax = std::max(mmax, q.m);
    nmax = std::max(nmax, q.n);
  }
  const size_t smem = sizeof(cxd) * (size_t)mmax * kNb;
  if (smem > 200 * 1024) return tn_set_error(ctx, TN_EUNSUPPORTED, "group qr: %lld rows exceed the panel kernel", (long long)mmax);
  TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_g_qr_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  const unsigned B = (unsigned)h.size();
  for (int64_t j0 = 0; j0 < nmax; j0 += kNb) {
    k_g_qr_panel<<<B, 256, sizeof(cxd) * (size_t)(mmax - j0) * kNb, ctx->stream>>>(d, j0);
    TN_LAUNCHED(ctx);
    if (j0 + kNb < nmax) {
      k_g_qr_apply<<<dim3(cdiv(nmax - j0 - 1, kSlab), B), 256, 0, ctx->stream>>>(d, j0, false);
      TN_LAUNCHED(ctx);
    }
  }
  k_g_qr_extract<<<dim3(blk(mmax * nmax, 256), B), 256, 0, ctx->stream>>>(d);
  TN_LAUNCHED(ctx);
  for (int64_t j0 = ((nmax - 1) / kNb) * kNb; j0 >= 0; j0 -= kNb) {
    k_g_qr_apply<<<dim3(cdiv(nmax - j0, kSlab), B), 256, 0, ctx->stream>>>(d, j0, true);
    TN_LAUNCHED(ctx);
  }
  return TN_OK;
}

// U (r leading columns) and Σ of every W (m ≥ n) by grouped one-sided Jacobi sweeps
tn_status_t g_svd_left(tn_ctx* ctx, std::vector<JacD>& h, int* active, int* rotated) {
  if (h.empty()) return TN_OK;
  const int P = (int)h.size();
  int64_t mmax = 1, Nmax = 2;
  for (auto& j : h) {
    j.N = (int)(j.n + (j.n & 1));
    mmax = std::max(mmax, j.m);
    Nmax = std::max<int64_t>(Nmax, j.N);
  }
  if (mmax > 4096) return tn_set_error(ctx, TN_EUNSUPPORTED, "group svd: more than 4096 rows");
  JacD* d = nullptr;
  TN_RETURN_IF(upload(ctx, h, &d));
  std::vector<int> h_act(P, 1), h_rot(2 * P);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(active, h_act.data(), sizeof(int) * P, cudaMemcpyHostToDevice, ctx->stream));
  const double stop_ratio = sqrt(4.0 * sqrt((double)mmax) * 2.220446049250313e-16 * 1e-2);
  // one sweep (norm refresh + N−1 rounds over every instance) captured as a CUDA graph
  // and replayed until all instances have converged
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t ge = nullptr;
  TN_CHECK_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(rotated, 0, sizeof(int) * 2 * P, ctx->stream);
  k_g_colnorms<<<dim3(blk(32 * 512, 64), P), 256, 0, ctx->stream>>>(d, active);
  k_g_fro<<<(unsigned)P, 256, 0, ctx->stream>>>(d, active);
  const dim3 grid((unsigned)(Nmax / 2), (unsigned)P);
  for (int r = 0; r < Nmax - 1; ++r) {
    if (mmax <= 512)
      k_g_jacobi_step<128, 4><<<grid, 128, 0, ctx->stream>>>(d, r, active, rotated, P);
    else if (mmax <= 1024)
      k_g_jacobi_step<256, 4><<<grid, 256, 0, ctx->stream>>>(d, r, active, rotated, P);
    else if (mmax <= 2048)
      k_g_jacobi_step<256, 8><<<grid, 256, 0, ctx->stream>>>(d, r, active, rotated, P);
    else
      k_g_jacobi_step<256, 16><<<grid, 256, 0, ctx->stream>>>(d, r, active, rotated, P);
  }
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
  if (ce == cudaSuccess) ce = cudaGraphInstantiate(&ge, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return tn_set_error(ctx, TN_ECUDA, "group svd graph: %s", cudaGetErrorString(ce));
  struct GraphGuard {  // destroyed only after its last replay has finished
    cudaGraphExec_t g;
    cudaStream_t s;
    ~GraphGuard() {
      cudaStreamSynchronize(s);
      if (g) cudaGraphExecDestroy(g);
    }
  } guard{ge, ctx->stream};
  int n_active = P;
  for (int sweep = 0; sweep < 40 && n_active > 0; ++sweep) {
    TN_CHECK_CUDA(ctx, cudaGraphLaunch(ge, ctx->stream));
    ctx->launches += Nmax + 1;
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_rot.data(), rotated, sizeof(int) * 2 * P, cudaMemcpyDeviceToHost, ctx->stream));
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    n_active = 0;
    for (int b = 0; b < P; ++b) {
      float ratio;
      memcpy(&ratio, &h_rot[P + b], sizeof(float));
      h_act[b] = h_act[b] && h_rot[b] && ratio > stop_ratio;
      n_active += h_act[b];
    }
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(active, h_act.data(), sizeof(int) * P, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (n_active > 0) return tn_set_error(ctx, TN_ENOCONV, "group svd: no convergence within 40 sweeps");
  int P2 = 1;
  int64_t nmax = 1;
  for (auto& j : h) nmax = std::max(nmax, j.n);
  while (P2 < nmax) P2 <<= 1;
  const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)P2;  // ≤ 48 KB for n ≤ 4096
  k_g_svd_finish<<<(unsigned)P, 512, smem, ctx->stream>>>(d, P2);
  TN_LAUNCHED(ctx);
  const size_t csm = sizeof(cxd) * (size_t)nmax;
  TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_g_complete, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
  k_g_complete<<<(unsigned)P, 256, csm, ctx->stream>>>(d);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }
// descriptor tables of one step: at most 16 tables of ≤ 128 bytes per instance
size_t table_bytes(size_t n) { return 16 * al256(128 * (n + 1)) + 65536; }

}  // namespace

extern "C" {

tn_status_t tn_group_create(tn_ctx* ctx, int32_t B, const int32_t* L, int32_t d, const int64_t* bonds,
                            tn_group** out) {
  if (!ctx || !out || !L || !bonds || B < 1 || d < 1)
    return tn_set_error(ctx, TN_EINVAL, "tn_group_create: bad arguments");
  auto* g = new tn_group();
  g->ctx = ctx;
  g->B = B;
  g->d = d;
  g->L.assign(L, L + B);
  g->bond.resize(B);
  g->cap.resize(B);
  g->site.resize(B);
  g->lambda.resize(B);
  size_t total = 0, off = 0;
  for (int b = 0; b < B; ++b) {
    if (L[b] < 2) {
      delete g;
      return tn_set_error(ctx, TN_EINVAL, "tn_group_create: instance %d has fewer than 2 sites", b);
    }
    g->bond[b].assign(L[b] + 1, 1);
    for (int i = 1; i < L[b]; ++i) {
      const int64_t x = bonds[off + i - 1];
      if (x < 1) {
        delete g;
        return tn_set_error(ctx, TN_EINVAL, "tn_group_create: bond %d of instance %d < 1", i, b);
      }
      g->bond[b][i] = x;
    }
    off += L[b] - 1;
    g->bond0.push_back(g->bond[b]);
    g->cap[b].assign(L[b] + 1, 0);
    for (int i = 1; i <= L[b]; ++i) {
      const int64_t bl = g->bond[b][i - 1], br = g->bond[b][i];
      // a site's bytes, and their running total, must fit in 63 bits
      if (bl > INT64_MAX / (int64_t)sizeof(cxd) / d / br / 2 ||
          total > (size_t)INT64_MAX - al256(sizeof(cxd) * (size_t)(bl * d * br))) {
        delete g;
        return tn_set_error(ctx, TN_EINVAL, "tn_group_create: site %d of instance %d is too large", i, b);
      }
      g->cap[b][i] = bl * d * br;
      total += al256(sizeof(cxd) * (size_t)g->cap[b][i]);
    }
  }
  tn_status_t st = tn_dev_alloc(ctx, total, &g->block);
  if (st != TN_OK) {
    delete g;
    return st;
  }
  char* c = (char*)g->block;
  for (int b = 0; b < B; ++b) {
    g->site[b].assign(L[b] + 1, nullptr);
    for (int i = 1; i <= L[b]; ++i) {
      g->site[b][i] = (cxd*)c;
      c += al256(sizeof(cxd) * (size_t)g->cap[b][i]);
    }
  }
  ctx->refs++;
  *out = g;
  return TN_OK;
}

tn_status_t tn_group_destroy(tn_group* g) {
  if (!g) return TN_OK;
  tn_ctx* ctx = g->ctx;
  cudaStreamSynchronize(ctx->stream);
  tn_dev_free(ctx, g->block);
  delete g;
  ctx->refs--;
  if (ctx->refs == 0 && ctx->destroy_requested) ctx_release(ctx);
  return TN_OK;
}

tn_status_t tn_group_fill_random(tn_group* g, uint64_t seed) {
  if (!g) return TN_EINVAL;
  tn_ctx* ctx = g->ctx;
  g->bond = g->bond0;  // a fresh MPS of the creation shape
  for (auto& l : g->lambda) l.clear();
  for (int b = 0; b < g->B; ++b)
    for (int i = 1; i <= g->L[b]; ++i) {
      const int64_t e = g->bond[b][i - 1] * g->d * g->bond[b][i];
      const double scale = 1.0 / std::sqrt((double)(g->d * g->bond[b][i - 1]));
      const uint64_t s = seed * 0x9E3779B97F4A7C15ull ^ ((uint64_t)b << 32 | (uint64_t)i);
      k_g_fill<<<blk(e, 2048), 256, 0, ctx->stream>>>(g->site[b][i], e, s, scale);
      TN_LAUNCHED(ctx);
    }
  g->compressed = false;
  return TN_OK;
}

tn_status_t tn_group_set_site(tn_group* g, int32_t b, int32_t i, const void* h_data) {
  if (!g || !h_data || b < 0 || b >= g->B || i < 1 || i > g->L[b]) return tn_set_error(g ? g->ctx : nullptr, TN_EINVAL, "tn_group_set_site: bad arguments");
  const int64_t e = g->bond[b][i - 1] * g->d * g->bond[b][i];
  TN_CHECK_CUDA(g->ctx, cudaMemcpyAsync(g->site[b][i], h_data, sizeof(cxd) * e, cudaMemcpyHostToDevice, g->ctx->stream));
  TN_CHECK_CUDA(g->ctx, cudaStreamSynchronize(g->ctx->stream));
  return TN_OK;
}

tn_status_t tn_group_get_site(const tn_group* g, int32_t b, int32_t i, void* h_data) {
  if (!g || !h_data || b < 0 || b >= g->B || i < 1 || i > g->L[b]) return tn_set_error(g ? g->ctx : nullptr, TN_EINVAL, "tn_group_get_site: bad arguments");
  const int64_t e = g->bond[b][i - 1] * g->d * g->bond[b][i];
  TN_CHECK_CUDA(g->ctx, cudaMemcpyAsync(h_data, g->site[b][i], sizeof(cxd) * e, cudaMemcpyDeviceToHost, g->ctx->stream));
  TN_CHECK_CUDA(g->ctx, cudaStreamSynchronize(g->ctx->stream));
  return TN_OK;
}

tn_status_t tn_group_bond_dims(const tn_group* g, int32_t b, int64_t* h_bonds) {
  if (!g || !h_bonds || b < 0 || b >= g->B) return tn_set_error(g ? g->ctx : nullptr, TN_EINVAL, "tn_group_bond_dims: bad arguments");
  for (int i = 1; i < g->L[b]; ++i) h_bonds[i - 1] = g->bond[b][i];
  return TN_OK;
}

tn_status_t tn_group_lambda(const tn_group* g, int32_t b, double* h_lambda, int64_t* len) {
  if (!g || !len || b < 0 || b >= g->B) return tn_set_error(g ? g->ctx : nullptr, TN_EINVAL, "tn_group_lambda: bad arguments");
  if (!g->compressed) return tn_set_error(g->ctx, TN_EINVAL, "tn_group_lambda: the group has not been compressed");
  *len = (int64_t)g->lambda[b].size();
  if (h_lambda) memcpy(h_lambda, g->lambda[b].data(), sizeof(double) * g->lambda[b].size());
  return TN_OK;
}

tn_status_t tn_group_canonize_compress_norm(tn_group* g, const int64_t* maxdim, double* h_norms) {
  if (!g || !maxdim) return tn_set_error(g ? g->ctx : nullptr, TN_EINVAL, "tn_group_canonize_compress_norm: bad arguments");
  tn_ctx* ctx = g->ctx;
  const int B = g->B, d = g->d;
  for (int b = 0; b < B; ++b)
    if (maxdim[b] < 1) return tn_set_error(ctx, TN_EINVAL, "compress: maxdim must be a positive integer (instance %d)", b);
  int Lmax = 0;
  for (int b = 0; b < B; ++b) Lmax = std::max(Lmax, g->L[b]);
  // ---- A: QR sweep left→right ----
  for (int k = 1; k < Lmax; ++k) {
    std::vector<int> ids;
    for (int b = 0; b < B; ++b)
      if (k <= g->L[b] - 1) ids.push_back(b);
    if (ids.empty()) continue;
    size_t need = table_bytes(ids.size());
    for (int b : ids) {
      const int64_t m = g->bond[b][k - 1] * d, n = g->bond[b][k], n2 = d * g->bond[b][k + 1];
      need += al256(sizeof(cxd) * (size_t)(m * n)) * 2 + al256(sizeof(cxd) * (size_t)(n * n)) +
              al256(sizeof(cxd) * (size_t)(n + 1)) + al256(sizeof(cxd) * (size_t)(((n + kNb - 1) / kNb) * kNb * kNb)) +
              al256(sizeof(cxd) * (size_t)(n * n2));
    }
    TN_RETURN_IF(ws_reserve(ctx, need));
    std::vector<QrD> qr;
    std::vector<GemmD> mm;
    std::vector<CopyD> cq, cb;
    for (int b : ids) {
      const int64_t m = g->bond[b][k - 1] * d, n = g->bond[b][k], n2 = d * g->bond[b][k + 1];
      if (m < n) return tn_set_error(ctx, TN_EUNSUPPORTED, "group canonize: site %d of instance %d is wide", k, b);
      QrD q;
      q.m = m;
      q.n = n;
      q.W = ws_take<cxd>(ctx, (size_t)(m * n));
      q.Q = ws_take<cxd>(ctx, (size_t)(m * n));
      q.R = ws_take<cxd>(ctx, (size_t)(n * n));
      q.tau = ws_take<cxd>(ctx, (size_t)(n + 1));
      q.T = ws_take<cxd>(ctx, (size_t)(((n + kNb - 1) / kNb) * kNb * kNb));
      cxd* tmp = ws_take<cxd>(ctx, (size_t)(n * n2));
      qr.push_back(q);
      cq.push_back({g->site[b][k], q.W, m, m, m, n, 0});
      mm.push_back({q.R, g->site[b][k + 1], tmp, n, n2, n, n, n, n, 'N', 'N'});
      cb.push_back({tmp, g->site[b][k + 1], n, n, n, n2, 0});
    }
    TN_RETURN_IF(ws_check(ctx));
    TN_RETURN_IF(g_copy(ctx, cq));
    TN_RETURN_IF(g_qr(ctx, qr));
    std::vector<CopyD> cqo;
    for (size_t t = 0; t < ids.size(); ++t) cqo.push_back({qr[t].Q, g->site[ids[t]][k], qr[t].m, qr[t].m, qr[t].m, qr[t].n, 0});
    TN_RETURN_IF(g_copy(ctx, cqo));
    TN_RETURN_IF(g_gemm(ctx, mm));
    TN_RETURN_IF(g_copy(ctx, cb));
    g->steps_launched++;
  }
  // ---- B: LQ sweep right→left (site i_b = L_b − j) ----
  for (int j = 0; j < Lmax - 1; ++j) {
    std::vector<int> ids;
    for (int b = 0; b < B; ++b)
      if (g->L[b] - j >= 2) ids.push_back(b);
    if (ids.empty()) continue;
    size_t need = table_bytes(ids.size());
    for (int b : ids) {
      const int i = g->L[b] - j;
      const int64_t rows = g->bond[b][i - 1], cols = d * g->bond[b][i], m0 = g->bond[b][i - 2] * d;
      need += al256(sizeof(cxd) * (size_t)(rows * cols)) * 2 + al256(sizeof(cxd) * (size_t)(rows * rows)) +
              al256(sizeof(cxd) * (size_t)(rows + 1)) +
              al256(sizeof(cxd) * (size_t)(((rows + kNb - 1) / kNb) * kNb * kNb)) +
              al256(sizeof(cxd) * (size_t)(m0 * rows));
    }
    TN_RETURN_IF(ws_reserve(ctx, need));
    std::vector<QrD> qr;
    std::vector<CopyD> ct, cback, cprev;
    std::vector<GemmD> mm;
    for (int b : ids) {
      const int i = g->L[b] - j;
      // A_i (χ_{i−1} × d χ_i); its adjoint (d χ_i × χ_{i−1}) is tall
      const int64_t rows = g->bond[b][i - 1], cols = d * g->bond[b][i], m0 = g->bond[b][i - 2] * d;
      if (cols < rows) return tn_set_error(ctx, TN_EUNSUPPORTED, "group canonize: site %d of instance %d is tall", i, b);
      QrD q;
      q.m = cols;
      q.n = rows;
      q.W = ws_take<cxd>(ctx, (size_t)(rows * cols));
      q.Q = ws_take<cxd>(ctx, (size_t)(rows * cols));
      q.R = ws_take<cxd>(ctx, (size_t)(rows * rows));
      q.tau = ws_take<cxd>(ctx, (size_t)(rows + 1));
      q.T = ws_take<cxd>(ctx, (size_t)(((rows + kNb - 1) / kNb) * kNb * kNb));
      cxd* tmp = ws_take<cxd>(ctx, (size_t)(m0 * rows));
      qr.push_back(q);
      ct.push_back({g->site[b][i], q.W, rows, cols, rows, cols, 1});     // W = A_iᴴ
      cback.push_back({q.Q, g->site[b][i], cols, rows, cols, rows, 1});  // A_i = Qᴴ
      // A_{i−1} (m0 × χ_{i−1}) ← A_{i−1} Rᴴ
      mm.push_back({g->site[b][i - 1], q.R, tmp, m0, rows, rows, m0, rows, m0, 'N', 'C'});
      cprev.push_back({tmp, g->site[b][i - 1], m0, m0, m0, rows, 0});
    }
    TN_RETURN_IF(ws_check(ctx));
    TN_RETURN_IF(g_copy(ctx, ct));
    TN_RETURN_IF(g_qr(ctx, qr));
    TN_RETURN_IF(g_copy(ctx, cback));
    TN_RETURN_IF(g_gemm(ctx, mm));
    TN_RETURN_IF(g_copy(ctx, cprev));
    g->steps_launched++;
  }
  // ---- C: SVD sweep left→right with truncation ----
  std::vector<double> norms(B, 0.0);
  for (int k = 1; k < Lmax; ++k) {
    std::vector<int> ids;
    for (int b = 0; b < B; ++b)
      if (k <= g->L[b] - 1) ids.push_back(b);
    if (ids.empty()) continue;
    const int P = (int)ids.size();
    size_t need = table_bytes(ids.size()) + al256(sizeof(int) * (size_t)(3 * P + 4));
    for (int b : ids) {
      const int64_t m = g->bond[b][k - 1] * d, n = g->bond[b][k], n2 = d * g->bond[b][k + 1];
      const int64_t r = std::min<int64_t>(maxdim[b], std::min(m, n));
      need += al256(sizeof(cxd) * (size_t)(m * n)) + al256(sizeof(cxd) * (size_t)(m * r)) +
              al256(sizeof(double) * (size_t)(n + 1)) + al256(sizeof(double) * (size_t)n) + al256(sizeof(int) * (size_t)n) +
              al256(sizeof(cxd) * (size_t)(r * n)) + al256(sizeof(cxd) * (size_t)(r * n2));
    }
    TN_RETURN_IF(ws_reserve(ctx, need));
    int* active = ws_take<int>(ctx, (size_t)P + 1);
    int* rotated = ws_take<int>(ctx, (size_t)(2 * P + 2));
    std::vector<JacD> jd;
    std::vector<CopyD> cw, cu, cn;
    std::vector<GemmD> mz, mn;
    for (int b : ids) {
      const int64_t m = g->bond[b][k - 1] * d, n = g->bond[b][k], n2 = d * g->bond[b][k + 1];
      // thin SVD: min(m, n) values, the first min(maxdim, ·) kept (compress.jl:47-51); a
      // wide M_k (m < n, odd χ with maxdim = χ÷2) is fine for one-sided Jacobi: its n − m
      // surplus columns shrink to zero
      const int64_t r = std::min<int64_t>(maxdim[b], std::min(m, n));
      JacD q;
      q.m = m;
      q.n = n;
      q.r = r;
      q.N = 0;
      q.W = ws_take<cxd>(ctx, (size_t)(m * n));
      q.U = ws_take<cxd>(ctx, (size_t)(m * r));
      q.nrm = ws_take<double>(ctx, (size_t)(n + 1));  // column norms, then ‖W‖²_F
      q.S = ws_take<double>(ctx, (size_t)n);
      q.order = ws_take<int>(ctx, (size_t)n);
      cxd* Z = ws_take<cxd>(ctx, (size_t)(r * n));
      cxd* tmp = ws_take<cxd>(ctx, (size_t)(r * n2));
      jd.push_back(q);
      cw.push_back({g->site[b][k], q.W, m, m, m, n, 0});
      // Z (r × n) = U_rᴴ M_k ; next site (r × n2) = Z · A_{k+1} (n × n2)
      mz.push_back({q.U, g->site[b][k], Z, r, n, m, m, m, r, 'C', 'N'});
      mn.push_back({Z, g->site[b][k + 1], tmp, r, n2, n, r, n, r, 'N', 'N'});
      cu.push_back({q.U, g->site[b][k], m, m, m, r, 0});
      cn.push_back({tmp, g->site[b][k + 1], r, r, r, n2, 0});
    }
    TN_RETURN_IF(ws_check(ctx));
    TN_RETURN_IF(g_copy(ctx, cw));
    TN_RETURN_IF(g_svd_left(ctx, jd, active, rotated));
    TN_RETURN_IF(g_gemm(ctx, mz));  // reads M_k before it is overwritten
    TN_RETURN_IF(g_copy(ctx, cu));
    TN_RETURN_IF(g_gemm(ctx, mn));
    TN_RETURN_IF(g_copy(ctx, cn));
    // bond dimensions; Λ of the last bond
    std::vector<int> last;
    for (size_t t = 0; t < ids.size(); ++t) {
      const int b = ids[t];
      g->bond[b][k] = jd[t].r;
      if (k == g->L[b] - 1) last.push_back((int)t);
    }
    if (!last.empty()) {
      for (int t : last) {
        const int b = ids[t];
        g->lambda[b].resize(jd[t].r);
        TN_CHECK_CUDA(ctx, cudaMemcpyAsync(g->lambda[b].data(), jd[t].S, sizeof(double) * jd[t].r, cudaMemcpyDeviceToHost,
                                           ctx->stream));
      }
      TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      for (int t : last) {
        const int b = ids[t];
        double s2 = 0;
        for (double v : g->lambda[b]) s2 += v * v;
        norms[b] = std::sqrt(s2);
      }
    }
    g->steps_launched++;
  }
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  g->compressed = true;
  if (h_norms) memcpy(h_norms, norms.data(), sizeof(double) * B);
  return TN_OK;
}

}  // extern "C"
