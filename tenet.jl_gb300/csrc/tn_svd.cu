// K4 — batched one-sided (Hestenes) Jacobi SVD, complex FP64 / FP32.
//
// Replaces LAPACK gesdd behind Muscle.tensor_svd_thin (src/Operations/canonize.jl:41,97)
// and the SVD inside Muscle.simple_update (src/Operations/simple_update.jl:53-64).
//
// For A (m×n, m ≥ n) the columns of W = A are rotated pairwise until every pair is
// orthogonal to tol = 4·√m·ε; then σ_j = ‖w_j‖, u_j = w_j/σ_j and V accumulates the
// rotations.  Pairs follow the round-robin (circle) ordering, so one step touches n/2
// disjoint pairs that run in parallel:
//  * k_jacobi_step — one CTA per (pair, matrix): the three inner products ‖w_i‖²,
//    ‖w_j‖², w_iᴴw_j are reduced with warp shuffles and a 4-warp shared-memory combine,
//    then both columns of W and of V are rotated.  Columns stay in HBM/L2; a sweep is
//    n−1 launches.  This is the large-matrix path (TEBD θ at χ=256 is 512×512).
//  * k_jacobi_smem — one CTA per matrix with W and V resident in shared memory and all
//    sweeps inside the kernel (warp per pair, shuffle reductions); the path for the
//    many small bond matrices of batched canonisation.
// Both stop on a sweep without rotations or at the sweep cap (status TN_ENOCONV).
//
// The complex 2×2 rotation: with γ = |γ|e^{iφ}, ζ = (β−α)/(2|γ|),
// t = sgn(ζ)/(|ζ|+√(1+ζ²)), c = 1/√(1+t²), s = c·t:
//   w_i' = c·w_i − s·e^{−iφ}·w_j,   w_j' = s·e^{iφ}·w_i + c·w_j.
#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>

#include "tn_internal.cuh"

namespace {

// one-sided Jacobi converges quadratically at the end but only linearly while a wide,
// smoothly decaying spectrum (e.g. 512 values over 14 decades) is being sorted out: such
// matrices take 40-60 sweeps
constexpr int kMaxSweeps = 80;
constexpr size_t kSmemMax = 200 * 1024;

template <typename T>
__host__ __device__ inline T jacobi_tol(int64_t m) {
  const T eps = sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-7);
  return T(4) * sqrt(T(m > 1 ? m : 1)) * eps;
}

// circle method: players 0..N-1 (N even), round r in 0..N-2, pair k in 0..N/2-1
__device__ __forceinline__ void rr_pair(int N, int r, int k, int& i, int& j) {
  if (k == 0) {
    i = r % (N - 1);
    j = N - 1;
  } else {
    i = (r + k) % (N - 1);
    j = (r - k + (N - 1)) % (N - 1);
  }
  if (i > j) {
    int t = i;
    i = j;
    j = t;
  }
}

// Jacobi rotation of the pair (w_i, w_j) with α = ‖w_i‖², β = ‖w_j‖², γ = w_iᴴw_j:
// ζ = (β − α)/(2|γ|), t = sign(ζ)/(|ζ| + √(1+ζ²)), c = 1/√(1+t²), s = c·t, e^{iφ} = γ/|γ|.
// Square roots and divisions are the correctly rounded ones (an approximate reciprocal
// square root makes every rotation shrink the columns by an ulp, which adds up over
// thousands of rotations).  The apply test compares squares.  A rotation that rounds to
// the identity (t = 0 when ζ² overflows) is not applied, so the sweep can end.
template <typename T>
struct RotC {
  T c, tag;     // tag = t·|γ|: the exact change of the two squared column norms
  cx<T> se;     // s·e^{iφ}
  float ratio;  // |γ| / √(αβ), for the convergence monitor
  int apply;
};

// Squared column norms at or below the floor are numerically zero: the squares of their
// entries would be subnormal, so neither their norms nor their inner products carry any
// precision.  Such columns are left out of the rotations (and of the convergence test);
// the finaliser gives them orthonormal U columns.  Relative to an O(1) matrix this is far
// below the absolute accuracy of a Householder SVD (ε‖A‖).
// unit roundoff of T: columns with ‖w‖ ≤ ε‖A‖_F are numerically zero
template <typename T>
__host__ __device__ constexpr T jacobi_eps() {
  return sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-7);
}

template <typename T>
struct JacobiFloor;
template <>
struct JacobiFloor<double> {
  static constexpr double value = 1e-290;
};
template <>
struct JacobiFloor<float> {
  static constexpr float value = 1e-32f;
};

// negl: squared norm at or below which a column is numerically zero relative to its
// matrix (ε²·‖A‖²_F): one-sided Jacobi orthogonalises such columns only at the pace of
// a graded matrix (tens of sweeps with nearly every pair rotating), while their content
// is below the absolute accuracy of the factorisation anyway
template <typename T>
__device__ __forceinline__ RotC<T> make_rot_c(T alpha, T beta, cx<T> g, T tol, T negl) {
  RotC<T> R;
  R.c = T(1);
  R.tag = T(0);
  R.se = mkcx<T>(0, 0);
  R.apply = 0;
  R.ratio = 0.f;
  const T fl = negl > JacobiFloor<T>::value ? negl : JacobiFloor<T>::value;
  if (!(alpha > fl) || !(beta > fl)) return R;
  T ag;
  const T ab = alpha * beta;
  if (ab > JacobiFloor<T>::value) {
    // the usual scale: squares are exact enough (one square root on the critical path)
    const T ag2 = abs2(g);
    R.ratio = sqrtf((float)(ag2 / ab));
    R.apply = ag2 > tol * tol * ab && ag2 > T(0);
    if (!R.apply) return R;
    ag = sqrt(ag2);
  } else {
    // tiny columns: |γ| and √α·√β without squaring small quantities
    ag = hypot(g.x, g.y);
    const T sab = sqrt(alpha) * sqrt(beta);
    R.ratio = (float)(ag / sab);
    R.apply = ag > tol * sab && ag > T(0);
    if (!R.apply) return R;
  }
  const T zeta = (beta - alpha) / (T(2) * ag);
  const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  if (t == T(0)) {
    R.apply = 0;
    return R;
  }
  const T c = T(1) / sqrt(T(1) + t * t);
  const T s = c * t;
  R.c = c;
  R.tag = t * ag;
  R.se = mkcx<T>(s * (g.x / ag), s * (g.y / ag));
  return R;
}

// The rotation for the latency-bound small-matrix kernels: the same angle as make_rot_c
// from fewer long-latency operations on the one thread that forms it (1/|γ| once, no
// monitor ratio: another thread derives that off the critical path).
template <typename T>
__device__ __forceinline__ RotC<T> make_rot_lean(T alpha, T beta, cx<T> g, T tol, T negl) {
  RotC<T> R;
  R.c = T(1);
  R.tag = T(0);
  R.se = mkcx<T>(0, 0);
  R.apply = 0;
  R.ratio = 0.f;
  const T fl = negl > JacobiFloor<T>::value ? negl : JacobiFloor<T>::value;
  if (!(alpha > fl) || !(beta > fl)) return R;
  T ag;
  const T ab = alpha * beta;
  if (ab > JacobiFloor<T>::value) {
    const T ag2 = abs2(g);
    if (!(ag2 > tol * tol * ab && ag2 > T(0))) return R;
    ag = sqrt(ag2);
  } else {
    ag = hypot(g.x, g.y);
    if (!(ag > tol * (sqrt(alpha) * sqrt(beta)) && ag > T(0))) return R;
  }
  const T inv_ag = T(1) / ag;
  const T zeta = (beta - alpha) * (T(0.5) * inv_ag);
  const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
  if (t == T(0)) return R;
  const T c = T(1) / sqrt(T(1) + t * t);
  const T sn = c * t * inv_ag;
  R.apply = 1;
  R.c = c;
  R.tag = t * ag;
  R.se = mkcx<T>(sn * g.x, sn * g.y);
  return R;
}

// the convergence monitor of a pair, as make_rot_c computes it
template <typename T>
__device__ __forceinline__ float rot_ratio(T alpha, T beta, cx<T> g, T negl) {
  const T fl = negl > JacobiFloor<T>::value ? negl : JacobiFloor<T>::value;
  if (!(alpha > fl) || !(beta > fl)) return 0.f;
  const T ab = alpha * beta;
  if (ab > JacobiFloor<T>::value) return sqrtf((float)(abs2(g) / ab));
  return (float)(hypot(g.x, g.y) / (sqrt(alpha) * sqrt(beta)));
}

template <typename T>
__device__ __forceinline__ void rot_apply_c(T c, cx<T> se, cx<T>& wi, cx<T>& wj) {
  // wi' = c wi − conj(se) wj ; wj' = se wi + c wj
  const cx<T> a = c * wi - conjg(se) * wj;
  const cx<T> b = se * wi + c * wj;
  wi = a;
  wj = b;
}

// Register-resident step: one CTA per (pair, matrix); each thread keeps its R rows of
// both columns in registers from the load through the reduction to the rotation, so W is
// read and written once per step.  EXACT: reduce ‖w_i‖², ‖w_j‖² too (FP32); otherwise
// use the cached norms nrm[], updated analytically (α' = α − t|γ|, β' = β + t|γ|) and
// recomputed exactly at the start of every sweep (FP64).  V may be null (no
// accumulation: the caller recovers Vh from U and A).
// The rotation of columns (i, j) of matrix b by one CTA (shared by the per-round kernel
// and the persistent cooperative one).  nmat: matrices in the batch (‖W_b‖²_F sits at
// nrm[n·nmat + b]); counters: rotations of matrix b at cnt[b], the largest off-diagonal
// ratio (float bits) at ratio[b].
// LAT (cached norms, no truncation flags): the latency-bound form for the dataflow
// kernel — the cached norms and ‖A‖²_F are fetched with the columns, thread 0 forms only
// the rotation (make_rot_lean), and thread 32 updates the norms and counters.
template <typename T, int NT, int R, bool EXACT, bool LAT = false, bool PV = false>
__device__ __forceinline__ void jacobi_pair(int64_t m, int64_t n, int64_t b, int i, int j, cx<T>* W, int64_t sW,
                                            cx<T>* V, int64_t sV, T* nrm, int64_t nmat, int* cnt, int* ratio, T tol,
                                            const unsigned char* __restrict__ tail) {
  static_assert(!(LAT && EXACT), "the latency form uses cached norms");
  static_assert(!LAT || NT > 32, "the latency form needs a second warp");
  // both columns ranked below the kept set: their mutual orthogonality is never used
  if (!LAT && tail && tail[b * n + i] && tail[b * n + j]) return;
  T pre_al = 0, pre_be = 0, pre_f = 0;
  if (LAT && threadIdx.x == 0) {
    pre_al = nrm[b * n + i];
    pre_be = nrm[b * n + j];
    pre_f = nrm[n * nmat + b];
  }
  cx<T>* wi = W + b * sW + (int64_t)i * m;
  cx<T>* wj = W + b * sW + (int64_t)j * m;
  constexpr int NW = NT / 32;
  __shared__ T red[NW][4];
  cx<T> x[R], y[R];
  // PV (V accumulated, few rows per thread): the V columns (n ≤ m ≤ NT·R rows) are loaded
  // together with W's, so their latency overlaps the reduction instead of following the
  // rotation (without V the registers are left to occupancy)
  constexpr bool kPrefetchV = PV && R <= 4;
  constexpr int RV = kPrefetchV ? R : 1;
  cx<T> vx[RV], vy[RV];
  cx<T>* vi = V ? V + b * sV + (int64_t)i * n : nullptr;
  cx<T>* vj = V ? V + b * sV + (int64_t)j * n : nullptr;
  cx<T> g = mkcx<T>(0, 0);
  T al = 0, be = 0;
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int64_t t = threadIdx.x + (int64_t)q * NT;
    if (kPrefetchV && V && t < n) {
      vx[q < RV ? q : 0] = vi[t];
      vy[q < RV ? q : 0] = vj[t];
    }
    if (t < m) {
      x[q] = wi[t];
      y[q] = wj[t];
      cfma_cj(g, x[q], y[q]);
      if (EXACT) {
        al += abs2(x[q]);
        be += abs2(y[q]);
      }
    }
  }
  g.x = warp_sum(g.x);
  g.y = warp_sum(g.y);
  if (EXACT) {
    al = warp_sum(al);
    be = warp_sum(be);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[warp][0] = g.x;
    red[warp][1] = g.y;
    red[warp][2] = al;
    red[warp][3] = be;
  }
  __syncthreads();
  // one thread forms the rotation (FP64 square roots and divisions are scarce on this
  // part) and hands (c, s·e^{iφ}) to the block through shared memory
  __shared__ T s_rot[3];
  __shared__ int s_apply;
  if (LAT) {
    __shared__ T s_mon[6];
    if (threadIdx.x == 0) {
      g = mkcx<T>(0, 0);
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        g.x += red[w][0];
        g.y += red[w][1];
      }
      const T negl = jacobi_eps<T>() * jacobi_eps<T>() * pre_f;
      const RotC<T> Rt = make_rot_lean(pre_al, pre_be, g, tol, negl);
      s_apply = Rt.apply;
      s_rot[0] = Rt.c;
      s_rot[1] = Rt.se.x;
      s_rot[2] = Rt.se.y;
      s_mon[0] = pre_al;
      s_mon[1] = pre_be;
      s_mon[2] = g.x;
      s_mon[3] = g.y;
      s_mon[4] = negl;
      s_mon[5] = Rt.tag;
    }
    __syncthreads();
    const int apply = s_apply;
    if (threadIdx.x == 32) {
      const T al2 = s_mon[0], be2 = s_mon[1];
      if (al2 > T(0) && be2 > T(0))
        atomicMax(&ratio[b], __float_as_int(rot_ratio(al2, be2, mkcx<T>(s_mon[2], s_mon[3]), s_mon[4])));
      if (apply) {
        atomicAdd(&cnt[b], 1);
        nrm[b * n + i] = al2 - s_mon[5];
        nrm[b * n + j] = be2 + s_mon[5];
      }
    }
    if (!apply) return;
  } else if (threadIdx.x == 0) {
    g = mkcx<T>(0, 0);
    al = 0;
    be = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      g.x += red[w][0];
      g.y += red[w][1];
      al += red[w][2];
      be += red[w][3];
    }
    if (!EXACT) {
      al = nrm[b * n + i];
      be = nrm[b * n + j];
    }
    // ‖A‖²_F of this matrix, stored after the n·batch column norms by k_fro
    const T negl = jacobi_eps<T>() * jacobi_eps<T>() * nrm[n * nmat + b];
    RotC<T> Rt = make_rot_c(al, be, g, tol, negl);
    float monitor = Rt.ratio;
    if (tail && (tail[b * n + i] != tail[b * n + j]) && al > T(0) && be > T(0)) {
      // a kept column against a tail column: only the kept column is used, and the
      // rotation changes it by ρ·β_tail/α_kept (relative); below tol the pair is done
      const T ak = tail[b * n + i] ? be : al, at = tail[b * n + i] ? al : be;
      monitor = (float)((T)Rt.ratio * (at / ak));
      if (!(monitor > (float)tol)) Rt.apply = 0;
    }
    if (al > T(0) && be > T(0)) {
      // largest off-diagonal ratio of the sweep (positive floats order like their bits)
      atomicMax(&ratio[b], __float_as_int(monitor));
    }
    s_apply = Rt.apply;
    if (Rt.apply) {
      atomicAdd(&cnt[b], 1);
      nrm[b * n + i] = al - Rt.tag;
      nrm[b * n + j] = be + Rt.tag;
      s_rot[0] = Rt.c;
      s_rot[1] = Rt.se.x;
      s_rot[2] = Rt.se.y;
    }
  }
  if (!LAT) {
    __syncthreads();
    if (!s_apply) return;
  }
  const T c = s_rot[0];
  const cx<T> se = mkcx<T>(s_rot[1], s_rot[2]);
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int64_t t = threadIdx.x + (int64_t)q * NT;
    if (t < m) {
      rot_apply_c(c, se, x[q], y[q]);
      wi[t] = x[q];
      wj[t] = y[q];
    }
  }
  if (V && kPrefetchV) {
#pragma unroll
    for (int q = 0; q < RV; ++q) {
      const int64_t t = threadIdx.x + (int64_t)q * NT;
      if (t < n) {
        rot_apply_c(c, se, vx[q], vy[q]);
        vi[t] = vx[q];
        vj[t] = vy[q];
      }
    }
  } else if (V) {
    for (int64_t t = threadIdx.x; t < n; t += NT) {
      cx<T> a = vi[t], e = vj[t];
      rot_apply_c(c, se, a, e);
      vi[t] = a;
      vj[t] = e;
    }
  }
}

template <typename T, int NT, int R, bool EXACT, bool PV = false>
__global__ void __launch_bounds__(NT)
    k_jacobi_step_reg(int64_t m, int64_t n, int N, int r, cx<T>* W, int64_t sW, cx<T>* V, int64_t sV, T* nrm,
                      const int* active, int* rotated, T tol, const unsigned char* __restrict__ tail) {
  const int64_t b = blockIdx.y;
  if (!active[b]) return;
  int i, j;
  rr_pair(N, r, blockIdx.x, i, j);
  if (j >= n) return;
  jacobi_pair<T, NT, R, EXACT, false, PV>(m, n, b, i, j, W, sW, V, sV, nrm, gridDim.y, rotated, rotated + gridDim.y,
                                          tol, tail);
}

// ---------------------------------------------------------------------------------
// Block round of the FP32 pre-pass (m, n ≤ NT): the n columns form blocks of 8; the blocks
// play a round-robin tournament (NB − 1 outer rounds per sweep, one launch each), and the
// CTA of block pair (P, Q) of matrix b holds the 16 columns of W and V in registers — one
// row per thread — while it visits the 64 cross pairs (P_i, Q_k) in 8 inner rounds of 8
// disjoint pairs; in outer round 0 every block first visits its own 28 pairs (7 inner
// rounds over P and Q together).  Every column pair is visited once per sweep, as in the
// column-pair rounds, but W and V cross L2 once per outer round instead of once per pair
// round (63 instead of 511 passes at n = 512).  Per inner round the 8 pairs' α, β, γ
// (32 values) are reduced by a transposing butterfly (31 shuffles: lane l ends with the
// warp sum of value l), then across warps in shared memory; lanes 4k of warp 0 form the
// rotation of pair k exactly as make_rot_c does (with the truncation-aware tail rule of
// jacobi_pair), and every thread applies the 8 rotations to its row of W and V.
// Counters as k_jacobi_step_reg: rotations at cnt[b], the largest ratio at cnt[nmat + b].
// ---------------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void transpose_stage(float* v, int lane) {
  const bool up = (lane & H) != 0;
#pragma unroll
  for (int k = 0; k < H; ++k) {
    const float send = up ? v[k] : v[k + H];
    const float keep = up ? v[k + H] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, send, H);
  }
}

// Inner-round schedules with fixed register slots (so one round body serves every round
// and the kernel stays small enough for the instruction cache): the data move instead.
// Intra rounds pair slots (s, 7 − s), s < 4, inside each block (polygon method) and then
// rotate slots 0..6 by one, so after r rotations slot s holds original column (s + r) mod 7
// (slot 7 stays); cross rounds pair P slot k with Q slot k and then rotate the Q slots, so
// Q slot k holds original column (k + r) mod 8.  Seven (eight) rotations restore the order.
template <int OFF, int LEN>
__device__ __forceinline__ void rotate_slots(cxf* a) {
  const cxf t = a[OFF];
#pragma unroll
  for (int q = 0; q < LEN - 1; ++q) a[OFF + q] = a[OFF + q + 1];
  a[OFF + LEN - 1] = t;
}
__host__ __device__ constexpr int blk_slot_i(bool intra, int k) { return intra ? (k & 3) + (k >= 4 ? 8 : 0) : k; }
__host__ __device__ constexpr int blk_slot_j(bool intra, int k) { return intra ? 7 - (k & 3) + (k >= 4 ? 8 : 0) : 8 + k; }
// the original column (0..15 within the block pair) in a slot at inner round r
__host__ __device__ constexpr int blk_slot_orig(bool intra, int r, int slot) {
  return intra ? ((slot & 7) < 7 ? ((slot & 7) + r) % 7 : 7) + (slot & 8) : (slot < 8 ? slot : 8 + ((slot - 8) + r) % 8);
}

template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT)
    k_jacobi_block_f32(int64_t m, int64_t n, int NB, int R, cxf* __restrict__ W, cxf* __restrict__ V,
                       const float* __restrict__ nrm, const int* __restrict__ active, int* __restrict__ cnt, float tol,
                       const unsigned char* __restrict__ tail) {
  constexpr int NC = 16, NW = NT / 32;
  const int64_t b = blockIdx.y, nmat = gridDim.y;
  if (!active[b]) return;
  int P, Q;
  rr_pair(NB, R, blockIdx.x, P, Q);
  __shared__ int s_col[NC];
  __shared__ unsigned char s_tail[NC];
  __shared__ float red[2][NW][32];
  __shared__ int s_cnt, s_ratio;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < NC) {
    const int64_t c = t < 8 ? (int64_t)P * 8 + t : (int64_t)Q * 8 + (t - 8);
    s_col[t] = c < n ? (int)c : -1;
    s_tail[t] = (tail && c < n) ? tail[b * n + c] : 0;
  }
  if (t == 0) {
    s_cnt = 0;
    s_ratio = 0;
  }
  __syncthreads();
  cxf* Wb = W + b * m * n;
  cxf* Vb = V + b * n * n;
  cxf w[NC], v[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int col = s_col[c];
    w[c] = (col >= 0 && t < m) ? Wb[(int64_t)col * m + t] : mkcx<float>(0.f, 0.f);
    v[c] = (col >= 0 && t < n) ? Vb[(int64_t)col * n + t] : mkcx<float>(0.f, 0.f);
  }
  const float negl = jacobi_eps<float>() * jacobi_eps<float>() * nrm[n * nmat + b];

  // one inner round over 8 disjoint pairs (column slots i_k, j_k, compile-time after
  // unrolling).  One barrier per round: every warp sums the per-warp partials itself (in
  // the same order, so all warps form bit-identical rotations) from a double-buffered
  // table, and lanes 4k hand pair k's rotation to the other lanes by shuffles.
  int rb = 0;
  auto round = [&](const bool intra, const int r) {
    float val[32];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const cxf x = w[blk_slot_i(intra, k)], y = w[blk_slot_j(intra, k)];
      val[4 * k + 0] = x.x * x.x + x.y * x.y;
      val[4 * k + 1] = y.x * y.x + y.y * y.y;
      val[4 * k + 2] = x.x * y.x + x.y * y.y;
      val[4 * k + 3] = x.x * y.y - x.y * y.x;
    }
    transpose_stage<16>(val, lane);
    transpose_stage<8>(val, lane);
    transpose_stage<4>(val, lane);
    transpose_stage<2>(val, lane);
    transpose_stage<1>(val, lane);
    red[rb][warp][lane] = val[0];
    __syncthreads();
    float tot = 0.f;
#pragma unroll
    for (int q = 0; q < NW; ++q) tot += red[rb][q][lane];
    rb ^= 1;
    const int base = lane & ~3;
    const float al = __shfl_sync(0xffffffffu, tot, base);
    const float be = __shfl_sync(0xffffffffu, tot, base + 1);
    const cxf g = mkcx<float>(__shfl_sync(0xffffffffu, tot, base + 2), __shfl_sync(0xffffffffu, tot, base + 3));
    float rc = 1.f, rsx = 0.f, rsy = 0.f;
    int app = 0;
    if ((lane & 3) == 0) {
      const int k = lane >> 2;  // lane-dependent: the original columns at run time
      const int i = blk_slot_orig(intra, r, blk_slot_i(intra, k)), j = blk_slot_orig(intra, r, blk_slot_j(intra, k));
      if (s_col[i] >= 0 && s_col[j] >= 0 && !(s_tail[i] && s_tail[j])) {
        RotC<float> Rt = make_rot_c(al, be, g, tol, negl);
        float monitor = Rt.ratio;
        if (s_tail[i] != s_tail[j] && al > 0.f && be > 0.f) {
          const float ak = s_tail[i] ? be : al, at = s_tail[i] ? al : be;
          monitor = Rt.ratio * (at / ak);
          if (!(monitor > tol)) Rt.apply = 0;
        }
        app = Rt.apply;
        rc = Rt.c;
        rsx = Rt.se.x;
        rsy = Rt.se.y;
        if (warp == 0) {
          if (al > 0.f && be > 0.f) atomicMax(&s_ratio, __float_as_int(monitor));
          if (app) atomicAdd(&s_cnt, 1);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (__shfl_sync(0xffffffffu, app, 4 * k)) {
        const float c = __shfl_sync(0xffffffffu, rc, 4 * k);
        const cxf se = mkcx<float>(__shfl_sync(0xffffffffu, rsx, 4 * k), __shfl_sync(0xffffffffu, rsy, 4 * k));
        rot_apply_c(c, se, w[blk_slot_i(intra, k)], w[blk_slot_j(intra, k)]);
        rot_apply_c(c, se, v[blk_slot_i(intra, k)], v[blk_slot_j(intra, k)]);
      }
    }
  };
  if (R == 0) {
#pragma unroll 1
    for (int r = 0; r < 7; ++r) {
      round(true, r);
      rotate_slots<0, 7>(w);
      rotate_slots<8, 7>(w);
      rotate_slots<0, 7>(v);
      rotate_slots<8, 7>(v);
    }
  }
#pragma unroll 1
  for (int r = 0; r < 8; ++r) {
    round(false, r);
    rotate_slots<8, 8>(w);
    rotate_slots<8, 8>(v);
  }
  __syncthreads();  // warp 0's counter updates are complete before thread 0 reads them
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int col = s_col[c];
    if (col >= 0 && t < m) Wb[(int64_t)col * m + t] = w[c];
    if (col >= 0 && t < n) Vb[(int64_t)col * n + t] = v[c];
  }
  if (t == 0) {
    if (s_cnt) atomicAdd(&cnt[b], s_cnt);
    if (s_ratio) atomicMax(&cnt[nmat + b], s_ratio);
  }
}

// Persistent one-sided Jacobi for small matrices, where a round is far too little work to
// hide a launch: one cooperative launch runs every sweep of every matrix.  Rounds are
// separated by grid-wide barriers (all CTAs co-resident by construction of the cooperative
// launch); the exact column norms, ‖W‖²_F and the convergence test of each sweep are done
// on the device, so there is no host round trip until the end.  Every loop is bounded by
// max_sweeps.  ctl (ints, zeroed by the caller): [0, 2B) and [2B, 4B) the rotation
// counters / largest ratios of even and odd sweeps; [4B] any matrix still active; [4B+1]
// sweeps run; [4B+2 …] worst ratio (float bits) and its rotation count per sweep (≤ 64).
constexpr int kCoopDiag = 64;
template <typename T, int NT, int R>
__global__ void __launch_bounds__(NT)
    k_jacobi_coop(int64_t m, int64_t n, int N, cx<T>* W, cx<T>* V, T* nrm, int* active, int* ctl, int64_t batch, T tol,
                  int max_sweeps, float stop_ratio) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ T red[NT / 32];
  const int64_t G = gridDim.x, g = blockIdx.x;
  const int64_t pairs = N / 2, items = pairs * batch;
  const int64_t sW = m * n, sV = n * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* any = ctl + 4 * batch;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    int* cnt = ctl + (sweep & 1) * 2 * batch;
    int* rat = cnt + batch;
    // exact column norms, one warp per column (as k_col_norms)
    for (int64_t col = g * (NT / 32) + warp; col < n * batch; col += G * (NT / 32)) {
      const int64_t b = col / n, c = col % n;
      if (!active[b]) continue;
      const cx<T>* w = W + b * sW + c * m;
      T sq = 0;
      for (int64_t t = lane; t < m; t += 32) sq += abs2(w[t]);
      sq = warp_sum(sq);
      if (lane == 0) nrm[col] = sq;
    }
    grid.sync();
    // ‖W_b‖²_F, one CTA per matrix
    for (int64_t b = g; b < batch; b += G) {
      if (!active[b]) continue;
      T f = 0;
      for (int64_t c = threadIdx.x; c < n; c += NT) f += nrm[b * n + c];
      f = warp_sum(f);
      if (lane == 0) red[warp] = f;
      __syncthreads();
      if (threadIdx.x == 0) {
        T a = 0;
        for (int w = 0; w < NT / 32; ++w) a += red[w];
        nrm[n * batch + b] = a;
      }
      __syncthreads();
    }
    grid.sync();
    for (int r = 0; r < N - 1; ++r) {
      for (int64_t it = g; it < items; it += G) {
        const int64_t b = it / pairs;
        if (!active[b]) continue;
        int i, j;
        rr_pair(N, r, (int)(it % pairs), i, j);
        if (j >= n) continue;
        jacobi_pair<T, NT, R, false>(m, n, b, i, j, W, sW, V, sV, nrm, batch, cnt, rat, tol, nullptr);
        __syncthreads();
      }
      // the other parity's counters were last read before this sweep began
      if (r == 0 && g == 0)
        for (int64_t t = threadIdx.x; t < 2 * batch; t += NT) ctl[((sweep + 1) & 1) * 2 * batch + t] = 0;
      grid.sync();
    }
    if (g == 0 && threadIdx.x == 0) {
      int n_act = 0, worst_rot = 0;
      float worst = 0.f;
      for (int64_t b = 0; b < batch; ++b) {
        if (!active[b]) continue;
        const float rt = __int_as_float(rat[b]);
        if (rt > worst) {
          worst = rt;
          worst_rot = cnt[b];
        }
        const int a = cnt[b] > 0 && rt > stop_ratio;
        active[b] = a;
        n_act += a;
      }
      *any = n_act;
      ctl[4 * batch + 1] = sweep + 1;
      if (sweep < kCoopDiag) {
        ctl[4 * batch + 2 + sweep] = __float_as_int(worst);
        ctl[4 * batch + 2 + kCoopDiag + sweep] = worst_rot;
      }
    }
    grid.sync();
    if (*any == 0) break;
  }
}

// The same iteration with the per-round grid barrier replaced by dataflow: in the circle
// ordering a column held by slot k in round r was held in round r−1 by the slot
// rr_holder(N, r−1, column), so a CTA (one per pair slot and matrix) waits only for the
// two CTAs that last wrote its columns.  Each CTA publishes the round it finished
// (release at GPU scope after its writes) and polls its two predecessors (acquire);
// grid barriers remain only at sweep boundaries (norm refresh, stop test).  A poll that
// exceeds kFlowSpinLimit iterations sets the error word and moves on, so every CTA still
// reaches every barrier and the launch ends; the host reports the error.
constexpr long long kFlowSpinLimit = 1ll << 24;

__device__ __forceinline__ int rr_holder(int N, int r, int c) {
  if (c == N - 1 || c == r % (N - 1)) return 0;
  const int a = ((c - r) % (N - 1) + (N - 1)) % (N - 1);
  if (a >= 1 && a <= N / 2 - 1) return a;
  return ((r - c) % (N - 1) + (N - 1)) % (N - 1);
}

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T, int NT, int R>
__global__ void __launch_bounds__(NT)
    k_jacobi_flow(int64_t m, int64_t n, int N, cx<T>* W, cx<T>* V, T* nrm, int* active, int* ctl, int* done,
                  int64_t batch, T tol, int max_sweeps, float stop_ratio) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ T red[NT / 32];
  const int64_t G = gridDim.x, g = blockIdx.x;
  const int64_t pairs = N / 2;
  const int64_t b = g / pairs;
  const int k = (int)(g % pairs);
  const int64_t sW = m * n, sV = n * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* any = ctl + 4 * batch;
  int* err = ctl + 4 * batch + 2 + 2 * kCoopDiag;
  int* done_b = done + b * pairs;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    int* cnt = ctl + (sweep & 1) * 2 * batch;
    int* rat = cnt + batch;
    for (int64_t col = g * (NT / 32) + warp; col < n * batch; col += G * (NT / 32)) {
      const int64_t bb = col / n, c = col % n;
      if (!active[bb]) continue;
      const cx<T>* w = W + bb * sW + c * m;
      T sq = 0;
      for (int64_t t = lane; t < m; t += 32) sq += abs2(w[t]);
      sq = warp_sum(sq);
      if (lane == 0) nrm[col] = sq;
    }
    grid.sync();
    for (int64_t bb = g; bb < batch; bb += G) {
      if (!active[bb]) continue;
      T f = 0;
      for (int64_t c = threadIdx.x; c < n; c += NT) f += nrm[bb * n + c];
      f = warp_sum(f);
      if (lane == 0) red[warp] = f;
      __syncthreads();
      if (threadIdx.x == 0) {
        T a = 0;
        for (int w = 0; w < NT / 32; ++w) a += red[w];
        nrm[n * batch + bb] = a;
      }
      __syncthreads();
    }
    grid.sync();
    if (g == 0)  // the other parity's counters were last read before this sweep began
      for (int64_t t = threadIdx.x; t < 2 * batch; t += NT) ctl[((sweep + 1) & 1) * 2 * batch + t] = 0;
    if (active[b]) {
      for (int r = 0; r < N - 1; ++r) {
        int i, j;
        rr_pair(N, r, k, i, j);
        if (r > 0) {
          if (threadIdx.x == 0) {
            const int want = sweep * N + r;  // published by a holder when it finished round r−1
            const int h1 = rr_holder(N, r - 1, i), h2 = rr_holder(N, r - 1, j);
            long long spins = 0;
            while (ld_acquire_gpu(&done_b[h1]) < want || ld_acquire_gpu(&done_b[h2]) < want) {
              if (++spins > kFlowSpinLimit) {
                atomicExch(err, 1);
                break;
              }
            }
            __threadfence();
          }
          __syncthreads();
        }
        if (j < n) jacobi_pair<T, NT, R, false, true>(m, n, b, i, j, W, sW, V, sV, nrm, batch, cnt, rat, tol, nullptr);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) st_release_gpu(&done_b[k], sweep * N + r + 1);
      }
    }
    grid.sync();
    if (g == 0 && threadIdx.x == 0) {
      int n_act = 0, worst_rot = 0;
      float worst = 0.f;
      const int failed = *err;
      for (int64_t bb = 0; bb < batch; ++bb) {
        if (!active[bb]) continue;
        const float rt = __int_as_float(rat[bb]);
        if (rt > worst) {
          worst = rt;
          worst_rot = cnt[bb];
        }
        const int a = !failed && cnt[bb] > 0 && rt > stop_ratio;
        active[bb] = a;
        n_act += a;
      }
      *any = n_act;
      ctl[4 * batch + 1] = sweep + 1;
      if (sweep < kCoopDiag) {
        ctl[4 * batch + 2 + sweep] = __float_as_int(worst);
        ctl[4 * batch + 2 + kCoopDiag + sweep] = worst_rot;
      }
    }
    grid.sync();
    if (*any == 0) break;
  }
}

// nrm[b][c] = ‖w_c‖² (one warp per column)
template <typename T>
__global__ void k_col_norms(int64_t m, int64_t n, const cx<T>* W, int64_t sW, T* nrm, int64_t batch) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t col = gw; col < n * batch; col += nw) {
    const int64_t b = col / n, c = col % n;
    const cx<T>* w = W + b * sW + c * m;
    T s = 0;
    for (int64_t t = lane; t < m; t += 32) s += abs2(w[t]);
    s = warp_sum(s);
    if (lane == 0) nrm[col] = s;
  }
}

// nrm[n·batch + b] = Σ_c nrm[b][c] = ‖W_b‖²_F (fixed summation order: deterministic)
template <typename T>
__global__ void __launch_bounds__(256) k_fro(int64_t n, T* nrm, int64_t batch) {
  __shared__ T red[8];
  for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
    T f = 0;
    for (int64_t c = threadIdx.x; c < n; c += 256) f += nrm[b * n + c];
    f = warp_sum(f);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = f;
    __syncthreads();
    if (threadIdx.x == 0) {
      T a = 0;
      for (int w = 0; w < 8; ++w) a += red[w];
      nrm[n * batch + b] = a;
    }
    __syncthreads();
  }
}

// whole SVD of one matrix per CTA in shared memory (W m×n and V n×n resident)
template <typename T>
__global__ void __launch_bounds__(512)
    k_jacobi_smem(int64_t m, int64_t n, cx<T>* W, int64_t sW, cx<T>* V, int64_t sV, int* status, T tol,
                  int max_sweeps, bool v_given) {
  extern __shared__ unsigned char smem_raw[];
  cx<T>* sw = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* sv = sw + m * n;
  __shared__ int s_rot;
  const int64_t b = blockIdx.x;
  cx<T>* Wb = W + b * sW;
  cx<T>* Vb = V + b * sV;
  for (int64_t t = threadIdx.x; t < m * n; t += blockDim.x) sw[t] = Wb[t];
  for (int64_t t = threadIdx.x; t < n * n; t += blockDim.x) {
    int64_t r = t % n, c = t / n;
    sv[t] = v_given ? Vb[t] : mkcx<T>(r == c ? T(1) : T(0), 0);
  }
  __syncthreads();
  const int N = (int)(n + (n & 1));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  // ‖A‖²_F (invariant under the rotations) for the negligible-column threshold
  __shared__ T s_fro[16];
  {
    T f = 0;
    for (int64_t t = threadIdx.x; t < m * n; t += blockDim.x) f += abs2(sw[t]);
    f = warp_sum(f);
    if (lane == 0) s_fro[warp] = f;
    __syncthreads();
    if (threadIdx.x == 0) {
      T a = 0;
      for (int w = 0; w < nwarps; ++w) a += s_fro[w];
      s_fro[0] = a;
    }
    __syncthreads();
  }
  const T negl = jacobi_eps<T>() * jacobi_eps<T>() * s_fro[0];
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    for (int r = 0; r < N - 1; ++r) {
      for (int k = warp; k < N / 2; k += nwarps) {
        int i, j;
        rr_pair(N, r, k, i, j);
        if (j >= n) continue;
        cx<T>* wi = sw + (int64_t)i * m;
        cx<T>* wj = sw + (int64_t)j * m;
        T al = 0, be = 0;
        cx<T> g = mkcx<T>(0, 0);
        for (int64_t t = lane; t < m; t += 32) {
          cx<T> x = wi[t], y = wj[t];
          al += abs2(x);
          be += abs2(y);
          cfma_cj(g, x, y);
        }
        al = warp_sum(al);
        be = warp_sum(be);
        g.x = warp_sum(g.x);
        g.y = warp_sum(g.y);
        const RotC<T> R = make_rot_c(al, be, g, tol, negl);
        if (!R.apply) continue;
        if (lane == 0) s_rot = 1;
        for (int64_t t = lane; t < m; t += 32) {
          cx<T> x = wi[t], y = wj[t];
          rot_apply_c(R.c, R.se, x, y);
          wi[t] = x;
          wj[t] = y;
        }
        cx<T>* vi = sv + (int64_t)i * n;
        cx<T>* vj = sv + (int64_t)j * n;
        for (int64_t t = lane; t < n; t += 32) {
          cx<T> x = vi[t], y = vj[t];
          rot_apply_c(R.c, R.se, x, y);
          vi[t] = x;
          vj[t] = y;
        }
      }
      __syncthreads();
    }
    int any = s_rot;
    __syncthreads();
    if (!any) break;
  }
  for (int64_t t = threadIdx.x; t < m * n; t += blockDim.x) Wb[t] = sw[t];
  for (int64_t t = threadIdx.x; t < n * n; t += blockDim.x) Vb[t] = sv[t];
  if (threadIdx.x == 0) status[b] = sweep >= max_sweeps ? 1 : 0;
}

template <typename T>
__global__ void k_identity(int64_t n, cx<T>* V, int64_t sV, int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % n, c = t / n;
      V[b * sV + t] = mkcx<T>(r == c ? T(1) : T(0), 0);
    }
}

template <typename T>
__global__ void k_copy_mat(int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* W, int64_t sW,
                           int64_t batch) {
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
      int64_t r = t % m, c = t / m;
      W[b * sW + t] = A[b * sA + r + c * lda];
    }
}

// σ_j = ‖w_j‖ (FP64), then a descending order by a per-matrix bitonic sort in shared
// memory; order[b][j] = source column of the j-th largest σ.
template <typename T>
__global__ void __launch_bounds__(512)
    k_svd_order(int64_t m, int64_t n, const cx<T>* W, int64_t sW, double* S, int64_t sS, int* order) {
  extern __shared__ unsigned char smem_raw[];
  const int64_t b = blockIdx.x;
  int P2 = 1;
  while (P2 < n) P2 <<= 1;
  double* key = reinterpret_cast<double*>(smem_raw);
  int* idx = reinterpret_cast<int*>(key + P2);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t c = warp; c < P2; c += nwarps) {
    double s2 = 0;
    if (c < n) {
      const cx<T>* w = W + b * sW + c * m;
      for (int64_t t = lane; t < m; t += 32) s2 += (double)abs2(w[t]);
      s2 = warp_sum(s2);
    }
    if (lane == 0) {
      key[c] = c < n ? sqrt(s2) : -1.0;
      idx[c] = (int)c;
    }
  }
  __syncthreads();
  // bitonic sort, descending by key, ties by index ascending
  for (int size = 2; size <= P2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < P2; t += blockDim.x) {
        int p = t ^ stride;
        if (p > t) {
          bool desc = (t & size) == 0;
          double kt = key[t], kp = key[p];
          int it = idx[t], ip = idx[p];
          bool t_first = kt > kp || (kt == kp && it < ip);
          if (desc != t_first) {
            key[t] = kp;
            key[p] = kt;
            idx[t] = ip;
            idx[p] = it;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    S[b * sS + t] = key[t];
    order[b * n + t] = idx[t];
  }
}

// U(:, j) = W(:, order_j) / σ_j ; Vout(:, j) = V(:, order_j)  (as Vh = Vᴴ when vh)
template <typename T>
__global__ void k_svd_gather(int64_t m, int64_t n, const cx<T>* W, int64_t sW, const cx<T>* V, int64_t sV,
                             const double* S, int64_t sS, const int* order, cx<T>* U, int64_t sU, cx<T>* Vo,
                             int64_t sVo, bool vh, int64_t batch) {
  const int64_t b = blockIdx.y;
  if (b >= batch) return;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t % m, c = t / m;
    int src = order[b * n + c];
    double s = S[b * sS + c];
    T inv = s > 0 ? T(1.0 / s) : T(0);
    U[b * sU + t] = inv * W[b * sW + r + (int64_t)src * m];
  }
  if (!V || !Vo) return;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t % n, c = t / n;
    int src = order[b * n + c];
    cx<T> v = V[b * sV + r + (int64_t)src * n];
    if (vh)
      Vo[b * sVo + c + r * n] = conjg(v);  // Vh(c, r) = conj(V(r, c))
    else
      Vo[b * sVo + t] = v;
  }
}

// U columns of numerically zero σ (the columns the sweeps left alone, exact zeros of a
// rank-deficient matrix) get an orthonormal completion, as a Householder SVD's U has; one
// block per matrix, nothing to do (one pass over S) in the usual full-rank case
template <typename T>
__global__ void __launch_bounds__(256) k_svd_complete(int64_t m, int64_t n, cx<T>* U, int64_t sU, const double* S,
                                                      int64_t sS, double negl_rel, double floor_abs) {
  extern __shared__ unsigned char smem_raw[];
  cx<T>* c = reinterpret_cast<cx<T>*>(smem_raw);
  __shared__ double red[32];
  __shared__ int64_t first, next_k;
  const int64_t b = blockIdx.x;
  if (threadIdx.x == 0) first = negligible_start(S + b * sS, n, negl_rel, floor_abs);
  __syncthreads();
  if (first >= n) return;
  complete_columns<T>(m, n, first, U + b * sU, c, red, &next_k);
}

}  // namespace

template <typename T>
size_t svd_workspace(int64_t m, int64_t n, int64_t batch) {
  return ws_round(sizeof(cx<T>) * (size_t)(m * n * batch)) + ws_round(sizeof(cx<T>) * (size_t)(n * n * batch)) +
         ws_round(sizeof(int) * (size_t)(n * batch)) + ws_round(sizeof(int) * (size_t)(batch + 1)) +
         ws_round(sizeof(int) * (size_t)(2 * batch + 2)) + ws_round(sizeof(T) * (size_t)((n + 1) * batch));
}
template size_t svd_workspace<double>(int64_t, int64_t, int64_t);
template size_t svd_workspace<float>(int64_t, int64_t, int64_t);

// one round-robin step of the register kernel, instantiated by row count
// flags[b][j] = 1 for the columns of matrix b outside its `keep` largest norms (ties
// kept): one CTA per matrix, bitonic sort of a copy of the norms in shared memory.
template <typename T>
__global__ void __launch_bounds__(512) k_tail_flags(int64_t n, const T* __restrict__ nrm, int64_t keep,
                                                    unsigned char* __restrict__ flags) {
  extern __shared__ unsigned char smem_raw[];
  T* v = reinterpret_cast<T*>(smem_raw);
  const int64_t b = blockIdx.x;
  int64_t P2 = 1;
  while (P2 < n) P2 <<= 1;
  for (int64_t t = threadIdx.x; t < P2; t += blockDim.x) v[t] = t < n ? nrm[b * n + t] : T(-1);
  __syncthreads();
  for (int64_t k = 2; k <= P2; k <<= 1)
    for (int64_t jj = k >> 1; jj > 0; jj >>= 1) {
      for (int64_t t = threadIdx.x; t < P2; t += blockDim.x) {
        const int64_t u = t ^ jj;
        if (u > t) {
          const bool desc = (t & k) == 0;
          const T x = v[t], y = v[u];
          if (desc ? (x < y) : (x > y)) {
            v[t] = y;
            v[u] = x;
          }
        }
      }
      __syncthreads();
    }
  const T thr = v[keep - 1];
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) flags[b * n + t] = nrm[b * n + t] < thr ? 1 : 0;
}

template <typename T>
static tn_status_t update_tail_flags(tn_ctx* ctx, int64_t n, int64_t batch, const T* nrm, int64_t keep,
                                     unsigned char* flags) {
  int64_t P2 = 1;
  while (P2 < n) P2 <<= 1;
  k_tail_flags<T><<<(unsigned)batch, 512, sizeof(T) * (size_t)P2, ctx->stream>>>(n, nrm, keep, flags);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

template <typename T>
static tn_status_t launch_step(tn_ctx* ctx, int64_t m, int64_t n, int N, int r, cx<T>* W, cx<T>* V, T* nrm,
                               const int* active, int* rotated, T tol, unsigned gy,
                               const unsigned char* tail) {
  constexpr bool EX = sizeof(T) == 4;
  const dim3 grid(N / 2, gy);
  const int64_t sW = m * n, sV = n * n;
  if (m <= 512 && V)
    k_jacobi_step_reg<T, 128, 4, EX, true><<<grid, 128, 0, ctx->stream>>>(m, n, N, r, W, sW, V, sV, nrm, active, rotated,
                                                                         tol, tail);
  else if (m <= 512)
    k_jacobi_step_reg<T, 128, 4, EX><<<grid, 128, 0, ctx->stream>>>(m, n, N, r, W, sW, V, sV, nrm, active, rotated, tol, tail);
  else if (m <= 1024 && V)
    k_jacobi_step_reg<T, 256, 4, EX, true><<<grid, 256, 0, ctx->stream>>>(m, n, N, r, W, sW, V, sV, nrm, active, rotated,
                                                                         tol, tail);
  else if (m <= 1024)
    k_jacobi_step_reg<T, 256, 4, EX><<<grid, 256, 0, ctx->stream>>>(m, n, N, r, W, sW, V, sV, nrm, active, rotated, tol, tail);
  else if (m <= 2048)
    k_jacobi_step_reg<T, 256, 8, EX><<<grid, 256, 0, ctx->stream>>>(m, n, N, r, W, sW, V, sV, nrm, active, rotated, tol, tail);
  else if (m <= 4096)
    k_jacobi_step_reg<T, 256, 16, EX><<<grid, 256, 0, ctx->stream>>>(m, n, N, r, W, sW, V, sV, nrm, active, rotated, tol, tail);
  else
    return tn_set_error(ctx, TN_EUNSUPPORTED, "svd: more than 4096 rows");
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// matrices with at most this many columns take the persistent cooperative path
constexpr int64_t kCoopMaxN = 256;

// the whole Jacobi iteration of a small FP64 batch in one cooperative launch
template <typename T>
static tn_status_t jacobi_coop(tn_ctx* ctx, int64_t m, int64_t n, cx<T>* W, cx<T>* V, int64_t batch, int* active,
                               T* nrm, int max_sweeps, int* sweeps_out, bool* noconv_out) {
  constexpr int NT = 128, R = 4;  // m ≤ 512
  const int N = (int)(n + (n & 1));
  const int64_t items = (int64_t)(N / 2) * batch;
  int per_sm = 0;
  TN_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi_coop<T, NT, R>, NT, 0));
  int per_sm_flow = 0;
  TN_CHECK_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_flow, k_jacobi_flow<T, NT, R>, NT, 0));
  // dataflow rounds need one resident CTA per pair slot and matrix
  const bool flow = items <= (int64_t)std::max(per_sm_flow, 0) * ctx->num_sms;
  const int64_t G = flow ? items : std::min<int64_t>(items, (int64_t)std::max(per_sm, 1) * ctx->num_sms);
  const size_t nhdr = (size_t)(4 * batch + 2 + 2 * kCoopDiag + 1);
  const size_t nctl = nhdr + (flow ? (size_t)items : 0);
  int* ctl = nullptr;
  TN_RETURN_IF(ctx_flags(ctx, nctl, &ctl));
  TN_CHECK_CUDA(ctx, cudaMemsetAsync(ctl, 0, sizeof(int) * nctl, ctx->stream));
  std::vector<int> h_act(batch, 1);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(active, h_act.data(), sizeof(int) * batch, cudaMemcpyHostToDevice, ctx->stream));
  const T tol = jacobi_tol<T>(m);
  const float stop_ratio = (float)sqrt((double)tol * 1e-1);
  int64_t bt = batch;
  if (flow) {
    int* done = ctl + nhdr;
    void* args[] = {&m, &n, (void*)&N, &W, &V, &nrm, &active, &ctl, &done, &bt, (void*)&tol, &max_sweeps,
                    (void*)&stop_ratio};
    TN_CHECK_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_jacobi_flow<T, NT, R>, dim3((unsigned)G), dim3(NT),
                                                   args, 0, ctx->stream));
  } else {
    void* args[] = {&m, &n, (void*)&N, &W, &V, &nrm, &active, &ctl, &bt, (void*)&tol, &max_sweeps, (void*)&stop_ratio};
    TN_CHECK_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_jacobi_coop<T, NT, R>, dim3((unsigned)G), dim3(NT),
                                                   args, 0, ctx->stream));
  }
  TN_LAUNCHED(ctx);
  std::vector<int> h(nctl);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h.data(), ctl, sizeof(int) * nctl, cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int sweeps = h[4 * batch + 1];
  for (int k = 0; k < kCoopDiag && k < 64; ++k) {
    memcpy(&ctx->sweep_ratio[k], &h[4 * batch + 2 + k], sizeof(float));
    ctx->sweep_rotations[k] = h[4 * batch + 2 + kCoopDiag + k];
  }
  *sweeps_out = sweeps;
  *noconv_out = h[4 * batch] > 0;
  if (h[4 * batch + 2 + 2 * kCoopDiag])
    return tn_set_error(ctx, TN_ECUDA, "svd: a dataflow wait of the Jacobi rounds exceeded its limit");
  return TN_OK;
}

// sweeps of one phase after which the truncation-aware flags are dropped
constexpr int kTailSweeps = 8;

// Jacobi sweeps on W (m×n dense, batch stride m·n) accumulating into V (n×n dense; may
// be null on the large-matrix path).  V is set to the identity first unless v_given.
// nrm: n·batch reals of workspace.  The n−1 steps of a sweep (plus the flag reset and the
// norm refresh) are captured once into a CUDA graph, cached on the context by shape and
// buffer addresses, and replayed per sweep; the host reads one flag word per matrix
// after each sweep to stop converged matrices.
template <typename T>
//   tail / keep: truncation-aware mode (keep > 0, n ≤ 4096): only the `keep`
//     largest columns are wanted.  tail[b][j] flags the columns ranked below them;
//     rotations between two flagged columns are skipped.  The flags are refreshed from
//     the running column norms after each sweep that rotated fewer than half of its
//     pairs (always, when the flags were set by an earlier phase: tail_preset).
//   min_rot_frac: the sweeps of matrix b also stop once a sweep rotates no more than this
//     fraction of the pairs (a pre-pass whose residue a later phase removes).
static tn_status_t jacobi_core(tn_ctx* ctx, int64_t m, int64_t n, cx<T>* W, cx<T>* V, int64_t batch, bool v_given,
                               int* active, int* rotated, T* nrm, int max_sweeps, int* sweeps_out, bool* noconv_out,
                               unsigned char* tail = nullptr, int64_t keep = 0, bool tail_preset = false,
                               double min_rot_frac = 0.0, bool tail_fixed = false) {
  if (!(tail && keep > 0 && keep < n && n <= 4096)) {
    tail = nullptr;
    keep = 0;
  }
  const unsigned gy = (unsigned)batch;
  const T tol = jacobi_tol<T>(m);
  int sweeps = 0;
  bool noconv = false;
  const size_t smem_need = sizeof(cx<T>) * (size_t)(m * n + n * n);
  if (V && smem_need <= kSmemMax && n <= 256) {
    TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_jacobi_smem<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
    int threads = n >= 32 ? 512 : 128;
    k_jacobi_smem<T><<<gy, threads, smem_need, ctx->stream>>>(m, n, W, m * n, V, n * n, rotated, tol, max_sweeps,
                                                              v_given);
    TN_LAUNCHED(ctx);
    std::vector<int> st(batch);
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(st.data(), rotated, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream));
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t b = 0; b < batch; ++b) noconv |= st[b] != 0;
    sweeps = -1;
  } else if (sizeof(T) == 8 && !tail && min_rot_frac <= 0.0 && m <= 512 && n <= kCoopMaxN) {
    if (V && !v_given) {
      int64_t blocks = std::min<int64_t>((n * n + 255) / 256, 2048);
      k_identity<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(n, V, n * n, batch);
      TN_LAUNCHED(ctx);
    }
    TN_RETURN_IF(jacobi_coop<T>(ctx, m, n, W, V, batch, active, nrm, max_sweeps, &sweeps, &noconv));
  } else {
    if (V && !v_given) {
      int64_t blocks = std::min<int64_t>((n * n + 255) / 256, 2048);
      k_identity<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(n, V, n * n, batch);
      TN_LAUNCHED(ctx);
    }
    std::vector<int> h_act(batch, 1), h_rot(2 * batch);
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(active, h_act.data(), sizeof(int) * batch, cudaMemcpyHostToDevice, ctx->stream));
    const int N = (int)(n + (n & 1));
    // FP32 with V and m, n ≤ 512: block rounds (16 columns per CTA in registers)
    const bool blocked = sizeof(T) == 4 && V && m <= 512 && n <= 512 && n >= 32;
    const int NB0 = (int)((n + 7) / 8), NB = NB0 + (NB0 & 1);
    const int rounds = blocked ? NB - 1 : N - 1;
    // A sweep whose largest off-diagonal ratio is ρ leaves ~ρ² for the next one
    // (one-sided Jacobi converges quadratically); when ρ² is below tol/10 the next
    // sweep would rotate nothing and is skipped.
    const double stop_ratio = sqrt((double)tol * 1e-1);
    // graph for one sweep
    char key[256];
    snprintf(key, sizeof(key), "jac%zu:%lld:%lld:%lld:%p:%p:%p:%p:%p:%p", sizeof(T), (long long)m, (long long)n,
             (long long)batch, (void*)W, (void*)V, (void*)nrm, (void*)active, (void*)rotated, (void*)tail);
    cudaGraphExec_t ge = nullptr;
    auto it = ctx->graphs.find(key);
    if (it != ctx->graphs.end()) {
      ge = it->second;
    } else {
      if (ctx->graphs.size() > 256) {
        for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
        ctx->graphs.clear();
      }
      cudaGraph_t g = nullptr;
      TN_CHECK_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      cudaMemsetAsync(rotated, 0, sizeof(int) * 2 * batch, ctx->stream);
      int64_t nb = std::min<int64_t>((n * batch * 32 + 255) / 256, (int64_t)ctx->num_sms * 8);
      k_col_norms<T><<<(unsigned)std::max<int64_t>(nb, 1), 256, 0, ctx->stream>>>(m, n, W, m * n, nrm, batch);
      k_fro<T><<<(unsigned)std::min<int64_t>(batch, 65535), 256, 0, ctx->stream>>>(n, nrm, batch);
      tn_status_t st = TN_OK;
      if constexpr (sizeof(T) == 4) {
        if (blocked) {
          const dim3 grid((unsigned)(NB / 2), gy);
          for (int r = 0; r < NB - 1; ++r) {
            if (m <= 128 && n <= 128)
              k_jacobi_block_f32<128><<<grid, 128, 0, ctx->stream>>>(m, n, NB, r, W, V, nrm, active, rotated, tol, tail);
            else if (m <= 256 && n <= 256)
              k_jacobi_block_f32<256><<<grid, 256, 0, ctx->stream>>>(m, n, NB, r, W, V, nrm, active, rotated, tol, tail);
            else
              k_jacobi_block_f32<512><<<grid, 512, 0, ctx->stream>>>(m, n, NB, r, W, V, nrm, active, rotated, tol, tail);
            TN_LAUNCHED(ctx);
          }
        }
      }
      for (int r = 0; !blocked && r < N - 1 && st == TN_OK; ++r)
        st = launch_step<T>(ctx, m, n, N, r, W, V, nrm, active, rotated, tol, gy, tail);
      cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
      if (st != TN_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      if (e != cudaSuccess) return tn_set_error(ctx, TN_ECUDA, "svd graph capture: %s", cudaGetErrorString(e));
      e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return tn_set_error(ctx, TN_ECUDA, "svd graph instantiate: %s", cudaGetErrorString(e));
      ctx->graphs[key] = ge;
      ctx->launches -= rounds;  // counted again per replay below
    }
    if (tail && !tail_preset) TN_CHECK_CUDA(ctx, cudaMemsetAsync(tail, 0, (size_t)(n * batch), ctx->stream));
    const int64_t pairs = n * (n - 1) / 2;
    const int64_t min_rot = (int64_t)(min_rot_frac * (double)pairs);
    int n_active = (int)batch;
    for (sweeps = 0; sweeps < max_sweeps && n_active > 0; ++sweeps) {
      const int slot = prof_begin(ctx);
      TN_CHECK_CUDA(ctx, cudaGraphLaunch(ge, ctx->stream));
      if (slot >= 0) {
        // per round, every pair of every active matrix: wᵢᴴwⱼ (8m) + the two rotated
        // columns of W (24m) [+ of V (24n)]; W [and V] read and written once
        // (block rounds: W and V cross memory once per outer round, NB − 1 per sweep)
        const double pair_rounds = (double)(N - 1), act = (double)n_active;
        const double flops = pair_rounds * act * (N / 2) * (32.0 * m + (V ? 24.0 * n : 0.0));
        const double bytes = (double)rounds * act * 2.0 * sizeof(cx<T>) * ((double)m * n + (V ? (double)n * n : 0.0));
        prof_end(ctx, slot, sizeof(T) == 4 ? TN_PROF_JACOBI_F32 : TN_PROF_JACOBI_F64, rounds, flops, bytes);
      }
      ctx->launches += rounds + 2;  // norm refresh, ‖A‖_F, the rounds
      TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_rot.data(), rotated, sizeof(int) * 2 * batch, cudaMemcpyDeviceToHost,
                                         ctx->stream));
      TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (sweeps < (int)(sizeof(ctx->sweep_rotations) / sizeof(int))) {
        // the matrix with the largest off-diagonal ratio among those still active
        int64_t worst = 0;
        float wr = -1.f;
        for (int64_t b = 0; b < batch; ++b) {
          float ratio;
          memcpy(&ratio, &h_rot[batch + b], sizeof(float));
          if (h_act[b] && ratio > wr) {
            wr = ratio;
            worst = b;
          }
        }
        ctx->sweep_rotations[sweeps] = h_rot[worst];
        ctx->sweep_ratio[sweeps] = wr < 0.f ? 0.f : wr;
      }
      n_active = 0;
      int64_t max_rot = 0;
      for (int64_t b = 0; b < batch; ++b) {
        float ratio;
        memcpy(&ratio, &h_rot[batch + b], sizeof(float));
        if (h_act[b]) max_rot = std::max<int64_t>(max_rot, h_rot[b]);
        h_act[b] = h_act[b] && h_rot[b] && ratio > stop_ratio && h_rot[b] > min_rot;
        n_active += h_act[b];
      }
      if (tail && n_active > 0 && sweeps + 1 >= kTailSweeps) {
        // Without tail–tail rotations the kept columns converge like a subspace
        // iteration, at a rate set by the gap between the kept and the tail values; a
        // near-degenerate boundary (entanglement spectra of symmetric ground states)
        // makes that slow.  Clearing the flags turns the remaining sweeps into full,
        // quadratically convergent Jacobi (the captured sweep reads the flags).
        TN_CHECK_CUDA(ctx, cudaMemsetAsync(tail, 0, (size_t)(n * batch), ctx->stream));
        tail = nullptr;
      }
      if (tail && !tail_fixed && n_active > 0 && (tail_preset || 2 * max_rot < pairs))
        TN_RETURN_IF(update_tail_flags<T>(ctx, n, batch, nrm, keep, tail));
      TN_CHECK_CUDA(ctx, cudaMemcpyAsync(active, h_act.data(), sizeof(int) * batch, cudaMemcpyHostToDevice, ctx->stream));
    }
    noconv = n_active > 0;
  }
  if (sweeps_out) *sweeps_out = sweeps;
  if (noconv_out) *noconv_out = noconv;
  if (sizeof(T) == 4)
    ctx->last_sweeps_fp32 = sweeps;
  else
    ctx->last_sweeps_fp64 = sweeps;
  return TN_OK;
}

// σ, ordering, U = W/σ, V (or Vh) from converged W, V
template <typename T>
static tn_status_t jacobi_finalize(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* W, const cx<T>* V, int* order,
                                   cx<T>* U, int64_t sU, double* S, int64_t sS, cx<T>* Vo, int64_t sVo, bool vh,
                                   int64_t batch) {
  const unsigned gy = (unsigned)batch;
  int P2 = 1;
  while (P2 < n) P2 <<= 1;
  size_t smem = (sizeof(double) + sizeof(int)) * (size_t)P2;
  if (smem > kSmemMax) return tn_set_error(ctx, TN_EUNSUPPORTED, "svd: n too large for the sort");
  TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_svd_order<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
  k_svd_order<T><<<gy, 512, smem, ctx->stream>>>(m, n, W, m * n, S, sS, order);
  TN_LAUNCHED(ctx);
  int64_t blocks = std::min<int64_t>((m * n + 255) / 256, 1024);
  k_svd_gather<T><<<dim3((unsigned)blocks, gy), 256, 0, ctx->stream>>>(m, n, W, m * n, V, n * n, S, sS, order, U, sU,
                                                                        Vo, sVo, vh, batch);
  TN_LAUNCHED(ctx);
  const size_t csm = sizeof(cx<T>) * (size_t)n;
  if (csm <= kSmemMax) {
    TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_svd_complete<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
    const double e = (double)jacobi_eps<T>();
    k_svd_complete<T><<<gy, 256, csm, ctx->stream>>>(m, n, U, sU, S, sS, e * e, (double)JacobiFloor<T>::value);
    TN_LAUNCHED(ctx);
  }
  return TN_OK;
}

// U: m×n, S: n (FP64), Vo: V (n×n) or Vh when vh; workspace reserved by the caller
template <typename T>
static tn_status_t svd_tall_impl(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA,
                                 cx<T>* U, int64_t sU, double* S, int64_t sS, cx<T>* Vo, int64_t sVo, bool vh,
                                 int64_t batch, int* sweeps_out) {
  if (m < n) return tn_set_error(ctx, TN_EINVAL, "svd_tall: m < n");
  if (n == 0 || batch == 0) return TN_OK;
  if (batch > 65535) return tn_set_error(ctx, TN_EUNSUPPORTED, "svd: batch > 65535");
  cx<T>* W = ws_take<cx<T>>(ctx, (size_t)(m * n * batch));
  cx<T>* V = ws_take<cx<T>>(ctx, (size_t)(n * n * batch));
  int* order = ws_take<int>(ctx, (size_t)(n * batch));
  int* active = ws_take<int>(ctx, (size_t)(batch + 1));
  int* rotated = ws_take<int>(ctx, (size_t)(2 * batch + 2));
  T* nrm = ws_take<T>(ctx, (size_t)((n + 1) * batch));  // column norms, then ‖W_b‖²_F
  {
    int64_t blocks = std::min<int64_t>((m * n + 255) / 256, 2048);
    k_copy_mat<T><<<dim3((unsigned)blocks, (unsigned)batch), 256, 0, ctx->stream>>>(m, n, A, lda, sA, W, m * n, batch);
    TN_LAUNCHED(ctx);
  }
  bool noconv = false;
  ctx->last_sweeps_fp32 = 0;
  TN_RETURN_IF(jacobi_core<T>(ctx, m, n, W, V, batch, false, active, rotated, nrm, kMaxSweeps, sweeps_out, &noconv));
  TN_RETURN_IF(jacobi_finalize<T>(ctx, m, n, W, V, order, U, sU, S, sS, Vo, sVo, vh, batch));
  if (noconv) return tn_set_error(ctx, TN_ENOCONV, "Jacobi SVD did not converge within %d sweeps", kMaxSweeps);
  return TN_OK;
}

template <typename T>
tn_status_t svd_tall_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* A, int64_t lda, int64_t sA, cx<T>* U,
                        int64_t sU, double* S, int64_t sS, cx<T>* V, int64_t sV, int64_t batch, int* sweeps_out) {
  return svd_tall_impl<T>(ctx, m, n, A, lda, sA, U, sU, S, sS, V, sV, false, batch, sweeps_out);
}
template tn_status_t svd_tall_cx<double>(tn_ctx*, int64_t, int64_t, const cxd*, int64_t, int64_t, cxd*, int64_t,
                                         double*, int64_t, cxd*, int64_t, int64_t, int*);
template tn_status_t svd_tall_cx<float>(tn_ctx*, int64_t, int64_t, const cxf*, int64_t, int64_t, cxf*, int64_t,
                                        double*, int64_t, cxf*, int64_t, int64_t, int*);

// ---------------------------------------------------------------------------------
// mixed precision (C64 data): the Jacobi sweeps run first in FP32 — on GB300 the FP32
// pipe is ~64× the FP64 pipe — until the columns are orthogonal to FP32 accuracy.  The
// FP32 rotations V32 are lifted to FP64, re-orthonormalised by one series step
// V ← V (I − E/2 + 3E²/8 − 5E³/16), E = VᴴV − I, and W = A·V is formed in FP64; the FP64 Jacobi
// sweeps then only remove the O(1e-5) residual (quadratic convergence: two sweeps).
// Rotations, σ and the truncation decision stay FP64.
// ---------------------------------------------------------------------------------
__global__ void k_d2f(int64_t count, const cxd* __restrict__ a, int64_t lda, int64_t rows, cxf* __restrict__ b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t % rows, c = t / rows;
    cxd v = a[r + c * lda];
    b[t] = mkcx<float>((float)v.x, (float)v.y);
  }
}
__global__ void k_f2d(int64_t count, const cxf* __restrict__ a, cxd* __restrict__ b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    cxf v = a[t];
    b[t] = mkcx<double>(v.x, v.y);
  }
}

// E = G − I as complex float (G = VᴴV, n×n per matrix, dense; E at batch stride sE)
__global__ void k_gram_minus_identity_f32(int64_t n, int64_t batch, const cxd* G, cxf* E, int64_t sE) {
  const int64_t total = n * n * batch;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / (n * n), w = t % (n * n), r = w % n, c = w / n;
    cxd g = G[t];
    E[b * sE + w] = mkcx<float>((float)(g.x - (r == c ? 1.0 : 0.0)), (float)g.y);
  }
}
// G ← I − E/2 + 3E²/8 − 5E³/16 with E = G − I (FP64), E² (stride n²) and E³ (stride sE3)
// in FP32
__global__ void k_ortho_poly(int64_t n, int64_t batch, cxd* G, const cxf* E2, const cxf* E3, int64_t sE3) {
  const int64_t total = n * n * batch;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / (n * n), w = t % (n * n), r = w % n, c = w / n;
    const double id = r == c ? 1.0 : 0.0;
    const cxd g = G[t];
    const cxf e2 = E2[t], e3 = E3[b * sE3 + w];
    G[t] = mkcx<double>(id - 0.5 * (g.x - id) + 0.375 * (double)e2.x - 0.3125 * (double)e3.x,
                        -0.5 * g.y + 0.375 * (double)e2.y - 0.3125 * (double)e3.y);
  }
}

// ---------------------------------------------------------------------------------
// Refinement of the right singular vectors by matrix products (the truncated mixed path).
//
// The iteration is Ogita & Aishima's refinement of an approximate eigenvector basis
// (T. Ogita, K. Aishima, "Iterative refinement for symmetric eigenvalue decomposition",
// Japan J. Indust. Appl. Math. 35 (2018)) applied to AᴴA through W = A·V, so AᴴA is never
// formed: with R = I − VᴴV and S = WᴴW = Vᴴ(AᴴA)V,
//     λ_i = S_ii / (1 − R_ii),
//     E_ii = R_ii / 2,   E_ij = (S_ij + λ_j R_ij) / (λ_j − λ_i)   (i ≠ j),
//     V ← V + V·E,
// which converges quadratically once the columns are separated.  Every product is a
// split-BF16 tensor-core GEMM whose digit planes are scaled per row and per column, so
// S_ij is accurate to ~ε·σ_i·σ_j (graded, like one-sided Jacobi) and the σ_i come out
// with relative accuracy.  Per pair (i, j), with num = S_ij + λ_j R_ij, den = λ_j − λ_i,
// λ = max(λ_i, λ_j) and |num| the larger of |S_ij + λ_j R_ij| and |S_ij + λ_i R_ij| (the
// same for both orders of the pair):
//   * |num| ≤ kRefineNoise·λ and a relative gap below kRefineWideGap: the pair is converged
//     (its coupling is at the rounding level of the products); only the orthogonality
//     part R_ij/2 is applied, so no rotation is driven by noise;
//   * |num| ≤ kRefineStepMax·|den| and |den| > kRefineGapMin·λ: the first-order step;
//   * otherwise (a near-degenerate pair, or one the pre-pass left far from converged):
//     R_ij/2 only, and both columns are marked for the FP64 one-sided Jacobi of the
//     marked columns afterwards.
// Pairs of two tail columns (ranked below the kept set by the current λ) are only kept
// orthogonal.  The noise floor makes the steps that are applied at most
// kRefineNoise/kRefineGapMin (1e-8) when only rounding drives them, so the iteration
// ends: after a step of at most kRefineStop the deviation left is its square.
// ---------------------------------------------------------------------------------
constexpr double kRefineStepMax = 0.1;
constexpr double kRefineGapMin = 1e-6;
constexpr double kRefineNoise = 1e-14;
constexpr double kRefineWideGap = 1e-2;  // relative gap above which the noise floor does not apply
// The refinement's products use the context's digit planes in every iteration (fewer
// planes in the first iterations saved ~8 % of the GEMM time but left couplings of up to
// 1e-11 between neighbouring kept columns of U).  The noise floor and the gap floor of the
// pair rule follow the products' accuracy (~32·S·2^{1−7S} of the larger λ).
inline double refine_noise(int slices) { return std::max(kRefineNoise, 32.0 * slices * std::ldexp(1.0, 1 - 7 * slices)); }
inline double refine_gapmin(double noise) { return std::max(kRefineGapMin, 1e4 * noise); }
constexpr float kRefineStop = 1e-8f;
constexpr double kRefineNormMax = 0.5;  // ‖E‖_F above which the first-order steps diverge
constexpr int kRefineMaxIter = 6;

__global__ void k_set_identity_cxd(int64_t n, int64_t batch, cxd* X) {
  const int64_t total = n * n * batch;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = t % (n * n);
    X[t] = mkcx((w % n) == (w / n) ? 1.0 : 0.0, 0.0);
  }
}

// λ_i = Re S_ii / (1 − Re R_ii); stat[4b + 2] = max_i λ_i (float bits)
__global__ void k_refine_lambda(int64_t n, int64_t batch, const cxd* __restrict__ S, const cxd* __restrict__ R,
                                double* __restrict__ lam, int* stat) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * batch; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / n, i = t % n, d = b * n * n + i + i * n;
    const double l = S[d].x / (1.0 - R[d].x);
    lam[t] = l;
    if (l > 0.0) atomicMax(&stat[4 * b + 2], __float_as_int((float)l));
  }
}

// the pairs the refinement diagonalises: not two tail columns, neither column numerically
// zero (λ ≤ n·ε²·λ_max: its U column is completed orthonormally at the end)
__device__ __forceinline__ bool refine_pair(int64_t n, int64_t b, int64_t i, int64_t j, const unsigned char* tail,
                                            double li, double lj, const int* stat) {
  if (tail && tail[b * n + i] && tail[b * n + j]) return false;
  const double negl = (double)n * 4.93e-32 * (double)__int_as_float(stat[4 * b + 2]);
  return li > negl && lj > negl;
}

// E (in place over R) by the per-pair rule above; grid (·, batch), one matrix per grid
// row, so each warp reduces its statistics before one atomic per warp.  stat[4b] = the
// largest applied step |E_ij| (float bits), stat[4b + 1] = marked pairs, stat[4b + 3] =
// the largest |R_ij|; esq[b] = ‖E‖²_F of the applied steps.
__global__ void __launch_bounds__(256)
    k_refine_step(int64_t n, const cxd* __restrict__ S, cxd* RE, const double* __restrict__ lam,
                  const unsigned char* __restrict__ tail, int* stat, double* __restrict__ esq,
                  unsigned char* __restrict__ cluster, double noise, double gapmin) {
  const int64_t b = blockIdx.y, nn = n * n;
  const cxd* Sb = S + b * nn;
  cxd* Rb = RE + b * nn;
  float emax = 0.f, rmax = 0.f;
  double e2 = 0.0;
  int marked = 0;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nn; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = w % n, j = w / n;
    const cxd r = Rb[w];
    rmax = fmaxf(rmax, (float)sqrt(r.x * r.x + r.y * r.y));
    cxd e = mkcx(0.5 * r.x, 0.5 * r.y);
    if (i != j) {
      const double li = lam[b * n + i], lj = lam[b * n + j];
      if (refine_pair(n, b, i, j, tail, li, lj, stat)) {
        const double den = lj - li, big = fmax(li, lj);
        const cxd sij = Sb[w];
        const cxd num = mkcx(sij.x + lj * r.x, sij.y + lj * r.y);
        // the pair is classified by the larger of |num_ij| and |num_ji| = |S_ij + λ_i R_ij|,
        // so E_ij and E_ji always come from the same rule: then E_ij + conj(E_ji) = R_ij and
        // the first-order part of the new S_ij cancels (a pair split between the rules
        // would keep a coupling of the size of λ·R_ij)
        const double nx = sij.x + li * r.x, ny = sij.y + li * r.y;
        const double mag = fmax(sqrt(num.x * num.x + num.y * num.y), sqrt(nx * nx + ny * ny));
        if (mag <= noise * big && fabs(den) < kRefineWideGap * big) {
          // converged near-degenerate pair (at this iteration's product accuracy): a step
          // would be rounding over rounding, so orthogonality only.  A pair with a wide gap
          // is stepped however small its coupling: the step's error is the coupling's
          // (~ noise·big) over the gap, harmless, and skipping it would leave a relative
          // coupling of noise·√(λ_big/λ_small) in U between well-separated values
        } else if (mag <= kRefineStepMax * fabs(den) && fabs(den) > gapmin * big) {
          e = mkcx(num.x / den, num.y / den);
          const double st = mag / fabs(den);
          emax = fmaxf(emax, (float)st);
          e2 += st * st;
        } else {
          ++marked;
          cluster[b * n + i] = 1;
          cluster[b * n + j] = 1;
        }
      }
    }
    Rb[w] = e;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  }
  e2 = warp_sum(e2);
  marked = warp_sum(marked);
  if ((threadIdx.x & 31) == 0) {
    if (emax > 0.f) atomicMax(&stat[4 * b], __float_as_int(emax));
    if (rmax > 0.f) atomicMax(&stat[4 * b + 3], __float_as_int(rmax));
    if (marked) atomicAdd(&stat[4 * b + 1], marked);
    if (e2 > 0.0) atomicAdd(&esq[b], e2);
  }
}

// FP64 one-sided Jacobi of the marked columns of each matrix, in shared memory: one CTA
// per matrix, the k marked columns of W (m rows) loaded once; each round-robin round
// gives one warp per disjoint pair (dot products by warp shuffles, the rotation formed
// by every lane identically, as make_rot_c forms it for the sweep kernels); sweeps until
// one rotates nothing.  The same rotations are applied to the columns of V (n rows, in
// place in global memory) when V is given, so W = A·V still holds.  Inside the
// refinement this removes the marked pairs' coupling, which would otherwise feed every
// coupling of the marked columns back at the rate coupling/gap per iteration (linear
// convergence).  A rotation inside the marked set leaves the columns as orthogonal to
// the unmarked ones as they were.  status[b]: 0 done,
// 1 more than kmax marked columns (nothing changed), 2 not converged in max_sweeps.
// The column list is built by ballots in column order, so the result is deterministic.
template <int NT>
__global__ void __launch_bounds__(NT)
    k_cluster_jacobi(int64_t m, int64_t n, cxd* __restrict__ W, int64_t sW, cxd* __restrict__ V, int64_t sV,
                     const unsigned char* __restrict__ cluster, int kmax, double tol, const int* __restrict__ stat,
                     int max_sweeps, int* __restrict__ status) {
  extern __shared__ unsigned char smem_raw[];
  cxd* Ws = reinterpret_cast<cxd*>(smem_raw);
  int* idx = reinterpret_cast<int*>(Ws + (size_t)m * kmax);
  __shared__ int s_count, s_rot;
  constexpr int NW = NT / 32;
  const int64_t b = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    int count = 0;
    for (int64_t base = 0; base < n; base += 32) {
      const bool f = base + lane < n && cluster[b * n + base + lane];
      const unsigned mask = __ballot_sync(0xffffffffu, f);
      const int pos = count + __popc(mask & ((1u << lane) - 1u));
      if (f && pos < kmax) idx[pos] = (int)(base + lane);
      count += __popc(mask);
    }
    if (lane == 0) s_count = count;
  }
  __syncthreads();
  const int k = s_count;
  if (k > kmax) {
    if (threadIdx.x == 0) status[b] = 1;
    return;
  }
  if (threadIdx.x == 0) status[b] = 0;
  if (k < 2) return;
  cxd* Wb = W + b * sW;
  for (int c = 0; c < k; ++c)
    for (int64_t r = threadIdx.x; r < m; r += NT) Ws[(size_t)c * m + r] = Wb[(int64_t)idx[c] * m + r];
  const double negl = (double)n * 4.93e-32 * (double)__int_as_float(stat[4 * b + 2]);
  const int K = k + (k & 1);
  int sweep = 0;
  bool any = false;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    for (int r = 0; r < K - 1; ++r) {
      for (int p = warp; p < K / 2; p += NW) {
        int i, j;
        rr_pair(K, r, p, i, j);
        if (j >= k) continue;
        cxd* wi = Ws + (size_t)i * m;
        cxd* wj = Ws + (size_t)j * m;
        cxd g = mkcx(0.0, 0.0);
        double al = 0.0, be = 0.0;
        for (int64_t t = lane; t < m; t += 32) {
          const cxd x = wi[t], y = wj[t];
          cfma_cj(g, x, y);
          al += abs2(x);
          be += abs2(y);
        }
        g.x = warp_sum(g.x);
        g.y = warp_sum(g.y);
        al = warp_sum(al);
        be = warp_sum(be);
        const RotC<double> Rt = make_rot_c(al, be, g, tol, negl);
        if (!Rt.apply) continue;
        if (lane == 0) s_rot = 1;
        for (int64_t t = lane; t < m; t += 32) {
          cxd x = wi[t], y = wj[t];
          rot_apply_c(Rt.c, Rt.se, x, y);
          wi[t] = x;
          wj[t] = y;
        }
        if (V) {
          cxd* vi = V + b * sV + (int64_t)idx[i] * n;
          cxd* vj = V + b * sV + (int64_t)idx[j] * n;
          for (int64_t t = lane; t < n; t += 32) {
            cxd x = vi[t], y = vj[t];
            rot_apply_c(Rt.c, Rt.se, x, y);
            vi[t] = x;
            vj[t] = y;
          }
        }
      }
      __syncthreads();
    }
    const int rotated = s_rot;
    __syncthreads();
    if (!rotated) break;
    any = true;
  }
  if (sweep == max_sweeps && threadIdx.x == 0) status[b] = 2;
  if (!any) return;
  for (int c = 0; c < k; ++c)
    for (int64_t r = threadIdx.x; r < m; r += NT) Wb[(int64_t)idx[c] * m + r] = Ws[(size_t)c * m + r];
}

__global__ void k_scale_real_cxd(int64_t count, cxd* X, double f) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
    X[t] = mkcx(f * X[t].x, f * X[t].y);
}
tn_status_t scale_real_cxd(tn_ctx* ctx, cxd* X, int64_t count, double f) {
  k_scale_real_cxd<<<(unsigned)std::min<int64_t>((count + 255) / 256, 4096), 256, 0, ctx->stream>>>(count, X, f);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

// the FP64 check's flags: every column outside a near-degenerate pair counts as tail, so
// only pairs with a marked column are examined
__global__ void k_cluster_flags(int64_t count, const unsigned char* __restrict__ cluster, unsigned char* __restrict__ f) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
    f[t] = cluster[t] ? 0 : 1;
}

size_t svd_mixed_workspace(int64_t m, int64_t n, int64_t batch) {
  size_t s = 0;
  s += ws_round(sizeof(cxf) * (size_t)(m * n * batch));      // W32
  s += ws_round(sizeof(cxf) * (size_t)(n * n * batch));      // V32
  s += ws_round(sizeof(cxd) * (size_t)(m * n * batch));      // W64
  s += 2 * ws_round(sizeof(cxd) * (size_t)(n * n * batch));  // V64, G
  s += ws_round(sizeof(int) * (size_t)(n * batch));
  s += ws_round(sizeof(int) * (size_t)(batch + 1)) + ws_round(sizeof(int) * (size_t)(2 * batch + 2));
  s += ws_round(sizeof(double) * (size_t)((n + 1) * batch)) + ws_round(sizeof(float) * (size_t)((n + 1) * batch));
  s += ws_round(sizeof(cxd) * (size_t)(n * n * batch));  // V scratch when V is not wanted
  s += ws_round(sizeof(cxf) * (size_t)(n * n * batch));  // E³ when W32 has no room for it
  s += ws_round((size_t)(n * batch));                     // tail flags
  s += ws_round(sizeof(cxd) * (size_t)(n * n * batch));  // R / E of the refinement
  s += ws_round((size_t)(n * batch)) + ws_round(sizeof(int) * (size_t)(5 * batch + 4));  // cluster marks, stats
  return s;
}

tn_status_t svd_tall_mixed(tn_ctx* ctx, int64_t m, int64_t n, const cxd* A, int64_t lda, int64_t sA, cxd* U,
                           int64_t sU, double* S, int64_t sS, cxd* V, int64_t sV, int64_t batch, int64_t keep) {
  // V == nullptr: right vectors not wanted; the FP64 sweeps then skip accumulating them.
  // keep > 0 (only with V == nullptr): only the `keep` largest singular triplets are
  // wanted (a truncation to maxdim follows).  Columns ranked below keep + margin by the
  // running norms are the tail; rotations between two tail columns are skipped, and a
  // kept–tail pair stops rotating once the rotation would change the kept column by less
  // than tol relative (ρ·β_tail/α_kept ≤ tol), so the kept columns are exact to FP64 and
  // the tail entries of U and S are approximate (never used by the caller).
  if (m < n) return tn_set_error(ctx, TN_EINVAL, "svd_tall_mixed: m < n");
  const bool want_v = V != nullptr;
  if (n == 0 || batch == 0) return TN_OK;
  if (batch > 65535) return tn_set_error(ctx, TN_EUNSUPPORTED, "svd: batch > 65535");
  cxf* W32 = ws_take<cxf>(ctx, (size_t)(m * n * batch));
  cxf* V32 = ws_take<cxf>(ctx, (size_t)(n * n * batch));
  cxd* W64 = ws_take<cxd>(ctx, (size_t)(m * n * batch));
  cxd* V64 = ws_take<cxd>(ctx, (size_t)(n * n * batch));
  cxd* G = ws_take<cxd>(ctx, (size_t)(n * n * batch));
  cxf* G3 = ws_take<cxf>(ctx, (size_t)(n * n * batch));
  cxd* Vt = want_v ? nullptr : ws_take<cxd>(ctx, (size_t)(n * n * batch));
  if (!want_v) {
    V = Vt;
    sV = n * n;
  }
  int* order = ws_take<int>(ctx, (size_t)(n * batch));
  int* active = ws_take<int>(ctx, (size_t)(batch + 1));
  int* rotated = ws_take<int>(ctx, (size_t)(2 * batch + 2));
  double* nrm64 = ws_take<double>(ctx, (size_t)((n + 1) * batch));
  float* nrm32 = ws_take<float>(ctx, (size_t)((n + 1) * batch));
  unsigned char* tail = ws_take<unsigned char>(ctx, (size_t)(n * batch));
  cxd* RE = ws_take<cxd>(ctx, (size_t)(n * n * batch));
  unsigned char* cluster = ws_take<unsigned char>(ctx, (size_t)(n * batch));
  int* stat = ws_take<int>(ctx, (size_t)(5 * batch + 4));
  const int64_t keep_m = (!want_v && keep > 0) ? keep + std::max<int64_t>(16, keep / 8) : 0;
  for (int64_t b = 0; b < batch; ++b) {
    int64_t blocks = std::min<int64_t>((m * n + 255) / 256, 2048);
    k_d2f<<<(unsigned)blocks, 256, 0, ctx->stream>>>(m * n, A + b * sA, lda, m, W32 + b * m * n);
    TN_LAUNCHED(ctx);
  }
  bool noconv = false;
  // FP32 pre-pass, stopped once a sweep rotates ≤ 5 % of the pairs (the FP64 phase removes
  // the residue)
  TN_RETURN_IF(jacobi_core<float>(ctx, m, n, W32, V32, batch, false, active, rotated, nrm32, kMaxSweeps, nullptr, &noconv,
                                  (keep_m > 0 && keep_m < n) ? tail : nullptr, keep_m, false, 0.05));
  if (keep_m > 0 && keep_m < n) {
    // rank the columns by their FP32 norms (the pre-pass left them nearly orthogonal)
    int64_t nb = std::min<int64_t>((n * batch * 32 + 255) / 256, (int64_t)ctx->num_sms * 8);
    k_col_norms<float><<<(unsigned)std::max<int64_t>(nb, 1), 256, 0, ctx->stream>>>(m, n, W32, m * n, nrm32, batch);
    TN_LAUNCHED(ctx);
    TN_RETURN_IF(update_tail_flags<float>(ctx, n, batch, nrm32, keep_m, tail));
  }
  {
    int64_t cnt = n * n * batch;
    int64_t blocks = std::min<int64_t>((cnt + 255) / 256, 4096);
    k_f2d<<<(unsigned)blocks, 256, 0, ctx->stream>>>(cnt, V32, V64);
    TN_LAUNCHED(ctx);
  }
  if (keep_m > 0 && keep_m < n) {
    // truncated: refine V by matrix products (tensor pipe) instead of FP64 Jacobi sweeps
    const unsigned blocks = (unsigned)std::min<int64_t>((n * n * batch + 255) / 256, 4096);
    const unsigned lblocks = (unsigned)std::min<int64_t>((n * batch + 255) / 256, 1024);
    const cxd one = mkcx(1.0, 0.0), zero = mkcx(0.0, 0.0), mone = mkcx(-1.0, 0.0);
    std::vector<int> h_stat(4 * batch);
    std::vector<double> h_esq(batch);
    double* esq = nrm64 + n * batch;  // free during the refinement (the sweeps use it for ‖A‖²_F)
    int* cstat = stat + 4 * batch;    // status of the marked-column Jacobi
    const int kmax = (int)std::min<int64_t>(n, (int64_t)(kSmemMax / (sizeof(cxd) * (size_t)m + sizeof(int))));
    if (kmax >= 2)
      TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_cluster_jacobi<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)kSmemMax));
    // the marked-column Jacobi on W (and V when given); returns whether it ran
    auto cluster_jacobi = [&](cxd* Vr) -> tn_status_t {
      const size_t smem = sizeof(cxd) * (size_t)m * kmax + sizeof(int) * (size_t)kmax;
      TN_CHECK_CUDA(ctx, cudaMemsetAsync(cstat, 0, sizeof(int) * (size_t)batch, ctx->stream));
      k_cluster_jacobi<512><<<(unsigned)batch, 512, smem, ctx->stream>>>(m, n, W64, m * n, Vr, n * n, cluster, kmax,
                                                                          jacobi_tol<double>(m), stat, 40, cstat);
      TN_LAUNCHED(ctx);
      return TN_OK;
    };
    bool w_fresh = false, converged = false, diverged = false, cluster_ran = false;
    int clusters = 0;
    float emax = 0.f, rmax = 0.f;
    ctx->last_refine_iters = 0;
    for (int it = 0; it < kRefineMaxIter; ++it) {
      const double noise = refine_noise(ctx->split_slices);
      TN_CHECK_CUDA(ctx, cudaMemsetAsync(cluster, 0, (size_t)(n * batch), ctx->stream));
      if (!w_fresh)
        TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', m, n, n, one, A, lda, sA, V64, n, n * n, zero, W64, m,
                              m * n, batch));
      w_fresh = true;
      cluster_ran = false;
      TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'C', 'N', n, n, m, one, W64, m, m * n, W64, m, m * n, zero, G, n, n * n,
                            batch));
      k_set_identity_cxd<<<blocks, 256, 0, ctx->stream>>>(n, batch, RE);
      TN_LAUNCHED(ctx);
      TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'C', 'N', n, n, n, mone, V64, n, n * n, V64, n, n * n, one, RE, n, n * n,
                            batch));
      TN_CHECK_CUDA(ctx, cudaMemsetAsync(stat, 0, sizeof(int) * 4 * batch, ctx->stream));
      TN_CHECK_CUDA(ctx, cudaMemsetAsync(esq, 0, sizeof(double) * batch, ctx->stream));
      k_refine_lambda<<<lblocks, 256, 0, ctx->stream>>>(n, batch, G, RE, nrm64, stat);
      TN_LAUNCHED(ctx);
      // the kept set by the current λ (the pre-pass ranked the columns by FP32 norms, which
      // cannot order values below ~1e-7 of the largest)
      TN_RETURN_IF(update_tail_flags<double>(ctx, n, batch, nrm64, keep_m, tail));
      {
        const dim3 sg((unsigned)std::min<int64_t>((n * n + 255) / 256, std::max<int64_t>(1, 4096 / batch)),
                      (unsigned)batch);
        k_refine_step<<<sg, 256, 0, ctx->stream>>>(n, G, RE, nrm64, tail, stat, esq, cluster, noise,
                                                    refine_gapmin(noise));
        TN_LAUNCHED(ctx);
      }
      TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_stat.data(), stat, sizeof(int) * 4 * batch, cudaMemcpyDeviceToHost,
                                         ctx->stream));
      TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_esq.data(), esq, sizeof(double) * batch, cudaMemcpyDeviceToHost,
                                         ctx->stream));
      TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      emax = 0.f;
      rmax = 0.f;
      double enorm = 0.0;
      bool finite = true;
      clusters = 0;
      for (int64_t b = 0; b < batch; ++b) {
        float e, r;
        memcpy(&e, &h_stat[4 * b], sizeof(float));
        memcpy(&r, &h_stat[4 * b + 3], sizeof(float));
        finite = finite && std::isfinite(e) && std::isfinite(r) && std::isfinite(h_esq[b]);
        emax = std::max(emax, e);
        rmax = std::max(rmax, r);
        enorm = std::max(enorm, sqrt(h_esq[b]));
        clusters += h_stat[4 * b + 1];
      }
      ctx->last_refine_iters = it + 1;
      ctx->refine_trace[it][0] = emax;
      ctx->refine_trace[it][1] = rmax;
      ctx->refine_trace[it][2] = (float)enorm;
      ctx->refine_trace[it][3] = (float)clusters;
      // outside the quadratic regime (a basis the FP32 pre-pass could not resolve, e.g.
      // values below ~1e-7 of the largest inside the kept set): the first-order steps
      // would not converge, so the FP64 sweeps take over from the pre-pass basis
      if (!finite || enorm > kRefineNormMax || rmax > 0.25f || (it >= 3 && emax > 1e-3f)) {
        diverged = true;
        break;
      }
      if (emax == 0.f && rmax <= 1e-15f && clusters == 0) {  // nothing to correct: W = A·V is final
        converged = true;
        break;
      }
      // V ← V + V·E
      TN_CHECK_CUDA(ctx, cudaMemcpyAsync(V, V64, sizeof(cxd) * (size_t)(n * n * batch), cudaMemcpyDeviceToDevice,
                                         ctx->stream));
      TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', n, n, n, one, V64, n, n * n, RE, n, n * n, one, V, n, n * n,
                            batch));
      std::swap(V, V64);
      w_fresh = false;
      if (clusters > 0 && kmax >= 2) {
        // W = A·V for the new basis, then the marked pairs are rotated in both
        TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', m, n, n, one, A, lda, sA, V64, n, n * n, zero, W64, m,
                              m * n, batch));
        TN_RETURN_IF(cluster_jacobi(V64));
        w_fresh = cluster_ran = true;
      }
      // quadratic convergence: steps and non-orthogonality of at most kRefineStop leave
      // their squares (≤ 1e-16)
      if (emax <= kRefineStop && rmax <= kRefineStop) {
        converged = true;
        break;
      }
    }
    ctx->refine_outcome = converged ? 0 : (diverged ? 1 : 2);
    bool restored = false;
    if (!converged) {
      if (diverged) {
        // back to the pre-pass basis
        const int64_t cnt = n * n * batch;
        k_f2d<<<(unsigned)std::min<int64_t>((cnt + 255) / 256, 4096), 256, 0, ctx->stream>>>(cnt, V32, V64);
        TN_LAUNCHED(ctx);
      }
      // restore V's unitarity (V ← V + V·R/2, quadratic: the pre-pass leaves R ~ 1e-4)
      // and leave every pair with a kept column to the FP64 sweeps
      for (int rep = 0; rep < 3; ++rep) {
        k_set_identity_cxd<<<blocks, 256, 0, ctx->stream>>>(n, batch, RE);
        TN_LAUNCHED(ctx);
        TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'C', 'N', n, n, n, mone, V64, n, n * n, V64, n, n * n, one, RE, n,
                              n * n, batch));
        TN_RETURN_IF(scale_real_cxd(ctx, RE, n * n * batch, 0.5));
        TN_CHECK_CUDA(ctx, cudaMemcpyAsync(V, V64, sizeof(cxd) * (size_t)(n * n * batch), cudaMemcpyDeviceToDevice,
                                           ctx->stream));
        TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', n, n, n, one, V64, n, n * n, RE, n, n * n, one, V, n, n * n,
                              batch));
        std::swap(V, V64);
      }
      restored = true;
      w_fresh = false;
    }
    if (!w_fresh)
      TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', m, n, n, one, A, lda, sA, V64, n, n * n, zero, W64, m, m * n,
                            batch));
    ctx->last_sweeps_fp64 = 0;
    ctx->last_refine_clusters = clusters;
    bool sweep_marked = false;
    if (!restored && clusters > 0) {
      // pairs still marked at the end: the marked-column Jacobi (already run on this W
      // when the last iteration stepped); a matrix with more marked columns than fit, or
      // unconverged, takes the FP64 sweeps over the pairs with a marked column
      if (kmax < 2) {
        sweep_marked = true;
      } else {
        if (!cluster_ran) TN_RETURN_IF(cluster_jacobi(nullptr));
        std::vector<int> h_c(batch);
        TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_c.data(), cstat, sizeof(int) * batch, cudaMemcpyDeviceToHost, ctx->stream));
        TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int64_t b = 0; b < batch; ++b) sweep_marked |= h_c[b] != 0;
      }
    }
    ctx->refine_totals[0] += 1;
    ctx->refine_totals[1] += ctx->last_refine_iters;
    ctx->refine_totals[2] += clusters;
    ctx->refine_totals[3] += (restored || sweep_marked) ? 1 : 0;
    if (restored) {
      // unconverged refinement: FP64 one-sided Jacobi with the truncation flags finishes
      // (after a divergence the flags are derived afresh from the sweeps' own norms)
      TN_RETURN_IF(jacobi_core<double>(ctx, m, n, W64, nullptr, batch, true, active, rotated, nrm64, kMaxSweeps, nullptr,
                                        &noconv, tail, keep_m, !diverged));
    } else if (sweep_marked) {
      k_cluster_flags<<<lblocks, 256, 0, ctx->stream>>>(n * batch, cluster, tail);
      TN_LAUNCHED(ctx);
      TN_RETURN_IF(jacobi_core<double>(ctx, m, n, W64, nullptr, batch, true, active, rotated, nrm64, kMaxSweeps, nullptr,
                                        &noconv, tail, keep_m, true, 0.0, true));
    }
    TN_RETURN_IF(jacobi_finalize<double>(ctx, m, n, W64, nullptr, order, U, sU, S, sS, nullptr, 0, false, batch));
    if (noconv) return tn_set_error(ctx, TN_ENOCONV, "Jacobi SVD did not converge within %d sweeps", kMaxSweeps);
    return TN_OK;
  }
  // One orthonormalisation step: with E = VᴴV − I (FP64 GEMM),
  //   V ← V (I − E/2 + 3E²/8 − 5E³/16)   (the (I + E)^{-1/2} series; residual ~ (35/128)E⁴)
  // FP32 rotation accumulation leaves |E| ~ 1e-4, so E² and E³ need only ~1e-4 relative
  // accuracy: both are FP32 GEMMs.
  // the Gram matrix, V·(…) and W = A·V below are split-BF16 tensor-core GEMMs
  // (FP64-grade products; rotations, norms and the stop test stay FP64)
  TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'C', 'N', n, n, n, mkcx(1.0, 0.0), V64, n, n * n, V64, n, n * n,
                        mkcx(0.0, 0.0), G, n, n * n, batch));
  {
    const int64_t cnt = n * n * batch;
    const unsigned blocks = (unsigned)std::min<int64_t>((cnt + 255) / 256, 4096);
    // E (as FP32, in the W32 scratch: m ≥ n) and E² (in V32, no longer needed)
    // E in W32[0 : n²], E² in V32, E³ in W32[n² : 2n²] (W32 holds m·n ≥ n² per matrix; the
    // second half is used only when m ≥ 2n, otherwise E³ goes to a slot after E²)
    cxf* E = W32;
    cxf* E2 = V32;
    cxf* E3 = (m >= 2 * n) ? W32 + n * n : nullptr;
    const int64_t sE = m * n;
    k_gram_minus_identity_f32<<<blocks, 256, 0, ctx->stream>>>(n, batch, G, E, sE);
    TN_LAUNCHED(ctx);
    TN_RETURN_IF(gemm_cx<float>(ctx, 'N', 'N', n, n, n, mkcx(1.0f, 0.0f), E, n, sE, E, n, sE, mkcx(0.0f, 0.0f), E2, n,
                                n * n, batch));
    if (!E3) E3 = G3;
    TN_RETURN_IF(gemm_cx<float>(ctx, 'N', 'N', n, n, n, mkcx(1.0f, 0.0f), E2, n, n * n, E, n, sE, mkcx(0.0f, 0.0f), E3,
                                n, (E3 == W32 + n * n) ? sE : n * n, batch));
    k_ortho_poly<<<blocks, 256, 0, ctx->stream>>>(n, batch, G, E2, E3, (E3 == W32 + n * n) ? sE : n * n);
    TN_LAUNCHED(ctx);
  }
  TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', n, n, n, mkcx(1.0, 0.0), V64, n, n * n, G, n, n * n,
                        mkcx(0.0, 0.0), V, n, sV, batch));
  for (int64_t b = 0; b < batch; ++b)
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(V64 + b * n * n, V + b * sV, sizeof(cxd) * n * n, cudaMemcpyDeviceToDevice,
                                       ctx->stream));
  // W = A V  (FP64)
  TN_RETURN_IF(gemm_c64(ctx, TN_PREC_MIXED, 'N', 'N', m, n, n, mkcx(1.0, 0.0), A, lda, sA, V64, n, n * n,
                        mkcx(0.0, 0.0), W64, m, m * n, batch));
  TN_RETURN_IF(jacobi_core<double>(ctx, m, n, W64, want_v ? V64 : nullptr, batch, true, active, rotated, nrm64,
                                    kMaxSweeps, nullptr, &noconv, (keep_m > 0 && keep_m < n) ? tail : nullptr, keep_m,
                                    true));
  TN_RETURN_IF(jacobi_finalize<double>(ctx, m, n, W64, want_v ? V64 : nullptr, order, U, sU, S, sS, want_v ? V : nullptr,
                                       sV, false, batch));
  if (noconv) return tn_set_error(ctx, TN_ENOCONV, "Jacobi SVD did not converge within %d sweeps", kMaxSweeps);
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// left singular vectors and values only (m ≥ n): U m×n, S n.  The large-matrix path
// skips the V accumulation (~43 % of an FP64 sweep's work at m = n); callers recover the
// right factor they need from U and A.
// ---------------------------------------------------------------------------------
size_t svd_left_workspace(tn_precision_t prec, int64_t m, int64_t n, int64_t batch) {
  return prec == TN_PREC_MIXED ? svd_mixed_workspace(m, n, batch) : svd_workspace<double>(m, n, batch);
}

tn_status_t svd_left(tn_ctx* ctx, tn_precision_t prec, int64_t m, int64_t n, const cxd* A, int64_t lda, int64_t sA,
                     cxd* U, int64_t sU, double* S, int64_t sS, int64_t batch, int64_t keep) {
  if (m < n) return tn_set_error(ctx, TN_EINVAL, "svd_left: m < n");
  if (n == 0 || batch == 0) return TN_OK;
  if (batch > 65535) return tn_set_error(ctx, TN_EUNSUPPORTED, "svd: batch > 65535");
  if (prec == TN_PREC_MIXED) return svd_tall_mixed(ctx, m, n, A, lda, sA, U, sU, S, sS, nullptr, 0, batch, keep);
  cxd* W = ws_take<cxd>(ctx, (size_t)(m * n * batch));
  cxd* V = ws_take<cxd>(ctx, (size_t)(n * n * batch));
  int* order = ws_take<int>(ctx, (size_t)(n * batch));
  int* active = ws_take<int>(ctx, (size_t)(batch + 1));
  int* rotated = ws_take<int>(ctx, (size_t)(2 * batch + 2));
  double* nrm = ws_take<double>(ctx, (size_t)((n + 1) * batch));
  {
    int64_t blocks = std::min<int64_t>((m * n + 255) / 256, 2048);
    k_copy_mat<double><<<dim3((unsigned)blocks, (unsigned)batch), 256, 0, ctx->stream>>>(m, n, A, lda, sA, W, m * n,
                                                                                         batch);
    TN_LAUNCHED(ctx);
  }
  // the one-CTA shared-memory kernel needs V resident; the large path runs without it
  // small matrices: one CTA per matrix in shared memory when there are many of them; a
  // few (a DMRG or TEBD pair, one MPS) take the persistent cooperative sweeps instead,
  // which spread each round's pairs over many SMs (one SM's FP64 rate serialises a whole
  // SVD; no right vectors are needed here)
  const bool coop = m <= 512 && n <= kCoopMaxN;
  const bool small = sizeof(cxd) * (size_t)(m * n + n * n) <= kSmemMax && n <= 256 && !(coop && batch < 32);
  bool noconv = false;
  ctx->last_sweeps_fp32 = 0;
  TN_RETURN_IF(jacobi_core<double>(ctx, m, n, W, small ? V : nullptr, batch, false, active, rotated, nrm, kMaxSweeps,
                                   nullptr, &noconv));
  TN_RETURN_IF(jacobi_finalize<double>(ctx, m, n, W, nullptr, order, U, sU, S, sS, nullptr, 0, false, batch));
  if (noconv) return tn_set_error(ctx, TN_ENOCONV, "Jacobi SVD did not converge within %d sweeps", kMaxSweeps);
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// any-shape thin SVD: U m×k, S k, Vh k×n
// ---------------------------------------------------------------------------------
size_t svd_any_workspace(tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n, int64_t batch) {
  const int64_t mm = m >= n ? m : n, nn = m >= n ? n : m;
  const size_t es = dt == TN_C64 ? 16 : 8;
  const bool mixed = dt == TN_C64 && prec == TN_PREC_MIXED;
  size_t core = mixed ? svd_mixed_workspace(mm, nn, batch)
                      : (dt == TN_C64 ? svd_workspace<double>(mm, nn, batch) : svd_workspace<float>(mm, nn, batch));
  if (m >= n) return core + (mixed ? ws_round(es * (size_t)(n * n * batch)) : 0);
  return core + 2 * ws_round(es * (size_t)(m * n * batch));
}

template <typename T>
static tn_status_t svd_any_t(tn_ctx* ctx, tn_precision_t prec, int64_t m, int64_t n, const cx<T>* A, int64_t lda,
                             int64_t sA, cx<T>* U, int64_t sU, double* S, int64_t sS, cx<T>* Vh, int64_t sVh,
                             int64_t batch) {
  const bool mixed = prec == TN_PREC_MIXED && sizeof(T) == 8;
  if (m >= n) {
    if (mixed) {
      // V (n×n) into Vh then conjugate-transpose in place via a temporary
      cx<T>* Vt = ws_take<cx<T>>(ctx, (size_t)(n * n * batch));
      TN_RETURN_IF(svd_tall_mixed(ctx, m, n, (const cxd*)A, lda, sA, (cxd*)U, sU, S, sS, (cxd*)Vt, n * n, batch, 0));
      return transpose_cx<T>(ctx, n, n, Vt, n, n * n, Vh, n, sVh, batch, true);
    }
    return svd_tall_impl<T>(ctx, m, n, A, lda, sA, U, sU, S, sS, Vh, sVh, true, batch, nullptr);
  }
  // A = (Aᴴ)ᴴ:  Aᴴ (n×m) = U' S V'ᴴ  ⇒  U = V' (m×m), Vh = U'ᴴ (m×n)
  cx<T>* B = ws_take<cx<T>>(ctx, (size_t)(m * n * batch));
  TN_RETURN_IF(transpose_cx<T>(ctx, m, n, A, lda, sA, B, n, m * n, batch, true));
  cx<T>* Up = ws_take<cx<T>>(ctx, (size_t)(n * m * batch));  // U' (n×m)
  if (mixed) {
    TN_RETURN_IF(svd_tall_mixed(ctx, n, m, (const cxd*)B, n, m * n, (cxd*)Up, n * m, S, sS, (cxd*)U, sU, batch, 0));
  } else {
    TN_RETURN_IF(svd_tall_impl<T>(ctx, n, m, B, n, m * n, Up, n * m, S, sS, U, sU, false, batch, nullptr));
  }
  return transpose_cx<T>(ctx, n, m, Up, n, n * m, Vh, m, sVh, batch, true);
}

tn_status_t svd_any(tn_ctx* ctx, tn_dtype_t dt, tn_precision_t prec, int64_t m, int64_t n, const void* A,
                    int64_t lda, int64_t sA, void* U, int64_t sU, double* S, int64_t sS, void* Vh, int64_t sVh,
                    int64_t batch) {
  if (dt == TN_C64)
    return svd_any_t<double>(ctx, prec, m, n, (const cxd*)A, lda, sA, (cxd*)U, sU, S, sS, (cxd*)Vh, sVh, batch);
  if (dt == TN_C32)
    return svd_any_t<float>(ctx, prec, m, n, (const cxf*)A, lda, sA, (cxf*)U, sU, S, sS, (cxf*)Vh, sVh, batch);
  return tn_set_error(ctx, TN_EUNSUPPORTED, "svd: only C64 and C32 are implemented");
}

// ---------------------------------------------------------------------------------
// Allocation-free thin SVD.
//
// Some callers cannot allocate device memory at the point where they need an SVD:
// real-time loops whose memory was fixed up front, or hosts that hand the library a
// stream but no allocator (and no tn_ctx with its workspace arena).
// tn_svd_thin_noalloc serves them: it takes only the caller's input and output buffers
// and keeps its scratch (W, V, column norms, the sort order and two flag words) in one
// file-scope device array of kNoAllocScratchBytes.  Every GPU that loads the library
// holds that array until the process exits.  The call waits on its stream once per
// Jacobi sweep (to read the convergence flag), so it returns with the work complete.
// ---------------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB per device
constexpr int64_t kNoAllocMaxRows = 4096;                   // rows a Jacobi step holds
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
constexpr int kNoAllocMaxDevices = 64;
void* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// The host-side name g_noalloc_scratch is only a stand-in for the device array; its
// device address is looked up once per device (with that device current) and cached.
tn_status_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return tn_set_error(nullptr, TN_ECUDA, "tn_svd_thin_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return tn_set_error(nullptr, TN_EUNSUPPORTED, "tn_svd_thin_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return tn_set_error(nullptr, TN_ECUDA, "tn_svd_thin_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return TN_OK;
}

__global__ void k_noalloc_flags(int* active, int* rotated) {
  if (threadIdx.x == 0) {
    *active = 1;
    *rotated = 0;
  }
}

inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

extern "C" tn_status_t tn_svd_thin_noalloc(void* stream, int64_t m, int64_t n, const void* d_A, int64_t lda,
                                          void* d_U, double* d_S, void* d_Vh) {
  if (m < 1 || n < 1 || m < n)
    return tn_set_error(nullptr, TN_EINVAL, "tn_svd_thin_noalloc: need m >= n >= 1 (pass the adjoint for m < n)");
  if (lda < m) return tn_set_error(nullptr, TN_EINVAL, "tn_svd_thin_noalloc: lda < m");
  if (!d_A || !d_U || !d_S || !d_Vh) return tn_set_error(nullptr, TN_EINVAL, "tn_svd_thin_noalloc: null pointer");
  // the Jacobi step keeps a column pair in registers, 16 rows per thread of a 256-thread
  // CTA at most: taller matrices are refused here, as the context SVD refuses them
  if (m > kNoAllocMaxRows)
    return tn_set_error(nullptr, TN_EUNSUPPORTED, "tn_svd_thin_noalloc: %lld rows; at most %lld are supported",
                        (long long)m, (long long)kNoAllocMaxRows);
  // scratch layout: W (m×n) | V (n×n) | column norms (n) | order (n) | active | rotated
  const size_t oW = 0, oV = oW + al256(sizeof(cxd) * (size_t)(m * n)), oN = oV + al256(sizeof(cxd) * (size_t)(n * n)),
               oO = oN + al256(sizeof(double) * (size_t)(n + 1)), oF = oO + al256(sizeof(int) * (size_t)n),
               total = oF + 256;
  if (total > kNoAllocScratchBytes)
    return tn_set_error(nullptr, TN_EINVAL,
                        "tn_svd_thin_noalloc: %lld x %lld needs %zu bytes of scratch; the limit is %zu "
                        "((m*n + n*n)*16 + n*12 + ~1 KiB <= 16 MiB, e.g. 1024 x 512)",
                        (long long)m, (long long)n, total, kNoAllocScratchBytes);
  void* base = nullptr;
  TN_RETURN_IF(noalloc_scratch(&base));
  char* sc = static_cast<char*>(base);
  cxd* W = reinterpret_cast<cxd*>(sc + oW);
  cxd* V = reinterpret_cast<cxd*>(sc + oV);
  double* nrm = reinterpret_cast<double*>(sc + oN);
  int* order = reinterpret_cast<int*>(sc + oO);
  int* active = reinterpret_cast<int*>(sc + oF);
  int* rotated = active + 1;
  cudaStream_t st = (cudaStream_t)stream;
#define NA_CHECK(call)                                                                                      \
  do {                                                                                                      \
    cudaError_t _e = (call);                                                                                \
    if (_e != cudaSuccess)                                                                                  \
      return tn_set_error(nullptr, TN_ECUDA, "tn_svd_thin_noalloc: %s: %s", #call, cudaGetErrorString(_e)); \
  } while (0)
  // the array keeps the previous call's contents: everything read below is written first
  k_copy_mat<double><<<(unsigned)std::min<int64_t>((m * n + 255) / 256, 2048), 256, 0, st>>>(
      m, n, (const cxd*)d_A, lda, 0, W, m * n, 1);
  NA_CHECK(cudaGetLastError());
  k_identity<double><<<(unsigned)std::min<int64_t>((n * n + 255) / 256, 2048), 256, 0, st>>>(n, V, n * n, 1);
  NA_CHECK(cudaGetLastError());
  k_noalloc_flags<<<1, 32, 0, st>>>(active, rotated);
  NA_CHECK(cudaGetLastError());
  const double tol = jacobi_tol<double>(m);
  const int N = (int)(n + (n & 1));
  const dim3 grid(N / 2, 1);
  bool converged = false;
  for (int sweep = 0; sweep < kMaxSweeps && !converged; ++sweep) {
    NA_CHECK(cudaMemsetAsync(rotated, 0, 2 * sizeof(int), st));
    k_col_norms<double><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, 1216)), 256, 0, st>>>(
        m, n, W, m * n, nrm, 1);
    NA_CHECK(cudaGetLastError());
    k_fro<double><<<1, 256, 0, st>>>(n, nrm, 1);
    NA_CHECK(cudaGetLastError());
    for (int r = 0; r < N - 1; ++r) {
      if (m <= 512)
        k_jacobi_step_reg<double, 128, 4, false><<<grid, 128, 0, st>>>(m, n, N, r, W, m * n, V, n * n, nrm, active,
                                                                        rotated, tol, nullptr);
      else if (m <= 1024)
        k_jacobi_step_reg<double, 256, 4, false><<<grid, 256, 0, st>>>(m, n, N, r, W, m * n, V, n * n, nrm, active,
                                                                        rotated, tol, nullptr);
      else if (m <= 2048)
        k_jacobi_step_reg<double, 256, 8, false><<<grid, 256, 0, st>>>(m, n, N, r, W, m * n, V, n * n, nrm, active,
                                                                        rotated, tol, nullptr);
      else  // m <= kNoAllocMaxRows = 256 threads x 16 rows
        k_jacobi_step_reg<double, 256, 16, false><<<grid, 256, 0, st>>>(m, n, N, r, W, m * n, V, n * n, nrm, active,
                                                                         rotated, tol, nullptr);
      NA_CHECK(cudaGetLastError());
    }
    int h_rot = 0;  // host stack word: no allocation
    NA_CHECK(cudaMemcpyAsync(&h_rot, rotated, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CHECK(cudaStreamSynchronize(st));
    converged = h_rot == 0;
  }
  int P2 = 1;
  while (P2 < n) P2 <<= 1;
  const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)P2;
  if (smem > 48 * 1024)
    NA_CHECK(cudaFuncSetAttribute(k_svd_order<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
  k_svd_order<double><<<1, 512, smem, st>>>(m, n, W, m * n, d_S, 0, order);
  NA_CHECK(cudaGetLastError());
  k_svd_gather<double><<<dim3((unsigned)std::min<int64_t>((m * n + 255) / 256, 1024), 1), 256, 0, st>>>(
      m, n, W, m * n, V, n * n, d_S, 0, order, (cxd*)d_U, 0, (cxd*)d_Vh, 0, true, 1);
  NA_CHECK(cudaGetLastError());
  if (sizeof(cxd) * (size_t)n <= kSmemMax) {
    NA_CHECK(cudaFuncSetAttribute(k_svd_complete<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
    k_svd_complete<double><<<1, 256, sizeof(cxd) * (size_t)n, st>>>(
        m, n, (cxd*)d_U, 0, d_S, 0, jacobi_eps<double>() * jacobi_eps<double>(), JacobiFloor<double>::value);
    NA_CHECK(cudaGetLastError());
  }
  NA_CHECK(cudaStreamSynchronize(st));
#undef NA_CHECK
  if (!converged)
    return tn_set_error(nullptr, TN_ENOCONV, "tn_svd_thin_noalloc: no convergence within %d sweeps", kMaxSweeps);
  return TN_OK;
}

extern "C" tn_status_t tn_svd_last_sweeps(tn_ctx* ctx, int32_t* fp32_sweeps, int32_t* fp64_sweeps,
                                          int32_t* rotations, int32_t n_rot) {
  if (!ctx) return TN_EINVAL;
  if (fp32_sweeps) *fp32_sweeps = ctx->last_sweeps_fp32;
  if (fp64_sweeps) *fp64_sweeps = ctx->last_sweeps_fp64;
  for (int i = 0; rotations && i < n_rot && i < 64; ++i) rotations[i] = ctx->sweep_rotations[i];
  return TN_OK;
}

extern "C" tn_status_t tn_svd_refine_stats(tn_ctx* ctx, int64_t* totals, int32_t reset) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, totals, "tn_svd_refine_stats: null output");
  for (int i = 0; i < 4; ++i) totals[i] = ctx->refine_totals[i];
  if (reset)
    for (int i = 0; i < 4; ++i) ctx->refine_totals[i] = 0;
  return TN_OK;
}

extern "C" tn_status_t tn_svd_last_refine(tn_ctx* ctx, float* trace, int32_t* iterations, int32_t* outcome) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, trace && iterations && outcome, "tn_svd_last_refine: null output");
  *iterations = ctx->last_refine_iters;
  *outcome = ctx->refine_outcome;
  for (int k = 0; k < ctx->last_refine_iters && k < 8; ++k)
    for (int q = 0; q < 4; ++q) trace[4 * k + q] = ctx->refine_trace[k][q];
  return TN_OK;
}

extern "C" tn_status_t tn_svd_last_ratios(tn_ctx* ctx, float* ratios, int32_t n) {
  if (!ctx || !ratios) return TN_EINVAL;
  for (int i = 0; i < n && i < 64; ++i) ratios[i] = ctx->sweep_ratio[i];
  return TN_OK;
}

extern "C" tn_status_t tn_svd_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, int64_t m, int64_t n,
                                   const void* A, int64_t lda, int64_t strideA, void* U, int64_t strideU, double* S,
                                   int64_t strideS, void* Vh, int64_t strideVh, int64_t batch) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, m >= 0 && n >= 0 && batch >= 0, "tn_svd_thin: negative size");
  TN_ARG(ctx, lda >= (m > 1 ? m : 1), "tn_svd_thin: lda < m");
  TN_ARG(ctx, (m == 0 || n == 0 || batch == 0) || (A && U && S && Vh), "tn_svd_thin: null pointer");
  TN_ARG(ctx, dtype == TN_C64 || dtype == TN_C32, "tn_svd_thin: only C64 and C32 are implemented");
  TN_RETURN_IF(ws_reserve(ctx, svd_any_workspace(dtype, prec, m, n, batch)));
  return svd_any(ctx, dtype, prec, m, n, A, lda, strideA, U, strideU, S, strideS, Vh, strideVh, batch);
}
