// Device-resident MPS and the Tenet operations on it, with the canonical-form trait kept
// in native code.  Every site tensor stays in HBM between calls; only bond dimensions,
// the form and scalar results cross to the host.
//
//   site i (1-based): (χ_{i-1}, d, χ_i) ComplexF64, column-major — Tenet's (:l, :o, :r)
//   order (src/Components/MPS.jl:50-94) with the open-end bonds χ_0 = χ_L = 1.
//
// A tn_mps holds B ≥ 1 instances that share L, d, the canonical form and the bond
// dimensions, and are advanced in lockstep by every operation (batched kernels: one
// launch serves all B instances).  Instance b of site i lives at site[i] + b·cap[i].
// When truncation ranks differ between instances the common bond dimension is the
// largest kept rank and each instance's surplus singular values are set to zero before
// √S is absorbed, so every instance carries exactly its own truncated state.
//
// Algorithms restated from Tenet.jl v0.10.3:
//   gauge move            generic_canonize_site!       src/Operations/canonize.jl:23-76
//   bond gauge move       generic_bond_canonize_site!  src/Operations/canonize.jl:78-116
//   form transitions      generic_mps_canonize!        src/Operations/canonize.jl:121-252
//   compress / truncate!  generic_mps_compress!        src/Operations/compress.jl:21-69
//   simple update         simple_update!(::MPS, op)    src/Operations/simple_update.jl:20-92
//   overlap               overlap(::MPS, ::MPS)        src/Operations/overlap.jl:36-50
//   amplitude             overlap(::ProductState, ψ)   src/Operations/overlap.jl:22-32
//   norm / normalize!                                   src/Operations/norm.jl:17-37, normalize.jl:15-37
#include <algorithm>
#include <cmath>
#include <vector>

#include "tn_mps_internal.cuh"

// Output sizing callback of the gate core: called once the kept rank r is known; returns
// where A' and B' go with their instance strides (it may grow and move buffers: the gate
// inputs have been consumed by then).
typedef tn_status_t (*su_out_fn)(void* arg, int64_t r, cxd** Aout, int64_t* sAout, cxd** Bout, int64_t* sBout);

namespace {

inline int64_t sz(const tn_mps* p, int i) { return p->bond[i - 1] * p->d * p->bond[i]; }

const cxd kOne = {1.0, 0.0};
const cxd kZero = {0.0, 0.0};

// strided copy of B instances of `elems` elements
tn_status_t copy_instances(tn_ctx* ctx, cxd* dst, size_t dst_stride, const cxd* src, size_t src_stride, size_t elems,
                           int B) {
  if (elems == 0 || B == 0) return TN_OK;
  TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(dst, dst_stride * sizeof(cxd), src, src_stride * sizeof(cxd), elems * sizeof(cxd),
                                       B, cudaMemcpyDeviceToDevice, ctx->stream));
  return TN_OK;
}

__global__ void k_set_one(cxd* x, int64_t stride, int64_t B) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < B; b += (int64_t)gridDim.x * blockDim.x) {
    x[b * stride].x = 1.0;
    x[b * stride].y = 0.0;
  }
}

tn_status_t set_one(tn_ctx* ctx, cxd* x, int64_t stride, int64_t B) {
  k_set_one<<<(unsigned)((B + 127) / 128), 128, 0, ctx->stream>>>(x, stride, B);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

tn_status_t ensure_site(tn_mps* p, int i, size_t elems) {
  if (elems <= p->cap[i]) return TN_OK;
  tn_ctx* ctx = p->ctx;
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  void* np = nullptr;
  TN_RETURN_IF(tn_dev_alloc(ctx, elems * sizeof(cxd) * p->B, &np));
  if (p->site[i]) {
    tn_status_t st = copy_instances(ctx, (cxd*)np, elems, p->site[i], p->cap[i], (size_t)sz(p, i), p->B);
    if (st == TN_OK) {
      const cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) st = tn_set_error(ctx, TN_ECUDA, "site growth: %s", cudaGetErrorString(e));
    }
    if (st != TN_OK) {  // the site keeps its old storage
      tn_dev_free(ctx, np);
      return st;
    }
    TN_RETURN_IF(tn_dev_free(ctx, p->site[i]));
  }
  p->site[i] = (cxd*)np;
  p->cap[i] = elems;
  return TN_OK;
}

tn_status_t ensure_lam(tn_mps* p, int64_t n) {
  if ((size_t)n <= p->lam_cap) return TN_OK;
  tn_ctx* ctx = p->ctx;
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (p->lam) TN_RETURN_IF(tn_dev_free(ctx, p->lam));
  p->lam = nullptr;  // (an allocation failure below leaves no Λ storage, not a freed one)
  p->lam_cap = 0;
  p->lam_len = 0;    // the growth does not keep the old values
  void* np = nullptr;
  size_t c = std::max<size_t>(n, 64);
  TN_RETURN_IF(tn_dev_alloc(ctx, c * sizeof(double) * p->B, &np));
  p->lam = (double*)np;
  p->lam_cap = c;
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// gauge moves (canonize.jl:23-116), all B instances at once
// ---------------------------------------------------------------------------------

// factorise site i across bond (i, i+1) — QR, or SVD keeping Λ — and push the
// non-isometric factor into site i+1
tn_status_t gauge_right(tn_mps* p, int i, bool svd_lambda) {
  tn_ctx* ctx = p->ctx;
  const int B = p->B;
  const int64_t chl = p->bond[i - 1], chr = p->bond[i], d = p->d;
  // size-1 bonds are skipped by the QR move (canonize.jl:38); the bond-canonical move
  // still factorises them so that a Λ of length 1 exists for norm / compress
  if (chr == 1 && !svd_lambda) return TN_OK;
  const int64_t m = chl * d, n = chr, k = std::min(m, n);
  const int64_t nbc = d * p->bond[i + 1];  // columns of site i+1 as (χ_i × d χ_{i+1})
  size_t need = ws_round(sizeof(cxd) * (size_t)(B * k * n)) + ws_round(sizeof(cxd) * (size_t)(B * k * nbc));
  if (svd_lambda)
    need += ws_round(sizeof(cxd) * (size_t)(B * m * k)) + svd_any_workspace(TN_C64, p->prec, m, n, B);
  else
    need += qr_workspace<double>(m, n, B);
  TN_RETURN_IF(ws_reserve(ctx, need));
  cxd* R = ws_take<cxd>(ctx, (size_t)(B * k * n));
  cxd* tmp = ws_take<cxd>(ctx, (size_t)(B * k * nbc));
  if (svd_lambda) {
    cxd* U = ws_take<cxd>(ctx, (size_t)(B * m * k));
    TN_RETURN_IF(ensure_lam(p, k));
    TN_RETURN_IF(svd_any(ctx, TN_C64, p->prec, m, n, p->site[i], m, p->cap[i], U, m * k, p->lam, p->lam_cap, R, k * n, B));
    TN_RETURN_IF(copy_instances(ctx, p->site[i], p->cap[i], U, m * k, m * k, B));
    p->lam_len = k;
  } else {
    TN_RETURN_IF(qr_cx<double>(ctx, m, n, p->site[i], m, p->cap[i], p->site[i], p->cap[i], R, k * n, B));
  }
  TN_RETURN_IF(gemm_c64(ctx, p->prec, 'N', 'N', k, nbc, n, kOne, R, k, k * n, p->site[i + 1], n, p->cap[i + 1], kZero,
                        tmp, k, k * nbc, B));
  TN_RETURN_IF(ensure_site(p, i + 1, (size_t)(k * nbc)));
  TN_RETURN_IF(copy_instances(ctx, p->site[i + 1], p->cap[i + 1], tmp, k * nbc, k * nbc, B));
  p->bond[i] = k;
  return TN_OK;
}

// factorise site i across bond (i-1, i); the non-isometric part goes into site i-1
tn_status_t gauge_left(tn_mps* p, int i, bool svd_lambda) {
  tn_ctx* ctx = p->ctx;
  const int B = p->B;
  const int64_t chl = p->bond[i - 1], chr = p->bond[i], d = p->d;
  if (chl == 1 && !svd_lambda) return TN_OK;
  const int64_t m = d * chr, n = chl, k = std::min(m, n);  // Mᴴ is (d χ_r) × χ_l
  const int64_t rows_b = p->bond[i - 2] * d;                // site i-1 as (χ_{i-2} d × χ_{i-1})
  size_t need = 2 * ws_round(sizeof(cxd) * (size_t)(B * m * n)) + ws_round(sizeof(cxd) * (size_t)(B * k * n)) +
                ws_round(sizeof(cxd) * (size_t)(B * rows_b * k));
  need += svd_lambda ? svd_any_workspace(TN_C64, p->prec, m, n, B) : qr_workspace<double>(m, n, B);
  TN_RETURN_IF(ws_reserve(ctx, need));
  cxd* Mh = ws_take<cxd>(ctx, (size_t)(B * m * n));
  cxd* Q = ws_take<cxd>(ctx, (size_t)(B * m * n));
  cxd* R = ws_take<cxd>(ctx, (size_t)(B * k * n));
  cxd* tmp = ws_take<cxd>(ctx, (size_t)(B * rows_b * k));
  TN_RETURN_IF(transpose_cx<double>(ctx, n, m, p->site[i], n, p->cap[i], Mh, m, m * n, B, true));
  if (svd_lambda) {
    TN_RETURN_IF(ensure_lam(p, k));
    TN_RETURN_IF(svd_any(ctx, TN_C64, p->prec, m, n, Mh, m, m * n, Q, m * n, p->lam, p->lam_cap, R, k * n, B));
    p->lam_len = k;
  } else {
    TN_RETURN_IF(qr_cx<double>(ctx, m, n, Mh, m, m * n, Q, m * n, R, k * n, B));
  }
  // new site i = Qᴴ (k × d χ_r)
  TN_RETURN_IF(transpose_cx<double>(ctx, m, k, Q, m, m * n, p->site[i], k, p->cap[i], B, true));
  // site i-1 ← B · Rᴴ
  TN_RETURN_IF(gemm_c64(ctx, p->prec, 'N', 'C', rows_b, k, n, kOne, p->site[i - 1], rows_b, p->cap[i - 1], R, k, k * n,
                        kZero, tmp, rows_b, rows_b * k, B));
  TN_RETURN_IF(ensure_site(p, i - 1, (size_t)(rows_b * k)));
  TN_RETURN_IF(copy_instances(ctx, p->site[i - 1], p->cap[i - 1], tmp, rows_b * k, rows_b * k, B));
  p->bond[i - 1] = k;
  return TN_OK;
}

// absorb Λ into a neighbouring site along the bond (canonize.jl:198,209)
tn_status_t absorb_lambda(tn_mps* p, int i, bool into_left_index) {
  tn_ctx* ctx = p->ctx;
  int64_t dims[3] = {p->bond[i - 1], p->d, p->bond[i]};
  int axis = into_left_index ? 0 : 2;
  if (dims[axis] != p->lam_len)
    return tn_set_error(ctx, TN_EINVAL, "absorb: Λ length %lld does not match bond %lld", (long long)p->lam_len,
                        (long long)dims[axis]);
  for (int b = 0; b < p->B; ++b)
    TN_RETURN_IF(tn_hadamard(ctx, TN_C64, 3, dims, axis, p->site[i] + b * p->cap[i], p->lam + b * p->lam_cap,
                             p->site[i] + b * p->cap[i]));
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// form transitions (canonize.jl:121-252)
// ---------------------------------------------------------------------------------
tn_status_t canonize_mixed(tn_mps* p, int lo, int hi);

tn_status_t mixed_to_mixed(tn_mps* p, int lo, int hi) {
  if (p->kind == TN_FORM_MIXED && p->lo == lo && p->hi == hi) return TN_OK;
  const int src_left = p->lo, src_right = p->hi;
  const int dst_left = lo - 1, dst_right = hi + 1;
  for (int i = src_left; i <= dst_left; ++i) TN_RETURN_IF(gauge_right(p, i, false));
  for (int i = src_right; i >= dst_right; --i) TN_RETURN_IF(gauge_left(p, i, false));
  p->kind = TN_FORM_MIXED;
  p->lo = lo;
  p->hi = hi;
  return TN_OK;
}

// SVD of `site` across bond (a, a+1) without absorbing Λ (canonize.jl:78-116)
tn_status_t bond_gauge(tn_mps* p, int site, int a) {
  p->lam_len = 0;
  if (site == a) return gauge_right(p, site, true);
  return gauge_left(p, site, true);
}

tn_status_t canonize_bond(tn_mps* p, int a) {
  const int na = a, nb = a + 1;
  if (p->kind == TN_FORM_NONCANONICAL) {
    p->kind = TN_FORM_MIXED;
    p->lo = 1;
    p->hi = p->L;
  }
  if (p->kind == TN_FORM_BOND) {
    if (p->lo == na) return TN_OK;
    const int old_min = p->lo, old_max = p->hi;
    // BondCanonical → BondCanonical (canonize.jl:221-246) goes through Bond → Mixed
    int target;
    if (old_max <= na)
      target = na;
    else if (nb <= old_min)
      target = nb;
    else
      return tn_set_error(p->ctx, TN_EINVAL, "Cannot canonize from bond %d-%d to bond %d-%d", old_min, old_max, na, nb);
    TN_RETURN_IF(canonize_mixed(p, target, target));
    TN_RETURN_IF(bond_gauge(p, target, a));
    p->kind = TN_FORM_BOND;
    p->lo = na;
    p->hi = nb;
    return TN_OK;
  }
  // Mixed → Bond (canonize.jl:151-179)
  const int old_min = p->lo, old_max = p->hi;
  int target;
  if (old_max <= na)
    target = na;
  else if (nb <= old_min)
    target = nb;
  else if (old_min <= na && nb <= old_max)
    target = na;
  else
    return tn_set_error(p->ctx, TN_EINVAL, "Cannot canonize from mixed %d..%d to bond %d-%d", old_min, old_max, na, nb);
  TN_RETURN_IF(mixed_to_mixed(p, target, target));
  TN_RETURN_IF(bond_gauge(p, target, a));
  p->kind = TN_FORM_BOND;
  p->lo = na;
  p->hi = nb;
  return TN_OK;
}

tn_status_t canonize_mixed(tn_mps* p, int lo, int hi) {
  if (p->kind == TN_FORM_NONCANONICAL) {
    p->kind = TN_FORM_MIXED;
    p->lo = 1;
    p->hi = p->L;
  }
  if (p->kind == TN_FORM_BOND) {
    // Bond → Mixed (canonize.jl:181-219): absorb Λ to one side, then sweep
    const int old_min = p->lo, old_max = p->hi;
    if (old_max <= lo) {
      TN_RETURN_IF(absorb_lambda(p, old_max, true));
      p->kind = TN_FORM_MIXED;
      p->lo = p->hi = old_max;
    } else if (hi <= old_min) {
      TN_RETURN_IF(absorb_lambda(p, old_min, false));
      p->kind = TN_FORM_MIXED;
      p->lo = p->hi = old_min;
    } else {
      return tn_set_error(p->ctx, TN_EINVAL, "Cannot canonize from bond %d-%d to mixed %d..%d", old_min, old_max, lo, hi);
    }
    p->lam_len = 0;
  }
  return mixed_to_mixed(p, lo, hi);
}

}  // namespace

tn_status_t mps_ensure_site(tn_mps* p, int i, size_t elems) { return ensure_site(p, i, elems); }


// ---------------------------------------------------------------------------------
// simple update core (Muscle.simple_update with AbsorbEqually), batched
// A (chl·d1 × chm), B (chm × d2·chr), G (d1 d2 × d1 d2) column-major, instance strides
// sA, sB; G shared by all instances.  Reserves the workspace itself.
// absorb (the same two-site state in every case, A'B' = the truncated θ):
//   kAbsorbEqually  A' = U√S, B' = √S Vh (Tenet's AbsorbEqually)
//   kAbsorbRight    A' = U, B' = S·Vh: A' is already left-isometric when the centre moves
//                   on to the right
//   kAbsorbLeft     A' = U·S, B' = Vh: B' is already right-isometric when the centre
//                   moves on to the left.  With n ≥ m the SVD runs on θᴴ, whose left
//                   vectors are V: B' = V[:, :r]ᴴ exactly isometric and A' = θ·V[:, :r]
//                   (no division by S).
// ---------------------------------------------------------------------------------
tn_status_t simple_update_core(tn_ctx* ctx, tn_precision_t prec, int64_t chl, int64_t d1, int64_t chm, int64_t d2,
                               int64_t chr, const cxd* A, int64_t sA, const cxd* Bm, int64_t sB, const cxd* dG,
                               int64_t maxdim, double threshold, int64_t batch, su_out_fn out_fn, void* out_arg,
                               double* Sout, int64_t* rank_out, int absorb) {
  const int64_t m = chl * d1, n = d2 * chr, k = std::min(m, n), dd = d1 * d2;
  // U-only SVDs (one factor from the Jacobi sweeps, the other by one GEMM):
  //   m ≥ n (the saturated TEBD case, θ square), not absorbing left: U and S of θ, then
  //     B' = √S Vh = diag(1/√s) Uᴴ θ (or S·Vh = Uᴴθ)
  //   n ≥ m, absorbing left: V and S from θᴴ, then A' = θ·V
  //   otherwise (absorbing left with m > n, or n > m not absorbing left) the full SVD
  const bool left_of_adj = absorb == kAbsorbLeft && n >= m;
  const bool left_only = absorb != kAbsorbLeft && m >= n;
  const size_t svd_ws = left_of_adj ? svd_left_workspace(prec, n, m, batch)
                                    : (left_only ? svd_left_workspace(prec, m, n, batch)
                                                 : svd_any_workspace(TN_C64, prec, m, n, batch));
  size_t need = 2 * ws_round(sizeof(cxd) * (size_t)(batch * m * n)) + ws_round(sizeof(cxd) * (size_t)(batch * m * k)) +
                ws_round(sizeof(double) * (size_t)(batch * k)) + ws_round(sizeof(cxd) * (size_t)(batch * k * n)) +
                svd_ws;
  TN_RETURN_IF(ws_reserve(ctx, need));
  cxd* th0 = ws_take<cxd>(ctx, (size_t)(batch * m * n));
  cxd* th = ws_take<cxd>(ctx, (size_t)(batch * m * n));
  cxd* U = ws_take<cxd>(ctx, (size_t)(batch * m * k));
  double* S = ws_take<double>(ctx, (size_t)(batch * k));
  cxd* Vh = ws_take<cxd>(ctx, (size_t)(batch * k * n));
  // θ0 = A (χl d1 × χm) · B (χm × d2 χr)
  TN_RETURN_IF(gemm_c64(ctx, prec, 'N', 'N', m, n, chm, kOne, A, m, sA, Bm, chm, sB, kZero, th0, m, m * n, batch));
  // θ[l, (a b), r] = Σ G[(a b), (a' b')] θ0[l, (a' b'), r] — batched over (r, instance),
  // which are contiguous blocks of chl·dd elements
  TN_RETURN_IF(apply_phys(ctx, chl, dd, chr * batch, th0, th, dG));
  if (left_of_adj) {
    // θᴴ (n × m) in θ0's buffer; its left vectors V (n × k) go to the Vh buffer
    TN_RETURN_IF(adjoint_cxd(ctx, m, n, th, m, m * n, th0, n, n * m, batch));
    TN_RETURN_IF(svd_left(ctx, prec, n, m, th0, n, n * m, Vh, n * k, S, k, batch, maxdim > 0 && maxdim < m ? maxdim : 0));
  } else if (left_only) {  // at most maxdim values survive the truncation below
    TN_RETURN_IF(svd_left(ctx, prec, m, n, th, m, m * n, U, m * k, S, k, batch, maxdim > 0 && maxdim < n ? maxdim : 0));
  } else {
    TN_RETURN_IF(svd_any(ctx, TN_C64, prec, m, n, th, m, m * n, U, m * k, S, k, Vh, k * n, batch));
  }
  int64_t r = 0;
  TN_RETURN_IF(rank_select_batched(ctx, S, k, k, batch, maxdim, threshold, &r, nullptr));
  if (prec != TN_PREC_NATIVE) TN_RETURN_IF(split_gemm_check(ctx));  // the stream has drained: one word
  cxd *Aout = nullptr, *Bout = nullptr;
  int64_t sAo = 0, sBo = 0;
  TN_RETURN_IF(out_fn(out_arg, r, &Aout, &sAo, &Bout, &sBo));
  if (left_of_adj) {
    // B' = V[:, :r]ᴴ; A' = θ V[:, :r], columns beyond an instance's own rank (S = 0) zeroed
    TN_RETURN_IF(adjoint_cxd(ctx, n, r, Vh, n, n * k, Bout, r, sBo, batch));
    TN_RETURN_IF(gemm_c64(ctx, prec, 'N', 'N', m, r, n, kOne, th, m, m * n, Vh, n, n * k, kZero, Aout, m, sAo, batch));
    TN_RETURN_IF(scale_cols_mode(ctx, Aout, m, r, m, S, sAo, k, batch, 0));
  } else {
    // A' = U[:, :r] (· √S or · S below)
    TN_RETURN_IF(copy_matrix_cxd(ctx, m * r, 1, U, m * r, Aout, m * r, m * k, sAo, batch));
    if (absorb == kAbsorbLeft) {
      // (m > n) B' = Vh[:r, :], A' = U S
      TN_RETURN_IF(scale_cols_mode(ctx, Aout, m, r, m, S, sAo, k, batch, 1));
      TN_RETURN_IF(copy_matrix_cxd(ctx, r, n, Vh, k, Bout, r, k * n, sBo, batch));
    } else if (absorb == kAbsorbRight) {
      if (left_only) {
        // B' = S Vh = U[:, :r]ᴴ θ, rows beyond an instance's own rank (S = 0) zeroed
        TN_RETURN_IF(
            gemm_c64(ctx, prec, 'C', 'N', r, n, m, kOne, U, m, m * k, th, m, m * n, kZero, Bout, r, sBo, batch));
        TN_RETURN_IF(scale_rows_mode(ctx, Bout, r, n, r, S, sBo, k, batch, 0));
      } else {
        TN_RETURN_IF(copy_matrix_cxd(ctx, r, n, Vh, k, Bout, r, k * n, sBo, batch));
        TN_RETURN_IF(scale_rows_mode(ctx, Bout, r, n, r, S, sBo, k, batch, 1));
      }
    } else if (left_only) {
      TN_RETURN_IF(scale_cols_sqrt<double>(ctx, Aout, m, r, m, S, sAo, k, batch));
      // B' = diag(1/√s) U[:, :r]ᴴ θ
      TN_RETURN_IF(
          gemm_c64(ctx, prec, 'C', 'N', r, n, m, kOne, U, m, m * k, th, m, m * n, kZero, Bout, r, sBo, batch));
      TN_RETURN_IF(scale_rows_invsqrt(ctx, Bout, r, n, r, S, sBo, k, batch));
    } else {
      TN_RETURN_IF(scale_cols_sqrt<double>(ctx, Aout, m, r, m, S, sAo, k, batch));
      // B' = √S Vh[:r, :]
      TN_RETURN_IF(copy_matrix_cxd(ctx, r, n, Vh, k, Bout, r, k * n, sBo, batch));
      TN_RETURN_IF(scale_rows_sqrt<double>(ctx, Bout, r, n, r, S, sBo, k, batch));
    }
  }
  if (Sout)
    TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(Sout, sizeof(double) * r, S, sizeof(double) * k, sizeof(double) * r, batch,
                                         cudaMemcpyDeviceToDevice, ctx->stream));
  *rank_out = r;
  return TN_OK;
}

namespace {

struct PairOut {
  tn_mps* p;
  int a;
};
tn_status_t pair_out(void* arg, int64_t r, cxd** Aout, int64_t* sAo, cxd** Bout, int64_t* sBo) {
  PairOut* e = (PairOut*)arg;
  tn_mps* p = e->p;
  const int64_t m = p->bond[e->a - 1] * p->d, n = p->d * p->bond[e->a + 1];
  TN_RETURN_IF(ensure_site(p, e->a, (size_t)(m * r)));
  TN_RETURN_IF(ensure_site(p, e->a + 1, (size_t)(r * n)));
  *Aout = p->site[e->a];
  *sAo = p->cap[e->a];
  *Bout = p->site[e->a + 1];
  *sBo = p->cap[e->a + 1];
  return TN_OK;
}

// kAbsorbRight: site a keeps U (left-isometric) and site a+1 all of S, so the form becomes
// MixedCanonical(a+1) — the same state as AbsorbEqually's MixedCanonical([a, a+1]), with
// the first of the next centre move's two QR factorisations already done; kAbsorbLeft
// mirrors it (site a+1 = Vh, MixedCanonical(a)) for a centre moving on to the left
tn_status_t apply_gate2(tn_mps* p, int a, const cxd* dG, int64_t maxdim, double threshold,
                        int absorb = kAbsorbEqually) {
  const int64_t d = p->d;
  PairOut e{p, a};
  int64_t r = 0;
  TN_RETURN_IF(simple_update_core(p->ctx, p->prec, p->bond[a - 1], d, p->bond[a], d, p->bond[a + 1], p->site[a],
                                  p->cap[a], p->site[a + 1], p->cap[a + 1], dG, maxdim, threshold, p->B, pair_out, &e,
                                  nullptr, &r, absorb));
  p->bond[a] = r;
  if (absorb != kAbsorbEqually) {
    p->kind = TN_FORM_MIXED;
    p->lo = p->hi = absorb == kAbsorbRight ? a + 1 : a;
  }
  return TN_OK;
}

tn_status_t apply_gate1(tn_mps* p, int i, const cxd* dG) {
  tn_ctx* ctx = p->ctx;
  const int64_t d = p->d, chl = p->bond[i - 1], chr = p->bond[i], e = chl * d * chr;
  TN_RETURN_IF(ws_reserve(ctx, ws_round(sizeof(cxd) * (size_t)(p->B * e))));
  cxd* tmp = ws_take<cxd>(ctx, (size_t)(p->B * e));
  // new[l, a, r] = Σ_b G[a, b] A[l, b, r]  (batched over r within each instance)
  for (int b = 0; b < p->B; ++b)
    TN_RETURN_IF(apply_phys(ctx, chl, d, chr, p->site[i] + b * p->cap[i], tmp + b * e, dG));
  return copy_instances(ctx, p->site[i], p->cap[i], tmp, e, e, p->B);
}

tn_status_t upload_gates(tn_mps* p, const void* h, size_t elems) {
  tn_ctx* ctx = p->ctx;
  if (elems > p->gates_cap) {
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (p->gates) TN_RETURN_IF(tn_dev_free(ctx, p->gates));
    p->gates = nullptr;  // a failed allocation below must not leave the freed buffer in use
    p->gates_cap = 0;
    void* np = nullptr;
    TN_RETURN_IF(tn_dev_alloc(ctx, elems * sizeof(cxd), &np));
    p->gates = (cxd*)np;
    p->gates_cap = elems;
  }
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(p->gates, h, elems * sizeof(cxd), cudaMemcpyHostToDevice, ctx->stream));
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// environments (overlap.jl:36-50): F (χb × χa) ← Bᴴ · (F · A), all instances
// ---------------------------------------------------------------------------------
tn_status_t overlap_impl(const tn_mps* a, const tn_mps* b, double* h_out) {
  tn_ctx* ctx = a->ctx;
  const int L = a->L, d = a->d, B = a->B;
  int64_t mx = 1;
  for (int i = 0; i <= L; ++i) mx = std::max({mx, a->bond[i], b->bond[i]});
  const size_t env = (size_t)(mx * mx), t = (size_t)(mx * d * mx);
  TN_RETURN_IF(ws_reserve(ctx, 2 * ws_round(sizeof(cxd) * env * B) + ws_round(sizeof(cxd) * t * B)));
  cxd* F = ws_take<cxd>(ctx, env * B);
  cxd* F2 = ws_take<cxd>(ctx, env * B);
  cxd* T = ws_take<cxd>(ctx, t * B);
  TN_RETURN_IF(set_one(ctx, F, env, B));
  for (int i = 1; i <= L; ++i) {
    const int64_t xa = a->bond[i - 1], xa2 = a->bond[i], yb = b->bond[i - 1], yb2 = b->bond[i];
    // T (yb × d xa2) = F (yb × xa) · A (xa × d xa2)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', yb, d * xa2, xa, kOne, F, yb, env, a->site[i], xa, a->cap[i], kZero, T,
                                 yb, t, B));
    // F2 (yb2 × xa2) = B_matᴴ ((yb d) × yb2)ᴴ · T ((yb d) × xa2)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', yb2, xa2, yb * d, kOne, b->site[i], yb * d, b->cap[i], T, yb * d, t,
                                 kZero, F2, yb2, env, B));
    std::swap(F, F2);
  }
  TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(h_out, sizeof(cxd), F, env * sizeof(cxd), sizeof(cxd), B, cudaMemcpyDeviceToHost,
                                       ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

// Sampling step at one site for every shot q (one block per shot): marginals
// p_s = Σ_r |T[q, s, r]|² of the projected site T = P·A (the sites to the right are right
// isometries), outcome s by inverse CDF of the caller's uniform u (scaled by Σ_s p_s),
// new projector row P[q, :] = T[q, s, :] / √p_s (sample.jl:34-70).  d ≤ 32.
__global__ void __launch_bounds__(128) k_sample_site(int64_t ns, int d, int64_t chr, const cxd* __restrict__ T,
                                                     const double* __restrict__ u, int64_t L, int site,
                                                     cxd* __restrict__ P, int32_t* __restrict__ out, int last) {
  __shared__ double red[4][32];
  __shared__ double p[32];
  __shared__ int s_choice;
  const int64_t q = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = 0; s < d; ++s) {
    double acc = 0;
    for (int64_t r = threadIdx.x; r < chr; r += blockDim.x) acc += abs2(T[q + ((int64_t)s + (int64_t)d * r) * ns]);
    acc = warp_sum(acc);
    if (lane == 0) red[warp][s] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0;
    for (int s = 0; s < d; ++s) {
      p[s] = red[0][s] + red[1][s] + red[2][s] + red[3][s];
      tot += p[s];
    }
    const double target = u[q * L + site] * tot;
    double c = 0;
    int ch = d - 1;
    for (int s = 0; s < d; ++s) {
      c += p[s];
      if (target < c) {
        ch = s;
        break;
      }
    }
    while (ch > 0 && p[ch] == 0.0) --ch;  // never pick an outcome of probability zero
    s_choice = ch;
    out[q * L + site] = ch + 1;  // 1-based, as the reference's samples
  }
  __syncthreads();
  if (last) return;
  const int ch = s_choice;
  const double sc = p[ch] > 0 ? 1.0 / sqrt(p[ch]) : 0.0;
  for (int64_t r = threadIdx.x; r < chr; r += blockDim.x) {
    const cxd t = T[q + ((int64_t)ch + (int64_t)d * r) * ns];
    P[q + r * ns] = mkcx(t.x * sc, t.y * sc);
  }
}

tn_status_t check_site_arg(const tn_mps* p, int32_t b, int32_t i) {
  if (b < 0 || b >= p->B) return tn_set_error(p->ctx, TN_EINVAL, "instance %d out of range (B=%d)", b, p->B);
  if (i < 1 || i > p->L) return tn_set_error(p->ctx, TN_EINVAL, "site %d out of range", i);
  return TN_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" {

tn_status_t tn_mps_create_batched(tn_ctx* ctx, int32_t B, int32_t L, int32_t d, const int64_t* bond_dims,
                                  int64_t max_bond, tn_precision_t prec, tn_mps** out) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, L >= 2 && d >= 1 && out, "tn_mps_create: need L >= 2, d >= 1");
  TN_ARG(ctx, B >= 1 && B <= 8192, "tn_mps_create: batch must be in 1..8192");
  TN_ARG(ctx, bond_dims != nullptr, "tn_mps_create: null bond_dims");
  tn_mps* p = new tn_mps();
  p->ctx = ctx;
  p->L = L;
  p->d = d;
  p->B = B;
  p->prec = prec;
  p->bond.assign(L + 1, 1);
  p->cap_bond.assign(L + 1, 1);
  for (int i = 1; i < L; ++i) {
    if (bond_dims[i - 1] < 1) {
      delete p;
      return tn_set_error(ctx, TN_EINVAL, "tn_mps_create: bond %d < 1", i);
    }
    p->bond[i] = bond_dims[i - 1];
    // the largest bond a gauge move or gate can produce: min(d^i, d^(L-i)), capped
    double lg = std::min(i, L - i) * std::log((double)d);
    int64_t clamp = lg > 40 ? (int64_t)1 << 40 : (int64_t)std::llround(std::pow((double)d, std::min(i, L - i)));
    int64_t c = max_bond > 0 ? std::min(max_bond, clamp) : p->bond[i];
    p->cap_bond[i] = std::max(c, p->bond[i]);
  }
  p->site.assign(L + 1, nullptr);
  p->cap.assign(L + 1, 0);
  for (int i = 1; i <= L; ++i) {
    // elements per instance, checked against int64 overflow (a capacity is a bond the caller
    // gave or d^min(i, L-i), both unbounded here)
    const int64_t cl = p->cap_bond[i - 1], cr = p->cap_bond[i];
    tn_status_t st = TN_OK;
    if (cl > INT64_MAX / (int64_t)sizeof(cxd) / B / d / cr)
      st = tn_set_error(ctx, TN_EINVAL, "tn_mps_create: site %d of %lld x %d x %lld elements is too large", i,
                        (long long)cl, d, (long long)cr);
    const size_t e = st == TN_OK ? (size_t)(cl * d * cr) : 0;
    if (st == TN_OK) st = ensure_site(p, i, e);
    if (st == TN_OK) {
      const cudaError_t ce = cudaMemsetAsync(p->site[i], 0, e * B * sizeof(cxd), ctx->stream);
      if (ce != cudaSuccess) st = tn_set_error(ctx, TN_ECUDA, "tn_mps_create: %s", cudaGetErrorString(ce));
    }
    if (st != TN_OK) {
      for (int j = 1; j <= L; ++j)
        if (p->site[j]) tn_dev_free(ctx, p->site[j]);
      delete p;
      return st;
    }
  }
  p->kind = TN_FORM_MIXED;
  p->lo = 1;
  p->hi = L;
  ctx->refs++;
  *out = p;
  return TN_OK;
}

tn_status_t tn_mps_create(tn_ctx* ctx, int32_t L, int32_t d, const int64_t* bond_dims, int64_t max_bond,
                          tn_precision_t prec, tn_mps** out) {
  return tn_mps_create_batched(ctx, 1, L, d, bond_dims, max_bond, prec, out);
}

tn_status_t tn_mps_batch_size(const tn_mps* p, int32_t* B) {
  if (!p || !B) return TN_EINVAL;
  *B = p->B;
  return TN_OK;
}

tn_status_t tn_mps_destroy(tn_mps* p) {
  if (!p) return TN_OK;
  tn_ctx* ctx = p->ctx;
  cudaStreamSynchronize(ctx->stream);
  for (int i = 1; i <= p->L; ++i)
    if (p->site[i]) tn_dev_free(ctx, p->site[i]);
  if (p->lam) tn_dev_free(ctx, p->lam);
  if (p->gates) tn_dev_free(ctx, p->gates);
  delete p;
  if (--ctx->refs == 0 && ctx->destroy_requested) ctx_release(ctx);
  return TN_OK;
}

tn_status_t tn_mps_copy(const tn_mps* src, tn_mps** out) {
  if (!src || !out) return TN_EINVAL;
  tn_ctx* ctx = src->ctx;
  std::vector<int64_t> b(src->bond.begin() + 1, src->bond.end() - 1);
  tn_mps* p = nullptr;
  TN_RETURN_IF(tn_mps_create_batched(ctx, src->B, src->L, src->d, b.data(), 0, src->prec, &p));
  for (int i = 1; i <= src->L; ++i) {
    tn_status_t st = ensure_site(p, i, src->cap[i]);
    if (st == TN_OK) st = copy_instances(ctx, p->site[i], p->cap[i], src->site[i], src->cap[i], (size_t)sz(src, i), src->B);
    if (st != TN_OK) {
      tn_mps_destroy(p);
      return st;
    }
  }
  p->cap_bond = src->cap_bond;
  p->kind = src->kind;
  p->lo = src->lo;
  p->hi = src->hi;
  if (src->lam_len > 0) {
    tn_status_t st = ensure_lam(p, src->lam_len);
    if (st == TN_OK) {
      const cudaError_t e = cudaMemcpy2DAsync(p->lam, p->lam_cap * sizeof(double), src->lam,
                                              src->lam_cap * sizeof(double), src->lam_len * sizeof(double), src->B,
                                              cudaMemcpyDeviceToDevice, ctx->stream);
      if (e != cudaSuccess) st = tn_set_error(ctx, TN_ECUDA, "tn_mps_copy: %s", cudaGetErrorString(e));
    }
    if (st != TN_OK) {
      tn_mps_destroy(p);
      return st;
    }
    p->lam_len = src->lam_len;
  }
  *out = p;
  return TN_OK;
}

tn_status_t tn_mps_set_instance_site(tn_mps* p, int32_t b, int32_t i, int64_t chl, int64_t chr, const void* h) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_RETURN_IF(check_site_arg(p, b, i));
  TN_ARG(ctx, h != nullptr, "tn_mps_set_site: null data");
  TN_ARG(ctx, (i > 1 || chl == 1) && (i < p->L || chr == 1), "tn_mps_set_site: open-end bonds must be 1");
  TN_ARG(ctx, chl == p->bond[i - 1] && chr == p->bond[i],
         "tn_mps_set_site: bond dimensions differ from the MPS's (set them at creation)");
  TN_RETURN_IF(ensure_site(p, i, (size_t)(chl * p->d * chr)));
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(p->site[i] + (size_t)b * p->cap[i], h, sizeof(cxd) * chl * p->d * chr,
                                     cudaMemcpyHostToDevice, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_mps_get_instance_site(const tn_mps* p, int32_t b, int32_t i, void* h) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_RETURN_IF(check_site_arg(p, b, i));
  TN_ARG(ctx, h != nullptr, "tn_mps_get_site: null output");
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h, p->site[i] + (size_t)b * p->cap[i], sizeof(cxd) * sz(p, i),
                                     cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_mps_set_instance_sites(tn_mps* p, int32_t b, const void* const* h) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_RETURN_IF(check_site_arg(p, b, 1));
  TN_ARG(ctx, h != nullptr, "tn_mps_set_instance_sites: null data");
  for (int i = 1; i <= p->L; ++i) TN_ARG(ctx, h[i - 1] != nullptr, "tn_mps_set_instance_sites: null site");
  for (int i = 1; i <= p->L; ++i) {
    TN_RETURN_IF(ensure_site(p, i, (size_t)sz(p, i)));
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(p->site[i] + (size_t)b * p->cap[i], h[i - 1], sizeof(cxd) * sz(p, i),
                                       cudaMemcpyHostToDevice, ctx->stream));
  }
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_mps_get_instance_sites(const tn_mps* p, int32_t b, void* const* h) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_RETURN_IF(check_site_arg(p, b, 1));
  TN_ARG(ctx, h != nullptr, "tn_mps_get_instance_sites: null output");
  for (int i = 1; i <= p->L; ++i) TN_ARG(ctx, h[i - 1] != nullptr, "tn_mps_get_instance_sites: null site");
  for (int i = 1; i <= p->L; ++i)
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h[i - 1], p->site[i] + (size_t)b * p->cap[i], sizeof(cxd) * sz(p, i),
                                       cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_mps_set_site(tn_mps* p, int32_t i, int64_t chl, int64_t chr, const void* h) {
  return tn_mps_set_instance_site(p, 0, i, chl, chr, h);
}

tn_status_t tn_mps_get_site(const tn_mps* p, int32_t i, void* h) { return tn_mps_get_instance_site(p, 0, i, h); }

tn_status_t tn_mps_bond_dims(const tn_mps* p, int64_t* h) {
  if (!p || !h) return TN_EINVAL;
  for (int i = 1; i < p->L; ++i) h[i - 1] = p->bond[i];
  return TN_OK;
}

tn_status_t tn_mps_set_precision(tn_mps* p, tn_precision_t prec) {
  if (!p) return TN_EINVAL;
  p->prec = prec;
  return TN_OK;
}

tn_status_t tn_mps_form(const tn_mps* p, int32_t* kind, int32_t* lo, int32_t* hi) {
  if (!p || !kind || !lo || !hi) return TN_EINVAL;
  *kind = p->kind;
  *lo = p->lo;
  *hi = p->hi;
  return TN_OK;
}

tn_status_t tn_mps_set_form(tn_mps* p, int32_t kind, int32_t lo, int32_t hi) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, kind == TN_FORM_NONCANONICAL || kind == TN_FORM_MIXED, "tn_mps_set_form: only NonCanonical or Mixed");
  if (kind == TN_FORM_MIXED) TN_ARG(ctx, 1 <= lo && lo <= hi && hi <= p->L, "tn_mps_set_form: bad centre");
  TN_ARG(ctx, p->kind != TN_FORM_BOND, "tn_mps_set_form: the MPS holds a Λ; canonize it to a mixed form first");
  p->kind = kind;
  p->lo = kind == TN_FORM_MIXED ? lo : 1;
  p->hi = kind == TN_FORM_MIXED ? hi : p->L;
  return TN_OK;
}

tn_status_t tn_mps_get_lambda(const tn_mps* p, double* h, int64_t* len) {
  if (!p || !len) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, p->kind == TN_FORM_BOND, "tn_mps_get_lambda: MPS is not bond-canonical");
  *len = p->lam_len;
  if (h && p->lam_len > 0) {
    TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(h, sizeof(double) * p->lam_len, p->lam, sizeof(double) * p->lam_cap,
                                         sizeof(double) * p->lam_len, p->B, cudaMemcpyDeviceToHost, ctx->stream));
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return TN_OK;
}

tn_status_t tn_mps_canonize_mixed(tn_mps* p, int32_t lo, int32_t hi) {
  if (!p) return TN_EINVAL;
  TN_ARG(p->ctx, 1 <= lo && lo <= hi && hi <= p->L, "canonize: centre out of range");
  return canonize_mixed(p, lo, hi);
}

tn_status_t tn_mps_canonize_bond(tn_mps* p, int32_t a) {
  if (!p) return TN_EINVAL;
  TN_ARG(p->ctx, 1 <= a && a < p->L, "canonize: bond out of range");
  return canonize_bond(p, a);
}

tn_status_t tn_mps_compress(tn_mps* p, int32_t a, int64_t maxdim, double threshold) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  // compress.jl:30-32
  TN_ARG(ctx, maxdim > 0 || threshold > 0, "Either `maxdim` or `threshold` must be specified");
  TN_ARG(ctx, 0 <= a && a < p->L, "compress: bond out of range");
  if (a == 0) {
    for (int i = 1; i < p->L; ++i) TN_RETURN_IF(tn_mps_compress(p, i, maxdim, threshold));
    return TN_OK;
  }
  TN_RETURN_IF(canonize_bond(p, a));
  if (p->lam_len == 0) return TN_OK;
  const int64_t k = p->lam_len;
  int64_t r = 0;
  TN_RETURN_IF(rank_select_batched(ctx, p->lam, k, p->lam_cap, p->B, maxdim, threshold, &r, nullptr));
  if (r == k) return TN_OK;
  // site a (χl d × k): the first r columns are a column-major prefix; site a+1 (k × d χr)
  // keeps its first r rows
  const int64_t n = p->d * p->bond[a + 1];
  TN_RETURN_IF(ws_reserve(ctx, ws_round(sizeof(cxd) * (size_t)(p->B * r * n))));
  cxd* tmp = ws_take<cxd>(ctx, (size_t)(p->B * r * n));
  TN_RETURN_IF(copy_matrix_cxd(ctx, r, n, p->site[a + 1], k, tmp, r, p->cap[a + 1], r * n, p->B));
  TN_RETURN_IF(copy_instances(ctx, p->site[a + 1], p->cap[a + 1], tmp, r * n, r * n, p->B));
  p->bond[a] = r;
  p->lam_len = r;
  return TN_OK;
}

tn_status_t tn_mps_simple_update(tn_mps* p, int32_t n_sites, int32_t a, const void* h_G, int64_t maxdim,
                                 double threshold) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, h_G != nullptr, "simple_update: null gate");
  TN_ARG(ctx, n_sites == 1 || n_sites == 2, "Operator must act on one or two sites");
  TN_ARG(ctx, a >= 1 && (int64_t)a + n_sites - 1 <= p->L, "Operator plugs must be present in the MPS");
  size_t ge = n_sites == 1 ? (size_t)(p->d * p->d) : (size_t)(p->d * p->d * p->d * p->d);
  TN_RETURN_IF(upload_gates(p, h_G, ge));
  TN_RETURN_IF(canonize_mixed(p, a, a + n_sites - 1));
  if (n_sites == 1) return apply_gate1(p, a, p->gates);
  return apply_gate2(p, a, p->gates, maxdim, threshold);
}

tn_status_t tn_mps_evolve_brickwork(tn_mps* p, int32_t n_layers, const int32_t* starts, const int32_t* n_gates,
                                    const void* h_gates, int64_t maxdim, double threshold) {
  return tn_mps_evolve_layers(p, n_layers, starts, n_gates, nullptr, h_gates, maxdim, threshold);
}

tn_status_t tn_mps_evolve_layers(tn_mps* p, int32_t n_layers, const int32_t* starts, const int32_t* n_gates,
                                 const int32_t* reverse, const void* h_gates, int64_t maxdim, double threshold) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, n_layers >= 0 && starts && n_gates && h_gates, "evolve: bad arguments");
  size_t total = 0;
  const size_t g4 = (size_t)p->d * p->d * p->d * p->d;
  for (int l = 0; l < n_layers; ++l) {
    TN_ARG(ctx, n_gates[l] >= 0 && starts[l] >= 1 && (int64_t)starts[l] + 2 * (int64_t)n_gates[l] - 1 <= p->L,
           "evolve: layer out of range");
    total += (size_t)n_gates[l] * g4;
  }
  if (total == 0) return TN_OK;
  TN_RETURN_IF(upload_gates(p, h_gates, total));
  size_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    const bool rev = reverse && reverse[l];
    for (int q = 0; q < n_gates[l]; ++q) {
      // gates are stored left to right; a reversed layer applies them right to left
      const int g = rev ? n_gates[l] - 1 - q : q;
      const int a = starts[l] + 2 * g;
      // within a layer the next gate lies further along the sweep: S goes to the site on
      // that side, whose QR (LQ) the centre move needs anyway, and the other site is left
      // isometric.  The last gate of a layer keeps Tenet's AbsorbEqually, so every layer
      // (and the call) ends in the reference's form (MixedCanonical([a, a+1])) and split.
      const int absorb = q + 1 < n_gates[l] ? (rev ? kAbsorbLeft : kAbsorbRight) : kAbsorbEqually;
      TN_RETURN_IF(canonize_mixed(p, a, a + 1));
      TN_RETURN_IF(apply_gate2(p, a, p->gates + (size_t)g * g4 + off, maxdim, threshold, absorb));
    }
    off += (size_t)n_gates[l] * g4;
  }
  return TN_OK;
}

tn_status_t tn_mps_overlap(const tn_mps* a, const tn_mps* b, double* h_out) {
  if (!a || !b || !h_out) return TN_EINVAL;
  TN_ARG(a->ctx, a->L == b->L && a->d == b->d, "overlap: nsites differ");
  TN_ARG(a->ctx, a->B == b->B, "overlap: batch sizes differ");
  TN_ARG(a->ctx, a->ctx == b->ctx, "overlap: MPS belong to different contexts");
  TN_ARG(a->ctx, a->kind != TN_FORM_BOND && b->kind != TN_FORM_BOND,
         "overlap: absorb Λ first (canonize the MPS to a mixed form)");
  return overlap_impl(a, b, h_out);
}

tn_status_t tn_mps_norm(tn_mps* p, double* h_out) {
  if (!p || !h_out) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  if (p->kind == TN_FORM_NONCANONICAL) {
    p->kind = TN_FORM_MIXED;
    p->lo = 1;
    p->hi = p->L;
  }
  if (p->kind == TN_FORM_BOND) return norms_batched(ctx, false, p->lam_len, p->lam, p->lam_cap, p->B, h_out);
  const int c = p->lo;
  TN_RETURN_IF(canonize_mixed(p, c, c));
  return norms_batched(ctx, true, sz(p, c), p->site[c], p->cap[c], p->B, h_out);
}

tn_status_t tn_mps_normalize(tn_mps* p) {
  if (!p) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  std::vector<double> nrm(p->B);
  TN_RETURN_IF(tn_mps_norm(p, nrm.data()));
  for (int b = 0; b < p->B; ++b) {
    TN_ARG(ctx, nrm[b] > 0, "normalize: zero norm");
    if (p->kind == TN_FORM_BOND)
      TN_RETURN_IF(tn_scale(ctx, TN_F64, p->lam_len, p->lam + b * p->lam_cap, 1.0 / nrm[b]));
    else
      TN_RETURN_IF(tn_scale(ctx, TN_C64, sz(p, p->lo), p->site[p->lo] + b * p->cap[p->lo], 1.0 / nrm[b]));
  }
  return TN_OK;
}

tn_status_t tn_mps_amplitude(const tn_mps* p, const void* h_vectors, double* h_out) {
  if (!p || !h_vectors || !h_out) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, p->kind != TN_FORM_BOND, "amplitude: absorb Λ first (canonize the MPS to a mixed form)");
  const int L = p->L, d = p->d, B = p->B;
  int64_t mx = 1;
  for (int i = 0; i <= L; ++i) mx = std::max(mx, p->bond[i]);
  const size_t ve = (size_t)(mx * d);
  TN_RETURN_IF(ws_reserve(ctx, 2 * ws_round(sizeof(cxd) * ve * B) + ws_round(sizeof(cxd) * (size_t)(L * d))));
  cxd* e = ws_take<cxd>(ctx, ve * B);
  cxd* u = ws_take<cxd>(ctx, ve * B);
  cxd* v = ws_take<cxd>(ctx, (size_t)(L * d));
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(v, h_vectors, sizeof(cxd) * L * d, cudaMemcpyHostToDevice, ctx->stream));
  TN_RETURN_IF(set_one(ctx, e, ve, B));
  for (int i = 1; i <= L; ++i) {
    const int64_t xl = p->bond[i - 1], xr = p->bond[i];
    // u (1 × d xr) = e (1 × xl) · A (xl × d xr)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', 1, d * xr, xl, kOne, e, 1, ve, p->site[i], xl, p->cap[i], kZero, u, 1,
                                 ve, B));
    // e (1 × xr) = vᵀ (1 × d) · u as (d × xr)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'T', 'N', 1, xr, d, kOne, v + (int64_t)(i - 1) * d, d, 0, u, d, ve, kZero, e, 1,
                                 ve, B));
  }
  TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(h_out, sizeof(cxd), e, ve * sizeof(cxd), sizeof(cxd), B, cudaMemcpyDeviceToHost,
                                       ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

tn_status_t tn_mps_local_expectations(const tn_mps* p, const void* h_op, double* h_out) {
  if (!p || !h_op || !h_out) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, p->kind != TN_FORM_BOND, "expectation: absorb Λ first (canonize the MPS to a mixed form)");
  const int L = p->L, d = p->d, B = p->B;
  int64_t mx = 1;
  for (int i = 0; i <= L; ++i) mx = std::max(mx, p->bond[i]);
  // right environments R_2..R_{L+1} kept; the left environment is swept
  const size_t env = (size_t)(mx * mx), t = (size_t)(mx * d * mx);
  size_t need = (size_t)(L + 4) * ws_round(sizeof(cxd) * env * B) + 3 * ws_round(sizeof(cxd) * t * B) +
                ws_round(sizeof(cxd) * (size_t)(d * d));
  TN_RETURN_IF(ws_reserve(ctx, need));
  std::vector<cxd*> R(L + 2);
  for (int i = 0; i <= L + 1; ++i) R[i] = ws_take<cxd>(ctx, env * B);
  cxd* F = ws_take<cxd>(ctx, env * B);
  cxd* F2 = ws_take<cxd>(ctx, env * B);
  cxd* T1 = ws_take<cxd>(ctx, t * B);
  cxd* T2 = ws_take<cxd>(ctx, t * B);
  cxd* OA = ws_take<cxd>(ctx, t * B);
  cxd* dO = ws_take<cxd>(ctx, (size_t)(d * d));
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(dO, h_op, sizeof(cxd) * d * d, cudaMemcpyHostToDevice, ctx->stream));
  TN_RETURN_IF(set_one(ctx, F, env, B));
  TN_RETURN_IF(set_one(ctx, R[L + 1], env, B));
  for (int i = L; i > 1; --i) {
    const int64_t x = p->bond[i - 1], x2 = p->bond[i];
    // T1 (x d × x2) = A (x d × x2) · R_{i+1} (x2 × x2)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', x * d, x2, x2, kOne, p->site[i], x * d, p->cap[i], R[i + 1], x2, env,
                                 kZero, T1, x * d, t, B));
    // R_i (x × x) = T1 as (x × d x2) · A as (x × d x2)ᴴ
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'C', x, x, d * x2, kOne, T1, x, t, p->site[i], x, p->cap[i], kZero, R[i], x,
                                 env, B));
  }
  std::vector<double> val(2 * B), nrm(2 * B);
  for (int i = 1; i <= L; ++i) {
    const int64_t x = p->bond[i - 1], x2 = p->bond[i];
    for (int pass = 0; pass < (i == 1 ? 2 : 1); ++pass) {
      const cxd* Ain = p->site[i];
      int64_t sAin = p->cap[i];
      if (pass == 0) {
        // OA[l, a, r] = Σ_b O[a, b] A[l, b, r]
        for (int b = 0; b < B; ++b) TN_RETURN_IF(apply_phys(ctx, x, d, x2, p->site[i] + b * p->cap[i], OA + b * t, dO));
        Ain = OA;
        sAin = t;
      }
      TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', x, d * x2, x, kOne, F, x, env, Ain, x, sAin, kZero, T1, x, t, B));
      TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', x * d, x2, x2, kOne, T1, x * d, t, R[i + 1], x2, env, kZero, T2, x * d,
                                   t, B));
      TN_RETURN_IF(zdotc_batched(ctx, x * d * x2, p->site[i], p->cap[i], T2, t, B, pass == 0 ? val.data() : nrm.data()));
      if (pass == 0)
        for (int b = 0; b < B; ++b) {
          h_out[2 * ((size_t)b * L + i - 1)] = val[2 * b];
          h_out[2 * ((size_t)b * L + i - 1) + 1] = val[2 * b + 1];
        }
    }
    if (i < L) {
      // F ← Aᴴ · (F · A)
      TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', x, d * x2, x, kOne, F, x, env, p->site[i], x, p->cap[i], kZero, T1, x,
                                   t, B));
      TN_RETURN_IF(gemm_cx<double>(ctx, 'C', 'N', x2, x2, x * d, kOne, p->site[i], x * d, p->cap[i], T1, x * d, t, kZero,
                                   F2, x2, env, B));
      std::swap(F, F2);
    }
  }
  // divide by ⟨ψ|ψ⟩ per instance
  for (int b = 0; b < B; ++b) {
    const double nx = nrm[2 * b], ny = nrm[2 * b + 1], nn = nx * nx + ny * ny;
    for (int i = 0; i < L; ++i) {
      double* o = h_out + 2 * ((size_t)b * L + i);
      const double a = o[0], c = o[1];
      o[0] = (a * nx + c * ny) / nn;
      o[1] = (c * nx - a * ny) / nn;
    }
  }
  return TN_OK;
}

// sample(ψ, nsamples) (src/Operations/sample.jl:20-72) for one instance, with the
// caller's uniforms (nshots × L, row-major) in place of the reference's RNG: moves the
// orthogonality centre to site 1 (canonize!(ψ, MixedCanonical(1)), as the reference does
// on a copy), then sweeps the sites once with all shots batched (one GEMM per site).
tn_status_t tn_mps_sample(tn_mps* p, int32_t instance, int64_t nshots, const double* h_uniforms, int32_t* h_out) {
  if (!p || !h_uniforms || !h_out) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  TN_ARG(ctx, instance >= 0 && instance < p->B, "sample: instance out of range");
  TN_ARG(ctx, nshots >= 1, "sample: nshots must be positive");
  TN_ARG(ctx, p->d <= 32, "sample: physical dimension above 32");
  TN_RETURN_IF(tn_mps_canonize_mixed(p, 1, 1));
  const int L = p->L, d = p->d;
  int64_t mx = 1;
  for (int i = 0; i <= L; ++i) mx = std::max(mx, p->bond[i]);
  const size_t need = ws_round(sizeof(cxd) * (size_t)(nshots * mx)) + ws_round(sizeof(cxd) * (size_t)(nshots * d * mx)) +
                      ws_round(sizeof(double) * (size_t)(nshots * L)) + ws_round(sizeof(int32_t) * (size_t)(nshots * L));
  TN_RETURN_IF(ws_reserve(ctx, need));
  cxd* P = ws_take<cxd>(ctx, (size_t)(nshots * mx));
  cxd* T = ws_take<cxd>(ctx, (size_t)(nshots * d * mx));
  double* U = ws_take<double>(ctx, (size_t)(nshots * L));
  int32_t* O = ws_take<int32_t>(ctx, (size_t)(nshots * L));
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(U, h_uniforms, sizeof(double) * nshots * L, cudaMemcpyHostToDevice, ctx->stream));
  TN_RETURN_IF(set_one(ctx, P, 1, nshots));
  for (int i = 1; i <= L; ++i) {
    const int64_t xl = p->bond[i - 1], xr = p->bond[i];
    const cxd* A = p->site[i] + (size_t)instance * p->cap[i];
    // T (nshots × d xr) = P (nshots × xl) · A (xl × d xr)
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', nshots, d * xr, xl, kOne, P, nshots, 0, A, xl, 0, kZero, T, nshots, 0, 1));
    k_sample_site<<<(unsigned)nshots, 128, 0, ctx->stream>>>(nshots, d, xr, T, U, L, i - 1, P, O, i == L ? 1 : 0);
    TN_LAUNCHED(ctx);
  }
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(h_out, O, sizeof(int32_t) * nshots * L, cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// MPO × MPS evolution (src/Operations/evolve.jl:19-137).  MPO site i is column-major
// (w_{i-1}, d_out, d_in, w_i) C64, w_0 = w_L = 1, d_out = d_in = d.
// ---------------------------------------------------------------------------------
namespace {

typedef double2 pd2;  // permute_t element for ComplexF64

// direct method (evolve.jl:19-46) for every instance: new site i = A_i · W_i over the
// physical index with (χ, w) fused on both bonds, χ fastest; then MixedCanonical(all)
tn_status_t evolve_mpo_direct(tn_mps* p, const std::vector<const cxd*>& hW, const std::vector<int64_t>& w) {
  tn_ctx* ctx = p->ctx;
  const int L = p->L, d = p->d, B = p->B;
  std::vector<cxd*> nsite(L + 1, nullptr);
  std::vector<size_t> ncap(L + 1, 0);
  // new site i into nsite[i]; on any failure the caller frees every nsite[] made so far
  auto build_site = [&](int i) -> tn_status_t {
    const int64_t l = p->bond[i - 1], r = p->bond[i], a = w[i - 1], b = w[i];
    const int64_t nel = l * a * d * r * b;
    const size_t need = ws_round(sizeof(cxd) * (size_t)(a * d * d * b)) * 2 +
                        ws_round(sizeof(cxd) * (size_t)(l * r * d * B)) + 2 * ws_round(sizeof(cxd) * (size_t)(nel * B));
    TN_RETURN_IF(ws_reserve(ctx, need));
    void* np = nullptr;
    TN_RETURN_IF(tn_dev_alloc(ctx, sizeof(cxd) * (size_t)nel * B, &np));
    nsite[i] = (cxd*)np;
    ncap[i] = (size_t)nel;
    cxd* W0 = ws_take<cxd>(ctx, (size_t)(a * d * d * b));
    cxd* W1 = ws_take<cxd>(ctx, (size_t)(a * d * d * b));
    cxd* A1 = ws_take<cxd>(ctx, (size_t)(l * r * d * B));
    cxd* C1 = ws_take<cxd>(ctx, (size_t)(nel * B));
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(W0, hW[i - 1], sizeof(cxd) * a * d * d * b, cudaMemcpyHostToDevice, ctx->stream));
    // A' (l, r, s) per instance: dims (l, s, r, B), instance stride = capacity
    {
      const int64_t dims[4] = {l, d, r, B};
      const int64_t str[4] = {1, l, l * d, (int64_t)p->cap[i]};
      const int32_t perm[4] = {0, 2, 1, 3};
      TN_RETURN_IF(permute_t<pd2>(ctx, 4, dims, str, perm, (const pd2*)p->site[i], (pd2*)A1, false));
    }
    // W' (s, a, o, b) from W (a, o, s, b)
    {
      const int64_t dims[4] = {a, d, d, b};
      const int32_t perm[4] = {2, 0, 1, 3};
      TN_RETURN_IF(permute_t<pd2>(ctx, 4, dims, nullptr, perm, (const pd2*)W0, (pd2*)W1, false));
    }
    // C' ((l r) × (a o b)) = A' ((l r) × s) · W' (s × (a o b)), batched over instances
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', l * r, a * d * b, d, kOne, A1, l * r, l * r * d, W1, d, 0, kZero, C1,
                                 l * r, nel, B));
    // new site (l, a, o, r, b) from C' (l, r, a, o, b)
    {
      const int64_t dims[6] = {l, r, a, d, b, B};
      const int32_t perm[6] = {0, 2, 3, 1, 4, 5};
      TN_RETURN_IF(permute_t<pd2>(ctx, 6, dims, nullptr, perm, (const pd2*)C1, (pd2*)nsite[i], false));
    }
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // W0 came from pageable host memory
    return TN_OK;
  };
  for (int i = 1; i <= L; ++i) {
    const tn_status_t st = build_site(i);
    if (st != TN_OK) {
      cudaStreamSynchronize(ctx->stream);
      for (int j = 1; j <= i; ++j)
        if (nsite[j]) tn_dev_free(ctx, nsite[j]);
      return st;
    }
  }
  for (int i = 1; i <= L; ++i) {
    TN_RETURN_IF(tn_dev_free(ctx, p->site[i]));
    p->site[i] = nsite[i];
    p->cap[i] = ncap[i];
  }
  for (int i = 1; i < L; ++i) {
    p->bond[i] *= w[i];
    p->cap_bond[i] = std::max(p->cap_bond[i], p->bond[i]);
  }
  p->kind = TN_FORM_MIXED;  // canonize!(ψ, MixedCanonical(sites(ψ))): no arithmetic
  p->lo = 1;
  p->hi = L;
  p->lam_len = 0;
  return TN_OK;
}

// zip-up (evolve.jl:49-129), every instance of the MPS in lockstep: the carried block,
// the contractions and the truncated SVDs are batched over the B instances (instance
// stride = the largest block), the common new bond is the largest kept rank, and an
// instance's surplus singular values are zero (rank_select_batched), so each instance
// carries exactly its own truncated state
tn_status_t evolve_mpo_zipup(tn_mps* p, const std::vector<const cxd*>& hW, const std::vector<int64_t>& w,
                             int64_t maxdim, double threshold) {
  tn_ctx* ctx = p->ctx;
  const int L = p->L, d = p->d, B = p->B;
  std::vector<int64_t> ob(p->bond);  // bonds before the sweep
  int64_t mx = 1, wm = 1;
  for (int i = 0; i <= L; ++i) {
    mx = std::max(mx, ob[i]);
    wm = std::max(wm, w[i]);
  }
  const int64_t km = std::max<int64_t>(d * mx * wm, 1);  // largest carried bond before truncation
  const int64_t big = km * d * mx * wm;                   // largest (k o) × (r b) block
  const int64_t rows = km * d, cols = mx * wm, kk = std::min(rows, cols);
  const size_t need = 2 * ws_round(sizeof(cxd) * (size_t)(wm * d * d * wm)) +
                      5 * ws_round(sizeof(cxd) * (size_t)(big * B)) + ws_round(sizeof(cxd) * (size_t)(rows * kk * B)) +
                      ws_round(sizeof(double) * (size_t)(kk * B)) + ws_round(sizeof(cxd) * (size_t)(kk * cols * B)) +
                      svd_any_workspace(TN_C64, p->prec, rows, cols, B);
  TN_RETURN_IF(ws_reserve(ctx, need));
  cxd* W0 = ws_take<cxd>(ctx, (size_t)(wm * d * d * wm));
  cxd* W1 = ws_take<cxd>(ctx, (size_t)(wm * d * d * wm));
  cxd* R = ws_take<cxd>(ctx, (size_t)(big * B));
  cxd* X = ws_take<cxd>(ctx, (size_t)(big * B));
  cxd* Y = ws_take<cxd>(ctx, (size_t)(big * B));
  cxd* T = ws_take<cxd>(ctx, (size_t)(big * B));
  cxd* Tm = ws_take<cxd>(ctx, (size_t)(big * B));
  cxd* U = ws_take<cxd>(ctx, (size_t)(rows * kk * B));
  double* S = ws_take<double>(ctx, (size_t)(kk * B));
  cxd* Vh = ws_take<cxd>(ctx, (size_t)(kk * cols * B));
  TN_RETURN_IF(set_one(ctx, R, big, B));  // the carried block before site 1: (k = 1, χ_0 = 1, w_0 = 1)
  int64_t k = 1;
  for (int i = 1; i <= L; ++i) {
    const int64_t c = ob[i - 1], r = ob[i], a = w[i - 1], b = w[i];
    TN_CHECK_CUDA(ctx, cudaMemcpyAsync(W0, hW[i - 1], sizeof(cxd) * a * d * d * b, cudaMemcpyHostToDevice, ctx->stream));
    // R (k, c, a) → (k, a, c) per instance (the last mode is the instance, stride big)
    {
      const int64_t dims[4] = {k, c, a, B};
      const int64_t str[4] = {1, k, k * c, big};
      const int32_t perm[4] = {0, 2, 1, 3};
      TN_RETURN_IF(permute_t<pd2>(ctx, 4, dims, str, perm, (const pd2*)R, (pd2*)Y, false));
    }
    // X ((k a) × (s r)) = R' ((k a) × c) · A (c × (s r)), Y packed at stride k·a·c
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', k * a, d * r, c, kOne, Y, k * a, k * a * c, p->site[i], c, p->cap[i],
                                 kZero, X, k * a, big, B));
    // X (k, a, s, r) → (k, r, a, s) per instance;  W (a, o, s, b) → (a, s, o, b)
    {
      const int64_t dims[5] = {k, a, d, r, B};
      const int64_t str[5] = {1, k, k * a, k * a * d, big};
      const int32_t perm[5] = {0, 3, 1, 2, 4};
      TN_RETURN_IF(permute_t<pd2>(ctx, 5, dims, str, perm, (const pd2*)X, (pd2*)Y, false));
      const int64_t wd[4] = {a, d, d, b};
      const int32_t wp[4] = {0, 2, 1, 3};
      TN_RETURN_IF(permute_t<pd2>(ctx, 4, wd, nullptr, wp, (const pd2*)W0, (pd2*)W1, false));
    }
    // T ((k r) × (o b)) = Y ((k r) × (a s)) · W' ((a s) × (o b)); Y packed at stride k·r·a·d
    TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', k * r, d * b, a * d, kOne, Y, k * r, k * r * a * d, W1, a * d, 0, kZero,
                                 T, k * r, big, B));
    // T (k, r, o, b) → (k, o, r, b): the matrix ((k o) × (r b)), packed at stride m·n
    const int64_t m = k * d, n = r * b;
    {
      const int64_t dims[5] = {k, r, d, b, B};
      const int64_t str[5] = {1, k, k * r, k * r * d, big};
      const int32_t perm[5] = {0, 2, 1, 3, 4};
      TN_RETURN_IF(permute_t<pd2>(ctx, 5, dims, str, perm, (const pd2*)T, (pd2*)Tm, false));
    }
    if (i == L) {  // last site: (k, o, 1)
      TN_RETURN_IF(ensure_site(p, i, (size_t)(k * d)));
      TN_RETURN_IF(copy_instances(ctx, p->site[i], p->cap[i], Tm, (size_t)(m * n), (size_t)(k * d), B));
      p->bond[i - 1] = k;
      break;
    }
    const int64_t kmin = std::min(m, n);
    TN_RETURN_IF(svd_any(ctx, TN_C64, p->prec, m, n, Tm, m, m * n, U, m * kmin, S, kmin, Vh, kmin * n, B));
    int64_t rk = 0;
    TN_RETURN_IF(rank_select_batched(ctx, S, kmin, kmin, B, maxdim, threshold, &rk, nullptr));
    // site i = U[:, :rk] as (k, o, rk);  R = diag(S[:rk]) Vh[:rk, :] as (rk, r, b)
    TN_RETURN_IF(ensure_site(p, i, (size_t)(m * rk)));
    TN_RETURN_IF(copy_instances(ctx, p->site[i], p->cap[i], U, (size_t)(m * kmin), (size_t)(m * rk), B));
    TN_RETURN_IF(copy_matrix_cxd(ctx, rk, n, Vh, kmin, R, rk, kmin * n, big, B));
    TN_RETURN_IF(scale_rows_mode(ctx, R, rk, n, rk, S, big, kmin, B, 1));
    p->bond[i - 1] = k;
    k = rk;
    TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // W0 came from pageable host memory
  }
  for (int i = 1; i < L; ++i) p->cap_bond[i] = std::max(p->cap_bond[i], p->bond[i]);
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  p->lam_len = 0;  // the reference leaves the form as it was set before the sweep
  return TN_OK;
}

}  // namespace

extern "C" {

tn_status_t tn_mps_evolve_mpo(tn_mps* p, const void* const* h_mpo_sites, const int64_t* mpo_bonds, int32_t algorithm,
                              int64_t maxdim, double threshold) {
  if (!p || !h_mpo_sites) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  const int L = p->L;
  std::vector<int64_t> w(L + 1, 1);
  for (int i = 1; i < L; ++i) {
    TN_ARG(ctx, mpo_bonds && mpo_bonds[i - 1] >= 1, "evolve: MPO bond dimensions must be positive");
    w[i] = mpo_bonds[i - 1];
  }
  std::vector<const cxd*> hW(L);
  for (int i = 0; i < L; ++i) {
    TN_ARG(ctx, h_mpo_sites[i] != nullptr, "evolve: null MPO site");
    hW[i] = (const cxd*)h_mpo_sites[i];
  }
  if (algorithm == 0) return evolve_mpo_direct(p, hW, w);
  TN_ARG(ctx, algorithm == 1, "evolve: algorithm must be 0 (direct) or 1 (zip-up)");
  TN_ARG(ctx, maxdim > 0 || threshold > 0, "Either `maxdim` or `threhold` must be specified");
  if (p->kind == TN_FORM_BOND) TN_RETURN_IF(tn_mps_canonize_mixed(p, p->lo, p->lo));  // absorb Λ
  return evolve_mpo_zipup(p, hW, w, maxdim, threshold);
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// dump / load of a device MPS (warm restart of a pool, hand-over between processes).
// File: 8-byte magic "TNMPS001", int32 L, d, B, form kind, lo, hi, precision, int64
// lambda length, int64 bonds[0..L], then for each instance and site the column-major
// (χ_{i-1}, d, χ_i) ComplexF64 data, then Λ (B × lambda length doubles) if bond-canonical.
// ---------------------------------------------------------------------------------
namespace {
const char kMagic[8] = {'T', 'N', 'M', 'P', 'S', '0', '0', '1'};
}

extern "C" {

tn_status_t tn_mps_save(const tn_mps* p, const char* path) {
  if (!p || !path) return TN_EINVAL;
  tn_ctx* ctx = p->ctx;
  FILE* f = fopen(path, "wb");
  if (!f) return tn_set_error(ctx, TN_EINVAL, "tn_mps_save: cannot open %s", path);
  const int32_t hdr[7] = {p->L, p->d, p->B, p->kind, p->lo, p->hi, (int32_t)p->prec};
  const int64_t lam_len = p->kind == TN_FORM_BOND ? p->lam_len : 0;
  bool ok = fwrite(kMagic, 1, 8, f) == 8 && fwrite(hdr, sizeof(int32_t), 7, f) == 7 &&
            fwrite(&lam_len, sizeof(int64_t), 1, f) == 1 &&
            fwrite(p->bond.data(), sizeof(int64_t), p->L + 1, f) == (size_t)(p->L + 1);
  std::vector<cxd> buf;
  for (int b = 0; b < p->B && ok; ++b)
    for (int i = 1; i <= p->L && ok; ++i) {
      buf.resize((size_t)sz(p, i));
      if (cudaMemcpyAsync(buf.data(), p->site[i] + (size_t)b * p->cap[i], sizeof(cxd) * buf.size(),
                          cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
          cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        fclose(f);
        return tn_set_error(ctx, TN_ECUDA, "tn_mps_save: device read failed");
      }
      ok = fwrite(buf.data(), sizeof(cxd), buf.size(), f) == buf.size();
    }
  if (ok && lam_len > 0) {
    std::vector<double> lam((size_t)(lam_len * p->B));
    for (int b = 0; b < p->B; ++b)
      cudaMemcpyAsync(lam.data() + (size_t)b * lam_len, p->lam + (size_t)b * p->lam_cap, sizeof(double) * lam_len,
                      cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      fclose(f);
      return tn_set_error(ctx, TN_ECUDA, "tn_mps_save: device read failed");
    }
    ok = fwrite(lam.data(), sizeof(double), lam.size(), f) == lam.size();
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? TN_OK : tn_set_error(ctx, TN_EINVAL, "tn_mps_save: write to %s failed", path);
}

tn_status_t tn_mps_shape(const tn_mps* p, int32_t* L, int32_t* d, int32_t* B) {
  if (!p) return TN_EINVAL;
  if (L) *L = p->L;
  if (d) *d = p->d;
  if (B) *B = p->B;
  return TN_OK;
}

tn_status_t tn_mps_load(tn_ctx* ctx, const char* path, int64_t max_bond, tn_mps** out) {
  if (!ctx || !path || !out) return TN_EINVAL;
  FILE* f = fopen(path, "rb");
  if (!f) return tn_set_error(ctx, TN_EINVAL, "tn_mps_load: cannot open %s", path);
  char magic[8];
  int32_t hdr[7];
  int64_t lam_len = 0;
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, kMagic, 8) == 0 && fread(hdr, sizeof(int32_t), 7, f) == 7 &&
            fread(&lam_len, sizeof(int64_t), 1, f) == 1;
  const int32_t L = hdr[0], d = hdr[1], B = hdr[2];
  ok = ok && L >= 2 && L <= (1 << 20) && d >= 1 && d <= 1024 && B >= 1 && B <= 8192 && lam_len >= 0;
  std::vector<int64_t> bond(ok ? L + 1 : 0);
  ok = ok && fread(bond.data(), sizeof(int64_t), L + 1, f) == (size_t)(L + 1) && bond[0] == 1 && bond[L] == 1;
  for (int i = 1; ok && i < L; ++i) ok = bond[i] >= 1 && bond[i] <= (int64_t)1 << 24;
  if (!ok) {
    fclose(f);
    return tn_set_error(ctx, TN_EINVAL, "tn_mps_load: %s is not an MPS dump", path);
  }
  tn_mps* p = nullptr;
  tn_status_t st = tn_mps_create_batched(ctx, B, L, d, bond.data() + 1, max_bond, (tn_precision_t)hdr[6], &p);
  if (st != TN_OK) {
    fclose(f);
    return st;
  }
  std::vector<cxd> buf;
  for (int b = 0; b < B && st == TN_OK; ++b)
    for (int i = 1; i <= L && st == TN_OK; ++i) {
      buf.resize((size_t)sz(p, i));
      if (fread(buf.data(), sizeof(cxd), buf.size(), f) != buf.size())
        st = tn_set_error(ctx, TN_EINVAL, "tn_mps_load: %s is truncated", path);
      else
        st = tn_mps_set_instance_site(p, b, i, p->bond[i - 1], p->bond[i], buf.data());
    }
  if (st == TN_OK && hdr[3] == TN_FORM_BOND && lam_len > 0) {
    std::vector<double> lam((size_t)(lam_len * B));
    if (fread(lam.data(), sizeof(double), lam.size(), f) != lam.size()) {
      st = tn_set_error(ctx, TN_EINVAL, "tn_mps_load: %s is truncated", path);
    } else {
      st = ensure_lam(p, lam_len);
      for (int b = 0; b < B && st == TN_OK; ++b)
        if (cudaMemcpyAsync(p->lam + (size_t)b * p->lam_cap, lam.data() + (size_t)b * lam_len, sizeof(double) * lam_len,
                            cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
          st = tn_set_error(ctx, TN_ECUDA, "tn_mps_load: upload failed");
      if (st == TN_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        st = tn_set_error(ctx, TN_ECUDA, "tn_mps_load: upload failed");
      p->lam_len = lam_len;
    }
  }
  fclose(f);
  if (st != TN_OK) {
    tn_mps_destroy(p);
    return st;
  }
  p->kind = hdr[3];
  p->lo = hdr[4];
  p->hi = hdr[5];
  *out = p;
  return TN_OK;
}

}  // extern "C"
