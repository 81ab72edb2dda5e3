// Mode-labelled factorisations: Muscle.tensor_qr_thin / Muscle.tensor_svd_thin on a
// dense tensor whose modes carry integer labels (the Julia binding maps Tenet's Index
// values to them).  The tensor is matricised by the labels given for the left side (a
// permutation when they are not already leading), factorised, and the outputs come back
// as labelled tensors: Q (q modes…, virtual), R (virtual, other modes…); U (u modes…, s),
// S, Vh (s, other modes…), the SVD truncated like compress! (maxdim, then the absolute
// threshold) with the kept rank returned.
#include <algorithm>
#include <vector>

#include "tn_internal.cuh"

namespace {

int find_mode(const int32_t* modes, int n, int32_t m) {
  for (int i = 0; i < n; ++i)
    if (modes[i] == m) return i;
  return -1;
}

// left-side positions in A (in the caller's order), then the remaining positions in A's
// order; dims of both sides
tn_status_t split_modes(tn_ctx* ctx, const tn_tensor* A, int32_t n_left, const int32_t* left, int32_t new_mode,
                        std::vector<int32_t>* perm, int64_t* m, int64_t* n) {
  TN_ARG(ctx, A && A->rank >= 1 && A->rank <= TN_MAX_RANK, "labelled factorisation: rank out of range");
  TN_ARG(ctx, n_left >= 0 && n_left <= A->rank && (n_left == 0 || left), "labelled factorisation: bad left modes");
  for (int i = 0; i < A->rank; ++i) {
    TN_ARG(ctx, find_mode(A->modes, i, A->modes[i]) < 0, "labelled factorisation: repeated mode");
    TN_ARG(ctx, A->dims[i] >= 1, "labelled factorisation: empty dimension");
  }
  TN_ARG(ctx, find_mode(A->modes, A->rank, new_mode) < 0, "labelled factorisation: the new mode is already in use");
  perm->clear();
  *m = 1;
  *n = 1;
  for (int j = 0; j < n_left; ++j) {
    const int p = find_mode(A->modes, A->rank, left[j]);
    TN_ARG(ctx, p >= 0, "labelled factorisation: a left mode is not a mode of the tensor");
    TN_ARG(ctx, std::find(perm->begin(), perm->end(), p) == perm->end(), "labelled factorisation: repeated left mode");
    perm->push_back(p);
    *m *= A->dims[p];
  }
  for (int i = 0; i < A->rank; ++i)
    if (std::find(perm->begin(), perm->end(), i) == perm->end()) {
      perm->push_back(i);
      *n *= A->dims[i];
    }
  TN_ARG(ctx, A->rank < TN_MAX_RANK, "labelled factorisation: rank limit (the output adds a mode)");
  return TN_OK;
}

bool identity(const std::vector<int32_t>& p) {
  for (size_t i = 0; i < p.size(); ++i)
    if (p[i] != (int32_t)i) return false;
  return true;
}

// A as a dense m×n matrix (a permuted copy in the workspace when needed)
tn_status_t matricise(tn_ctx* ctx, tn_dtype_t dtype, const tn_tensor* A, const std::vector<int32_t>& perm,
                      const void** out) {
  if (identity(perm)) {
    *out = A->data;
    return TN_OK;
  }
  int64_t numel = 1;
  for (int i = 0; i < A->rank; ++i) numel *= A->dims[i];
  void* t = ws_take<char>(ctx, dtype_size(dtype) * (size_t)numel);
  TN_RETURN_IF(tn_permute(ctx, dtype, A->rank, A->dims, nullptr, perm.data(), A->data, t, 0));
  *out = t;
  return TN_OK;
}

void describe(tn_tensor* t, const tn_tensor* A, const std::vector<int32_t>& pos, int64_t k, int32_t new_mode,
              bool new_first) {
  int r = 0;
  if (new_first) {
    t->dims[r] = k;
    t->modes[r++] = new_mode;
  }
  for (int32_t p : pos) {
    t->dims[r] = A->dims[p];
    t->modes[r++] = A->modes[p];
  }
  if (!new_first) {
    t->dims[r] = k;
    t->modes[r++] = new_mode;
  }
  t->rank = r;
}

}  // namespace

extern "C" tn_status_t tn_tensor_qr_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, const tn_tensor* A,
                                         int32_t n_q, const int32_t* q_modes, int32_t virtual_mode, tn_tensor* Q,
                                         tn_tensor* R) {
  (void)prec;
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, Q && R, "tn_tensor_qr_thin: null output");
  TN_ARG(ctx, dtype == TN_C64 || dtype == TN_C32, "tn_tensor_qr_thin: only C64 and C32 are implemented");
  std::vector<int32_t> perm;
  int64_t m = 0, n = 0;
  TN_RETURN_IF(split_modes(ctx, A, n_q, q_modes, virtual_mode, &perm, &m, &n));
  TN_ARG(ctx, A->data && Q->data && R->data, "tn_tensor_qr_thin: null data");
  const int64_t k = std::min(m, n);
  const size_t es = dtype_size(dtype);
  TN_RETURN_IF(ws_reserve(ctx, ws_round(es * (size_t)(m * n)) +
                                   (dtype == TN_C64 ? qr_workspace<double>(m, n, 1) : qr_workspace<float>(m, n, 1))));
  const void* M = nullptr;
  TN_RETURN_IF(matricise(ctx, dtype, A, perm, &M));
  if (dtype == TN_C64)
    TN_RETURN_IF(qr_cx<double>(ctx, m, n, (const cxd*)M, m, 0, (cxd*)Q->data, 0, (cxd*)R->data, 0, 1));
  else
    TN_RETURN_IF(qr_cx<float>(ctx, m, n, (const cxf*)M, m, 0, (cxf*)Q->data, 0, (cxf*)R->data, 0, 1));
  describe(Q, A, std::vector<int32_t>(perm.begin(), perm.begin() + n_q), k, virtual_mode, false);
  describe(R, A, std::vector<int32_t>(perm.begin() + n_q, perm.end()), k, virtual_mode, true);
  return TN_OK;
}

extern "C" tn_status_t tn_tensor_svd_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, const tn_tensor* A,
                                          int32_t n_u, const int32_t* u_modes, int32_t s_mode, int64_t maxdim,
                                          double abs_threshold, tn_tensor* U, double* d_S, tn_tensor* Vh,
                                          int64_t* rank_out) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, U && Vh && d_S && rank_out, "tn_tensor_svd_thin: null output");
  TN_ARG(ctx, dtype == TN_C64 || dtype == TN_C32, "tn_tensor_svd_thin: only C64 and C32 are implemented");
  std::vector<int32_t> perm;
  int64_t m = 0, n = 0;
  TN_RETURN_IF(split_modes(ctx, A, n_u, u_modes, s_mode, &perm, &m, &n));
  TN_ARG(ctx, A->data && U->data && Vh->data, "tn_tensor_svd_thin: null data");
  const int64_t k = std::min(m, n);
  const size_t es = dtype_size(dtype);
  TN_RETURN_IF(ws_reserve(ctx, ws_round(es * (size_t)(m * n)) + ws_round(es * (size_t)(m * k)) +
                                   ws_round(es * (size_t)(k * n)) + ws_round(sizeof(double) * (size_t)k) +
                                   svd_any_workspace(dtype, prec, m, n, 1)));
  const void* M = nullptr;
  TN_RETURN_IF(matricise(ctx, dtype, A, perm, &M));
  char* Uw = ws_take<char>(ctx, es * (size_t)(m * k));
  char* Vw = ws_take<char>(ctx, es * (size_t)(k * n));
  double* Sw = ws_take<double>(ctx, (size_t)k);
  TN_RETURN_IF(svd_any(ctx, dtype, prec, m, n, M, m, 0, Uw, 0, Sw, 0, Vw, 0, 1));
  int64_t r = 0;
  TN_RETURN_IF(rank_select(ctx, Sw, k, maxdim, abs_threshold, &r));
  // U: the first r columns are a column-major prefix; Vh: the first r rows, compacted to
  // leading dimension r; S: the first r values
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(U->data, Uw, es * (size_t)(m * r), cudaMemcpyDeviceToDevice, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaMemcpy2DAsync(Vh->data, es * (size_t)r, Vw, es * (size_t)k, es * (size_t)r, (size_t)n,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(d_S, Sw, sizeof(double) * (size_t)r, cudaMemcpyDeviceToDevice, ctx->stream));
  describe(U, A, std::vector<int32_t>(perm.begin(), perm.begin() + n_u), r, s_mode, false);
  describe(Vh, A, std::vector<int32_t>(perm.begin() + n_u, perm.end()), r, s_mode, true);
  *rank_out = r;
  TN_RETURN_IF(split_gemm_check(ctx));
  return TN_OK;
}
