// Muscle-level entry points: binary_einsum (tn_contract) and simple_update.
//
// tn_contract plans a pairwise contraction the way Muscle.binary_einsum does — classify
// the mode labels, permute both operands to matrix form, one (batched) GEMM, permute the
// result to the requested mode order — but skips every permutation that is the identity
// and folds transposed operands into the GEMM's op flags instead of copying them.
#include <algorithm>
#include <vector>

#include "tn_internal.cuh"

typedef tn_status_t (*su_out_fn)(void* arg, int64_t r, cxd** Aout, int64_t* sAout, cxd** Bout, int64_t* sBout);
tn_status_t simple_update_core(tn_ctx* ctx, tn_precision_t prec, int64_t chl, int64_t d1, int64_t chm, int64_t d2,
                               int64_t chr, const cxd* A, int64_t sA, const cxd* Bm, int64_t sB, const cxd* dG,
                               int64_t maxdim, double threshold, int64_t batch, su_out_fn out_fn, void* out_arg,
                               double* Sout, int64_t* rank_out, int absorb = kAbsorbEqually);

namespace {

int find(const int32_t* modes, int r, int32_t m) {
  for (int i = 0; i < r; ++i)
    if (modes[i] == m) return i;
  return -1;
}

bool is_identity(const std::vector<int32_t>& p) {
  for (size_t i = 0; i < p.size(); ++i)
    if (p[i] != (int32_t)i) return false;
  return true;
}

}  // namespace

extern "C" tn_status_t tn_contract(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, const tn_tensor* a,
                                   const tn_tensor* b, tn_tensor* c) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, a && b && c, "tn_contract: null tensor");
  TN_ARG(ctx, a->rank >= 0 && a->rank <= TN_MAX_RANK && b->rank >= 0 && b->rank <= TN_MAX_RANK &&
                  c->rank >= 0 && c->rank <= TN_MAX_RANK,
         "tn_contract: rank out of range");
  for (int i = 0; i < a->rank; ++i) TN_ARG(ctx, find(a->modes, i, a->modes[i]) < 0, "tn_contract: repeated mode in a");
  for (int i = 0; i < b->rank; ++i) TN_ARG(ctx, find(b->modes, i, b->modes[i]) < 0, "tn_contract: repeated mode in b");
  for (int i = 0; i < c->rank; ++i) TN_ARG(ctx, find(c->modes, i, c->modes[i]) < 0, "tn_contract: repeated mode in c");
  // classify
  std::vector<int> M, N, K, H;  // positions: M,K in a; N in b; H in a
  for (int i = 0; i < a->rank; ++i) {
    int32_t m = a->modes[i];
    bool inb = find(b->modes, b->rank, m) >= 0, inc = find(c->modes, c->rank, m) >= 0;
    if (inb && inc)
      H.push_back(i);
    else if (inb)
      K.push_back(i);
    else if (inc)
      M.push_back(i);
    else
      return tn_set_error(ctx, TN_EINVAL, "tn_contract: mode %d of a appears in neither b nor c", m);
  }
  for (int i = 0; i < b->rank; ++i) {
    int32_t m = b->modes[i];
    bool ina = find(a->modes, a->rank, m) >= 0, inc = find(c->modes, c->rank, m) >= 0;
    if (!ina) {
      if (!inc) return tn_set_error(ctx, TN_EINVAL, "tn_contract: mode %d of b appears in neither a nor c", m);
      N.push_back(i);
    }
  }
  for (int i = 0; i < c->rank; ++i) {
    int32_t m = c->modes[i];
    TN_ARG(ctx, find(a->modes, a->rank, m) >= 0 || find(b->modes, b->rank, m) >= 0,
           "tn_contract: output mode missing from both inputs");
  }
  // shared dims must agree
  for (int i : K) TN_ARG(ctx, a->dims[i] == b->dims[find(b->modes, b->rank, a->modes[i])], "tn_contract: contracted dims differ");
  for (int i : H) TN_ARG(ctx, a->dims[i] == b->dims[find(b->modes, b->rank, a->modes[i])], "tn_contract: batch dims differ");
  int64_t m = 1, n = 1, k = 1, h = 1;
  for (int i : M) m *= a->dims[i];
  for (int i : N) n *= b->dims[i];
  for (int i : K) k *= a->dims[i];
  for (int i : H) h *= a->dims[i];
  // fill c dims
  for (int i = 0; i < c->rank; ++i) {
    int ia = find(a->modes, a->rank, c->modes[i]);
    c->dims[i] = ia >= 0 ? a->dims[ia] : b->dims[find(b->modes, b->rank, c->modes[i])];
  }
  if (m * n * h == 0) return TN_OK;
  TN_ARG(ctx, a->data && b->data && c->data, "tn_contract: null data");
  const size_t es = dtype_size(dtype);
  // a → (M, K, H) as op 'N', or (K, M, H) as op 'T'
  std::vector<int32_t> pa_n, pa_t, pb_n, pb_t;
  for (int i : M) pa_n.push_back(i);
  for (int i : K) pa_n.push_back(i);
  for (int i : H) pa_n.push_back(i);
  for (int i : K) pa_t.push_back(i);
  for (int i : M) pa_t.push_back(i);
  for (int i : H) pa_t.push_back(i);
  // b's K order must follow a's K order
  std::vector<int> Kb, Hb;
  for (int i : K) Kb.push_back(find(b->modes, b->rank, a->modes[i]));
  for (int i : H) Hb.push_back(find(b->modes, b->rank, a->modes[i]));
  for (int i : Kb) pb_n.push_back(i);
  for (int i : N) pb_n.push_back(i);
  for (int i : Hb) pb_n.push_back(i);
  for (int i : N) pb_t.push_back(i);
  for (int i : Kb) pb_t.push_back(i);
  for (int i : Hb) pb_t.push_back(i);
  char opa = 'N', opb = 'N';
  bool perm_a = true, perm_b = true;
  if (is_identity(pa_n)) perm_a = false;
  else if (is_identity(pa_t)) { perm_a = false; opa = 'T'; }
  if (is_identity(pb_n)) perm_b = false;
  else if (is_identity(pb_t)) { perm_b = false; opb = 'T'; }
  // output order (M, N, H) → c modes
  std::vector<int32_t> out_modes;
  for (int i : M) out_modes.push_back(a->modes[i]);
  for (int i : N) out_modes.push_back(b->modes[i]);
  for (int i : H) out_modes.push_back(a->modes[i]);
  std::vector<int32_t> pc(c->rank);
  for (int i = 0; i < c->rank; ++i) pc[i] = find(out_modes.data(), (int)out_modes.size(), c->modes[i]);
  const bool perm_c = !is_identity(pc);
  size_t need = 0;
  if (perm_a) need += ws_round(es * (size_t)(m * k * h));
  if (perm_b) need += ws_round(es * (size_t)(k * n * h));
  if (perm_c) need += ws_round(es * (size_t)(m * n * h));
  need += gemm_any_workspace(dtype, prec, m, n, k);
  TN_RETURN_IF(ws_reserve(ctx, need));
  const void* A = a->data;
  const void* B = b->data;
  void* C = c->data;
  if (perm_a) {
    void* t = ws_take<char>(ctx, es * (size_t)(m * k * h));
    TN_RETURN_IF(tn_permute(ctx, dtype, a->rank, a->dims, nullptr, pa_n.data(), a->data, t, 0));
    A = t;
  }
  if (perm_b) {
    void* t = ws_take<char>(ctx, es * (size_t)(k * n * h));
    TN_RETURN_IF(tn_permute(ctx, dtype, b->rank, b->dims, nullptr, pb_n.data(), b->data, t, 0));
    B = t;
  }
  if (perm_c) C = ws_take<char>(ctx, es * (size_t)(m * n * h));
  const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
  const int64_t lda = opa == 'N' ? m : k, ldb = opb == 'N' ? k : n;
  TN_RETURN_IF(gemm_any(ctx, dtype, prec, opa, opb, m, n, k, one, A, std::max<int64_t>(lda, 1), m * k, B,
                        std::max<int64_t>(ldb, 1), k * n, zero, C, std::max<int64_t>(m, 1), m * n, h));
  if (perm_c) {
    int64_t dims_t[TN_MAX_RANK];
    int r = 0;
    for (int i : M) dims_t[r++] = a->dims[i];
    for (int i : N) dims_t[r++] = b->dims[i];
    for (int i : H) dims_t[r++] = a->dims[i];
    TN_RETURN_IF(tn_permute(ctx, dtype, r, dims_t, nullptr, pc.data(), C, c->data, 0));
  }
  return TN_OK;
}

namespace {
struct FixedOut {
  cxd* A;
  cxd* B;
};
tn_status_t fixed_out(void* arg, int64_t, cxd** Aout, int64_t* sA, cxd** Bout, int64_t* sB) {
  FixedOut* f = (FixedOut*)arg;
  *Aout = f->A;
  *Bout = f->B;
  *sA = 0;
  *sB = 0;
  return TN_OK;
}
}  // namespace

extern "C" tn_status_t tn_simple_update(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, int64_t chl, int64_t d1,
                                        int64_t chm, int64_t d2, int64_t chr, const void* A, const void* B,
                                        const void* G, int64_t maxdim, double threshold, void* Aout, void* Bout,
                                        double* Sout, int64_t* rank) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, dtype == TN_C64, "tn_simple_update: only C64 is implemented");
  TN_ARG(ctx, chl >= 1 && d1 >= 1 && chm >= 1 && d2 >= 1 && chr >= 1, "tn_simple_update: sizes must be >= 1");
  TN_ARG(ctx, A && B && G && Aout && Bout && rank, "tn_simple_update: null pointer");
  FixedOut f{(cxd*)Aout, (cxd*)Bout};
  return simple_update_core(ctx, prec, chl, d1, chm, d2, chr, (const cxd*)A, 0, (const cxd*)B, 0, (const cxd*)G, maxdim,
                            threshold, 1, fixed_out, &f, Sout, rank);
}

extern "C" tn_status_t tn_simple_update_absorb(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, int64_t chl,
                                               int64_t d1, int64_t chm, int64_t d2, int64_t chr, const void* A,
                                               const void* B, const void* G, int64_t maxdim, double threshold,
                                               int32_t absorb, void* Aout, void* Bout, double* Sout, int64_t* rank) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, absorb == TN_ABSORB_EQUALLY || absorb == TN_ABSORB_U || absorb == TN_ABSORB_V,
         "tn_simple_update_absorb: absorb must be TN_ABSORB_EQUALLY, TN_ABSORB_U or TN_ABSORB_V");
  if (absorb == TN_ABSORB_EQUALLY)
    return tn_simple_update(ctx, dtype, prec, chl, d1, chm, d2, chr, A, B, G, maxdim, threshold, Aout, Bout, Sout,
                            rank);
  TN_ARG(ctx, dtype == TN_C64, "tn_simple_update_absorb: only C64 is implemented");
  TN_ARG(ctx, chl >= 1 && d1 >= 1 && chm >= 1 && d2 >= 1 && chr >= 1, "tn_simple_update_absorb: sizes must be >= 1");
  TN_ARG(ctx, A && B && G && Aout && Bout && rank, "tn_simple_update_absorb: null pointer");
  FixedOut f{(cxd*)Aout, (cxd*)Bout};
  return simple_update_core(ctx, prec, chl, d1, chm, d2, chr, (const cxd*)A, 0, (const cxd*)B, 0, (const cxd*)G, maxdim,
                            threshold, 1, fixed_out, &f, Sout, rank,
                            absorb == TN_ABSORB_U ? kAbsorbLeft : kAbsorbRight);
}
