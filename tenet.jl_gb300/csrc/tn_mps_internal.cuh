// The device MPS handle shared by the translation units that operate on it.
#pragma once

#include <vector>

#include "tn_internal.cuh"

struct tn_mps {
  tn_ctx* ctx = nullptr;
  int L = 0, d = 0, B = 1;
  std::vector<int64_t> bond;      // L+1 entries, bond[0] = bond[L] = 1
  std::vector<int64_t> cap_bond;  // storage caps per bond
  std::vector<cxd*> site;         // 1-based: site[1..L], B instances each
  std::vector<size_t> cap;        // elements reserved per site and instance (= instance stride)
  int kind = TN_FORM_MIXED, lo = 1, hi = 1;
  double* lam = nullptr;  // Λ at the bond-canonical centre, B instances at stride lam_cap
  int64_t lam_len = 0;
  size_t lam_cap = 0;
  tn_precision_t prec = TN_PREC_NATIVE;
  cxd* gates = nullptr;  // device copy of gates
  size_t gates_cap = 0;
};

// grow the storage of site i (all instances) to at least `elems` elements per instance,
// keeping its current contents
tn_status_t mps_ensure_site(tn_mps* p, int i, size_t elems);
