// Device-resident query server over a pool of MPS with continuous batching.
//
// Queries are the reference's operations on a fixed MPS:
//   amplitude  ⟨bits|ψ⟩ = overlap(ProductState(bits), ψ)          src/Operations/overlap.jl:22-32
//   ⟨O_i⟩      = overlap(ψ, O_i ψ) / overlap(ψ, ψ)                src/Operations/overlap.jl:36-50
//   overlap    ⟨ψ_b|ψ_a⟩                                           src/Operations/overlap.jl:36-50
//
// Pool.  Each registered MPS keeps on the device its site tensors A_i and, computed once
// at registration from the left environments Lf_i (sites 1..i) and the right
// environments R_i (sites i..L), the environment-dressed sites X_i = Lf_{i-1} A_i R_{i+1}
// (same shape as A_i).  ⟨ψ|ψ⟩ = Lf_L, and an expectation value is one O(d χ²)
// reduction, ⟨ψ|O_i|ψ⟩ = Σ conj(A_i) · O · X_i, instead of a sweep over L sites.
//
// Scheduling.  A worker thread owns the device work.  Submitted queries wait in a FIFO.
// Whenever a job finishes (a host callback on its stream) or a query arrives, the worker
//   * retires finished jobs (results were copied to pinned host memory on the stream);
//   * admits waiting queries while job slots and workspace are free: amplitude and
//     expectation queries are gathered into one short job (up to max_batch) on the main
//     stream — at most two short jobs are in flight, so a new batch forms while the
//     previous one runs; each overlap is its own job on one of the overlap streams.
// Workspace comes from one device arena carved first-fit; a query that does not fit
// waits until running jobs return their blocks.  The arena and the pool together are
// capped by the HBM budget.  Within a short job, amplitudes of one MPS are computed
// together: per site one GEMM E (nq × χl) · A (χl × d χr) and a selection of the
// physical component by each query's product vector.  Every query's numbers are computed
// by the same sequence of operations alone or in a batch.  Precision: FP64 throughout, or
// (mixed servers) amplitude chains and overlap sweeps as FP32 GEMMs over FP32 copies of
// the sites, the scalar result returned in FP64; ⟨O_i⟩ always FP64.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tn_internal.cuh"

namespace {

constexpr int kOvlStreams = 4;
constexpr int kMaxShort = 2;      // short jobs in flight on the main stream
constexpr int kMaxOverlaps = 8;   // overlap jobs in flight
constexpr int kExpBlocks = 128;   // partial sums per expectation query
constexpr size_t kAlign = 256;

const cxd kOne = {1.0, 0.0};
const cxd kZero = {0.0, 0.0};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
size_t al(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }
size_t cxb(int64_t n) { return al(sizeof(cxd) * (size_t)n); }
unsigned nblk(int64_t n, int cap = 4096) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, cap));
}

// ---------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void k_fill_one(cx<T>* x, int64_t stride, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i * stride].x = T(1);
    x[i * stride].y = T(0);
  }
}
// precision conversions: FP32 copies of the pool sites; FP32 results back to FP64
__global__ void k_d2f_cx(int64_t n, const cxd* __restrict__ a, cxf* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = mkcx((float)a[i].x, (float)a[i].y);
}
__global__ void k_f2d_cx(int64_t n, const cxf* __restrict__ a, cxd* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = mkcx((double)a[i].x, (double)a[i].y);
}

// E'[q, r] = Σ_s v_q[site, s] · P[q, s + d r]   (P: nq × d χr, E': nq × χr, both ld nq)
template <typename T>
__global__ void k_amp_select(int64_t nq, int64_t chr, int d, const cx<T>* __restrict__ P, const cxd* __restrict__ vec,
                             int64_t vstride, int64_t voff, cx<T>* __restrict__ E) {
  const int64_t total = nq * chr;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t % nq, r = t / nq;
    cx<T> acc = mkcx(T(0), T(0));
    for (int s = 0; s < d; ++s) {
      const cxd v = vec[q * vstride + voff + s];
      cfma(acc, mkcx((T)v.x, (T)v.y), P[q + (s + (int64_t)d * r) * nq]);
    }
    E[q + r * nq] = acc;
  }
}

// partial sums of Σ_{b,s,r} conj(A[b,s,r]) Σ_t O[s,t] T2[b,t,r]  (A, T2: xl × d × xr)
__global__ void __launch_bounds__(256) k_expect_partial(int64_t xl, int d, int64_t xr, const cxd* __restrict__ A,
                                                        const cxd* __restrict__ T2, const cxd* __restrict__ O,
                                                        cxd* __restrict__ partial) {
  cxd acc = {0, 0};
  const int64_t total = xl * xr;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = idx % xl, r = idx / xl;
    for (int s = 0; s < d; ++s) {
      cxd ot = {0, 0};
      for (int t = 0; t < d; ++t) cfma(ot, O[s + d * t], T2[b + xl * (t + (int64_t)d * r)]);
      cfma_cj(acc, A[b + xl * (s + (int64_t)d * r)], ot);
    }
  }
  __shared__ double sx[8], sy[8];
  double x = warp_sum(acc.x), y = warp_sum(acc.y);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sx[w] = x;
    sy[w] = y;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tx = 0, ty = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      tx += sx[i];
      ty += sy[i];
    }
    partial[blockIdx.x] = mkcx(tx, ty);
  }
}

// out = Σ p[i] in a fixed order (one block of 128 threads)
__global__ void k_sum_partials(const cxd* __restrict__ p, int n, cxd* __restrict__ out) {
  __shared__ double sx[128], sy[128];
  double x = 0, y = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    x += p[i].x;
    y += p[i].y;
  }
  sx[threadIdx.x] = x;
  sy[threadIdx.x] = y;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = mkcx(sx[0], sy[0]);
}

// Gaussian fill for generated pool MPS: counter-based hash (splitmix64 finaliser) → two
// uniforms → Box–Muller; entries (g1 + i g2)/√2 · scale
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__global__ void k_fill_gauss(cxd* x, int64_t n, uint64_t seed, double scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix64(seed ^ mix64(2 * (uint64_t)i));
    const uint64_t h2 = mix64(seed ^ mix64(2 * (uint64_t)i + 1));
    const double u1 = ((h1 >> 11) + 1) * (1.0 / 9007199254740992.0);  // (0, 1]
    const double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);        // [0, 1)
    const double rad = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    x[i].x = rad * cs * scale * 0.70710678118654752;
    x[i].y = rad * sn * scale * 0.70710678118654752;
  }
}

// ---------------------------------------------------------------------------------
// host structures
// ---------------------------------------------------------------------------------
struct PoolMPS {
  int L = 0, d = 0;
  std::vector<int64_t> bond;  // 0..L
  std::vector<cxd*> site;     // 1..L
  std::vector<cxd*> dressed;  // 1..L   X_i = Lf_{i-1} A_i R_{i+1}: χ_{i-1} × d × χ_i
  std::vector<cxf*> site32;   // 1..L   FP32 copies of A_i (mixed-precision servers)
  void* block = nullptr;
  size_t bytes = 0;
  int64_t maxbond = 1;
  double norm2 = 0;
  int inflight = 0;
};

struct Query {
  int64_t ticket = 0;
  int kind = 0, a = -1, b = -1, site = 0;
  std::vector<cxd> data;  // amplitude: L×d product vectors; expectation: d×d operator
  double t_submit = 0;
};

struct Result {
  bool done = false;
  tn_status_t status = TN_OK;
  cxd value = {0, 0};
  double latency = 0;
  std::string err;
};

// first-fit allocator over one device block
struct Arena {
  char* base = nullptr;
  size_t cap = 0;
  std::map<size_t, size_t> free_;  // offset → size
  void reset(char* b, size_t c) {
    base = b;
    cap = c;
    free_.clear();
    if (c) free_[0] = c;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = al(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, o = it->first + bytes;
      free_.erase(it);
      if (rest) free_[o] = rest;
      return true;
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = al(bytes);
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

}  // namespace
struct tn_server;
namespace {

struct Job {
  tn_server* S = nullptr;
  bool overlap = false;
  cudaStream_t stream = nullptr;
  size_t off = 0, bytes = 0;  // arena block
  size_t res_off = 0;         // results in the pinned slot
  std::vector<int64_t> tickets;
  std::vector<double> scale, submit;
  std::vector<int> refs;
  int slot = -1;  // pinned slot
  std::atomic<int> finished{0};
};

struct PinnedSlot {
  void* h = nullptr;
  size_t cap = 0;
  bool busy = false;
};

}  // namespace

struct tn_server {
  tn_ctx* ctx = nullptr;
  tn_precision_t prec = TN_PREC_NATIVE;
  int device = 0;
  cudaStream_t s_main = nullptr, s_reg = nullptr, s_ovl[kOvlStreams] = {};
  int ovl_rr = 0;
  size_t budget = 0;
  int max_batch = 64;
  void* arena_mem = nullptr;
  Arena arena;
  std::vector<PinnedSlot> slots;
  // mu guards: pending, results, counters, pool membership (with exec_mu for changes)
  std::mutex mu, exec_mu;
  std::condition_variable cv, cv_done;
  uint64_t events = 0;
  std::deque<Query> pending;
  std::unordered_map<int64_t, Result> results;
  std::unordered_map<int, PoolMPS> pool;
  std::vector<std::unique_ptr<Job>> jobs;
  int short_inflight = 0, ovl_inflight = 0;
  int next_id = 0;
  int64_t next_ticket = 1;
  std::thread worker;
  bool stop = false;
  int64_t completed = 0, short_jobs = 0, overlap_jobs = 0, max_batch_seen = 0, deferred = 0;
};

namespace {

thread_local std::string t_serve_error;

tn_status_t serr(tn_status_t st, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_serve_error = buf;
  return st;
}

size_t pool_bytes(const tn_server* S) {
  size_t b = 0;
  for (auto& kv : S->pool) b += kv.second.bytes;
  return b;
}

// device bytes one query adds to a job (upper bound, see launch_short / launch_overlap)
size_t query_bytes(const tn_server* S, const Query& q) {
  auto it = S->pool.find(q.a);
  if (it == S->pool.end()) return 0;
  const PoolMPS& p = it->second;
  const int64_t mx = p.maxbond, d = p.d;
  if (q.kind == TN_Q_AMPLITUDE) return cxb(mx) + cxb(d * mx) + cxb(p.L * d) + cxb(1);
  if (q.kind == TN_Q_EXPECTATION) return cxb(kExpBlocks) + cxb(d * d) + cxb(1);
  auto jt = S->pool.find(q.b);
  const int64_t mb = jt == S->pool.end() ? mx : std::max(mx, jt->second.maxbond);
  return 2 * cxb(mb * mb) + cxb(mb * d * mb) + cxb(1);
}

void CUDART_CB job_done_cb(void* arg) {
  Job* j = static_cast<Job*>(arg);
  tn_server* S = j->S;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    j->finished.store(1);
    S->events++;
  }
  S->cv.notify_all();
}

tn_status_t ensure_slot(tn_server* S, int slot, size_t bytes) {
  PinnedSlot& ps = S->slots[slot];
  if (ps.cap >= bytes) return TN_OK;
  if (ps.h) cudaFreeHost(ps.h);
  ps.h = nullptr;
  ps.cap = 0;
  const size_t cap = std::max<size_t>(bytes + bytes / 2, 1 << 16);
  if (cudaHostAlloc(&ps.h, cap, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    ps.h = nullptr;
    return tn_set_error(S->ctx, TN_ENOMEM, "serve: pinned staging of %zu bytes failed", cap);
  }
  ps.cap = cap;
  return TN_OK;
}

int free_slot(tn_server* S) {
  for (size_t i = 0; i < S->slots.size(); ++i)
    if (!S->slots[i].busy) return (int)i;
  return -1;
}

// ⟨b|a⟩ environment sweep on ctx->stream; returns the device location of the scalar
// sites in the sweep's precision: the FP64 sites, or their FP32 copies
inline const cxd* site_of(const PoolMPS& p, int i, cxd*) { return p.site[i]; }
inline const cxf* site_of(const PoolMPS& p, int i, cxf*) { return p.site32[i]; }

template <typename T>
tn_status_t overlap_sweep(tn_ctx* ctx, const PoolMPS& a, const PoolMPS& b, cx<T>* F, cx<T>* F2, cx<T>* Tm, cx<T>** res) {
  const int d = a.d;
  const cx<T> one = mkcx(T(1), T(0)), zero = mkcx(T(0), T(0));
  k_fill_one<T><<<1, 32, 0, ctx->stream>>>(F, 1, 1);
  TN_LAUNCHED(ctx);
  for (int i = 1; i <= a.L; ++i) {
    const int64_t xa = a.bond[i - 1], xa2 = a.bond[i], yb = b.bond[i - 1], yb2 = b.bond[i];
    // T (yb × d xa2) = F (yb × xa) · A (xa × d xa2);  F2 (yb2 × xa2) = B_matᴴ · T
    TN_RETURN_IF(gemm_cx<T>(ctx, 'N', 'N', yb, d * xa2, xa, one, F, yb, 0, site_of(a, i, (cx<T>*)nullptr), xa, 0, zero,
                            Tm, yb, 0, 1));
    TN_RETURN_IF(gemm_cx<T>(ctx, 'C', 'N', yb2, xa2, yb * d, one, site_of(b, i, (cx<T>*)nullptr), yb * d, 0, Tm, yb * d,
                            0, zero, F2, yb2, 0, 1));
    std::swap(F, F2);
  }
  *res = F;
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// job launch (worker thread, exec_mu held, mu not held)
// ---------------------------------------------------------------------------------
tn_status_t launch_short(tn_server* S, Job* job, std::vector<Query>& qs) {
  tn_ctx* ctx = S->ctx;
  ctx->stream = job->stream;
  const int n = (int)qs.size();
  // group amplitudes per MPS (in arrival order), expectation values in arrival order
  std::vector<int> amp_ids;
  std::unordered_map<int, std::vector<int>> amp;
  std::vector<int> exps;
  for (int k = 0; k < n; ++k) {
    if (qs[k].kind == TN_Q_AMPLITUDE) {
      if (!amp.count(qs[k].a)) amp_ids.push_back(qs[k].a);
      amp[qs[k].a].push_back(k);
    } else {
      exps.push_back(k);
    }
  }
  // layout: [upload: V per amp group | O per exp] [results] [E, P per amp group] [T1 T2] [partials]
  size_t up_bytes = 0;
  for (int id : amp_ids) up_bytes += cxb((int64_t)amp[id].size() * S->pool.at(id).L * S->pool.at(id).d);
  for (int k : exps) up_bytes += cxb((int64_t)S->pool.at(qs[k].a).d * S->pool.at(qs[k].a).d);
  TN_RETURN_IF(ensure_slot(S, job->slot, up_bytes + cxb(n)));
  char* hst = (char*)S->slots[job->slot].h;
  char* dev = S->arena.base + job->off;
  char* dup = dev;
  size_t o = 0;
  std::vector<cxd*> dV(amp_ids.size()), dO(exps.size());
  for (size_t g = 0; g < amp_ids.size(); ++g) {
    const PoolMPS& p = S->pool.at(amp_ids[g]);
    dV[g] = (cxd*)(dev + o);
    cxd* h = (cxd*)(hst + o);
    for (size_t q = 0; q < amp[amp_ids[g]].size(); ++q)
      memcpy(h + q * p.L * p.d, qs[amp[amp_ids[g]][q]].data.data(), sizeof(cxd) * p.L * p.d);
    o += cxb((int64_t)amp[amp_ids[g]].size() * p.L * p.d);
  }
  for (size_t e = 0; e < exps.size(); ++e) {
    const PoolMPS& p = S->pool.at(qs[exps[e]].a);
    dO[e] = (cxd*)(dev + o);
    memcpy(hst + o, qs[exps[e]].data.data(), sizeof(cxd) * p.d * p.d);
    o += cxb((int64_t)p.d * p.d);
  }
  if (o) TN_CHECK_CUDA(ctx, cudaMemcpyAsync(dup, hst, o, cudaMemcpyHostToDevice, ctx->stream));
  cxd* results = (cxd*)(dev + o);
  o += cxb(n);
  job->tickets.resize(n);
  job->scale.assign(n, 1.0);
  job->submit.resize(n);
  int slot = 0;
  std::vector<int> order(n);  // slot → query index
  for (size_t g = 0; g < amp_ids.size(); ++g) {
    const PoolMPS& p = S->pool.at(amp_ids[g]);
    const std::vector<int>& ks = amp[amp_ids[g]];
    const int64_t nq = (int64_t)ks.size(), d = p.d;
    cxd* E = (cxd*)(dev + o);
    o += cxb(nq * p.maxbond);
    cxd* P = (cxd*)(dev + o);
    o += cxb(nq * d * p.maxbond);
    if (S->prec == TN_PREC_MIXED) {  // FP32 chain over the FP32 site copies (the buffers fit twice)
      cxf* E32 = (cxf*)E;
      cxf* P32 = (cxf*)P;
      const cxf one = mkcx(1.f, 0.f), zero = mkcx(0.f, 0.f);
      k_fill_one<float><<<nblk(nq), 256, 0, ctx->stream>>>(E32, 1, nq);
      TN_LAUNCHED(ctx);
      for (int i = 1; i <= p.L; ++i) {
        const int64_t xl = p.bond[i - 1], xr = p.bond[i];
        TN_RETURN_IF(gemm_cx<float>(ctx, 'N', 'N', nq, d * xr, xl, one, E32, nq, 0, p.site32[i], xl, 0, zero, P32, nq, 0, 1));
        k_amp_select<float><<<nblk(nq * xr), 256, 0, ctx->stream>>>(nq, xr, (int)d, P32, dV[g], p.L * d,
                                                                     (int64_t)(i - 1) * d, E32);
        TN_LAUNCHED(ctx);
      }
      k_f2d_cx<<<nblk(nq), 256, 0, ctx->stream>>>(nq, E32, results + slot);
      TN_LAUNCHED(ctx);
    } else {
      k_fill_one<double><<<nblk(nq), 256, 0, ctx->stream>>>(E, 1, nq);
      TN_LAUNCHED(ctx);
      for (int i = 1; i <= p.L; ++i) {
        const int64_t xl = p.bond[i - 1], xr = p.bond[i];
        TN_RETURN_IF(gemm_cx<double>(ctx, 'N', 'N', nq, d * xr, xl, kOne, E, nq, 0, p.site[i], xl, 0, kZero, P, nq, 0, 1));
        k_amp_select<double><<<nblk(nq * xr), 256, 0, ctx->stream>>>(nq, xr, (int)d, P, dV[g], p.L * d,
                                                                      (int64_t)(i - 1) * d, E);
        TN_LAUNCHED(ctx);
      }
      TN_CHECK_CUDA(ctx, cudaMemcpyAsync(results + slot, E, sizeof(cxd) * nq, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    for (int64_t q = 0; q < nq; ++q) order[slot + q] = ks[q];
    slot += (int)nq;
  }
  if (!exps.empty()) {
    cxd* part = (cxd*)(dev + o);
    o += cxb(kExpBlocks * (int64_t)exps.size());
    for (size_t e = 0; e < exps.size(); ++e) {
      const Query& q = qs[exps[e]];
      const PoolMPS& p = S->pool.at(q.a);
      const int i = q.site, d = p.d;
      const int64_t xl = p.bond[i - 1], xr = p.bond[i];
      const unsigned blocks = (unsigned)std::min<int64_t>(kExpBlocks, std::max<int64_t>(1, (xl * xr + 255) / 256));
      // ⟨ψ|O_i|ψ⟩ = Σ_{b,s,r} conj(A_i[b,s,r]) Σ_t O[s,t] X_i[b,t,r]
      k_expect_partial<<<blocks, 256, 0, ctx->stream>>>(xl, d, xr, p.site[i], p.dressed[i], dO[e],
                                                        part + kExpBlocks * e);
      TN_LAUNCHED(ctx);
      k_sum_partials<<<1, 128, 0, ctx->stream>>>(part + kExpBlocks * e, (int)blocks, results + slot);
      TN_LAUNCHED(ctx);
      order[slot] = exps[e];
      ++slot;
    }
  }
  if (o > job->bytes) return tn_set_error(ctx, TN_ECUDA, "serve: job layout %zu exceeds its block %zu", o, job->bytes);
  job->res_off = up_bytes;
  cxd* hres = (cxd*)(hst + up_bytes);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(hres, results, sizeof(cxd) * n, cudaMemcpyDeviceToHost, ctx->stream));
  for (int s = 0; s < n; ++s) {
    const Query& q = qs[order[s]];
    job->tickets[s] = q.ticket;
    job->submit[s] = q.t_submit;
    job->scale[s] = q.kind == TN_Q_EXPECTATION ? 1.0 / S->pool.at(q.a).norm2 : 1.0;
  }
  TN_CHECK_CUDA(ctx, cudaLaunchHostFunc(ctx->stream, job_done_cb, job));
  return TN_OK;
}

tn_status_t launch_overlap(tn_server* S, Job* job, const Query& q) {
  tn_ctx* ctx = S->ctx;
  ctx->stream = job->stream;
  const PoolMPS& a = S->pool.at(q.a);
  const PoolMPS& b = S->pool.at(q.b);
  const int64_t mb = std::max(a.maxbond, b.maxbond);
  TN_RETURN_IF(ensure_slot(S, job->slot, cxb(1)));
  char* dev = S->arena.base + job->off;
  cxd* F = (cxd*)dev;
  cxd* F2 = (cxd*)(dev + cxb(mb * mb));
  cxd* T = (cxd*)(dev + 2 * cxb(mb * mb));
  cxd* res = nullptr;
  if (S->prec == TN_PREC_MIXED) {  // FP32 environment sweep over the FP32 site copies
    cxf* r32 = nullptr;
    TN_RETURN_IF(overlap_sweep<float>(ctx, a, b, (cxf*)F, (cxf*)F2, (cxf*)T, &r32));
    res = (cxd*)(r32 == (cxf*)F ? F2 : F);  // the buffer the sweep did not end in
    k_f2d_cx<<<1, 32, 0, ctx->stream>>>(1, r32, res);
    TN_LAUNCHED(ctx);
  } else {
    TN_RETURN_IF(overlap_sweep<double>(ctx, a, b, F, F2, T, &res));
  }
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(S->slots[job->slot].h, res, sizeof(cxd), cudaMemcpyDeviceToHost, ctx->stream));
  job->tickets = {q.ticket};
  job->submit = {q.t_submit};
  job->scale = {1.0};
  TN_CHECK_CUDA(ctx, cudaLaunchHostFunc(ctx->stream, job_done_cb, job));
  return TN_OK;
}

// ---------------------------------------------------------------------------------
// worker
// ---------------------------------------------------------------------------------
void finish_tickets(tn_server* S, const std::vector<int64_t>& tickets, const std::vector<double>& submit,
                    tn_status_t st, const std::string& err, const cxd* vals, const std::vector<double>* scale) {
  const double t = now_s();
  for (size_t k = 0; k < tickets.size(); ++k) {
    Result& r = S->results[tickets[k]];
    r.done = true;
    r.status = st;
    r.err = err;
    r.latency = t - submit[k];
    if (st == TN_OK && vals) r.value = mkcx(vals[k].x * (*scale)[k], vals[k].y * (*scale)[k]);
  }
  S->completed += (int64_t)tickets.size();
}

void release_job(tn_server* S, Job* j) {  // mu held
  S->arena.release(j->off, j->bytes);
  if (j->slot >= 0) S->slots[j->slot].busy = false;
  for (int id : j->refs) {
    auto it = S->pool.find(id);
    if (it != S->pool.end()) it->second.inflight--;
  }
  if (j->overlap)
    S->ovl_inflight--;
  else
    S->short_inflight--;
}

void retire(tn_server* S) {  // exec_mu held
  std::lock_guard<std::mutex> lock(S->mu);
  bool any = false;
  for (auto it = S->jobs.begin(); it != S->jobs.end();) {
    Job* j = it->get();
    if (!j->finished.load()) {
      ++it;
      continue;
    }
    const cxd* vals = (const cxd*)((const char*)S->slots[j->slot].h + j->res_off);
    finish_tickets(S, j->tickets, j->submit, TN_OK, "", vals, &j->scale);
    release_job(S, j);
    it = S->jobs.erase(it);
    any = true;
  }
  if (any) S->cv_done.notify_all();
}

void fail_job(tn_server* S, std::unique_ptr<Job> j, tn_status_t st) {
  // the stream may hold part of the job: let it drain before the workspace is reused
  cudaStreamSynchronize(j->stream);
  cudaGetLastError();
  std::lock_guard<std::mutex> lock(S->mu);
  finish_tickets(S, j->tickets, j->submit, st, S->ctx->last_error, nullptr, nullptr);
  release_job(S, j.get());
  S->cv_done.notify_all();
}

void admit_and_launch(tn_server* S) {  // exec_mu held
  std::vector<std::pair<std::unique_ptr<Job>, std::vector<Query>>> todo;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    std::vector<Query> keep;
    // queries whose MPS disappeared fail here
    std::vector<Query> batch;
    size_t batch_bytes = cxb(1);
    bool short_open = S->short_inflight < kMaxShort;
    std::deque<Query> rest;
    while (!S->pending.empty()) {
      Query q = std::move(S->pending.front());
      S->pending.pop_front();
      if (!S->pool.count(q.a) || (q.kind == TN_Q_OVERLAP && !S->pool.count(q.b))) {
        finish_tickets(S, {q.ticket}, {q.t_submit}, TN_EINVAL, "serve: the MPS was removed", nullptr, nullptr);
        S->cv_done.notify_all();
        continue;
      }
      const size_t need = query_bytes(S, q);
      if (q.kind == TN_Q_OVERLAP) {
        const int slot = free_slot(S);
        size_t off = 0;
        if (S->ovl_inflight < kMaxOverlaps && slot >= 0 && S->arena.alloc(need, &off)) {
          auto j = std::make_unique<Job>();
          j->S = S;
          j->overlap = true;
          j->stream = S->s_ovl[S->ovl_rr++ % kOvlStreams];
          j->off = off;
          j->bytes = al(need);
          j->slot = slot;
          j->refs = {q.a, q.b};
          S->slots[slot].busy = true;
          S->pool[q.a].inflight++;
          S->pool[q.b].inflight++;
          S->ovl_inflight++;
          S->overlap_jobs++;
          std::vector<Query> one;
          one.push_back(std::move(q));
          todo.emplace_back(std::move(j), std::move(one));
        } else {
          if (S->ovl_inflight < kMaxOverlaps && slot >= 0) S->deferred++;
          rest.push_back(std::move(q));
        }
        continue;
      }
      if (short_open && (int)batch.size() < S->max_batch && batch_bytes + need <= S->arena.cap) {
        batch_bytes += need;
        batch.push_back(std::move(q));
      } else {
        rest.push_back(std::move(q));
      }
    }
    if (!batch.empty()) {
      const int slot = free_slot(S);
      size_t off = 0;
      // shrink the batch until its block fits (the rest waits for memory)
      while (!batch.empty() && (slot < 0 || !S->arena.alloc(batch_bytes, &off))) {
        S->deferred++;
        batch_bytes -= query_bytes(S, batch.back());
        rest.push_front(std::move(batch.back()));
        batch.pop_back();
        if (slot < 0) break;
      }
      if (!batch.empty() && slot >= 0) {
        auto j = std::make_unique<Job>();
        j->S = S;
        j->overlap = false;
        j->stream = S->s_main;
        j->off = off;
        j->bytes = al(batch_bytes);
        j->slot = slot;
        for (auto& q : batch) {
          j->refs.push_back(q.a);
          S->pool[q.a].inflight++;
        }
        S->slots[slot].busy = true;
        S->short_inflight++;
        S->short_jobs++;
        S->max_batch_seen = std::max<int64_t>(S->max_batch_seen, (int64_t)batch.size());
        todo.emplace_back(std::move(j), std::move(batch));
      } else {
        for (auto it = batch.rbegin(); it != batch.rend(); ++it) rest.push_front(std::move(*it));
      }
    }
    // keep arrival order for what waits
    std::sort(rest.begin(), rest.end(), [](const Query& x, const Query& y) { return x.ticket < y.ticket; });
    S->pending = std::move(rest);
  }
  for (auto& t : todo) {
    Job* j = t.first.get();
    tn_status_t st = j->overlap ? launch_overlap(S, j, t.second[0]) : launch_short(S, j, t.second);
    if (st != TN_OK) {
      j->tickets.clear();
      j->submit.clear();
      for (auto& q : t.second) {
        j->tickets.push_back(q.ticket);
        j->submit.push_back(q.t_submit);
      }
      fail_job(S, std::move(t.first), st);
      continue;
    }
    std::lock_guard<std::mutex> lock(S->mu);
    S->jobs.push_back(std::move(t.first));
  }
}

void worker_main(tn_server* S) {
  cudaSetDevice(S->device);
  uint64_t seen = 0;
  while (true) {
    {
      std::unique_lock<std::mutex> lock(S->mu);
      S->cv.wait(lock, [&] { return S->events != seen || (S->stop && S->pending.empty() && S->jobs.empty()); });
      seen = S->events;
      if (S->stop && S->pending.empty() && S->jobs.empty()) return;
    }
    std::lock_guard<std::mutex> ex(S->exec_mu);
    retire(S);
    admit_and_launch(S);
  }
}

// ---------------------------------------------------------------------------------
// pool registration (exec_mu held)
// ---------------------------------------------------------------------------------
tn_status_t pool_alloc(tn_server* S, int L, int d, const int64_t* bonds, PoolMPS& p) {
  tn_ctx* ctx = S->ctx;
  p.L = L;
  p.d = d;
  p.bond.assign(L + 1, 1);
  for (int i = 1; i < L; ++i) {
    if (bonds[i - 1] < 1) return serr(TN_EINVAL, "serve: bond %d < 1", i);
    p.bond[i] = bonds[i - 1];
    p.maxbond = std::max(p.maxbond, p.bond[i]);
  }
  // every site's elements, and the pool entry's bytes, must stay far inside 63 bits
  const int64_t kMaxElems = (int64_t)1 << 40;
  int64_t elems = 0;
  for (int i = 1; i <= L; ++i) {
    const int64_t bl = p.bond[i - 1], br = p.bond[i];
    if (bl > kMaxElems / d / br || elems > kMaxElems - bl * d * br)
      return serr(TN_EINVAL, "serve: the MPS has more than 2^40 elements");
    elems += bl * d * br;
  }
  size_t bytes = 0;
  for (int i = 1; i <= L; ++i) bytes += cxb(p.bond[i - 1] * d * p.bond[i]);
  bytes *= 2;  // A_i and X_i
  if (S->prec == TN_PREC_MIXED)
    for (int i = 1; i <= L; ++i) bytes += al(sizeof(cxf) * (size_t)(p.bond[i - 1] * d * p.bond[i]));
  if (S->budget && ctx->in_use + bytes > S->budget)
    return serr(TN_ENOMEM, "serve: the MPS needs %zu bytes; %zu of the %zu-byte HBM budget are in use", bytes,
                ctx->in_use, S->budget);
  tn_status_t st = tn_dev_alloc(ctx, bytes, &p.block);
  if (st != TN_OK) return serr(st, "%s", ctx->last_error.c_str());
  p.bytes = bytes;
  char* c = (char*)p.block;
  p.site.assign(L + 1, nullptr);
  p.dressed.assign(L + 1, nullptr);
  for (int i = 1; i <= L; ++i) {
    p.site[i] = (cxd*)c;
    c += cxb(p.bond[i - 1] * d * p.bond[i]);
  }
  for (int i = 1; i <= L; ++i) {
    p.dressed[i] = (cxd*)c;
    c += cxb(p.bond[i - 1] * d * p.bond[i]);
  }
  if (S->prec == TN_PREC_MIXED) {
    p.site32.assign(L + 1, nullptr);
    for (int i = 1; i <= L; ++i) {
      p.site32[i] = (cxf*)c;
      c += al(sizeof(cxf) * (size_t)(p.bond[i - 1] * d * p.bond[i]));
    }
  }
  return TN_OK;
}

// X_i and ⟨ψ|ψ⟩; sites already on the device (stream s_reg).  The left environments
// Lf_0..Lf_L are kept in the context workspace for the duration of the call; the right
// environment sweep then forms X_i = (Lf_{i-1} A_i) R_{i+1} site by site from right to
// left with two ping-pong R buffers.
tn_status_t pool_register(tn_server* S, PoolMPS& p, int32_t* id) {
  tn_ctx* ctx = S->ctx;
  ctx->stream = S->s_reg;
  const int L = p.L, d = p.d;
  const int64_t mx = p.maxbond;
  size_t need = 4 * cxb(mx * d * mx) + 4 * kAlign;
  for (int i = 0; i <= L; ++i) need += cxb(p.bond[i] * p.bond[i]);
  tn_status_t st = ws_reserve(ctx, need);
  cxd* normslot = nullptr;
  if (st == TN_OK) {
    cxd* T = ws_take<cxd>(ctx, (size_t)(mx * d * mx));
    cxd* T1 = ws_take<cxd>(ctx, (size_t)(mx * d * mx));
    cxd* Ra = ws_take<cxd>(ctx, (size_t)(mx * mx));
    cxd* Rb = ws_take<cxd>(ctx, (size_t)(mx * mx));
    std::vector<cxd*> Lf(L + 1);
    for (int i = 0; i <= L; ++i) Lf[i] = ws_take<cxd>(ctx, (size_t)(p.bond[i] * p.bond[i]));
    k_fill_one<double><<<1, 32, 0, ctx->stream>>>(Lf[0], 1, 1);
    k_fill_one<double><<<1, 32, 0, ctx->stream>>>(Ra, 1, 1);  // R_{L+1}
    ctx->launches += 2;
    for (int i = 1; i <= L && st == TN_OK; ++i) {
      const int64_t x = p.bond[i - 1], x2 = p.bond[i];
      // Lf_i (x2 × x2) = Aᴴ ((x d) × x2)ᴴ · (Lf_{i-1} (x × x) · A (x × d x2))
      st = gemm_cx<double>(ctx, 'N', 'N', x, d * x2, x, kOne, Lf[i - 1], x, 0, p.site[i], x, 0, kZero, T, x, 0, 1);
      if (st == TN_OK)
        st = gemm_cx<double>(ctx, 'C', 'N', x2, x2, x * d, kOne, p.site[i], x * d, 0, T, x * d, 0, kZero, Lf[i], x2, 0,
                             1);
    }
    normslot = Lf[L];
    cxd* Rn = Ra;  // R_{i+1}
    cxd* Rf = Rb;
    for (int i = L; i >= 1 && st == TN_OK; --i) {
      const int64_t x = p.bond[i - 1], x2 = p.bond[i];
      // X_i ((x d) × x2) = (Lf_{i-1} (x × x) · A (x × d x2)) · R_{i+1} (x2 × x2)
      st = gemm_cx<double>(ctx, 'N', 'N', x, d * x2, x, kOne, Lf[i - 1], x, 0, p.site[i], x, 0, kZero, T1, x, 0, 1);
      if (st == TN_OK)
        st = gemm_cx<double>(ctx, 'N', 'N', x * d, x2, x2, kOne, T1, x * d, 0, Rn, x2, 0, kZero, p.dressed[i], x * d, 0,
                             1);
      if (i == 1 || st != TN_OK) break;
      // R_i (x × x) = (A ((x d) × x2) · R_{i+1}) as (x × d x2) · A as (x × d x2)ᴴ
      st = gemm_cx<double>(ctx, 'N', 'N', x * d, x2, x2, kOne, p.site[i], x * d, 0, Rn, x2, 0, kZero, T, x * d, 0, 1);
      if (st == TN_OK)
        st = gemm_cx<double>(ctx, 'N', 'C', x, x, d * x2, kOne, T, x, 0, p.site[i], x, 0, kZero, Rf, x, 0, 1);
      std::swap(Rn, Rf);
    }
    for (int i = 1; i <= L && st == TN_OK && S->prec == TN_PREC_MIXED; ++i) {
      const int64_t e = p.bond[i - 1] * d * p.bond[i];
      k_d2f_cx<<<nblk(e), 256, 0, ctx->stream>>>(e, p.site[i], p.site32[i]);
      ctx->launches++;
    }
  }
  cxd h = {0, 0};
  if (st == TN_OK && cudaMemcpyAsync(&h, normslot, sizeof(cxd), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
    st = tn_set_error(ctx, TN_ECUDA, "serve: norm read-back failed");
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && st == TN_OK)
    st = tn_set_error(ctx, TN_ECUDA, "serve: registration failed: %s", cudaGetErrorString(cudaGetLastError()));
  if (st == TN_OK && !(h.x > 0 && std::isfinite(h.x))) st = tn_set_error(ctx, TN_EINVAL, "serve: ⟨ψ|ψ⟩ = %g", h.x);
  if (st != TN_OK) {
    std::string msg = ctx->last_error;
    tn_dev_free(ctx, p.block);
    return serr(st, "%s", msg.c_str());
  }
  p.norm2 = h.x;
  std::lock_guard<std::mutex> lock(S->mu);
  *id = S->next_id++;
  S->pool[*id] = std::move(p);
  return TN_OK;
}

std::vector<int64_t> clamped_bonds(int L, int d, int64_t chi) {
  std::vector<int64_t> b(L - 1);
  for (int i = 1; i < L; ++i) {
    const int e = std::min(i, L - i);
    int64_t cap = 1;
    for (int k = 0; k < e && cap < chi; ++k) cap *= d;
    b[i - 1] = std::min(chi, cap);
  }
  return b;
}

}  // namespace

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" {

tn_status_t tn_serve_create(int32_t device, size_t hbm_budget, size_t work_bytes, int32_t max_batch,
                            tn_precision_t precision, tn_server** out) {
  if (!out) return serr(TN_EINVAL, "tn_serve_create: null output");
  if (precision != TN_PREC_NATIVE && precision != TN_PREC_MIXED)
    return serr(TN_EINVAL, "tn_serve_create: precision must be native or mixed");
  if (work_bytes < (1 << 20)) return serr(TN_EINVAL, "tn_serve_create: work_bytes must be at least 1 MiB");
  if (hbm_budget && work_bytes >= hbm_budget)
    return serr(TN_EINVAL, "tn_serve_create: work_bytes (%zu) must be below the HBM budget (%zu)", work_bytes,
                hbm_budget);
  tn_ctx* ctx = nullptr;
  tn_status_t st = tn_create(&ctx, device);
  if (st != TN_OK) return serr(st, "%s", tn_last_error_string(nullptr));
  auto* S = new tn_server();
  S->ctx = ctx;
  S->device = device;
  S->budget = hbm_budget;
  S->max_batch = max_batch > 0 ? max_batch : 64;
  S->prec = precision;
  // short jobs (amplitudes, ⟨O_i⟩) get the highest stream priority: their thread blocks
  // are scheduled ahead of the long overlap sweeps as SMs free up
  int prio_low = 0, prio_high = 0;
  cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  bool ok = cudaStreamCreateWithPriority(&S->s_main, cudaStreamNonBlocking, prio_high) == cudaSuccess &&
            cudaStreamCreateWithFlags(&S->s_reg, cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; k < kOvlStreams && ok; ++k)
    ok = cudaStreamCreateWithPriority(&S->s_ovl[k], cudaStreamNonBlocking, prio_low) == cudaSuccess;
  if (ok) {
    st = tn_dev_alloc(ctx, work_bytes, &S->arena_mem);
    ok = st == TN_OK;
  }
  if (!ok) {
    std::string msg = ctx->last_error.empty() ? "stream creation failed" : ctx->last_error;
    tn_serve_destroy(S);
    return serr(TN_ENOMEM, "tn_serve_create: %s", msg.c_str());
  }
  S->arena.reset((char*)S->arena_mem, work_bytes);
  S->slots.resize(kMaxShort + kMaxOverlaps + 2);
  S->worker = std::thread(worker_main, S);
  *out = S;
  return TN_OK;
}

tn_status_t tn_serve_destroy(tn_server* S) {
  if (!S) return TN_OK;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    S->events++;
  }
  S->cv.notify_all();
  if (S->worker.joinable()) S->worker.join();  // drains pending queries and running jobs
  if (S->s_main) cudaStreamSynchronize(S->s_main);
  for (auto s : S->s_ovl)
    if (s) cudaStreamSynchronize(s);
  tn_ctx* ctx = S->ctx;
  ctx->stream = ctx->own_stream;
  for (auto& kv : S->pool) tn_dev_free(ctx, kv.second.block);
  if (S->arena_mem) tn_dev_free(ctx, S->arena_mem);
  for (auto& ps : S->slots)
    if (ps.h) cudaFreeHost(ps.h);
  if (S->s_main) cudaStreamDestroy(S->s_main);
  if (S->s_reg) cudaStreamDestroy(S->s_reg);
  for (auto s : S->s_ovl)
    if (s) cudaStreamDestroy(s);
  tn_destroy(ctx);
  delete S;
  return TN_OK;
}

tn_status_t tn_serve_add_mps(tn_server* S, int32_t L, int32_t d, const int64_t* bond_dims, const void* const* h_sites,
                             int32_t* id) {
  if (!S || !id || !h_sites || (L > 1 && !bond_dims) || L < 1 || d < 1)
    return serr(TN_EINVAL, "tn_serve_add_mps: bad arguments");
  std::lock_guard<std::mutex> ex(S->exec_mu);
  PoolMPS p;
  TN_RETURN_IF(pool_alloc(S, L, d, bond_dims, p));
  S->ctx->stream = S->s_reg;
  for (int i = 1; i <= L; ++i) {
    if (cudaMemcpyAsync(p.site[i], h_sites[i - 1], sizeof(cxd) * p.bond[i - 1] * d * p.bond[i], cudaMemcpyHostToDevice,
                        S->s_reg) != cudaSuccess) {
      cudaStreamSynchronize(S->s_reg);
      tn_dev_free(S->ctx, p.block);
      return serr(TN_ECUDA, "tn_serve_add_mps: upload of site %d failed", i);
    }
  }
  return pool_register(S, p, id);
}

tn_status_t tn_serve_add_random_mps(tn_server* S, int32_t L, int32_t d, int64_t chi, uint64_t seed, int32_t* id) {
  if (!S || !id || L < 2 || d < 1 || chi < 1) return serr(TN_EINVAL, "tn_serve_add_random_mps: bad arguments");
  std::lock_guard<std::mutex> ex(S->exec_mu);
  std::vector<int64_t> bonds = clamped_bonds(L, d, chi);
  PoolMPS p;
  TN_RETURN_IF(pool_alloc(S, L, d, bonds.data(), p));
  tn_ctx* ctx = S->ctx;
  ctx->stream = S->s_reg;
  for (int i = 1; i <= L; ++i) {
    const int64_t e = p.bond[i - 1] * d * p.bond[i];
    // variance 1/(d χ_{i-1}) per entry: the mean transfer map keeps ⟨ψ|ψ⟩ of order one
    const double scale = 1.0 / std::sqrt((double)(d * p.bond[i - 1]));
    k_fill_gauss<<<nblk(e), 256, 0, ctx->stream>>>(p.site[i], e, seed * 0x9E3779B97F4A7C15ull + (uint64_t)i, scale);
    ctx->launches++;
  }
  return pool_register(S, p, id);
}

tn_status_t tn_serve_remove_mps(tn_server* S, int32_t id) {
  if (!S) return serr(TN_EINVAL, "tn_serve_remove_mps: null server");
  std::lock_guard<std::mutex> ex(S->exec_mu);
  void* block = nullptr;
  {
    std::unique_lock<std::mutex> lock(S->mu);
    auto it = S->pool.find(id);
    if (it == S->pool.end()) return serr(TN_EINVAL, "tn_serve_remove_mps: unknown id %d", id);
    // running jobs that read it finish first (they retire without the worker: it waits
    // for exec_mu, so completion is observed here)
    while (it->second.inflight > 0) {
      lock.unlock();
      for (auto& j : S->jobs) cudaStreamSynchronize(j->stream);
      lock.lock();
      for (auto jt = S->jobs.begin(); jt != S->jobs.end();) {
        Job* j = jt->get();
        if (j->finished.load()) {
          finish_tickets(S, j->tickets, j->submit, TN_OK, "",
                         (const cxd*)((const char*)S->slots[j->slot].h + j->res_off), &j->scale);
          release_job(S, j);
          jt = S->jobs.erase(jt);
        } else {
          ++jt;
        }
      }
      S->cv_done.notify_all();
      it = S->pool.find(id);
    }
    block = it->second.block;
    S->pool.erase(it);
  }
  return tn_dev_free(S->ctx, block) == TN_OK ? TN_OK : serr(TN_ECUDA, "%s", S->ctx->last_error.c_str());
}

tn_status_t tn_serve_mps_info(tn_server* S, int32_t id, int32_t* L, int32_t* d, int64_t* bond_dims, double* norm2) {
  if (!S || !L || !d) return serr(TN_EINVAL, "tn_serve_mps_info: bad arguments");
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->pool.find(id);
  if (it == S->pool.end()) return serr(TN_EINVAL, "tn_serve_mps_info: unknown id %d", id);
  *L = it->second.L;
  *d = it->second.d;
  if (bond_dims)
    for (int i = 1; i < it->second.L; ++i) bond_dims[i - 1] = it->second.bond[i];
  if (norm2) *norm2 = it->second.norm2;
  return TN_OK;
}

tn_status_t tn_serve_get_site(tn_server* S, int32_t id, int32_t site, void* h_data) {
  if (!S || !h_data) return serr(TN_EINVAL, "tn_serve_get_site: bad arguments");
  std::lock_guard<std::mutex> ex(S->exec_mu);
  cxd* src = nullptr;
  size_t bytes = 0;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->pool.find(id);
    if (it == S->pool.end()) return serr(TN_EINVAL, "tn_serve_get_site: unknown id %d", id);
    const PoolMPS& p = it->second;
    if (site < 1 || site > p.L) return serr(TN_EINVAL, "tn_serve_get_site: site %d out of range", site);
    src = p.site[site];
    bytes = sizeof(cxd) * p.bond[site - 1] * p.d * p.bond[site];
  }
  if (cudaMemcpyAsync(h_data, src, bytes, cudaMemcpyDeviceToHost, S->s_reg) != cudaSuccess ||
      cudaStreamSynchronize(S->s_reg) != cudaSuccess)
    return serr(TN_ECUDA, "tn_serve_get_site: copy failed");
  return TN_OK;
}

tn_status_t tn_serve_submit(tn_server* S, const tn_query* q, int64_t* ticket) {
  if (!S || !q || !ticket) return serr(TN_EINVAL, "tn_serve_submit: bad arguments");
  Query Q;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    if (S->stop) return serr(TN_EINVAL, "tn_serve_submit: the server is shutting down");
    auto it = S->pool.find(q->mps);
    if (it == S->pool.end()) return serr(TN_EINVAL, "tn_serve_submit: unknown MPS id %d", q->mps);
    const PoolMPS& p = it->second;
    Q.kind = q->kind;
    Q.a = q->mps;
    Q.b = q->mps_b;
    Q.site = q->site;
    if (q->kind == TN_Q_AMPLITUDE) {
      if (!q->data) return serr(TN_EINVAL, "tn_serve_submit: an amplitude needs L×d product vectors");
      Q.data.assign((const cxd*)q->data, (const cxd*)q->data + (size_t)p.L * p.d);
    } else if (q->kind == TN_Q_EXPECTATION) {
      if (!q->data) return serr(TN_EINVAL, "tn_serve_submit: an expectation value needs a d×d operator");
      if (q->site < 1 || q->site > p.L) return serr(TN_EINVAL, "tn_serve_submit: site %d out of range", q->site);
      Q.data.assign((const cxd*)q->data, (const cxd*)q->data + (size_t)p.d * p.d);
    } else if (q->kind == TN_Q_OVERLAP) {
      auto jt = S->pool.find(q->mps_b);
      if (jt == S->pool.end()) return serr(TN_EINVAL, "tn_serve_submit: unknown MPS id %d", q->mps_b);
      if (jt->second.L != p.L || jt->second.d != p.d)
        return serr(TN_EINVAL, "tn_serve_submit: an overlap needs two MPS of equal length and physical dimension");
    } else {
      return serr(TN_EINVAL, "tn_serve_submit: unknown query kind %d", q->kind);
    }
    const size_t need = query_bytes(S, Q) + cxb(1);
    if (need > S->arena.cap)
      return serr(TN_ENOMEM, "tn_serve_submit: the query needs %zu bytes of workspace; the server has %zu", need,
                  S->arena.cap);
    Q.ticket = S->next_ticket++;
    Q.t_submit = now_s();
    *ticket = Q.ticket;
    S->results[Q.ticket] = Result();
    S->pending.push_back(std::move(Q));
    S->events++;
  }
  S->cv.notify_all();
  return TN_OK;
}

tn_status_t tn_serve_wait(tn_server* S, int64_t ticket, double timeout_s, double* h_value, double* latency_s) {
  if (!S) return serr(TN_EINVAL, "tn_serve_wait: null server");
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->results.find(ticket);
  if (it == S->results.end()) return serr(TN_EINVAL, "tn_serve_wait: unknown ticket %lld", (long long)ticket);
  const auto limit = std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0.0);
  if (!S->cv_done.wait_for(lock, limit, [&] { return S->results[ticket].done; }))
    return serr(TN_ETIMEOUT, "tn_serve_wait: ticket %lld not done within %.3f s", (long long)ticket, timeout_s);
  Result r = S->results[ticket];
  S->results.erase(ticket);
  if (r.status != TN_OK) return serr(r.status, "serve: %s", r.err.c_str());
  if (h_value) {
    h_value[0] = r.value.x;
    h_value[1] = r.value.y;
  }
  if (latency_s) *latency_s = r.latency;
  return TN_OK;
}

tn_status_t tn_serve_stats(tn_server* S, int64_t* h_stats) {
  if (!S || !h_stats) return serr(TN_EINVAL, "tn_serve_stats: bad arguments");
  std::lock_guard<std::mutex> lock(S->mu);
  h_stats[0] = S->completed;
  h_stats[1] = S->short_jobs;
  h_stats[2] = S->overlap_jobs;
  h_stats[3] = S->max_batch_seen;
  h_stats[4] = S->deferred;
  h_stats[5] = (int64_t)pool_bytes(S);
  h_stats[6] = (int64_t)S->pending.size();
  h_stats[7] = (int64_t)(S->short_inflight + S->ovl_inflight);
  return TN_OK;
}

const char* tn_serve_last_error(void) { return t_serve_error.c_str(); }

}  // extern "C"
