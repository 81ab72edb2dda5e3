// K2 (tensor cores) — TMA-fed tcgen05 GEMM with the accumulator in TMEM, kind::tf32.
//
//   C (M×N, column-major) = Σ_p  A_p ᵀ · B_p      over 1 or 3 operand pairs p
//
// Both operands are K-major (the contraction index contiguous), which is the layout the
// contraction planner produces with the permutation kernel.  Precision modes:
//   * TF32      — one pass (A, B), FP32 accumulation;
//   * 3×TF32    — three passes A_hi·B_hi + (A_hi·B_lo + A_lo·B_hi), where x_hi is x
//                 rounded to nearest TF32 and x_lo = x − x_hi exactly; the hi·hi pass and
//                 the two small correction passes accumulate in separate TMEM
//                 accumulators (the corrections would otherwise be lost to the large
//                 accumulator's alignment) and are summed in the epilogue: FP32-grade
//                 products from the TF32 tensor pipe.
// Complex operands use the real 4M form as one real GEMM of twice the size:
//   [Re C; Im C] = [[Ar, −Ai], [Ai, Ar]] · [Br; Bi]
// built by a prep kernel that also does the hi/lo split, with an epilogue that writes the
// two row blocks back as interleaved complex.
//
// CTA (128 threads) per 128×256 output tile, tiles visited in bands of 8 row tiles so
// the resident CTAs share their operand panels in L2.  Thread 0 issues TMA loads
// (128-byte swizzle, 4-stage ring of 48 KB stages with full/empty mbarriers), thread 32
// issues tcgen05.mma (M=128, N=256, K=8 per instruction; accumulator = 256 TMEM
// columns) and commits each stage back to its empty barrier; all four warps then drain
// TMEM with tcgen05.ld (warp w owns accumulator rows 32w…32w+31).  Every mbarrier wait is bounded: on timeout the kernel records an error
// word, skips the remaining work, and still releases its TMEM.
#include <cuda.h>

#include <cstring>

#include "tn_internal.cuh"

namespace {

constexpr int BM = 128, BN = 256, BKB = 128;  // tile: 128×256 outputs, 128 bytes of K
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * BKB, B_BYTES = BN * BKB;
constexpr int SMEM_BYTES = STAGES * (A_BYTES + B_BYTES) + 1024 /*align*/ + 256 /*barriers*/;
constexpr long long kSpinLimit = 1ll << 28;
constexpr int kGroupM = 8;

struct Maps {
  CUtensorMap a[2];  // A_hi, A_lo
  CUtensorMap b[2];  // B_hi, B_lo
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false (and the error word set) if the phase never completes
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (long long i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  atomicExch(err, 1);
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(const void* p) {
  const uint64_t addr = (uint64_t)smem_u32(p);
  uint64_t d = (addr & 0x3FFFFull) >> 4;  // start address
  d |= 1ull << 16;                        // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset: 8 rows × 128 B
  d |= 1ull << 46;                        // descriptor version for tcgen05
  d |= 2ull << 61;                        // 128-byte swizzle
  return d;
}
// instruction descriptor: D f32, A/B tf32, both K-major, N = BN, M = BM
constexpr uint32_t kIdescTF32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                                ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(a), "l"(b), "r"(kIdescTF32), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

template <int EPI>  // 0: real C (float); 1: complex interleaved from [Re; Im] row blocks
__global__ void __launch_bounds__(128, 1)
    k_gemm_tf32(const __grid_constant__ Maps maps, int passes, int M, int N, int K, float* __restrict__ C,
                int64_t ldc, int Mh, float alpha, float beta, int* err) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t base_u = smem_u32(smem_raw);
  unsigned char* smem = smem_raw + ((1024 - (base_u & 1023)) & 1023);
  unsigned char* sA = smem;
  unsigned char* sB = smem + STAGES * A_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * (A_BYTES + B_BYTES));
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* done = bars + 2 * STAGES;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // grouped tile order: consecutive CTAs sweep the N tiles of a band of kGroupM row tiles,
  // so the CTAs resident at one time share their A and B panels in L2
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const int per_group = kGroupM * tiles_n;
  const int grp = (int)blockIdx.x / per_group, first_m = grp * kGroupM;
  const int gsize = min(kGroupM, tiles_m - first_m);
  const int in_grp = (int)blockIdx.x % per_group;
  const int m0 = (first_m + in_grp % gsize) * BM, n0 = (in_grp / gsize) * BN;
  const uint32_t tcols = passes > 1 ? 2 * BN : BN;  // hi·hi accumulator [+ corrections]
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(tcols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  const int nk = (K + 31) / 32;  // 32 fp32 = 128 bytes of K per tile
  const int total = passes * nk;
  if (tid == 0) {
    // producer
    for (int t = 0; t < total; ++t) {
      const int s = t % STAGES;
      if (t >= STAGES && !mbar_wait(&empty[s], ((t / STAGES) & 1) ^ 1, err)) break;
      const int pass = t / nk, kt = t % nk;
      const CUtensorMap* am = &maps.a[pass == 2 ? 1 : 0];
      const CUtensorMap* bm = &maps.b[pass == 1 ? 1 : 0];
      mbar_expect_tx(&full[s], A_BYTES + B_BYTES);
      tma_load_2d(sA + s * A_BYTES, am, &full[s], kt * 32, m0);
      tma_load_2d(sB + s * B_BYTES, bm, &full[s], kt * 32, n0);
    }
  } else if (tid == 32) {
    // MMA issuer
    bool ok = true;
    for (int t = 0; t < total && ok; ++t) {
      const int s = t % STAGES;
      ok = mbar_wait(&full[s], (t / STAGES) & 1, err);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int pass = t / nk;
      const uint32_t acc = tmem + (pass > 0 ? (uint32_t)BN : 0u);  // corrections: their own accumulator
      const bool first = (t % nk == 0) && pass <= 1;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {  // 4 × (K = 8 tf32 = 32 bytes)
        const uint64_t a = sdesc(sA + s * A_BYTES) + (uint64_t)((kk * 32) >> 4);
        const uint64_t b = sdesc(sB + s * B_BYTES) + (uint64_t)((kk * 32) >> 4);
        mma_tf32(acc, a, b, (first && kk == 0) ? 0u : 1u);
      }
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  __syncwarp();
  // epilogue: all 4 warps
  const bool ok = mbar_wait(done, 0, err);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (passes > 1) {  // add the correction accumulator
        uint32_t q[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(q[0]), "=r"(q[1]), "=r"(q[2]), "=r"(q[3]), "=r"(q[4]), "=r"(q[5]), "=r"(q[6]), "=r"(q[7]),
              "=r"(q[8]), "=r"(q[9]), "=r"(q[10]), "=r"(q[11]), "=r"(q[12]), "=r"(q[13]), "=r"(q[14]), "=r"(q[15])
            : "r"(taddr + (uint32_t)BN));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) r[j] = __float_as_uint(__uint_as_float(r[j]) + __uint_as_float(q[j]));
      }
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (col >= N) break;
          float v = alpha * __uint_as_float(r[j]);
          float* dst;
          if (EPI == 0)
            dst = C + row + (int64_t)col * ldc;
          else
            dst = C + 2 * ((int64_t)(row % Mh) + (int64_t)col * ldc) + (row >= Mh ? 1 : 0);
          if (beta != 0.f) v += beta * *dst;
          *dst = v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols) : "memory");
}

// ---------------------------------------------------------------------------------
// operand preparation: K-major real planes (hi, lo) with K padded to Kp (multiple of 32)
// ---------------------------------------------------------------------------------
// x rounded to the nearest TF32 value (10-bit mantissa, ties away from zero): the
// remainder x − hi is exact in FP32 and at most half a TF32 unit
__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// element (r, c) of op(X) for a column-major complex X with leading dimension ld
__device__ __forceinline__ cxf ld_op(const cxf* X, int64_t ld, char op, int64_t r, int64_t c) {
  if (op == 'N') return X[r + c * ld];
  cxf v = X[c + r * ld];
  if (op == 'C') v.y = -v.y;
  return v;
}

// A' (rows i' < 2M, K-major, pitch Kp): i' < M → [Ar, −Ai], i' ≥ M → [Ai, Ar]
__global__ void k_prep_a_cx(int64_t M, int64_t K, int64_t Kp, const cxf* A, int64_t lda, char op, float* hi, float* lo) {
  const int64_t total = 2 * M * Kp;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t kp = t % Kp, ip = t / Kp;
    float v = 0.f;
    if (kp < 2 * K) {
      const int64_t i = ip % M, k = kp % K;
      const cxf a = ld_op(A, lda, op, i, k);
      const bool top = ip < M, left = kp < K;
      v = top ? (left ? a.x : -a.y) : (left ? a.y : a.x);
    }
    const float h = tf32_hi(v);
    hi[t] = h;
    if (lo) lo[t] = v - h;
  }
}
// A' for op(A) = A (M-major source): 32×32 tiles of A staged through shared memory so
// that both the reads (along i) and the K-major writes (along k) are coalesced; the four
// quadrants [Ar, −Ai; Ai, Ar] of the tile are written from the staged tile.  Columns
// kp ≥ 2K of A' (the padding) are written by k_prep_a_pad.
__global__ void __launch_bounds__(256) k_prep_a_cx_n(int64_t M, int64_t K, int64_t Kp, const cxf* __restrict__ A,
                                                     int64_t lda, float* __restrict__ hi, float* __restrict__ lo) {
  __shared__ cxf tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 × 8
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + tx, k = k0 + r;
    tile[r][tx] = (i < M && k < K) ? A[i + k * lda] : mkcx(0.f, 0.f);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + r, k = k0 + tx;
    if (i >= M || k >= K) continue;
    const cxf a = tile[tx][r];
    const float q[4] = {a.x, -a.y, a.y, a.x};  // (top,left) (top,right) (bottom,left) (bottom,right)
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t ip = i + (u >= 2 ? M : 0), kp = k + ((u & 1) ? K : 0);
      const float v = q[u], h = tf32_hi(v);
      hi[ip * Kp + kp] = h;
      if (lo) lo[ip * Kp + kp] = v - h;
    }
  }
}
__global__ void k_prep_a_pad(int64_t M2, int64_t K2, int64_t Kp, float* hi, float* lo) {
  const int64_t w = Kp - K2, total = M2 * w;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ip = t / w, kp = K2 + t % w;
    hi[ip * Kp + kp] = 0.f;
    if (lo) lo[ip * Kp + kp] = 0.f;
  }
}
// B' (columns j < N, K-major, pitch Kp): [Br; Bi]
__global__ void k_prep_b_cx(int64_t N, int64_t K, int64_t Kp, const cxf* B, int64_t ldb, char op, float* hi, float* lo) {
  const int64_t total = N * Kp;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t kp = t % Kp, j = t / Kp;
    float v = 0.f;
    if (kp < 2 * K) {
      const cxf b = ld_op(B, ldb, op, kp % K, j);
      v = kp < K ? b.x : b.y;
    }
    const float h = tf32_hi(v);
    hi[t] = h;
    if (lo) lo[t] = v - h;
  }
}
// real: A' (M rows, K-major) from op(A); B' (N columns, K-major) from op(B)
__global__ void k_prep_re(int64_t R, int64_t K, int64_t Kp, const float* X, int64_t ld, bool kmajor_src, float* hi,
                          float* lo) {
  const int64_t total = R * Kp;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t kp = t % Kp, r = t / Kp;
    float v = 0.f;
    if (kp < K) v = kmajor_src ? X[kp + r * ld] : X[r + kp * ld];
    const float h = tf32_hi(v);
    hi[t] = h;
    if (lo) lo[t] = v - h;
  }
}

EncodeTiledFn encode_fn(tn_ctx* ctx) { return tn_encode_tiled_fn(ctx); }

// K-major operand: rows × Kp floats, row pitch Kp·4 bytes; box 32 floats × box_rows
tn_status_t make_map(tn_ctx* ctx, CUtensorMap* map, const float* base, int64_t rows, int64_t Kp, uint32_t box_rows) {
  EncodeTiledFn fn = encode_fn(ctx);
  if (!fn) return TN_ECUDA;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(Kp * 4)};
  cuuint32_t box[2] = {32, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tn_set_error(ctx, TN_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return TN_OK;
}

unsigned blocks_for(tn_ctx* ctx, int64_t n) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)ctx->num_sms * 16;
  return (unsigned)std::max<int64_t>(1, std::min(b, cap));
}

}  // namespace

// the driver's cuTensorMapEncodeTiled, looked up once through the runtime
EncodeTiledFn tn_encode_tiled_fn(tn_ctx* ctx) {
  static EncodeTiledFn fn = nullptr;
  if (fn) return fn;
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p) {
    tn_set_error(ctx, TN_ECUDA, "cuTensorMapEncodeTiled unavailable");
    return nullptr;
  }
  fn = (EncodeTiledFn)p;
  return fn;
}

// Workspace (bytes) for tc_gemm on the given shape.
// K-major operands are stored with K padded to a multiple of 4 floats (the 16-byte TMA
// pitch rule) and at least one 32-float box; the last box reads past K as zeros.
static inline int64_t padded_k(bool complex_in, int64_t k) {
  int64_t kk = complex_in ? 2 * k : k;
  kk = (kk + 3) / 4 * 4;
  return kk < 32 ? 32 : kk;
}

size_t tc_gemm_workspace(bool complex_in, int passes, int64_t m, int64_t n, int64_t k) {
  const int64_t Kp = padded_k(complex_in, k);
  const int64_t Ma = complex_in ? 2 * m : m;
  const int copies = passes > 1 ? 2 : 1;
  return copies * (ws_round(4 * (size_t)(Ma * Kp)) + ws_round(4 * (size_t)(n * Kp))) + ws_round(sizeof(int) * 4);
}

// C (m×n) = op(A)·op(B) on the TF32 tensor pipe (passes: 1 = TF32, 3 = 3×TF32).
// complex_in: A, B, C are interleaved complex (C64 data must be converted by the caller);
// otherwise real float.  beta applies to C (real).  Workspace reserved by the caller.
tn_status_t tc_gemm(tn_ctx* ctx, bool complex_in, int passes, char opa, char opb, int64_t m, int64_t n, int64_t k,
                    float alpha, const void* A, int64_t lda, const void* B, int64_t ldb, float beta, void* C, int64_t ldc) {
  if (m == 0 || n == 0) return TN_OK;
  const int64_t Kp = padded_k(complex_in, k);
  const int64_t Ma = complex_in ? 2 * m : m;
  if (Ma > (1ll << 31) - 128 || n > (1ll << 31) - 128) return tn_set_error(ctx, TN_EUNSUPPORTED, "tc_gemm: too large");
  const bool split = passes > 1;
  float* Ahi = ws_take<float>(ctx, (size_t)(Ma * Kp));
  float* Bhi = ws_take<float>(ctx, (size_t)(n * Kp));
  float* Alo = split ? ws_take<float>(ctx, (size_t)(Ma * Kp)) : nullptr;
  float* Blo = split ? ws_take<float>(ctx, (size_t)(n * Kp)) : nullptr;
  int* err = ws_take<int>(ctx, 4);
  TN_CHECK_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  if (complex_in) {
    if (opa == 'N') {
      k_prep_a_cx_n<<<dim3(cdiv(m, 32), cdiv(k, 32)), 256, 0, ctx->stream>>>(m, k, Kp, (const cxf*)A, lda, Ahi, Alo);
      TN_LAUNCHED(ctx);
      if (Kp > 2 * k) {
        k_prep_a_pad<<<blocks_for(ctx, Ma * (Kp - 2 * k)), 256, 0, ctx->stream>>>(Ma, 2 * k, Kp, Ahi, Alo);
        TN_LAUNCHED(ctx);
      }
    } else {
      k_prep_a_cx<<<blocks_for(ctx, Ma * Kp), 256, 0, ctx->stream>>>(m, k, Kp, (const cxf*)A, lda, opa, Ahi, Alo);
      TN_LAUNCHED(ctx);
    }
    k_prep_b_cx<<<blocks_for(ctx, n * Kp), 256, 0, ctx->stream>>>(n, k, Kp, (const cxf*)B, ldb, opb, Bhi, Blo);
    TN_LAUNCHED(ctx);
  } else {
    // A' rows are the m rows of op(A): K-major source when op(A) = Aᵀ
    k_prep_re<<<blocks_for(ctx, m * Kp), 256, 0, ctx->stream>>>(m, k, Kp, (const float*)A, lda, opa != 'N', Ahi, Alo);
    TN_LAUNCHED(ctx);
    k_prep_re<<<blocks_for(ctx, n * Kp), 256, 0, ctx->stream>>>(n, k, Kp, (const float*)B, ldb, opb == 'N', Bhi, Blo);
    TN_LAUNCHED(ctx);
  }
  Maps maps;
  memset(&maps, 0, sizeof(maps));
  TN_RETURN_IF(make_map(ctx, &maps.a[0], Ahi, Ma, Kp, BM));
  TN_RETURN_IF(make_map(ctx, &maps.b[0], Bhi, n, Kp, BN));
  if (split) {
    TN_RETURN_IF(make_map(ctx, &maps.a[1], Alo, Ma, Kp, BM));
    TN_RETURN_IF(make_map(ctx, &maps.b[1], Blo, n, Kp, BN));
  } else {
    maps.a[1] = maps.a[0];
    maps.b[1] = maps.b[0];
  }
  const int64_t tiles = (int64_t)cdiv(Ma, BM) * cdiv(n, BN);
  if (tiles > 0x7fffffffll) return tn_set_error(ctx, TN_EUNSUPPORTED, "tc_gemm: too many tiles");
  const dim3 grid((unsigned)tiles);
  if (complex_in) {
    TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_gemm_tf32<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    k_gemm_tf32<1><<<grid, 128, SMEM_BYTES, ctx->stream>>>(maps, passes, (int)Ma, (int)n, (int)Kp, (float*)C, ldc,
                                                           (int)m, alpha, beta, err);
  } else {
    TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_gemm_tf32<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    k_gemm_tf32<0><<<grid, 128, SMEM_BYTES, ctx->stream>>>(maps, passes, (int)Ma, (int)n, (int)Kp, (float*)C, ldc,
                                                           (int)m, alpha, beta, err);
  }
  TN_LAUNCHED(ctx);
  int* hp = reinterpret_cast<int*>(ctx->pinned);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(hp, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hp[0]) return tn_set_error(ctx, TN_ETIMEOUT, "tc_gemm: a pipeline wait timed out");
  return TN_OK;
}
