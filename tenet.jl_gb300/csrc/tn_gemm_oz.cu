// K2c — ComplexF64 GEMM from exact BF16 digit planes on the tcgen05 tensor pipe
// (an error-free splitting in the manner of Ozaki, Ogita, Oishi & Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012)).
//
//   C = alpha · op(A) · op(B) + beta · C          (A, B, C ComplexF64, column-major)
//
// Splitting.  Every row i of op(A) gets a power-of-two scale σ_i ≥ max_k(|Re a_ik|,
// |Im a_ik|) and every column j of op(B) a scale τ_j.  Each real part v of an entry is
// cut into S signed digits of b bits (b ≤ 8):
//     v = σ · 2^{2-b} · Σ_{p=0}^{S-1} d_p · 2^{-bp} + r,   |d_p| ≤ 2^{b-1} integers,
//     |r| ≤ 2^{1-bS} σ,
// computed exactly (the top digit rint(2^{b-2}·v/σ) in FP64 — one bit of headroom, so the
// carry from the lower digits keeps it within 2^{b-1} — the others as balanced base-2^b
// digits of the remainder held as one int64).  Every digit is an integer of magnitude
// ≤ 2^{b-1} ≤ 128, exactly representable in BF16.
//
// Products.  Complex arithmetic uses the real 4M form with Re/Im rows interleaved:
//     A''[2i]   = [Re a_i·, −Im a_i·],  A''[2i+1] = [Im a_i·, Re a_i·]   (2m × 2k)
//     B''[j]    = [Re b_·j,  Im b_·j]                                      (n × 2k)
// so that (A''·B''ᵀ)[2i + c, j] is Re (c = 0) or Im (c = 1) of (op(A)·op(B))_ij.  The
// digit planes D^A_p, D^B_q (p, q < S) are multiplied on the tensor pipe (kind::f16,
// BF16 inputs, FP32 accumulation) for every pair with p + q < S, and all pairs of one
// level L = p + q accumulate into one TMEM accumulator.  A level holds at most S pairs
// of K = 2k products of magnitude ≤ 2^{2b-2}, so its sum is an integer ≤ S·K·2^{2b-2};
// b is the widest digit with S·K·2^{2b-2} ≤ 2^24, which keeps the FP32 accumulation
// exact, and contractions too long for b = 7 are split on the host into chunks that
// accumulate into C.  The epilogue combines the levels exactly in int64 (the FP64 pipe
// is the scarce one on this part) and applies σ_i τ_j 2^{4-2b} in FP64:
//     c_ij = σ_i τ_j 2^{4-2b} Σ_L 2^{-bL} acc_L.
// The only approximation is the dropped pairs (p + q ≥ S) and the digit remainders, of
// relative size ~S·2^{1-bS} per product: S = 8, b = 7 gives ~52 bits, FP64-grade products.
//
// Kernel.  One CTA (6 warps) per 128×64 tile of the real 4M product, for one batch
// instance.  Warp 4 lane 0 issues TMA loads: per K stage (64 BF16 = 128 bytes, 128-byte
// swizzle) all S digit planes of the B tile into one of two B buffers, then the S planes
// of the A tile through a 4-slot ring.  Warp 5 lane 0 issues tcgen05.mma (M=128, N=64,
// K=16): for plane p of A it multiplies every resident B plane q < S − p into level
// p + q (TMEM columns 64·(p+q)…).  Warps 0-3 then read the S level accumulators with
// tcgen05.ld (warp w owns rows 32w…32w+31), combine them in int64, exchange Re/Im with
// the neighbouring lane and write interleaved complex C.  Every mbarrier wait is
// bounded: on timeout the kernel records an error word, skips the remaining work and
// still releases its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "tn_internal.cuh"

namespace {

constexpr int OZ_BM = 128, OZ_BN = 64, OZ_BK = 64;  // tile 128×64, 64 BF16 (128 B) of K per stage
constexpr int OZ_MAX_S = 8;
constexpr int OZ_A_RING = 4;
constexpr int OZ_A_TILE = OZ_BM * OZ_BK * 2;  // 16 KB
constexpr int OZ_B_TILE = OZ_BN * OZ_BK * 2;  // 8 KB
constexpr int OZ_THREADS = 192;
constexpr long long kOzSpin = 1ll << 24;

inline int oz_smem_bytes(int S) { return OZ_A_RING * OZ_A_TILE + 2 * S * OZ_B_TILE + 1024 + 256; }

struct OzMaps {
  CUtensorMap a;  // digit planes of A'': (2k, 2m, S·batch), plane-major
  CUtensorMap b;  // digit planes of B'': (2k, n, S·batch)
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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (long long i = 0; i < kOzSpin; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  atomicExch(err, 1);
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(const void* p) {
  const uint64_t addr = (uint64_t)smem_u32(p);
  uint64_t d = (addr & 0x3FFFFull) >> 4;
  d |= 1ull << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= 1ull << 46;
  d |= 2ull << 61;
  return d;
}
// instruction descriptor, kind::f16: D f32, A and B bf16, both K-major, N = 64, M = 128
constexpr uint32_t kIdescBF16 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_BN >> 3) << 17) | ((uint32_t)(OZ_BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(a), "l"(b), "r"(kIdescBF16), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// grid: (tiles_m · tiles_n, batch); 192 threads
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_gemm_oz(const __grid_constant__ OzMaps maps, int S, int bits, int M2, int N, int K2, int batch, cxd* __restrict__ C,
              int64_t ldc, int64_t sC, const double* __restrict__ sig, const double* __restrict__ tau, cxd alpha,
              cxd beta, int beta_zero, int m_complex, int* err) {
  extern __shared__ unsigned char smem_raw[];
  const uint32_t base_u = smem_u32(smem_raw);
  unsigned char* smem = smem_raw + ((1024 - (base_u & 1023)) & 1023);
  unsigned char* sA = smem;                               // OZ_A_RING tiles
  unsigned char* sB = smem + OZ_A_RING * OZ_A_TILE;       // 2 buffers × S tiles
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + 2 * S * OZ_B_TILE);
  uint64_t* a_full = bars;                  // [OZ_A_RING]
  uint64_t* a_empty = bars + OZ_A_RING;     // [OZ_A_RING]
  uint64_t* b_full = bars + 2 * OZ_A_RING;  // [2]
  uint64_t* b_empty = b_full + 2;           // [2]
  uint64_t* done = b_empty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_m = (M2 + OZ_BM - 1) / OZ_BM;
  const int m0 = ((int)blockIdx.x % tiles_m) * OZ_BM, n0 = ((int)blockIdx.x / tiles_m) * OZ_BN;
  const int bidx = (int)blockIdx.y;
  const uint32_t tcols = S <= 4 ? 256u : 512u;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(tcols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
    for (int s = 0; s < OZ_A_RING; ++s) {
      mbar_init(&a_full[s], 1);
      mbar_init(&a_empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&b_full[s], 1);
      mbar_init(&b_empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const int nks = (K2 + OZ_BK - 1) / OZ_BK;

  if (warp == 4) {
    if (lane == 0) {
      // producer: per K stage, the S planes of the B tile, then the S planes of the A tile
      int ta = 0;
      bool ok = true;
      for (int ks = 0; ks < nks && ok; ++ks) {
        const int kb = ks & 1;
        if (ks >= 2 && !(ok = mbar_wait(&b_empty[kb], ((ks >> 1) & 1) ^ 1, err))) break;
        mbar_expect_tx(&b_full[kb], (uint32_t)(S * OZ_B_TILE));
        for (int q = 0; q < S; ++q)
          tma_load_3d(sB + (kb * S + q) * OZ_B_TILE, &maps.b, &b_full[kb], ks * OZ_BK, n0, q * batch + bidx);
        for (int p = 0; p < S; ++p, ++ta) {
          const int slot = ta % OZ_A_RING;
          if (ta >= OZ_A_RING && !(ok = mbar_wait(&a_empty[slot], ((ta / OZ_A_RING) & 1) ^ 1, err))) break;
          mbar_expect_tx(&a_full[slot], (uint32_t)OZ_A_TILE);
          tma_load_3d(sA + slot * OZ_A_TILE, &maps.a, &a_full[slot], ks * OZ_BK, m0, p * batch + bidx);
        }
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      // MMA issuer: plane p of A against every resident plane q < S - p of B, level p + q
      int ta = 0;
      bool ok = true;
      for (int ks = 0; ks < nks && ok; ++ks) {
        const int kb = ks & 1;
        if (!(ok = mbar_wait(&b_full[kb], (ks >> 1) & 1, err))) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int p = 0; p < S; ++p, ++ta) {
          const int slot = ta % OZ_A_RING;
          if (!(ok = mbar_wait(&a_full[slot], (ta / OZ_A_RING) & 1, err))) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint64_t a0 = sdesc(sA + slot * OZ_A_TILE);
          for (int q = 0; q < S - p; ++q) {
            const uint64_t b0 = sdesc(sB + (kb * S + q) * OZ_B_TILE);
            const uint32_t d = tmem + (uint32_t)((p + q) * OZ_BN);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)  // 4 × (K = 16 BF16 = 32 bytes)
              mma_bf16(d, a0 + (uint64_t)kk * 2, b0 + (uint64_t)kk * 2, (ks > 0 || p > 0 || kk > 0) ? 1u : 0u);
          }
          mma_commit(&a_empty[slot]);
        }
        mma_commit(&b_empty[kb]);
      }
      mma_commit(done);
    }
  } else {
    // epilogue: warps 0-3
    const bool ok = mbar_wait(done, 0, err);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
      const int row = m0 + warp * 32 + lane;  // real row of the 4M product: 2i + (0 Re | 1 Im)
      const int i = row >> 1;
      const bool re_lane = (lane & 1) == 0;
      // The levels are recombined exactly in int64 on the integer pipe (GB300's FP64 pipe
      // is ~1/70 of its FP32 pipe, and an FP64 Horner step per level and output kept it
      // busier than the tensor pipe): H = Σ_L acc_L · 2^{b(S−1−L)−D}, each acc_L an
      // integer of magnitude ≤ 2^24 (exact in FP32), D = max(0, b(S−1) − 37) so that
      // |H| < 2^62; the levels below 2^D are rounded to nearest (an error of at most
      // S/2 units of 2^{D−b(S−1)} relative to acc_0, below 2^-60 of the largest term).
      // One conversion to FP64 per output, then the scales σ_i τ_j 2^{4−2b+D−b(S−1)}.
      const int D = bits * (S - 1) > 37 ? bits * (S - 1) - 37 : 0;
      const double si =
          (row < M2) ? ldexp(sig[(int64_t)bidx * m_complex + i], 4 - 2 * bits + D - bits * (S - 1)) : 0.0;
      const bool alpha_one = alpha.x == 1.0 && alpha.y == 0.0;
      cxd* Cb = C + (int64_t)bidx * sC;
#pragma unroll 1
      for (int cb = 0; cb < OZ_BN; cb += 16) {
        long long h[16];
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) h[j] = 0;
        for (int L = 0; L < S; ++L) {
          tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(L * OZ_BN + cb), v);
          const int sh = bits * (S - 1 - L) - D;
          if (sh >= 0) {
#pragma unroll
            for (int j = 0; j < 16; ++j) h[j] += (long long)__float2int_rn(v[j]) * (1ll << sh);
          } else {
            const long long half = 1ll << (-sh - 1);
#pragma unroll
            for (int j = 0; j < 16; ++j) h[j] += ((long long)__float2int_rn(v[j]) + half) >> (-sh);
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + cb + j;
          const double x = (double)h[j];
          const double y = __shfl_xor_sync(0xffffffffu, x, 1);
          if (row < M2 && col < N && re_lane) {
            const double s = si * tau[(int64_t)bidx * N + col];
            const cxd c = mkcx(s * x, s * y);
            cxd* dst = Cb + i + (int64_t)col * ldc;
            cxd out = alpha_one ? c : alpha * c;
            if (!beta_zero) out = out + beta * *dst;
            *dst = out;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols) : "memory");
}

// ---------------------------------------------------------------------------------
// operand preparation
// ---------------------------------------------------------------------------------
// op(X) as a K-major "row" matrix X̃ (rows r, contraction index c): X̃(r, c) =
// base[r + c·ld] (r_contig) or base[c + r·ld], conjugated when conj.
struct OpView {
  const cxd* base;
  int64_t ld, stride;  // leading dimension, instance stride
  bool r_contig, conj;
};
__device__ __forceinline__ cxd view_at(const OpView& v, int64_t b, int64_t r, int64_t c) {
  cxd x = v.r_contig ? v.base[b * v.stride + r + c * v.ld] : v.base[b * v.stride + c + r * v.ld];
  if (v.conj) x.y = -x.y;
  return x;
}

// σ_r = the smallest power of two ≥ max_c max(|Re X̃(r,c)|, |Im X̃(r,c)|) (1 for a zero row);
// one warp per row
__global__ void k_oz_scales(OpView v, int64_t R, int64_t K, int64_t batch, double* __restrict__ out) {
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w < R * batch; w += warps) {
    const int64_t b = w / R, r = w % R;
    double mx = 0.0;
    for (int64_t c = lane; c < K; c += 32) {
      const cxd x = view_at(v, b, r, c);
      mx = fmax(mx, fmax(fabs(x.x), fabs(x.y)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
      double s = 1.0;
      if (mx > 0.0) {
        int e;
        const double f = frexp(mx, &e);  // mx = f·2^e, f ∈ [0.5, 1)
        s = ldexp(1.0, f == 0.5 ? e - 1 : e);
      }
      out[b * R + r] = s;
    }
  }
}

__device__ __forceinline__ unsigned short bf16_bits(double d) {
  return __bfloat16_as_ushort(__float2bfloat16_rn((float)d));  // |d| ≤ 128 integer: exact
}

// digit planes of one operand.  a_form: A'' rows 2r (Re) / 2r+1 (Im) with columns
// [Re | −Im] / [Im | Re]; otherwise B'' rows r with columns [Re | Im].  Planes are
// stored plane-major: out[(p·batch + b)·rows'·pitch + row'·pitch + col].  32×32 tiles of
// X̃ are staged through shared memory so that reads follow the source's contiguous index
// and writes the contraction index.
__global__ void __launch_bounds__(256)
    k_oz_split(OpView v, int64_t R, int64_t K, int64_t batch, int S, int bits, bool a_form, const double* __restrict__ scale,
               int64_t pitch, unsigned short* __restrict__ out) {
  __shared__ cxd tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32, c0 = (int64_t)blockIdx.y * 32, b = blockIdx.z;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 × 8
  for (int u = ty; u < 32; u += 8) {
    // tile[c][r]; the fast thread index follows the source's contiguous dimension
    const int64_t r = v.r_contig ? r0 + tx : r0 + u, c = v.r_contig ? c0 + u : c0 + tx;
    const cxd x = (r < R && c < K) ? view_at(v, b, r, c) : mkcx(0.0, 0.0);
    if (v.r_contig)
      tile[u][tx] = x;
    else
      tile[tx][u] = x;
  }
  __syncthreads();
  const int64_t rows_out = a_form ? 2 * R : R;
  const int64_t plane = rows_out * pitch;
  for (int u = ty; u < 32; u += 8) {
    const int64_t r = r0 + u, c = c0 + tx;
    if (r >= R || c >= K) continue;
    const cxd x = tile[tx][u];
    // The top digit is rint(x) in FP64; the remainder (|·| ≤ ½) becomes one integer of
    // b·(S−1) fraction bits (≤ 2^55: exact in int64), whose balanced base-2^b digits are
    // peeled off from the bottom with integer operations (the FP64 pipe is the scarce one
    // on this part); the carry left after S−1 digits (−1, 0 or 1) goes to the top digit.
    const double inv = ldexp(1.0 / scale[b * R + r], bits - 2);  // powers of two: exact
    const double xr = x.x * inv, xi = x.y * inv;
    const double tr = rint(xr), ti = rint(xi);
    const double lo_scale = ldexp(1.0, bits * (S - 1));
    long long Xr = llrint((xr - tr) * lo_scale), Xi = llrint((xi - ti) * lo_scale);
    const long long half = 1ll << (bits - 1), mask = (1ll << bits) - 1;
    int dr[OZ_MAX_S], di[OZ_MAX_S];
#pragma unroll
    for (int p = OZ_MAX_S - 1; p >= 1; --p) {
      if (p < S) {
        const long long lr = ((Xr + half) & mask) - half, li = ((Xi + half) & mask) - half;
        Xr = (Xr - lr) >> bits;
        Xi = (Xi - li) >> bits;
        dr[p] = (int)lr;
        di[p] = (int)li;
      }
    }
    dr[0] = (int)tr + (int)Xr;
    di[0] = (int)ti + (int)Xi;
#pragma unroll
    for (int p = 0; p < OZ_MAX_S; ++p) {
      if (p >= S) break;
      unsigned short* o = out + ((int64_t)p * batch + b) * plane;
      const double vr = (double)dr[p], vi = (double)di[p];
      if (a_form) {
        o[(2 * r) * pitch + c] = bf16_bits(vr);
        o[(2 * r) * pitch + K + c] = bf16_bits(-vi);
        o[(2 * r + 1) * pitch + c] = bf16_bits(vi);
        o[(2 * r + 1) * pitch + K + c] = bf16_bits(vr);
      } else {
        o[r * pitch + c] = bf16_bits(vr);
        o[r * pitch + K + c] = bf16_bits(vi);
      }
    }
  }
}

tn_status_t make_map3(tn_ctx* ctx, CUtensorMap* map, const void* base, int64_t K2, int64_t rows, int64_t planes,
                      int64_t pitch, uint32_t box_rows) {
  EncodeTiledFn fn = tn_encode_tiled_fn(ctx);
  if (!fn) return TN_ECUDA;
  cuuint64_t dims[3] = {(cuuint64_t)K2, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch * 2), (cuuint64_t)(pitch * 2 * rows)};
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tn_set_error(ctx, TN_ECUDA, "cuTensorMapEncodeTiled (split GEMM) failed (%d)", (int)r);
  return TN_OK;
}

OpView make_view(const cxd* base, int64_t ld, int64_t stride, char op, bool is_a) {
  OpView v;
  v.base = base;
  v.ld = ld;
  v.stride = stride;
  v.conj = op == 'C';
  // A: X̃ = op(A) (rows i): 'N' → A[i + c·lda] (r-contiguous).  B: X̃ = op(B)ᵀ (rows j):
  // 'N' → B[c + j·ldb] (c-contiguous); 'T'/'C' → B[j + c·ldb].
  v.r_contig = is_a ? (op == 'N') : (op != 'N');
  return v;
}

// the split GEMM's error word (sticky until split_gemm_check reads it)
tn_status_t oz_error_word(tn_ctx* ctx, int** out) {
  if (!ctx->oz_err) {
    void* p = nullptr;
    TN_RETURN_IF(tn_dev_alloc(ctx, 256, &p));
    TN_CHECK_CUDA(ctx, cudaMemsetAsync(p, 0, sizeof(int), ctx->stream));
    ctx->oz_err = static_cast<int*>(p);
  }
  *out = ctx->oz_err;
  return TN_OK;
}

// the split GEMM's operand planes, kept in a scratch of the context's own: grown (after
// the stream has drained) when a larger product needs it
tn_status_t oz_scratch(tn_ctx* ctx, size_t bytes, char** out) {
  if (bytes > ctx->oz_cap) {
    if (ctx->oz_ws) {
      TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      TN_RETURN_IF(tn_dev_free(ctx, ctx->oz_ws));
      ctx->oz_ws = nullptr;
      ctx->oz_cap = 0;
    }
    void* p = nullptr;
    TN_RETURN_IF(tn_dev_alloc(ctx, bytes, &p));
    ctx->oz_ws = static_cast<char*>(p);
    ctx->oz_cap = bytes;
  }
  *out = ctx->oz_ws;
  return TN_OK;
}

}  // namespace

tn_status_t gemm_c64_split(tn_ctx* ctx, int S, char opa, char opb, int64_t m, int64_t n, int64_t k, cxd alpha,
                           const cxd* A, int64_t lda, int64_t sA, const cxd* B, int64_t ldb, int64_t sB, cxd beta,
                           cxd* C, int64_t ldc, int64_t sC, int64_t batch) {
  if (m == 0 || n == 0 || batch == 0) return TN_OK;
  if (S < 2 || S > OZ_MAX_S) return tn_set_error(ctx, TN_EINVAL, "split GEMM: slices must be in [2, %d]", OZ_MAX_S);
  if (batch > 65535) return tn_set_error(ctx, TN_EUNSUPPORTED, "split GEMM: batch > 65535");
  if (k == 0) return gemm_cx<double>(ctx, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
  // a level's FP32 sum is exact while S·(2k)·2^{2b-2} ≤ 2^24: the widest such digit b
  // (at most 8); contractions that would need b < 7 run in chunks of k sized for b = 7,
  // the later chunks accumulating into C (beta = 1)
  int bits = 8;
  while (bits > 1 && (double)S * (double)(2 * k) * ldexp(1.0, 2 * bits - 2) > 16777216.0) --bits;
  const int64_t kmax = std::max<int64_t>(32, (4096 / S) / 2 / 32 * 32);
  if (bits < 7 && k > kmax) {
    for (int64_t k0 = 0; k0 < k; k0 += kmax) {
      const int64_t kc = std::min(kmax, k - k0);
      const cxd* Ac = (opa == 'N') ? A + k0 * lda : A + k0;
      const cxd* Bc = (opb == 'N') ? B + k0 : B + k0 * ldb;
      TN_RETURN_IF(gemm_c64_split(ctx, S, opa, opb, m, n, kc, alpha, Ac, lda, sA, Bc, ldb, sB,
                                  k0 == 0 ? beta : mkcx(1.0, 0.0), C, ldc, sC, batch));
    }
    return TN_OK;
  }
  const int64_t M2 = 2 * m, K2 = 2 * k, pitch = (K2 + 7) / 8 * 8;
  if (M2 > (1ll << 30) || n > (1ll << 30)) return tn_set_error(ctx, TN_EUNSUPPORTED, "split GEMM: too large");
  const size_t bytesA = ws_round(2 * (size_t)(S * batch * M2 * pitch));
  const size_t bytesB = ws_round(2 * (size_t)(S * batch * n * pitch));
  const size_t bytesS = ws_round(sizeof(double) * (size_t)(batch * m)) + ws_round(sizeof(double) * (size_t)(batch * n));
  char* ws = nullptr;
  int* err = nullptr;
  TN_RETURN_IF(oz_error_word(ctx, &err));
  TN_RETURN_IF(oz_scratch(ctx, bytesA + bytesB + bytesS, &ws));
  unsigned short* dA = reinterpret_cast<unsigned short*>(ws);
  unsigned short* dB = reinterpret_cast<unsigned short*>(ws + bytesA);
  double* sig = reinterpret_cast<double*>(ws + bytesA + bytesB);
  double* tau = sig + ws_round(sizeof(double) * (size_t)(batch * m)) / sizeof(double);
  const OpView va = make_view(A, lda, sA, opa, true), vb = make_view(B, ldb, sB, opb, false);
  const int prep_slot = prof_begin(ctx);
  {
    const int64_t rows = m * batch;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((rows + 7) / 8, (int64_t)ctx->num_sms * 16));
    k_oz_scales<<<blocks, 256, 0, ctx->stream>>>(va, m, k, batch, sig);
    TN_LAUNCHED(ctx);
    const int64_t cols = n * batch;
    const unsigned bb = (unsigned)std::max<int64_t>(1, std::min<int64_t>((cols + 7) / 8, (int64_t)ctx->num_sms * 16));
    k_oz_scales<<<bb, 256, 0, ctx->stream>>>(vb, n, k, batch, tau);
    TN_LAUNCHED(ctx);
    k_oz_split<<<dim3(cdiv(m, 32), cdiv(k, 32), (unsigned)batch), 256, 0, ctx->stream>>>(va, m, k, batch, S, bits, true,
                                                                                       sig, pitch, dA);
    TN_LAUNCHED(ctx);
    k_oz_split<<<dim3(cdiv(n, 32), cdiv(k, 32), (unsigned)batch), 256, 0, ctx->stream>>>(vb, n, k, batch, S, bits,
                                                                                       false, tau, pitch, dB);
    TN_LAUNCHED(ctx);
  }
  if (prep_slot >= 0)  // read op(A), op(B) once, write their digit planes and scales
    prof_end(ctx, prep_slot, TN_PROF_SPLIT_PREP, 4, 0.0,
             2.0 * 16.0 * ((double)m * k + (double)k * n) * batch + 2.0 * S * ((double)M2 + n) * K2 * batch);
  OzMaps maps;
  memset(&maps, 0, sizeof(maps));
  TN_RETURN_IF(make_map3(ctx, &maps.a, dA, K2, M2, (int64_t)S * batch, pitch, OZ_BM));
  TN_RETURN_IF(make_map3(ctx, &maps.b, dB, K2, n, (int64_t)S * batch, pitch, OZ_BN));
  const int64_t tiles = (int64_t)cdiv(M2, OZ_BM) * cdiv(n, OZ_BN);
  if (tiles > 0x7fffffffll) return tn_set_error(ctx, TN_EUNSUPPORTED, "split GEMM: too many tiles");
  const int smem = oz_smem_bytes(S);
  TN_CHECK_CUDA(ctx, cudaFuncSetAttribute(k_gemm_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const bool beta_zero = beta.x == 0.0 && beta.y == 0.0;
  const int slot = prof_begin(ctx);
  k_gemm_oz<<<dim3((unsigned)tiles, (unsigned)batch), OZ_THREADS, smem, ctx->stream>>>(
      maps, S, bits, (int)M2, (int)n, (int)K2, (int)batch, C, ldc, sC, sig, tau, alpha, beta, beta_zero ? 1 : 0, (int)m, err);
  TN_LAUNCHED(ctx);
  if (slot >= 0)  // tensor-pipe flops of the S(S+1)/2 real products it issues; planes read once, C written
    prof_end(ctx, slot, TN_PROF_GEMM_SPLIT, 1, S * (S + 1) / 2 * 2.0 * M2 * n * K2 * batch,
             (2.0 * S * ((double)M2 + n) * K2 + 16.0 * m * n * (beta_zero ? 1 : 2)) * batch);
  return TN_OK;
}

// Shapes below these bounds stay on the FP64 CUDA cores: the split path's operand
// preparation and 128×64 tiles cost more than they save there.
static bool split_pays(int64_t m, int64_t n, int64_t k) { return m >= 32 && n >= 32 && k >= 32 && m * n >= 8192; }

tn_status_t gemm_c64(tn_ctx* ctx, tn_precision_t prec, char opa, char opb, int64_t m, int64_t n, int64_t k, cxd alpha,
                     const cxd* A, int64_t lda, int64_t sA, const cxd* B, int64_t ldb, int64_t sB, cxd beta, cxd* C,
                     int64_t ldc, int64_t sC, int64_t batch) {
  if ((prec == TN_PREC_MIXED || prec == TN_PREC_SPLIT_BF16) && split_pays(m, n, k))
    return gemm_c64_split(ctx, ctx->split_slices, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC,
                          batch);
  return gemm_cx<double>(ctx, opa, opb, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
}

// status of the split GEMMs enqueued since the last check: a pipeline wait that ran out
// is reported here (after the stream has drained)
tn_status_t split_gemm_check(tn_ctx* ctx) {
  if (!ctx->oz_err) return TN_OK;
  int* hp = reinterpret_cast<int*>(ctx->pinned);
  TN_CHECK_CUDA(ctx, cudaMemcpyAsync(hp, ctx->oz_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TN_CHECK_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hp[0]) {
    TN_CHECK_CUDA(ctx, cudaMemsetAsync(ctx->oz_err, 0, sizeof(int), ctx->stream));
    return tn_set_error(ctx, TN_ETIMEOUT, "split GEMM: a pipeline wait timed out");
  }
  return TN_OK;
}

extern "C" tn_status_t tn_set_split_slices(tn_ctx* ctx, int32_t slices) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, slices >= 2 && slices <= OZ_MAX_S, "tn_set_split_slices: slices must be in [2, 8]");
  ctx->split_slices = slices;
  return TN_OK;
}
