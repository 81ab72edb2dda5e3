// K1 — index permutation.
//
// Replaces the `permutedims` that Muscle.binary_einsum / Muscle.fuse run before and
// after every BLAS call.  Every permutation is first reduced to its canonical form
// (size-1 modes dropped, modes that stay adjacent in both layouts fused).  If the
// input-contiguous mode is also the output-contiguous mode the copy is a plain
// coalesced gather; otherwise the two contiguous modes form a 32×32 tile staged in
// shared memory so that both the loads and the stores are coalesced.  Elements are
// moved whole: a ComplexF64 element is one 128-bit access.
#include <algorithm>

#include "tn_internal.cuh"

namespace {

__device__ __forceinline__ int64_t cdiv_dev(int64_t a) { return (a + 31) / 32; }

constexpr int kMaxDims = TN_MAX_RANK + 2;

struct PermPlan {
  int r;                     // number of modes (output order)
  int64_t n[kMaxDims];       // extent
  int64_t is[kMaxDims];      // input stride (elements)
  int64_t os[kMaxDims];      // output stride (elements)
};

template <typename E>
__device__ __forceinline__ E maybe_conj(E v, bool) {
  return v;
}
template <>
__device__ __forceinline__ float2 maybe_conj<float2>(float2 v, bool c) {
  if (c) v.y = -v.y;
  return v;
}
template <>
__device__ __forceinline__ double2 maybe_conj<double2>(double2 v, bool c) {
  if (c) v.y = -v.y;
  return v;
}

// one output element per thread; coalesced on the output side
template <typename E>
__global__ void k_permute_generic(PermPlan p, int64_t total, const E* __restrict__ in,
                                  E* __restrict__ out, bool conj) {
  for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < total;
       lin += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = lin, io = 0, oo = 0;
#pragma unroll 1
    for (int j = 0; j < p.r; ++j) {
      int64_t q = rem / p.n[j];
      int64_t c = rem - q * p.n[j];
      rem = q;
      io += c * p.is[j];
      oo += c * p.os[j];
    }
    out[oo] = maybe_conj(__ldg(in + io), conj);
  }
}

// the contiguous mode is the same in both layouts (e.g. (0, 2, 1)): each row of it is a
// contiguous run in the input and in the output, copied by one block with four
// independent 128-bit loads in flight per thread; the row's offsets are decoded once
template <typename E>
__global__ void __launch_bounds__(256) k_permute_rows(PermPlan p, int64_t rows, const E* __restrict__ in,
                                                      E* __restrict__ out, bool conj) {
  const int64_t n0 = p.n[0];
  for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    int64_t rem = row, io = 0, oo = 0;
#pragma unroll 1
    for (int j = 1; j < p.r; ++j) {
      const int64_t q = rem / p.n[j];
      const int64_t c = rem - q * p.n[j];
      rem = q;
      io += c * p.is[j];
      oo += c * p.os[j];
    }
    const E* src = in + io;
    E* dst = out + oo;
    for (int64_t base = threadIdx.x; base < n0; base += 4 * (int64_t)blockDim.x) {
      E v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t t = base + u * (int64_t)blockDim.x;
        if (t < n0) v[u] = __ldg(src + t);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t t = base + u * (int64_t)blockDim.x;
        if (t < n0) dst[t] = maybe_conj(v[u], conj);
      }
    }
  }
}

// 32×32 tile over (input-contiguous mode a, output-contiguous mode o); other modes in
// the batch.  Block (32, 8).
template <typename E>
__global__ void k_permute_tiled(PermPlan p, int ja, int jo, int64_t nbatch, const E* __restrict__ in,
                                E* __restrict__ out, bool conj) {
  __shared__ E tile[32][33];
  const int64_t Na = p.n[ja], No = p.n[jo];
  const int64_t ta = blockIdx.x % cdiv_dev(Na);
  const int64_t to = blockIdx.x / cdiv_dev(Na);
  for (int64_t b = blockIdx.y; b < nbatch; b += gridDim.y) {
    // decode batch index over the remaining modes
    int64_t rem = b, ib = 0, ob = 0;
#pragma unroll 1
    for (int j = 0; j < p.r; ++j) {
      if (j == ja || j == jo) continue;
      int64_t q = rem / p.n[j];
      int64_t c = rem - q * p.n[j];
      rem = q;
      ib += c * p.is[j];
      ob += c * p.os[j];
    }
    // load: threads run along a (input stride 1)
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
      int64_t ia = ta * 32 + threadIdx.x;
      int64_t io = to * 32 + threadIdx.y + 8 * rr;
      if (ia < Na && io < No) tile[threadIdx.y + 8 * rr][threadIdx.x] = __ldg(in + ib + ia + io * p.is[jo]);
    }
    __syncthreads();
    // store: threads run along o (output stride 1)
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
      int64_t io = to * 32 + threadIdx.x;
      int64_t ia = ta * 32 + threadIdx.y + 8 * rr;
      if (ia < Na && io < No)
        out[ob + io + ia * p.os[ja]] = maybe_conj(tile[threadIdx.x][threadIdx.y + 8 * rr], conj);
    }
    __syncthreads();
  }
}

void simplify(PermPlan& p) {
  PermPlan q;
  q.r = 0;
  for (int j = 0; j < p.r; ++j) {
    if (p.n[j] == 1) continue;
    if (q.r > 0) {
      int k = q.r - 1;
      if (p.is[j] == q.is[k] * q.n[k] && p.os[j] == q.os[k] * q.n[k]) {
        q.n[k] *= p.n[j];
        continue;
      }
    }
    q.n[q.r] = p.n[j];
    q.is[q.r] = p.is[j];
    q.os[q.r] = p.os[j];
    q.r++;
  }
  if (q.r == 0) {
    q.r = 1;
    q.n[0] = 1;
    q.is[0] = 1;
    q.os[0] = 1;
  }
  p = q;
}

template <typename E>
tn_status_t run_plan(tn_ctx* ctx, PermPlan p, const E* in, E* out, bool conj) {
  simplify(p);
  int64_t total = 1;
  for (int j = 0; j < p.r; ++j) total *= p.n[j];
  if (total == 0) return TN_OK;
  int ja = -1, jo = -1;
  for (int j = 0; j < p.r; ++j) {
    if (p.is[j] == 1 && ja < 0) ja = j;
    if (p.os[j] == 1 && jo < 0) jo = j;
  }
  const bool tiled = ja >= 0 && jo >= 0 && ja != jo && p.n[ja] >= 8 && p.n[jo] >= 8;
  if (ja == 0 && jo == 0 && p.r > 1 && p.n[0] >= 32) {
    const int64_t rows = total / p.n[0];
    const int64_t blocks = std::min<int64_t>(rows, (int64_t)ctx->num_sms * 16);
    k_permute_rows<E><<<(unsigned)blocks, 256, 0, ctx->stream>>>(p, rows, in, out, conj);
    TN_LAUNCHED(ctx);
    return TN_OK;
  }
  if (!tiled) {
    int threads = 256;
    int64_t blocks = (total + threads - 1) / threads;
    if (blocks > (int64_t)ctx->num_sms * 64) blocks = (int64_t)ctx->num_sms * 64;
    k_permute_generic<E><<<(unsigned)blocks, threads, 0, ctx->stream>>>(p, total, in, out, conj);
    TN_LAUNCHED(ctx);
    return TN_OK;
  }
  int64_t nbatch = total / (p.n[ja] * p.n[jo]);
  int64_t gx = (int64_t)cdiv(p.n[ja], 32) * cdiv(p.n[jo], 32);
  if (gx > 0x7fffffff) return tn_set_error(ctx, TN_EINVAL, "permute: tile grid too large");
  int64_t gy = nbatch < 65535 ? nbatch : 65535;
  dim3 grid((unsigned)gx, (unsigned)gy);
  k_permute_tiled<E><<<grid, dim3(32, 8), 0, ctx->stream>>>(p, ja, jo, nbatch, in, out, conj);
  TN_LAUNCHED(ctx);
  return TN_OK;
}

template <typename E>
tn_status_t permute_impl(tn_ctx* ctx, int rank, const int64_t* dims, const int64_t* in_strides,
                         const int32_t* perm, const E* in, E* out, bool conj) {
  PermPlan p;
  p.r = rank;
  int64_t dense[kMaxDims];
  int64_t s = 1;
  for (int i = 0; i < rank; ++i) {
    dense[i] = s;
    s *= dims[i];
  }
  int64_t os = 1;
  for (int j = 0; j < rank; ++j) {
    int src = perm[j];
    p.n[j] = dims[src];
    p.is[j] = in_strides ? in_strides[src] : dense[src];
    p.os[j] = os;
    os *= dims[src];
  }
  return run_plan<E>(ctx, p, in, out, conj);
}

}  // namespace

template <typename T>
tn_status_t permute_t(tn_ctx* ctx, int rank, const int64_t* dims, const int64_t* in_strides,
                      const int32_t* perm, const T* in, T* out, bool conj) {
  return permute_impl<T>(ctx, rank, dims, in_strides, perm, in, out, conj);
}
template tn_status_t permute_t<float>(tn_ctx*, int, const int64_t*, const int64_t*, const int32_t*,
                                      const float*, float*, bool);
template tn_status_t permute_t<double>(tn_ctx*, int, const int64_t*, const int64_t*,
                                       const int32_t*, const double*, double*, bool);
template tn_status_t permute_t<float2>(tn_ctx*, int, const int64_t*, const int64_t*,
                                       const int32_t*, const float2*, float2*, bool);
template tn_status_t permute_t<double2>(tn_ctx*, int, const int64_t*, const int64_t*,
                                        const int32_t*, const double2*, double2*, bool);

template <typename T>
tn_status_t transpose_cx(tn_ctx* ctx, int64_t m, int64_t n, const cx<T>* in, int64_t lda,
                         int64_t sIn, cx<T>* out, int64_t ldo, int64_t sOut, int64_t batch,
                         bool conj) {
  using E = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
  // output modes: (n, m, batch); out(j, i) = in(i, j)
  PermPlan p;
  p.r = 3;
  p.n[0] = n;
  p.is[0] = lda;
  p.os[0] = 1;
  p.n[1] = m;
  p.is[1] = 1;
  p.os[1] = ldo;
  p.n[2] = batch;
  p.is[2] = sIn;
  p.os[2] = sOut;
  return run_plan<E>(ctx, p, reinterpret_cast<const E*>(in), reinterpret_cast<E*>(out), conj);
}
template tn_status_t transpose_cx<float>(tn_ctx*, int64_t, int64_t, const cxf*, int64_t, int64_t,
                                         cxf*, int64_t, int64_t, int64_t, bool);
template tn_status_t transpose_cx<double>(tn_ctx*, int64_t, int64_t, const cxd*, int64_t, int64_t,
                                          cxd*, int64_t, int64_t, int64_t, bool);

extern "C" tn_status_t tn_permute(tn_ctx* ctx, tn_dtype_t dtype, int32_t rank, const int64_t* dims,
                                  const int64_t* in_strides, const int32_t* perm, const void* in,
                                  void* out, int32_t conj) {
  if (!ctx) return TN_EINVAL;
  TN_ARG(ctx, rank >= 1 && rank <= TN_MAX_RANK, "tn_permute: rank must be in 1..16");
  TN_ARG(ctx, dims && perm && in && out, "tn_permute: null pointer");
  bool seen[TN_MAX_RANK] = {false};
  for (int i = 0; i < rank; ++i) {
    TN_ARG(ctx, dims[i] >= 0, "tn_permute: negative extent");
    TN_ARG(ctx, perm[i] >= 0 && perm[i] < rank && !seen[perm[i]], "tn_permute: perm is not a permutation");
    seen[perm[i]] = true;
  }
  TN_ARG(ctx, !conj || dtype_complex(dtype), "tn_permute: conj needs a complex dtype");
  switch (dtype) {
    case TN_F32: return permute_impl<float>(ctx, rank, dims, in_strides, perm, (const float*)in, (float*)out, false);
    case TN_F64: return permute_impl<double>(ctx, rank, dims, in_strides, perm, (const double*)in, (double*)out, false);
    case TN_C32: return permute_impl<float2>(ctx, rank, dims, in_strides, perm, (const float2*)in, (float2*)out, conj != 0);
    case TN_C64: return permute_impl<double2>(ctx, rank, dims, in_strides, perm, (const double2*)in, (double2*)out, conj != 0);
  }
  return tn_set_error(ctx, TN_EINVAL, "tn_permute: bad dtype");
}
