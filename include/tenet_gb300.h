/*
 * tenet_gb300.h — C ABI of libtenetgb.so, the GB300 (sm_103a) implementation of the
 * tensor-network hot path of Tenet.jl v0.10.3: pairwise contraction of Tensors and the
 * QR/SVD factorisation + truncation behind canonize!, compress!/truncate!,
 * simple_update!/evolve!, overlap and norm on MPS.
 *
 * Tenet never does arithmetic itself: it calls Muscle.jl on Tangles.Tensor values.  The
 * entry points below are what a Julia `ccall` binding of those Muscle calls binds, plus
 * device-resident MPS operations that keep a whole sweep on the GPU.  Every function is
 * `extern "C"`, takes plain pointers and sizes, and returns a tn_status_t (0 = OK).
 *
 * Conventions
 *  - Arrays are column-major (Julia layout).  Complex values are interleaved (re, im),
 *    identical to Julia's Complex{Float64} / Complex{Float32}.
 *  - Pointers named d_* or documented as "device" are device pointers (from tn_alloc or
 *    any CUDA allocation on the context's device); "host" pointers are ordinary memory.
 *  - All work is enqueued on the context's stream (tn_set_stream); results written to
 *    host memory are complete when the call returns.
 *  - On error the call returns a status and tn_last_error_string() describes it.
 *  - A tn_ctx must not be used from two host threads at once (one context per thread
 *    or stream).
 */
#ifndef TENET_GB300_H
#define TENET_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mapped to ArgumentError / OutOfMemoryError / ErrorException by the
 *      Julia binding, like Tenet's @argcheck, src/Operations/compress.jl:30-32) ---- */
typedef int32_t tn_status_t;
#define TN_OK 0
#define TN_EINVAL 1       /* bad argument: shape, rank, mode labels, null pointer */
#define TN_ENOMEM 2       /* device allocation failed or the HBM budget is exhausted */
#define TN_ENOCONV 3      /* Jacobi SVD hit its sweep cap before convergence */
#define TN_ETIMEOUT 4     /* a bounded device wait or a serving deadline ran out */
#define TN_ECUDA 5        /* CUDA runtime error (message in tn_last_error_string) */
#define TN_EUNSUPPORTED 6 /* dtype / precision combination not implemented */

/* element types */
typedef enum { TN_F32 = 0, TN_F64 = 1, TN_C32 = 2, TN_C64 = 3 } tn_dtype_t;

/* arithmetic modes of the contraction GEMMs and factorisations.
 * TN_PREC_NATIVE: the dtype's own arithmetic on the CUDA cores (FP64 for C64/F64, FP32
 *   for C32/F32).
 * TN_PREC_MIXED: C32/F32 GEMMs as 3xTF32 split products on the tcgen05 tensor pipe
 *   (FP32-grade); C64 SVDs as an FP32 Jacobi pre-pass followed by FP64 Jacobi sweeps
 *   (FP64 is kept for the rotations, the truncation decision and norm/overlap
 *   accumulation); C64 GEMMs stay FP64.
 * TN_PREC_TF32: C32/F32 GEMMs as single-pass TF32 tensor-core products.
 * TN_PREC_SPLIT_BF16: C64 GEMMs from exact BF16 digit planes on the tcgen05 tensor pipe
 *   (tn_set_split_slices planes of 7 bits per operand, default 8: FP64-grade products);
 *   factorisations as TN_PREC_NATIVE. */
typedef enum { TN_PREC_NATIVE = 0, TN_PREC_MIXED = 1, TN_PREC_TF32 = 2, TN_PREC_SPLIT_BF16 = 3 } tn_precision_t;

#define TN_MAX_RANK 16

typedef struct tn_ctx tn_ctx;

/* ------------------------------------------------------------------------------------
 * context, memory, stream
 * ---------------------------------------------------------------------------------- */
tn_status_t tn_create(tn_ctx** ctx, int device);
tn_status_t tn_destroy(tn_ctx* ctx);
/* stream: a cudaStream_t (NULL = the context's own stream) */
tn_status_t tn_set_stream(tn_ctx* ctx, void* stream);
void* tn_get_stream(tn_ctx* ctx);
tn_status_t tn_sync(tn_ctx* ctx);
tn_status_t tn_alloc(tn_ctx* ctx, size_t bytes, void** dptr);
tn_status_t tn_free(tn_ctx* ctx, void* dptr);
tn_status_t tn_memcpy_h2d(tn_ctx* ctx, void* d_dst, const void* h_src, size_t bytes);
tn_status_t tn_memcpy_d2h(tn_ctx* ctx, void* h_dst, const void* d_src, size_t bytes);
tn_status_t tn_memcpy_d2d(tn_ctx* ctx, void* d_dst, const void* d_src, size_t bytes);
/* device HBM budget for MPS storage and workspaces (0 = unlimited) */
tn_status_t tn_set_hbm_budget(tn_ctx* ctx, size_t bytes);
tn_status_t tn_hbm_in_use(tn_ctx* ctx, size_t* bytes);
/* number of library kernels launched on this context since creation */
tn_status_t tn_kernel_launches(tn_ctx* ctx, int64_t* count);
const char* tn_last_error_string(tn_ctx* ctx);
const char* tn_version(void);
/* phase profiler: with enable != 0 the hot path brackets its phases by CUDA events on
 * the context's stream (each Jacobi sweep, each GEMM launch, each QR factorisation) and
 * tn_profile_read returns per class, since enabling: the kernel launches, the device
 * time (ms) and the algorithmic flops and bytes.  Classes: 0 Jacobi sweeps FP32, 1 Jacobi
 * sweeps FP64, 2 complex FP64 GEMM, 3 split-BF16 tensor-core GEMM (flops = the BF16
 * tensor-pipe products it issues), 4 its digit-plane preparation, 5 Householder QR,
 * 6 cooperative small-matrix Jacobi.  Enabling (or disabling) resets the totals. */
tn_status_t tn_profile_enable(tn_ctx* ctx, int32_t enable);
tn_status_t tn_profile_read(tn_ctx* ctx, int32_t cls, int64_t* launches, double* ms, double* flops,
                            double* bytes);
/* measured fused multiply-add rate of the CUDA cores (TFLOP/s): which 0 = FP32, 1 = FP64
 * (a register-resident FMA loop over every SM; the roofline denominator of CUDA-core
 * kernels) */
tn_status_t tn_pipe_peak(tn_ctx* ctx, int32_t which, double* tflops);
/* autotuner: with enable != 0 the first call of an unseen shape bucket times the
 * candidate launch configurations (QR panel and slab widths) and records the fastest.
 * tn_tuning_dump writes the table as text ("key v1 v2" lines; *needed = bytes incl. the
 * terminator); tn_tuning_load reads such text back (a tuning cache file; QR entries hold a
 * panel width in 1, 2, 4, …, 32 and a slab width in 1, 2, 4, anything else is TN_EINVAL). */
tn_status_t tn_set_autotune(tn_ctx* ctx, int32_t enable);
tn_status_t tn_tuning_dump(tn_ctx* ctx, char* buf, size_t len, size_t* needed);
tn_status_t tn_tuning_load(tn_ctx* ctx, const char* text);

/* ------------------------------------------------------------------------------------
 * K1 — index permutation (replaces Julia `permutedims` inside Muscle.binary_einsum and
 * Muscle.fuse; reached from binary_einsum call sites e.g. src/Operations/canonize.jl:61)
 * out = permutedims(in, perm); out is dense column-major with dims[perm[j]] at j.
 * in_strides may be NULL (dense column-major input).  perm is 0-based.
 * ---------------------------------------------------------------------------------- */
tn_status_t tn_permute(tn_ctx* ctx, tn_dtype_t dtype, int32_t rank, const int64_t* dims,
                       const int64_t* in_strides, const int32_t* perm, const void* d_in,
                       void* d_out, int32_t conj);

/* ------------------------------------------------------------------------------------
 * K2 — batched strided GEMM  C = alpha op(A) op(B) + beta C   (op: 'N', 'T', 'C')
 * alpha/beta are host scalars of the dtype's real type pair: for complex dtypes two
 * doubles (re, im); for real dtypes one double.  Replaces the BLAS gemm in
 * Muscle.binary_einsum.
 * ---------------------------------------------------------------------------------- */
tn_status_t tn_gemm(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, char opa, char opb,
                    int64_t m, int64_t n, int64_t k, const double* alpha, const void* d_A,
                    int64_t lda, int64_t strideA, const void* d_B, int64_t ldb,
                    int64_t strideB, const double* beta, void* d_C, int64_t ldc,
                    int64_t strideC, int64_t batch);

/* digit planes per operand of the TN_PREC_SPLIT_BF16 (and mixed C64) GEMMs, 2..8
 * (default 8): each plane carries 7 bits (8 for short contractions), so the products'
 * relative error is ~2^(-7·slices), and the tensor-pipe work grows as slices·(slices+1)/2
 * BF16 products.  Contractions longer than 4096/slices real terms run in chunks. */
tn_status_t tn_set_split_slices(tn_ctx* ctx, int32_t slices);

/* ------------------------------------------------------------------------------------
 * Muscle.binary_einsum(a, b; dims) on dense column-major tensors with integer mode
 * labels.  Modes of c that appear in both a and b are kept (Hadamard / batch modes,
 * the `dims=Index[]` case of src/Operations/canonize.jl:44); modes in both a and b but
 * not in c are contracted; every other mode must appear in exactly one input and in c.
 * c->dims is filled from a/b.  Call sites: canonize.jl:44,47,61,100;
 * simple_update.jl:34; overlap.jl:26-46.
 * ---------------------------------------------------------------------------------- */
typedef struct {
  int32_t rank;
  int64_t dims[TN_MAX_RANK];
  int32_t modes[TN_MAX_RANK];
  void* data; /* device, dense column-major */
} tn_tensor;

tn_status_t tn_contract(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec,
                        const tn_tensor* a, const tn_tensor* b, tn_tensor* c);

/* ------------------------------------------------------------------------------------
 * K3 — thin QR (Muscle.tensor_qr_thin, called at src/Operations/canonize.jl:58):
 * A (m×n, column-major, lda) = Q (m×k) R (k×n), k = min(m,n), batched with strides.
 * Blocked Householder: R has a real non-negative... (LAPACK sign convention: R_ii real).
 * ---------------------------------------------------------------------------------- */
tn_status_t tn_qr_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, int64_t m,
                       int64_t n, const void* d_A, int64_t lda, int64_t strideA, void* d_Q,
                       int64_t strideQ, void* d_R, int64_t strideR, int64_t batch);

/* ------------------------------------------------------------------------------------
 * K4 — thin SVD (Muscle.tensor_svd_thin, src/Operations/canonize.jl:41,97;
 * evolve.jl:62,92): A (m×n) = U diag(S) Vh, k = min(m,n), S real descending (always
 * FP64 on output), U m×k, Vh k×n.  One-sided Jacobi with warp-shuffle reductions.
 * ---------------------------------------------------------------------------------- */
tn_status_t tn_svd_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, int64_t m,
                        int64_t n, const void* d_A, int64_t lda, int64_t strideA, void* d_U,
                        int64_t strideU, double* d_S, int64_t strideS, void* d_Vh,
                        int64_t strideVh, int64_t batch);

/* Allocation-free thin SVD of a ComplexF64 matrix, m >= n (no counterpart in the
 * reference: it is an addition for callers that cannot allocate device memory where they
 * need the factorisation — loops whose memory is fixed up front, or hosts that have a
 * stream but no allocator and no tn_ctx).
 * Same outputs as tn_svd_thin: U (m×n), S (n, FP64, descending), Vh (n×n), dense
 * column-major, all caller-owned device buffers; no context, no cudaMalloc/cudaFree.
 * Scratch lives in a 16 MiB file-scope device array that every GPU loading the library
 * holds until exit, so (m·n + n²)·16 + n·12 + ~1 KiB must fit in 16 MiB (e.g. 1024×512);
 * larger sizes return TN_EINVAL, and more than 4096 rows TN_EUNSUPPORTED.  The first call
 * on each device looks up the array's device address.  Every call shares the array:
 * calls that overlap on the GPU (two streams, two host threads) race.  Runs on `stream`
 * (a cudaStream_t; NULL = the legacy default stream), synchronises that stream once per
 * Jacobi sweep to read the convergence flag, and returns after the work has completed.
 * Errors: tn_last_error_string(NULL). */
tn_status_t tn_svd_thin_noalloc(void* stream, int64_t m, int64_t n, const void* d_A, int64_t lda,
                                void* d_U, double* d_S, void* d_Vh);

/* ------------------------------------------------------------------------------------
 * Mode-labelled factorisations, the form the Julia binding of Muscle calls:
 *
 * Muscle.tensor_qr_thin(A; inds_q, inds_r, ind_virtual) (src/Operations/canonize.jl:58):
 * A is matricised as (q_modes…) × (its other modes, in A's order), factorised, and Q, R
 * come back as labelled tensors Q (q_modes…, virtual_mode), R (virtual_mode, others…).
 * Q->data / R->data are caller buffers of ≥ m·k and k·n elements (k = min(m, n)); the
 * library fills rank, dims and modes.
 *
 * Muscle.tensor_svd_thin(A; inds_u, inds_v, ind_s) (src/Operations/canonize.jl:41,97),
 * with compress!'s truncation (src/Operations/compress.jl:47-59) applied to the result:
 * keep min(maxdim, k) values (maxdim <= 0: no cap), then those with |s| > abs_threshold
 * (abs_threshold <= 0: none), at least one; *rank_out = the kept rank r.  U (u_modes…,
 * s_mode) holds the first r left vectors, d_S the r values (FP64, descending), Vh
 * (s_mode, others…) the first r right vectors, compacted (leading dimension r).  Buffers
 * as for the QR with k columns / rows.  Both: C64 or C32; TN_EINVAL when a label is
 * missing, repeated or the new mode is already used.
 * ---------------------------------------------------------------------------------- */
tn_status_t tn_tensor_qr_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, const tn_tensor* A,
                              int32_t n_q, const int32_t* q_modes, int32_t virtual_mode, tn_tensor* Q,
                              tn_tensor* R);
tn_status_t tn_tensor_svd_thin(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec, const tn_tensor* A,
                               int32_t n_u, const int32_t* u_modes, int32_t s_mode, int64_t maxdim,
                               double abs_threshold, tn_tensor* U, double* d_S, tn_tensor* Vh,
                               int64_t* rank_out);

/* diagnostics of the last SVD on this context: Jacobi sweeps run in FP32 (mixed
 * pre-pass) and in FP64 (-1: the one-CTA shared-memory kernel ran all sweeps), and the
 * number of rotations applied in each sweep of the first matrix (up to n_rot) */
tn_status_t tn_svd_last_sweeps(tn_ctx* ctx, int32_t* fp32_sweeps, int32_t* fp64_sweeps,
                               int32_t* rotations, int32_t n_rot);
/* cumulative statistics of the truncated mixed-precision SVD (the FP32 pre-pass + matrix-
 * product refinement of the kept right vectors) on this context: totals[0] calls,
 * totals[1] refinement iterations, totals[2] near-degenerate pairs handed to the FP64
 * one-sided Jacobi of the marked columns, totals[3] calls that needed full FP64 sweeps;
 * reset != 0 zeroes them after the read */
tn_status_t tn_svd_refine_stats(tn_ctx* ctx, int64_t* totals, int32_t reset);
/* the last truncated mixed-precision SVD: per refinement iteration k (< *iterations, at
 * most 8) trace[4k..4k+3] = the largest applied step |E_ij|, the largest |I − VᴴV|_ij,
 * the largest ‖E‖_F over the batch and the near-degenerate pairs marked; *outcome 0
 * converged, 1 left the quadratic regime (FP64 sweeps from the FP32 basis), 2 out of
 * iterations (FP64 sweeps from the refined basis) */
tn_status_t tn_svd_last_refine(tn_ctx* ctx, float* trace, int32_t* iterations, int32_t* outcome);
/* the largest off-diagonal ratio |w_iᴴw_j| / (‖w_i‖‖w_j‖) seen in each sweep of the
 * first matrix of the last multi-launch Jacobi phase (up to n values) */
tn_status_t tn_svd_last_ratios(tn_ctx* ctx, float* ratios, int32_t n);

/* truncation rank select: keep min(maxdim, k) values (maxdim <= 0: no cap), then those
 * with |s| > threshold (threshold <= 0: no threshold), at least one.  Mirrors
 * src/Operations/compress.jl:47-59.  S is a device array; rank written to *rank (host). */
tn_status_t tn_truncation_rank(tn_ctx* ctx, const double* d_S, int64_t k, int64_t maxdim,
                               double threshold, int64_t* rank);

/* ------------------------------------------------------------------------------------
 * K5 — small fused ops
 * ---------------------------------------------------------------------------------- */
/* Muscle.hadamard(t, s) along `axis` (src/Operations/canonize.jl:198,209):
 * out = t .* s (broadcast along axis); s is real FP64 of length dims[axis]. */
tn_status_t tn_hadamard(tn_ctx* ctx, tn_dtype_t dtype, int32_t rank, const int64_t* dims,
                        int32_t axis, const void* d_t, const double* d_s, void* d_out);
/* ||x||_2 accumulated in FP64 (LinearAlgebra.norm on a Tensor, norm.jl:27,33) */
tn_status_t tn_norm2(tn_ctx* ctx, tn_dtype_t dtype, int64_t n, const void* d_x,
                     double* h_out);
tn_status_t tn_scale(tn_ctx* ctx, tn_dtype_t dtype, int64_t n, void* d_x, double s);
/* Krylov-solver vector operations on ComplexF64 device vectors (the DMRG eigensolver):
 * h_out = ⟨x, y⟩ = Σ conj(x_i) y_i as (re, im); y += (ar + i·ai) x */
tn_status_t tn_dotc(tn_ctx* ctx, int64_t n, const void* d_x, const void* d_y, double* h_out);
tn_status_t tn_axpy(tn_ctx* ctx, int64_t n, double ar, double ai, const void* d_x, void* d_y);

/* Muscle.simple_update(A, ia, B, ib, bond, op, oa, ob; maxdim, absorb=AbsorbEqually())
 * (called at src/Operations/simple_update.jl:53-64): A (chl, d1, chm), B (chm, d2, chr),
 * G (d1, d2, d1, d2) indices [out_a, out_b, in_a, in_b]; θ = Σ G·A·B, thin SVD over
 * (chl,d1)|(d2,chr), keep (maxdim, threshold) as tn_truncation_rank, A' = U√S (chl,d1,k),
 * B' = √S Vh (k,d2,chr).  A_out/B_out must hold chl*d1*min(d1*chl, d2*chr) and
 * min(..)*d2*chr elements.  S_out (device, may be NULL) receives the kept values. */
tn_status_t tn_simple_update(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec,
                             int64_t chl, int64_t d1, int64_t chm, int64_t d2, int64_t chr,
                             const void* d_A, const void* d_B, const void* d_G,
                             int64_t maxdim, double threshold, void* d_Aout, void* d_Bout,
                             double* d_Sout, int64_t* rank);
/* the same with Muscle's `absorb` keyword: TN_ABSORB_EQUALLY (A' = U√S, B' = √S Vh, as
 * tn_simple_update), TN_ABSORB_U (A' = U·S, B' = Vh right-isometric) or TN_ABSORB_V
 * (A' = U left-isometric, B' = S·Vh).  Every mode gives the same A'B'. */
#define TN_ABSORB_EQUALLY 0
#define TN_ABSORB_V 1
#define TN_ABSORB_U 2
tn_status_t tn_simple_update_absorb(tn_ctx* ctx, tn_dtype_t dtype, tn_precision_t prec,
                                    int64_t chl, int64_t d1, int64_t chm, int64_t d2, int64_t chr,
                                    const void* d_A, const void* d_B, const void* d_G,
                                    int64_t maxdim, double threshold, int32_t absorb,
                                    void* d_Aout, void* d_Bout, double* d_Sout, int64_t* rank);

/* ------------------------------------------------------------------------------------
 * Device-resident MPS (src/Components/MPS.jl:13-94) with the canonical-form trait
 * (src/CanonicalForm.jl) kept in native code.  Site i (1-based) is a (χ_{i-1}, d, χ_i)
 * column-major C64 tensor; χ_0 = χ_L = 1.  The operations follow Tenet's algorithms:
 *  canonize (canonize.jl:121-252), compress (compress.jl:21-69), simple_update
 *  (simple_update.jl:82-92), overlap (overlap.jl:36-50), amplitude (overlap.jl:22-32),
 *  norm / normalize (norm.jl:17-37, normalize.jl:15-37).
 * ---------------------------------------------------------------------------------- */
typedef struct tn_mps tn_mps;

#define TN_FORM_NONCANONICAL 0
#define TN_FORM_MIXED 1
#define TN_FORM_BOND 2

/* create an MPS of L sites, physical dim d; bond_dims[L-1] initial bonds; max_bond caps
 * the storage reserved per site (0 = the initial bonds only, growing on demand). */
tn_status_t tn_mps_create(tn_ctx* ctx, int32_t L, int32_t d, const int64_t* bond_dims,
                          int64_t max_bond, tn_precision_t prec, tn_mps** out);
/* B instances advanced in lockstep by every operation (same L, d, form and bond
 * dimensions; different tensors).  Operations returning one value per MPS write B values
 * (instance-major).  Uneven truncation ranks are padded with zero singular values, so
 * each instance holds exactly its own truncated state. */
tn_status_t tn_mps_create_batched(tn_ctx* ctx, int32_t B, int32_t L, int32_t d,
                                  const int64_t* bond_dims, int64_t max_bond,
                                  tn_precision_t prec, tn_mps** out);
tn_status_t tn_mps_batch_size(const tn_mps* mps, int32_t* B);
tn_status_t tn_mps_set_instance_site(tn_mps* mps, int32_t b, int32_t site, int64_t chl,
                                     int64_t chr, const void* h_data);
tn_status_t tn_mps_get_instance_site(const tn_mps* mps, int32_t b, int32_t site, void* h_data);
/* Every site of instance b in one call: h[i-1] points at site i's column-major
 * (χ_{i-1}, d, χ_i) data (the MPS's current bonds).  The copies are issued back to back
 * and waited for once; page-locked host buffers make them DMA transfers. */
tn_status_t tn_mps_set_instance_sites(tn_mps* mps, int32_t b, const void* const* h);
tn_status_t tn_mps_get_instance_sites(const tn_mps* mps, int32_t b, void* const* h);
tn_status_t tn_mps_destroy(tn_mps* mps);
tn_status_t tn_mps_copy(const tn_mps* src, tn_mps** out);
/* host data of site i (1-based), column-major (χl, d, χr) C64 */
tn_status_t tn_mps_set_site(tn_mps* mps, int32_t site, int64_t chl, int64_t chr,
                            const void* h_data);
tn_status_t tn_mps_get_site(const tn_mps* mps, int32_t site, void* h_data);
tn_status_t tn_mps_bond_dims(const tn_mps* mps, int64_t* h_bonds /* L-1 */);
tn_status_t tn_mps_set_precision(tn_mps* mps, tn_precision_t prec);
/* form: kind + (lo, hi) sites for MIXED, (a, a+1) for BOND */
tn_status_t tn_mps_form(const tn_mps* mps, int32_t* kind, int32_t* lo, int32_t* hi);
tn_status_t tn_mps_set_form(tn_mps* mps, int32_t kind, int32_t lo, int32_t hi);
/* Λ at the bond-canonical centre (FP64 host array of B × χ_a) */
tn_status_t tn_mps_get_lambda(const tn_mps* mps, double* h_lambda, int64_t* len);

tn_status_t tn_mps_canonize_mixed(tn_mps* mps, int32_t lo, int32_t hi);
tn_status_t tn_mps_canonize_bond(tn_mps* mps, int32_t a /* bond a-(a+1) */);
/* bond a = 0: every bond 1..L-1 in turn; maxdim <= 0 / threshold <= 0 disable each cut */
tn_status_t tn_mps_compress(tn_mps* mps, int32_t a, int64_t maxdim, double threshold);
/* gate on sites (a) [n_sites = 1, G d×d] or (a, a+1) [n_sites = 2, G d×d×d×d];
 * G is a host array (column-major C64). */
tn_status_t tn_mps_simple_update(tn_mps* mps, int32_t n_sites, int32_t a, const void* h_G,
                                 int64_t maxdim, double threshold);
/* whole brickwork circuit: layers x gates; h_gates holds n_gates[l] 2-site gates of
 * d^4 C64 each per layer, layer l starting at bond starts[l]; gates applied left→right */
tn_status_t tn_mps_evolve_brickwork(tn_mps* mps, int32_t n_layers, const int32_t* starts,
                                    const int32_t* n_gates, const void* h_gates,
                                    int64_t maxdim, double threshold);
/* as tn_mps_evolve_brickwork, with a direction per layer: reverse[l] != 0 applies layer
 * l's gates right→left (its gates are still stored left→right in h_gates).  A sweep
 * that alternates direction (serpentine) starts each layer where the orthogonality
 * centre was left, instead of moving it back across the chain; reverse == NULL is
 * left→right everywhere.  Every gate is Tenet's simple_update! (canonize! to the pair,
 * contract, SVD, truncate) on the state as left by the previous gate. */
tn_status_t tn_mps_evolve_layers(tn_mps* mps, int32_t n_layers, const int32_t* starts,
                                 const int32_t* n_gates, const int32_t* reverse,
                                 const void* h_gates, int64_t maxdim, double threshold);
/* ⟨b|a⟩ = Σ a·conj(b); h_out = (re, im) per instance */
tn_status_t tn_mps_overlap(const tn_mps* a, const tn_mps* b, double* h_out);
tn_status_t tn_mps_norm(tn_mps* mps, double* h_out);
tn_status_t tn_mps_normalize(tn_mps* mps);
/* ⟨bits|ψ⟩ with product vectors (not conjugated): h_vectors is L×d C64 (site-major);
 * h_out = (re, im) per instance */
tn_status_t tn_mps_amplitude(const tn_mps* mps, const void* h_vectors, double* h_out);
/* ⟨ψ|O_i|ψ⟩/⟨ψ|ψ⟩ for every site i, O a host d×d C64; h_out is B×L×(re,im) */
tn_status_t tn_mps_local_expectations(const tn_mps* mps, const void* h_op, double* h_out);
/* sample(ψ, nshots) (src/Operations/sample.jl:20-72) of one instance: h_uniforms holds
 * nshots × L uniforms in [0, 1) (row-major; the caller's RNG replaces Julia's), h_out
 * receives nshots × L outcomes, 1-based like the reference's samples.  Moves the
 * orthogonality centre of `mps` to site 1 (the state is unchanged). */
tn_status_t tn_mps_sample(tn_mps* mps, int32_t instance, int64_t nshots, const double* h_uniforms, int32_t* h_out);
/* evolve!(ψ, MPO) (src/Operations/evolve.jl:19-137).  MPO site i is a host array,
 * column-major (w_{i-1}, d, d, w_i) = (left bond, output, input, right bond) C64, with
 * w_0 = w_L = 1; mpo_bonds holds w_1..w_{L-1}.  algorithm 0: direct contraction (every
 * instance; bonds become χ_i·w_i, form MixedCanonical(all)); 1: zip-up with truncation
 * (maxdim > 0 and/or threshold > 0; every instance, the common bond the largest kept rank
 * with each instance's surplus singular values zero). */
tn_status_t tn_mps_evolve_mpo(tn_mps* mps, const void* const* h_mpo_sites, const int64_t* mpo_bonds, int32_t algorithm,
                              int64_t maxdim, double threshold);
/* dmrg!(ψ, H; method) (src/Algorithms/DMRG.jl:45-461): ground-state search in place.
 * method 1 = Dmrg1 (DMRG.jl:45-210, bonds unchanged), 2 = Dmrg2 (DMRG.jl:212-459, pair
 * split by a thin SVD keeping min(maxdim, k) values; maxdim <= 0 means 128).  The local
 * eigensolver is KrylovKit's eigsolve(x0, 1, :LM; ishermitian = true, krylovdim, maxiter)
 * with tolerance tol (<= 0: 1e-12).  MPO sites as for tn_mps_evolve_mpo; mpo_count is 1
 * (one Hamiltonian for every instance) or B (h_mpo_sites[b*L + i] is site i+1 of
 * instance b's Hamiltonian; all share mpo_bonds).  h_energy receives B values: the
 * eigenvalue of the last local problem; h_history (optional) 2·nsweeps·B values: the
 * same after each half sweep.  Ends in MixedCanonical(site 1). */
tn_status_t tn_mps_dmrg(tn_mps* mps, const void* const* h_mpo_sites, const int64_t* mpo_bonds, int32_t mpo_count,
                        int32_t method, int32_t nsweeps, int64_t maxdim, int32_t krylovdim, int32_t maxiter, double tol,
                        double* h_energy, double* h_history);
/* Device time of the last tn_mps_dmrg on this context, per phase (ms): [0] gauge moves
 * (canonize!), [1] environment updates, [2] local eigensolves (with forming the pair),
 * [3] pair splits (Dmrg2); h_updates[0] = local updates timed, h_updates[1] = Jacobi
 * sweeps summed over the pair splits. */
tn_status_t tn_dmrg_last_stats(tn_ctx* ctx, double* h_ms, int64_t* h_updates);
/* dump / load of a device MPS (all instances, the form and Λ) as a raw file: magic
 * "TNMPS001", int32 L, d, B, form, lo, hi, precision, int64 Λ length, int64 bonds[0..L],
 * column-major ComplexF64 sites per instance, then Λ.  max_bond as tn_mps_create. */
tn_status_t tn_mps_save(const tn_mps* mps, const char* path);
tn_status_t tn_mps_shape(const tn_mps* mps, int32_t* L, int32_t* d, int32_t* B);
tn_status_t tn_mps_load(tn_ctx* ctx, const char* path, int64_t max_bond, tn_mps** out);

/* ---------------------------------------------------------------------------------
 * Query server: a device-resident pool of MPS answering amplitude, local expectation
 * value and overlap queries with continuous batching (src/Operations/overlap.jl:22-50).
 * The server owns its context, a worker thread, one high-priority stream for amplitude
 * and expectation batches, four overlap streams, and a workspace arena of work_bytes
 * carved per job.  A pool MPS holds its sites A_i and the environment-dressed sites
 * X_i = Lf_{i-1} A_i R_{i+1} (2× the site bytes); pool and arena together stay under
 * hbm_budget (0 = unlimited).  Queries wait until a job slot and workspace are free.
 * --------------------------------------------------------------------------------- */
typedef struct tn_server tn_server;

#define TN_Q_AMPLITUDE 0   /* ⟨bits|ψ⟩: data = L×d C64 product vectors, site-major, not conjugated */
#define TN_Q_EXPECTATION 1 /* ⟨ψ|O_site|ψ⟩/⟨ψ|ψ⟩: data = d×d C64 operator (column-major), site 1-based */
#define TN_Q_OVERLAP 2     /* ⟨ψ_{mps_b}|ψ_{mps}⟩: both MPS of equal L and d */

typedef struct {
  int32_t kind;
  int32_t mps;   /* pool id (the ket) */
  int32_t mps_b; /* overlap: pool id of the bra */
  int32_t site;  /* expectation value: operator site */
  const void* data;
} tn_query;

/* precision: TN_PREC_NATIVE (FP64 throughout) or TN_PREC_MIXED (pool MPS also keep FP32
 * copies of their sites; amplitude batches and overlap sweeps run as FP32 GEMMs with the
 * result returned in FP64, relative error ~1e-6; ⟨O_i⟩ stays FP64) */
tn_status_t tn_serve_create(int32_t device, size_t hbm_budget, size_t work_bytes, int32_t max_batch,
                            tn_precision_t precision, tn_server** out);
/* waits for every submitted query, then frees the pool and the device */
tn_status_t tn_serve_destroy(tn_server* srv);
/* host sites (column-major (χl, d, χr) C64) → pool; TN_ENOMEM past the budget */
tn_status_t tn_serve_add_mps(tn_server* srv, int32_t L, int32_t d, const int64_t* bond_dims /* L-1 */,
                             const void* const* h_sites, int32_t* id);
/* seeded Gaussian MPS generated on the device, bonds min(chi, d^min(i, L-i)), entries of
 * variance 1/(d χ_{i-1}) */
tn_status_t tn_serve_add_random_mps(tn_server* srv, int32_t L, int32_t d, int64_t chi, uint64_t seed, int32_t* id);
tn_status_t tn_serve_remove_mps(tn_server* srv, int32_t id);
tn_status_t tn_serve_mps_info(tn_server* srv, int32_t id, int32_t* L, int32_t* d, int64_t* bond_dims,
                              double* norm2);
tn_status_t tn_serve_get_site(tn_server* srv, int32_t id, int32_t site, void* h_data);
/* thread-safe; returns at once with a ticket */
tn_status_t tn_serve_submit(tn_server* srv, const tn_query* q, int64_t* ticket);
/* blocks until the ticket's result is ready (TN_ETIMEOUT after timeout_s); value =
 * (re, im); latency = submit → result on the host, seconds */
tn_status_t tn_serve_wait(tn_server* srv, int64_t ticket, double timeout_s, double* h_value, double* latency_s);
/* completed, short jobs, overlap jobs, largest batch, deferrals for memory, pool bytes,
 * pending, jobs in flight */
tn_status_t tn_serve_stats(tn_server* srv, int64_t* h_stats /* 8 */);
/* message of the last failed tn_serve_* call on this thread */
const char* tn_serve_last_error(void);

/* ---------------------------------------------------------------------------------
 * Grouped MPS batches: B independent MPS of different lengths L_b and bond dimensions
 * (physical dimension d shared), stored on the device and processed in lockstep by
 * grouped launches (each launch covers every instance with a site at that step, shapes
 * from a per-step descriptor table).  Sites are column-major (χ_{i-1}, d, χ_i) C64.
 * --------------------------------------------------------------------------------- */
typedef struct tn_group tn_group;
/* bonds: the L_b − 1 inner bond dimensions of every instance, concatenated */
tn_status_t tn_group_create(tn_ctx* ctx, int32_t B, const int32_t* L, int32_t d, const int64_t* bonds,
                            tn_group** out);
tn_status_t tn_group_destroy(tn_group* g);
/* seeded Gaussian sites generated on the device, entries of variance 1/(d χ_{i-1}),
 * with the bond dimensions given at creation (also after a compress) */
tn_status_t tn_group_fill_random(tn_group* g, uint64_t seed);
tn_status_t tn_group_set_site(tn_group* g, int32_t b, int32_t site, const void* h_data);
tn_status_t tn_group_get_site(const tn_group* g, int32_t b, int32_t site, void* h_data);
tn_status_t tn_group_bond_dims(const tn_group* g, int32_t b, int64_t* h_bonds /* L_b - 1 */);
/* for every instance b: canonize!(ψ_b, MixedCanonical(L_b)); compress!(ψ_b;
 * maxdim = maxdim[b]); h_norms[b] = norm(ψ_b) = ‖Λ_{L_b-1}‖ (canonize.jl:121-252,
 * compress.jl:21-69, norm.jl:31-34).  Afterwards sites 1..L_b-1 are left-isometric and
 * site L_b holds Λ_{L_b-1} absorbed; Λ_{L_b-1} is returned by tn_group_lambda.  The
 * initial bonds must satisfy χ_{i-1}·d ≥ χ_i and χ_{i}·d ≥ χ_{i-1} (rand(MPS) clamping). */
tn_status_t tn_group_canonize_compress_norm(tn_group* g, const int64_t* maxdim, double* h_norms);
tn_status_t tn_group_lambda(const tn_group* g, int32_t b, double* h_lambda, int64_t* len);

#ifdef __cplusplus
}
#endif
#endif /* TENET_GB300_H */
