/*
 * qsgpu.h -- C-ABI of the GB300 (sm_103a) block-sparse symmetric tensor
 * contraction library (libqsgpu.so).
 *
 * The library replaces the numerical core behind QSpace's MEX routines
 * contractQS / permuteQS / eigQS / svdQS and the Davidson re-orthogonalisation
 * step.  Host code (a MEX shim, a C++ application, or Python through ctypes)
 * passes block-sparse tensors as plain pointers; nothing in these signatures
 * is a torch or MATLAB type.
 *
 * Conventions
 *  - Every entry point returns qs_status; on failure qs_last_error() returns a
 *    thread-local message (the reference throws Wb::LogException, which the
 *    MEX layer turns into mexErrMsgIdAndTxt, Source/wblib.h:633-660).
 *  - A QSpace is described by qs_qspace_view (the MATLAB struct {Q,data,info}
 *    of Source/QSpace.hh:3092): int32 labels, per-block leg dimensions and
 *    column-major FP64 blocks (complex: interleaved {re,im}, the layout of
 *    wbcomplex) stored back to back at the given element offsets.
 *  - Index strings follow the reference ('12*', '1,3', '[2 3]*'): 1-based legs,
 *    a trailing '*' conjugates that operand (Source/wbindex.cc:482-540).
 *  - Permutations are 1-based over the output legs (Source/contractQS.cc:
 *    521-536); nperm = 0 means none.
 *  - Host buffers are borrowed read-only for the duration of the call.
 *    Results are owned by the caller and released with qs_result_free /
 *    qs_tensor_free.
 *  - One qs_ctx drives one CUDA stream on one device.  Calls on the same
 *    context must not overlap; different contexts may be used from
 *    different threads.
 */
#ifndef QSGPU_H
#define QSGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define QS_EXPORT __attribute__((visibility("default")))
#else
#define QS_EXPORT
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  QS_OK = 0,
  QS_ERR_ARG = 1,        /* malformed argument (index string, perm, sizes) */
  QS_ERR_SHAPE = 2,      /* inconsistent block dimensions                 */
  QS_ERR_LABEL = 3,      /* label / QDIM / itag inconsistency             */
  QS_ERR_CUDA = 4,       /* a CUDA runtime / library call failed          */
  QS_ERR_OOM = 5,        /* device memory exhausted or admission refused  */
  QS_ERR_TIMEOUT = 6,    /* a bounded device wait ran out                  */
  QS_ERR_UNSUPPORTED = 7,
  QS_ERR_INTERNAL = 8,
  QS_ERR_CANCELLED = 9,
  QS_ERR_NUMERIC = 10    /* e.g. split precision could not meet the tolerance */
} qs_status;

typedef enum {
  QS_PREC_FP64 = 0,   /* plain FP64 (DFMA) path: the drop-in                   */
  QS_PREC_SPLIT = 1   /* FP64 sliced into BF16 digits, tcgen05 products with
                         exact FP32 accumulation, compensated recombination   */
} qs_prec;

typedef struct qs_ctx qs_ctx;         /* device + stream + memory pool        */
typedef struct qs_result qs_result;   /* host-side result of a contraction    */
typedef struct qs_tensor qs_tensor;   /* device-resident QSpace               */

/* A block-sparse tensor in host memory (or, for qs_tensor_from_device, with
 * `data` a device pointer). */
typedef struct {
  int32_t rank;           /* number of legs r                                  */
  int32_t qdim;           /* labels per leg (QDIM; e.g. 2 for U(1)xU(1))       */
  int64_t nblk;           /* number of blocks                                  */
  const int32_t *q;       /* nblk x (rank*qdim), block-major: block i, leg k,
                             component j at q[(i*rank + k)*qdim + j]           */
  const int64_t *dims;    /* nblk x rank leg dimensions                        */
  const int64_t *offs;    /* nblk element offsets into data (complex: in
                             complex elements)                                 */
  const double *data;     /* blocks, column-major, back to back                */
  int32_t is_complex;     /* 0: float64, 1: complex128 interleaved             */
  const char *itags;      /* leg tags "L,s,R*" (a trailing '*' marks an
                             outgoing leg), or NULL: info.itags of the struct */
} qs_qspace_view;

typedef struct {
  int32_t prec;       /* qs_prec                                               */
  int32_t nslices;    /* split path: BF16 digits per operand; 0 = automatic     */
  double tol;         /* split path: target relative error (default 1e-12)     */
  int32_t flags;      /* QS_FLAG_*                                              */
} qs_opts;

#define QS_FLAG_NO_GRAPH 1      /* do not capture/replay the launch in a CUDA graph */
#define QS_FLAG_DETERMINISTIC 2 /* fixed reduction order (always true today)   */
#define QS_FLAG_AUTOTUNE 4      /* reusable plans: time the digit widths on the first run */

/* Per-call statistics (optional out-parameter). */
typedef struct {
  double flops;           /* FP64-equivalent flops: 2MNK real, 8MNK complex   */
  double bytes;           /* algorithmic bytes: inputs + output, once          */
  double device_ms;       /* device time of the contraction kernels            */
  int64_t npairs;         /* block pairs                                       */
  int64_t nblk_out;       /* output blocks                                     */
  int32_t nslices;        /* split path: digits used                           */
  int32_t digit_bits;     /* split path: bits per digit                        */
  double err_bound;       /* split path: a-priori relative error bound         */
  int32_t launches;       /* kernels launched by this call                     */
  int32_t pad_;
} qs_stats;

/* ---------------------------------------------------------------- basics */

QS_EXPORT const char *qs_last_error(void);
QS_EXPORT const char *qs_version(void);
QS_EXPORT qs_status qs_ctx_create(int device, qs_ctx **out);
QS_EXPORT void qs_ctx_destroy(qs_ctx *ctx);
/* cudaStream_t of the context (for event timing by the caller). */
QS_EXPORT void *qs_ctx_stream(qs_ctx *ctx);
QS_EXPORT qs_status qs_ctx_sync(qs_ctx *ctx);
/* Kernels launched on this context since creation (for launch accounting). */
QS_EXPORT int64_t qs_ctx_launches(const qs_ctx *ctx);
/* Phase timing (no counterpart in the reference; its WB_CLOCK timers,
 * Source/wbclock.hh:43-377, play this role on the CPU).  When enabled, each
 * contraction records CUDA events on the context stream around operand
 * preparation (digit slicing; empty for the FP64 path) and around the GEMM
 * kernel; qs_ctx_phase_ms waits for the most recent call and returns both
 * device times in milliseconds.  For qs_permuteQS / qs_permute_dev the first
 * time is that of the permute kernels and the second is zero. */
QS_EXPORT qs_status qs_ctx_set_timing(qs_ctx *ctx, int32_t enable);
QS_EXPORT qs_status qs_ctx_phase_ms(qs_ctx *ctx, double *prep_ms, double *gemm_ms);

/* ------------------------------------------------------- contractQS (host)
 * C = contractQS(A, ia, B, ib [,perm]) with host buffers in and out.
 * Replaces the MEX usage #1 path: contract_plain / CONTRACT_QS
 * (Source/contractQS.cc:505-632) -> QSpace::contract (Source/QSpace.cc:
 * 4296-4420) with contract_getIdxSet (:4131-4294) and contractDATA_group
 * (Source/QSpace_aux.cc:27-355).  Labels and block order are bit-exact;
 * block data match the reference's dgemm/zgemm results to FP rounding (FP64
 * path) or to opts->tol (split path).  Abelian symmetries (no CGR) only. */
QS_EXPORT qs_status qs_contractQS(qs_ctx *ctx,
                        const qs_qspace_view *A, const char *ia,
                        const qs_qspace_view *B, const char *ib,
                        const int32_t *perm, int32_t nperm,
                        const qs_opts *opts, qs_result **C, qs_stats *stats);

QS_EXPORT qs_status qs_result_info(const qs_result *C, int32_t *rank, int32_t *qdim,
                         int64_t *nblk, int64_t *nelem, int32_t *is_complex);
/* Copies labels (nblk*rank*qdim), dims (nblk*rank), offsets (nblk) and data
 * (nelem, x2 doubles when complex) into caller buffers; any may be NULL. */
/* Leg tags of the result as "a,b*,c" into buf (len bytes, NUL-terminated);
 * empty when the operands had none. */
QS_EXPORT qs_status qs_result_itags(const qs_result *C, char *buf, size_t len);
QS_EXPORT qs_status qs_result_copy(const qs_result *C, int32_t *q, int64_t *dims,
                         int64_t *offs, double *data);
QS_EXPORT void qs_result_free(qs_result *C);

/* --------------------------------------------------- device-resident API */
QS_EXPORT qs_status qs_tensor_upload(qs_ctx *ctx, const qs_qspace_view *A, qs_tensor **out);
QS_EXPORT qs_status qs_tensor_info(const qs_tensor *T, int32_t *rank, int32_t *qdim,
                         int64_t *nblk, int64_t *nelem, int32_t *is_complex);
QS_EXPORT qs_status qs_tensor_download(qs_ctx *ctx, const qs_tensor *T, int32_t *q,
                             int64_t *dims, int64_t *offs, double *data);
/* C = A + bfac * B for device tensors (plusQS, Source/plusQS.cc:11-45 with
 * QSpace::plus_plain, Source/QSpace.cc:3593-3700): blocks of the union of both
 * label sets in lexicographic label order, each the sum of the blocks present
 * (dims must agree), then SkipZeroData (rank-2 exemption as in contractQS).
 * Real + complex gives complex.  Abelian QSpaces. */
QS_EXPORT qs_status qs_plus_dev(qs_ctx *ctx, const qs_tensor *A, const qs_tensor *B, double bfac,
                      qs_tensor **C);
/* Labels, dims and element offsets of a device tensor (host copies of its
 * metadata only; any pointer may be NULL). */
QS_EXPORT qs_status qs_tensor_meta(const qs_tensor *T, int32_t *q, int64_t *dims, int64_t *offs);
/* Device pointer of the block data (for callers that keep data on device). */
QS_EXPORT const double *qs_tensor_data(const qs_tensor *T);
QS_EXPORT qs_status qs_tensor_itags(const qs_tensor *T, char *buf, size_t len);
QS_EXPORT void qs_tensor_free(qs_tensor *T);

/* ---------------------------------------------------------- wire container
 * A QSpace as one flat binary container (no counterpart in binary form: the
 * reference's container is the MATLAB struct {Q, data, info} of
 * Source/QSpace.hh:3005-3100, kept in .mat files).  Little-endian; a 128-byte
 * header ("QSPW", format version 1, complex flag, rank, qdim, nblk, data
 * extent, section offsets) followed by 64-byte aligned sections: labels
 * (int32, block-major as in qs_qspace_view), dims (int64), offsets (int64),
 * data (FP64 or interleaved complex128), itags ("a,b*,c" + NUL).  Abelian
 * QSpaces only (no info.cgr section).  Every offset and length is validated
 * before a view points into a buffer; a malformed container is QS_ERR_ARG. */
QS_EXPORT qs_status qs_wire_size(const qs_qspace_view *A, int64_t *bytes);
QS_EXPORT qs_status qs_wire_pack(const qs_qspace_view *A, void *buf, int64_t bytes);
/* Zero copy: *A points into buf (8-byte aligned) and is valid as long as it. */
QS_EXPORT qs_status qs_wire_view(const void *buf, int64_t bytes, qs_qspace_view *A);
/* Device tensors straight from / into a container: one host->device copy of
 * its data section, or one device->host copy into it. */
QS_EXPORT qs_status qs_tensor_from_wire(qs_ctx *ctx, const void *buf, int64_t bytes, qs_tensor **out);
QS_EXPORT qs_status qs_tensor_wire_size(const qs_tensor *T, int64_t *bytes);
QS_EXPORT qs_status qs_tensor_to_wire(qs_ctx *ctx, const qs_tensor *T, void *buf, int64_t bytes);
/* Same contraction as qs_contractQS with device-resident operands and result. */
QS_EXPORT qs_status qs_contract_dev(qs_ctx *ctx, const qs_tensor *A, const char *ia,
                          const qs_tensor *B, const char *ib,
                          const int32_t *perm, int32_t nperm,
                          const qs_opts *opts, qs_tensor **C, qs_stats *stats);

/* A batch of device-resident contractions C[r] = contractQS(A[r], ia[r], B[r],
 * ib[r] [,perm[r]]) whose block products all run in one grouped launch per
 * result element type (no reference counterpart: the reference contracts
 * one pair of QSpaces per call; the per-contraction semantics are those of
 * qs_contract_dev).  On the split path each contraction keeps the digit
 * plan it would get alone, so every result is bit-identical to the same
 * call alone.  perm and nperm may be NULL; C receives n tensors. */
QS_EXPORT qs_status qs_contract_batch(qs_ctx *ctx, int32_t n, const qs_tensor *const *A,
                                      const char *const *ia, const qs_tensor *const *B,
                                      const char *const *ib, const int32_t *const *perm,
                                      const int32_t *nperm, const qs_opts *opts, qs_tensor **C);

/* Cell contraction C = contractQS({X_0, X_1, ..., X_{n-1}} [,perm])
 * (Source/contractQS.cc:634-808, contractQS_itags) on device-resident
 * tensors: right to left, C = X_{n-1}, then C = X_k * C for k = n-2..0 over
 * the legs whose itags match (same name, opposite direction; the same
 * direction when one of the two carries a conj flag; Source/wbindex.cc:
 * 1512-1595).  conj[k] != 0 is the '*' option of X_k (conj may be NULL).
 * Every leg needs a non-empty itag.  perm (1-based; a partial permutation is
 * extended) applies to the final result; an empty intermediate result gives
 * an empty result. */
QS_EXPORT qs_status qs_contract_itags(qs_ctx *ctx, int32_t n, const qs_tensor *const *T,
                                      const int32_t *conj, const int32_t *perm, int32_t nperm,
                                      const qs_opts *opts, qs_tensor **C);

/* ---------------------------------------------------------- permuteQS
 * B = permuteQS(A, perm [,'conj']) (Source/permuteQS.cc:198-258;
 * QSpace::Permute Source/QSpace.hh:2670-2719): legs of labels and of every
 * block are reordered on the device, block order is unchanged. */
QS_EXPORT qs_status qs_permuteQS(qs_ctx *ctx, const qs_qspace_view *A,
                       const int32_t *perm, int32_t nperm, int32_t conj,
                       qs_result **B);
QS_EXPORT qs_status qs_permute_dev(qs_ctx *ctx, const qs_tensor *A, const int32_t *perm,
                         int32_t nperm, int32_t conj, qs_tensor **B);

/* ------------------------------------------------- grouped block products
 * The per-output-block seam of the reference (the OpenMP loop at
 * Source/QSpace.cc:4375-4393 calling contractDATA_group, which for each block
 * pair does Ck += afac * Ai*Bi, Source/QSpace_aux.cc:227-235 and
 * wbarray::contract Source/wbarray.cc:3389-3500 -> DZGEMM Source/
 * wbarray_blas.cc:121-213).  Pair p computes
 *     C[c_blk[p]] (+)= afac[p] * op(A_p) * op(B_p)
 * with op(A_p) an M x K and op(B_p) a K x N column-major view at the given
 * element offsets and leading dimensions; trans bit 0 transposes A (A stored
 * K x M), bit 1 transposes B (B stored N x K), bit 2 conjugates A, bit 3
 * conjugates B.  Pairs that share c_blk are summed in array order into the
 * same M x N output block (first pair overwrites).  All pointers are device
 * pointers; element type double or complex128 (is_complex).
 * How a block runs depends on the block alone (so a block gives the same
 * bits in any batch): a block whose pairs sum at most 8 along K is computed
 * directly in FP64 (always on the FP64 path; on the split path where the
 * tiles would mostly be padding, e.g. M = 1); a block with a summed depth of
 * thousands and few output tiles is cut along its depth into parts summed in
 * a fixed order (parts of at most 64 outputs reduced in FP64); every other
 * block runs through the grouped tiles of the chosen precision. */
typedef struct {
  int64_t npairs;
  const int32_t *M, *N, *K;
  const int64_t *a_off, *b_off, *c_off;
  const int32_t *lda, *ldb, *ldc;
  const int32_t *trans;
  const double *afac;     /* real CG / X-symbol factors                      */
  const int32_t *c_blk;   /* output block id per pair (pairs of one block are
                             contiguous)                                     */
  int32_t is_complex;
} qs_pair_list;

QS_EXPORT qs_status qs_grouped_gemm(qs_ctx *ctx, const qs_pair_list *pairs,
                          const double *A, const double *B, double *C,
                          const qs_opts *opts, qs_stats *stats);
/* Host-buffer form of the same call: A and B are copied in, C (c_elems
 * elements) is copied out; elements of C outside every output block come
 * back as zero.  Every access is checked against the given element counts. */
QS_EXPORT qs_status qs_grouped_gemm_host(qs_ctx *ctx, const qs_pair_list *pairs,
                               const double *A, int64_t a_elems,
                               const double *B, int64_t b_elems,
                               double *C, int64_t c_elems,
                               const qs_opts *opts, qs_stats *stats);

/* ------------------------------------------------ reusable grouped plans
 * No reference counterpart (the reference plans every contraction anew).  A
 * plan validates a pair list once, keeps its work lists and digit arena on
 * the device, and records its launch sequence as a CUDA graph on the first
 * run; later runs with the same A, B, C replay the graph (other pointers
 * record it again).  Repeated products over one block structure -- the
 * Davidson iterations of a DMRG site update, the steps of an NRG run --
 * then skip host planning.  opts->flags: QS_FLAG_NO_GRAPH launches directly;
 * QS_FLAG_AUTOTUNE times every digit width that meets opts->tol on the first
 * run and keeps the fastest (remembered per pair-list shape in the process;
 * stats->device_ms reports the winner's time).  A, B, C are device pointers
 * as for qs_grouped_gemm; runs are asynchronous on the context's stream.  A
 * plan is destroyed before its context. */
typedef struct qs_grouped_plan qs_grouped_plan;
QS_EXPORT qs_status qs_grouped_plan_create(qs_ctx *ctx, const qs_pair_list *pairs, const qs_opts *opts,
                                           qs_grouped_plan **out);
QS_EXPORT qs_status qs_grouped_plan_run(qs_grouped_plan *plan, const double *A, const double *B, double *C,
                                        qs_stats *stats);
QS_EXPORT void qs_grouped_plan_destroy(qs_grouped_plan *plan);

/* ------------------------------------- split grouped GEMM, no allocation
 * No reference counterpart: QSpace has no GPU path.  The same product as
 * qs_grouped_gemm with QS_PREC_SPLIT (opts NULL: split, tol 1e-12; any other
 * prec is QS_ERR_ARG), for callers that must not allocate device memory
 * while they run -- a host whose device memory is fully handed to another
 * allocator, or a serving loop that must not let cudaFree synchronise the
 * device.  It allocates no device memory: no cudaMalloc/cudaMallocAsync/
 * cudaFree, no memory pool, no library workspace (its host-side planning uses
 * ordinary host memory).  Its device scratch (work lists,
 * exponents, BF16 digits) is one file-scope array of
 * QS_STATIC_SCRATCH_BYTES per device and process; a pair list that needs
 * more is refused with QS_ERR_OOM before anything is launched.
 *  - The first call on each device looks the array up (cudaGetSymbolAddress)
 *    and clears its 4-byte error word, the only part that must start at
 *    zero; make that first call before any stream capture.  Everything else
 *    in the array is written before it is read in every call.
 *  - All calls in a process share the array of their device: calls that
 *    overlap in time (two host threads, two contexts) race on it and corrupt
 *    each other's results.  Serialise them.
 *  - Every output block runs through the tiles as it is: blocks that
 *    qs_grouped_gemm computes directly (a summed depth of at most 8) or cuts
 *    along their depth (a few outputs over thousands of terms) give the same
 *    product within the split error bound, not the same bits.
 *  - A, B, C are device pointers as for qs_grouped_gemm; the call returns
 *    after the product is complete: it synchronises the context's stream to
 *    read the error word, so it must not be called while that stream is
 *    being captured into a CUDA graph.
 *  - The array is device memory of every process that loads the module
 *    holding it: on each device where that module is loaded (at the first
 *    call with lazy module loading, at context creation with
 *    CUDA_MODULE_LOADING=EAGER), even if the entry point is never called,
 *    and until the process exits. */
#define QS_STATIC_SCRATCH_BYTES 33554432 /* 32 MiB */
QS_EXPORT qs_status qs_grouped_gemm_split_static(qs_ctx *ctx, const qs_pair_list *pairs,
                                                 const double *A, const double *B, double *C,
                                                 const qs_opts *opts, qs_stats *stats);

/* ------------------------------------------- device CG / X-symbol factors
 * The reference looks every block pair's X-symbol up in a host hash map
 * (X3Map gXS, Source/clebsch.hh:3911-4245), filled on first use by
 * X3Map::contractCGR (Source/clebsch_aux.cc:4073-4330) and consulted inside
 * the pair loop (Source/QSpace_aux.cc:27-355).  A qs_xcache is that store on
 * the device: the caller derives a 128-bit key (two uint64 words) from the
 * (CGT_a, ica, CGT_b, icb) tuple of a factor, puts the factors once, and the
 * keyed grouped product resolves every pair's factor on the device, so
 * repeated contractions pass keys only.  The key (2^64-1, 2^64-1) is
 * reserved.  A table holds up to `capacity` entries; a put beyond that is
 * refused with QS_ERR_OOM and leaves the table unchanged.  Puts synchronise
 * with the context's stream (they belong to warm-up). */
typedef struct qs_xcache qs_xcache;
QS_EXPORT qs_status qs_xcache_create(qs_ctx *ctx, int64_t capacity, qs_xcache **out);
QS_EXPORT void qs_xcache_destroy(qs_xcache *cache);
/* Inserts or overwrites n factors; keys holds 2n words. */
QS_EXPORT qs_status qs_xcache_put(qs_xcache *cache, int64_t n, const uint64_t *keys, const double *vals);
/* Looks n keys up on the device (host arrays in and out); found[i] = 0
 * marks a missing key, whose vals[i] is 0. */
QS_EXPORT qs_status qs_xcache_get(qs_xcache *cache, int64_t n, const uint64_t *keys, double *vals,
                                  int32_t *found);
QS_EXPORT qs_status qs_xcache_count(const qs_xcache *cache, int64_t *n);
/* qs_grouped_gemm with the factor of pair p looked up under the key
 * fkeys[2p], fkeys[2p+1] (host array); pairs->afac is ignored and may be
 * NULL.  The keys are looked up on the device, the factors come back (8
 * bytes per pair) and the product runs as qs_grouped_gemm with them, so it
 * gives the same bits as the listed-factor call.  The call waits for its
 * products.  A key missing from the table fails it with QS_ERR_ARG; the
 * products of that pair then used factor 0. */
QS_EXPORT qs_status qs_grouped_gemm_keyed(qs_ctx *ctx, const qs_pair_list *pairs, const uint64_t *fkeys,
                                          const qs_xcache *cache, const double *A, const double *B,
                                          double *C, const qs_opts *opts, qs_stats *stats);

/* ------------------------------------------------------- eigQS blocks
 * Hermitian eigendecomposition of every symmetry block on the device in FP64
 * (the OpenMP loop of QSpace::EigenSymmetric, Source/QSpace.cc:4789-4811,
 * calling wbEigenS -> dsyevd/zheevd, Source/wbarray_blas.cc:501-660).
 * blocks: n[i] x n[i] column-major at offs[i] (device pointer `H`); on return
 * `E` (device, sum n) holds ascending eigenvalues per block at eoffs[i] and
 * `U` (device, same layout as H) the eigenvectors. */
QS_EXPORT qs_status qs_eig_blocks(qs_ctx *ctx, int64_t nblk, const int64_t *n,
                        const int64_t *offs, const int64_t *eoffs,
                        const double *H, double *E, double *U,
                        int32_t is_complex);

/* Global truncation over all blocks' eigenvalues (markSet,
 * Source/gathered.cc:1822-1990, as used by EigenSymmetric :4814): marks the
 * Nkeep lowest, moved to the widest gap near the cut when deps > 0 (so that
 * degenerate multiplets stay together), capped by Etrunc when > 0.  Host
 * arrays; `keep` receives 0/1 per eigenvalue.  `qdim_w` (weighting by
 * multiplet dimension) must be NULL: weights are refused with
 * QS_ERR_UNSUPPORTED.
 * *nkeep_out receives NK exactly as markSet leaves it: min(Nkeep, N) (N = all
 * eigenvalues; Nkeep < 0 counts as N) when Etrunc > 0 and deps == 0, even
 * where Etrunc keeps fewer states; otherwise the number of kept states.  To
 * size buffers, count the 1s in `keep`.  *etrunc_out receives the
 * truncation energy. */
QS_EXPORT qs_status qs_mark_keep(int64_t nblk, const int64_t *n, const double *E,
                       const double *qdim_w, int64_t nkeep, double etrunc,
                       double deps, uint8_t *keep, int64_t *nkeep_out,
                       double *etrunc_out);

/* markSet's degeneracy averaging alone (Source/gathered.cc:1847-1866): the
 * levels of all blocks (n[i] back to back in E, host arrays) in stable
 * ascending order, clusters of consecutive levels closer than
 * deps * (max - min) replaced by their mean, written to E_out in E's order
 * (E_out may be E).  deps <= 0 copies E.  eigQS reports these levels when
 * deps > 0. */
QS_EXPORT qs_status qs_average_levels(int64_t nblk, const int64_t *n, const double *E, double deps,
                       double *E_out);

/* qs_mark_keep with the eigenvalues on the device (E: device array, blocks'
 * ascending eigenvalues back to back; n: host array of block sizes) and the
 * 0/1 flags written to the device array `keep`; NK and Etrunc as
 * qs_mark_keep reports them, from the same arithmetic (the stable order by
 * merging the blocks' runs and the degeneracy averaging run on the device;
 * only the values around the cut reach the host). */
QS_EXPORT qs_status qs_mark_keep_dev(qs_ctx *ctx, int64_t nblk, const int64_t *n, const double *E,
                       int64_t nkeep, double etrunc, double deps, uint8_t *keep,
                       int64_t *nkeep_out, double *etrunc_out);

/* eigQS on a device-resident block-diagonal rank-2 QSpace H (EigenSymmetric,
 * Source/QSpace.cc:4673-4939, with markSet): block eig on the device, the
 * global truncation (as qs_mark_keep) from the eigenvalues, and the kept /
 * discarded eigenvectors as new device tensors *AK / *AD (legs: H's first
 * leg and the eigenstate index, labels of H's block; blocks without kept
 * resp. discarded states are omitted).  The truncation runs on the device
 * (qs_mark_keep_dev): the eigenvalues reach the host only when E is given.  Optional host outputs: E (sum of the
 * block sizes) = ascending eigenvalues per block in H's block order, keep =
 * 0/1 per eigenvalue, NK as qs_mark_keep reports it (not always the kept
 * count: count the kept states from `keep` or from *AK's blocks) and the
 * truncation energy.  With deps > 0 the eigenvalues in E are the averaged
 * ones, as markSet writes them back for the reference's eigQS (clusters of
 * levels closer than deps times the spectral width share their mean;
 * qs_average_levels); a block's levels that the solver returned a rounding
 * out of order (degenerate levels) are made non-decreasing. */
QS_EXPORT qs_status qs_eigQS_dev(qs_ctx *ctx, const qs_tensor *H, int64_t nkeep, double etrunc,
                       double deps, qs_tensor **AK, qs_tensor **AD, double *E,
                       uint8_t *keep, int64_t *nkeep_out, double *etrunc_out);

/* The truncation of svdQS (SVD_Data::dmrgTruncate, Source/mpsortho.cc:
 * 616-700, markSet in descending order): given the singular values of every
 * block (k[i] values of block i back to back in S, host arrays), marks the
 * kept ones: those above stol (at least Nkmin of the largest when stol would
 * drop more), at most Nkeep (< 0: no limit).  Returns the kept count, the
 * discarded and the total weight (sums of S^2), and sfac, the factor that
 * rescales the kept values to the full norm. */
QS_EXPORT qs_status qs_svd_keep(int64_t nblk, const int64_t *k, const double *S, int64_t nkeep,
                      int64_t nkmin, double stol, uint8_t *keep, int64_t *nkeep_out,
                      double *s2t_out, double *s2tot_out, double *sfac_out);

/* -------------------------------------------------------- svdQS blocks
 * Thin SVD of every block (SVD_Data::blockSVD, Source/mpsortho.cc:546-613 ->
 * wbSVD -> dgesdd, Source/wbarray_blas.cc:995-1090).  Block i is m[i] x n[i]
 * column-major at offs[i]; outputs U (m x k), S (k), Vt (k x n) with
 * k = min(m, n) at uoffs/soffs/voffs.  Device pointers. */
QS_EXPORT qs_status qs_svd_blocks(qs_ctx *ctx, int64_t nblk, const int64_t *m,
                        const int64_t *n, const int64_t *offs,
                        const int64_t *uoffs, const int64_t *soffs,
                        const int64_t *voffs, const double *A, double *U,
                        double *S, double *Vt);

/* The same for real (is_complex = 0: FP64) or complex (is_complex = 1:
 * interleaved complex128, offsets in complex elements; Vt = V^H) blocks.
 * With max_sweeps = 0 and tol <= 0 blocks of at most 32 x 32 go to the
 * batched Jacobi solver and larger ones to the polar-decomposition SVD
 * (cuSOLVER Xgesvdp), spread over concurrent solver streams; a caller that
 * gives max_sweeps > 0 or tol > 0 gets one Jacobi SVD per block with that
 * sweep limit (0 = 100) and tolerance (<= 0: 1e-15).  A block that does
 * not converge fails the call with QS_ERR_NUMERIC (wbSVD stops on a LAPACK
 * info != 0, Source/wbarray_blas.cc:1040-1060). */
QS_EXPORT qs_status qs_svd_blocks_ex(qs_ctx *ctx, int64_t nblk, const int64_t *m,
                        const int64_t *n, const int64_t *offs,
                        const int64_t *uoffs, const int64_t *soffs,
                        const int64_t *voffs, int32_t is_complex,
                        const double *A, double *U, double *S, double *Vt,
                        int32_t max_sweeps, double tol);

/* ------------------------------------------- Davidson re-orthogonalisation
 * Double classical Gram-Schmidt of vector v (length n) against the nv
 * orthonormal columns of V (n x nv, column-major), then normalisation
 * (RunDavidson, Source/david2SiteQS.cc:440-470; GSProject twice).  Device
 * pointers, FP64.  *norm_out receives |v| before normalisation. */
QS_EXPORT qs_status qs_gs_reortho(qs_ctx *ctx, int64_t n, int64_t nv, const double *V,
                        double *v, double *norm_out);

/* ------------------------------------------------------------ serving loop
 * A continuous-batching request loop (no counterpart in the reference, whose
 * MEX calls are one at a time).  Requests are contractions and block
 * eigendecompositions (eigQS) of device-resident tensors; each runs on its
 * own slot stream once admitted by HBM footprint; completions are polled. */
typedef struct qs_server qs_server;
typedef struct {
  int32_t nslots;          /* concurrent requests on the device               */
  int32_t max_batch;       /* requests one slot runs in one grouped launch
                              (continuous batching); 0 = 16                  */
  int64_t hbm_budget;      /* bytes of scratch+output the server may hold      */
} qs_server_cfg;
QS_EXPORT qs_status qs_server_create(qs_ctx *ctx, const qs_server_cfg *cfg, qs_server **out);
QS_EXPORT void qs_server_destroy(qs_server *s);
/* Enqueue; returns a ticket.  Thread-safe. */
QS_EXPORT qs_status qs_server_submit(qs_server *s, const qs_tensor *A, const char *ia,
                           const qs_tensor *B, const char *ib,
                           const int32_t *perm, int32_t nperm,
                           const qs_opts *opts, int64_t *ticket);
/* Non-blocking poll (timeout_ms = 0) or bounded wait.  On completion *done = 1
 * and *C receives the result tensor (owned by the caller), *latency_ms the
 * submit-to-completion time. */
QS_EXPORT qs_status qs_server_poll(qs_server *s, int64_t ticket, int32_t timeout_ms,
                         int32_t *done, qs_tensor **C, double *latency_ms);
QS_EXPORT qs_status qs_server_cancel(qs_server *s, int64_t ticket);
/* qs_server_submit for a client with its own context `client` (same device;
 * NULL = the server's context): the request waits for the work queued on the
 * client's stream so far, and its result tensor belongs to the client's
 * context, so the client may keep using it on its own stream and frees it
 * there. */
QS_EXPORT qs_status qs_server_submit_from(qs_server *s, qs_ctx *client, const qs_tensor *A,
                                          const char *ia, const qs_tensor *B, const char *ib,
                                          const int32_t *perm, int32_t nperm, const qs_opts *opts,
                                          int64_t *ticket);
/* An eigQS request: qs_eigQS_dev of the device-resident rank-2 QSpace H
 * (EigenSymmetric + markSet, Source/QSpace.cc:4673-4939) with the truncation
 * options nkeep / etrunc / deps, run on a slot stream beside the contraction
 * batches (no counterpart in the reference).  H must stay alive until the
 * request completes. */
QS_EXPORT qs_status qs_server_submit_eig(qs_server *s, const qs_tensor *H, int64_t nkeep, double etrunc,
                                         double deps, int64_t *ticket);
/* The same for a client with its own context (as qs_server_submit_from). */
QS_EXPORT qs_status qs_server_submit_eig_from(qs_server *s, qs_ctx *client, const qs_tensor *H,
                                              int64_t nkeep, double etrunc, double deps, int64_t *ticket);
/* Completion of an eig request, as qs_server_poll: *AK / *AD receive the
 * kept / discarded eigenvector tensors (owned by the caller; NULL to drop),
 * E and keep (optional host arrays of sum(block sizes) entries) the
 * eigenvalues in H's block order and their 0/1 keep flags, NK and Etrunc as
 * qs_eigQS_dev reports them. */
QS_EXPORT qs_status qs_server_poll_eig(qs_server *s, int64_t ticket, int32_t timeout_ms, int32_t *done,
                                       qs_tensor **AK, qs_tensor **AD, double *E, uint8_t *keep,
                                       int64_t *nkeep_out, double *etrunc_out, double *latency_ms);

#ifdef __cplusplus
}
#endif
#endif /* QSGPU_H */
