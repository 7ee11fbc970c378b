// Internal declarations of libqsgpu: error handling, device work descriptors
// and the kernel launchers shared between the host planner (qs_plan.cpp,
// qs_capi.cpp) and the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <deque>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/qsgpu.h"

namespace qs {

// ------------------------------------------------------------------ errors
struct Error : std::runtime_error {
  qs_status code;
  Error(qs_status c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(qs_status code, const char *fmt, ...);
void set_last_error(const std::string &msg);

#define QS_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      ::qs::fail(QS_ERR_CUDA, "%s:%d %s -> %s", __FILE__, __LINE__, #call,   \
                 cudaGetErrorString(e_));                                    \
  } while (0)

// Check the most recent launch.
#define QS_LAUNCHED(ctx)                                                     \
  do {                                                                       \
    cudaError_t e_ = cudaGetLastError();                                     \
    if (e_ != cudaSuccess)                                                   \
      ::qs::fail(QS_ERR_CUDA, "%s:%d kernel launch -> %s", __FILE__,         \
                 __LINE__, cudaGetErrorString(e_));                          \
    (ctx)->launches++;                                                       \
  } while (0)

// ------------------------------------------------------------------ context
struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // factor tables made on this context: their device memory is released
  // with the context, so a table destroyed later touches no freed context
  std::vector<qs_xcache *> tables;
  int num_sms = 0;
  int64_t launches = 0;
  // device error word for bounded waits inside kernels (0 = ok)
  int *d_err = nullptr;
  // pooled scratch (grown on demand, stream ordered)
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  void *ensure_scratch(size_t bytes);
  // page-locked staging ring for work-list uploads: copies from it are
  // asynchronous, so the host plans the next call while the device works
  char *stage_buf = nullptr;      // host address
  char *stage_dev = nullptr;      // the same memory as the device sees it
  size_t stage_cap = 0;
  int64_t stage_head = 0;  // virtual write position (grows monotonically)
  struct StageMark {
    cudaEvent_t ev;
    int64_t start;
  };
  std::deque<StageMark> stage_q;    // copies in flight, oldest first
  std::vector<cudaEvent_t> stage_ev;  // recycled events
  void stage_upload(void *dst, const void *src, size_t bytes);
  void destroy_staging();
  // copy streams of the pipelined host-buffer path (created on first use)
  cudaStream_t h2d = nullptr, d2h = nullptr;
  void ensure_copy_streams();
  void destroy_copy_streams();
  // a second compute stream for independent kernels of one step (forked
  // from and joined back to `stream` with the two events; created on use,
  // released with the copy streams)
  cudaStream_t aux = nullptr;
  cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
  void ensure_aux();
  // cuSOLVER handle (created on first use)
  void *solver = nullptr;
  void *solver_lanes = nullptr;  // extra solver streams for concurrent blocks
  // phase timing: events around operand preparation and the GEMM kernel
  bool timing = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  bool ev_used = false;
  void mark(int i) {
    if (timing && ev[i]) {
      cudaEventRecord(ev[i], stream);
      if (i == 2) ev_used = true;
    }
  }
};

// --------------------------------------------- device work descriptors
// One block product C[c] (+)= afac * op(A) * op(B), element offsets in units
// of the element type (double or complex).
struct PairDesc {
  int64_t a_off, b_off;
  int32_t M, N, K;
  int32_t lda, ldb;
  int32_t trans;   // bit0 transA, bit1 transB, bit2 conjA, bit3 conjB
  double afac;
};
static_assert(sizeof(PairDesc) == 48, "PairDesc layout");

// Deep output blocks.  The grouped kernels give each output tile to one CTA
// for the block's whole summed depth, so a block with few tiles and a very
// deep sum (a reduced density matrix or an overlap over large bonds) would
// leave most SMs idle.  Such a block is cut along its depth into parts, each
// a temporary output block of its own (the pairs' K ranges split where the
// parts meet), and the parts are summed in a fixed order afterwards.  The
// decision depends on the block alone, so a block is cut the same way
// whatever else is in the launch.
struct DeepReduce {
  int64_t c_off;   // the block in C (elements)
  int64_t t_off;   // its first part in the temporary buffer (elements)
  int32_t M, N, ldc, nparts;  // parts are packed M x N, back to back
};
struct DeepSplit {
  std::vector<PairDesc> pairs;
  std::vector<int64_t> grp, coff;   // coff of part blocks: temporary-buffer offsets
  std::vector<int32_t> bM, bN, bldc;
  std::vector<char> part;           // block is a part (its coff is in the temporary buffer)
  std::vector<int32_t> src;         // pair of the input list each pair came from
  std::vector<DeepReduce> red;
  int64_t temp_elems = 0;
  // shifts the part blocks' offsets by the temporary buffer's element
  // offset from C
  void place(int64_t shift) {
    for (size_t b = 0; b < coff.size(); ++b)
      if (part[b]) coff[b] += shift;
  }
};
// Whether any block of the list is deep enough to be cut.
bool has_deep_blocks(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                     const std::vector<int32_t> &bM, const std::vector<int32_t> &bN);
// Cuts the deep blocks (except those marked in `keep`); false (and `out`
// untouched) when there are none.
bool split_deep(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                const std::vector<int32_t> &bM, const std::vector<int32_t> &bN,
                const std::vector<int64_t> &coff, const std::vector<int32_t> *bldc, DeepSplit &out,
                const std::vector<char> *keep = nullptr);
// C block = sum of its parts in part order (FP64 or complex128 elements).
void launch_reduce_parts(Ctx *ctx, const DeepReduce *d_red, int64_t nred, const double *T, double *C, bool cplx);

// Shallow output blocks: a summed depth of at most SHALLOW_K (applying a
// site operator over a leg of dimension 1 or 2, an outer product).  Tiled
// products would pad the depth to a full k-block and pay the epilogue per
// tile; these blocks are computed directly, one thread per output element,
// in FP64 (exact products, summed in pair and k order).
constexpr int64_t SHALLOW_K = 8;
bool is_shallow(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1);
// Whether the direct FP64 computation of a shallow block is estimated to be
// faster than the tiled split-precision one: FP64 rate against the tiles'
// padding (a block with one short side, e.g. M = 1, fills 1 of 32 or 128
// lines of every tile).  Used by the split path; the FP64 path computes every
// shallow block directly.
bool shallow_direct_wins(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1, int32_t M, int32_t N,
                         bool cplx);
// Runs the listed blocks (indices into grp / bM / ...) directly.
void run_shallow(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                 const std::vector<int32_t> &bM, const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
                 const std::vector<int32_t> *bldc, const std::vector<int64_t> &blocks, const double *A,
                 const double *B, double *C, bool cplx);
// Parts of deep output blocks with at most DOT_OUTPUTS elements on the FP64
// path: one CTA per output element reduces over the part's pairs and depth
// (a fixed partition and tree order); 64 x 64 tiles would compute 4096
// outputs for each of them.
constexpr int64_t DOT_OUTPUTS = 64;
void run_dot(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
             const std::vector<int32_t> &bM, const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
             const std::vector<int32_t> *bldc, const std::vector<int64_t> &blocks, const double *A,
             const double *B, double *C, bool cplx);
// The same with the work list prepared once on device memory owned by the
// caller (reusable plans): prepare, launch any number of times, release.
struct ShallowPlan {
  void *tasks = nullptr, *pairs = nullptr;
  int64_t ntasks = 0;
  bool cplx = false;
};
ShallowPlan shallow_prepare(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                            const std::vector<int32_t> &bM, const std::vector<int32_t> &bN,
                            const std::vector<int64_t> &coff, const std::vector<int32_t> *bldc,
                            const std::vector<int64_t> &blocks, bool cplx);
void shallow_launch(Ctx *ctx, const ShallowPlan &sp, const double *A, const double *B, double *C);
void shallow_release(ShallowPlan &sp);
// The blocks of a list with sel[b] set, as a list of their own (with the
// pairs' index in the input list in `src`).
struct BlockList {
  std::vector<PairDesc> pairs;
  std::vector<int64_t> grp, coff;
  std::vector<int32_t> bM, bN, bldc;
  std::vector<int32_t> src;
};
BlockList select_blocks(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                        const std::vector<int32_t> &bM, const std::vector<int32_t> &bN,
                        const std::vector<int64_t> &coff, const std::vector<int32_t> *bldc,
                        const std::vector<char> &sel);

// One output tile of one output block: the pairs [p0, p1) all write block c.
struct TileDesc {
  int64_t c_off;
  int32_t p0, p1;
  int32_t m0, n0;
  int32_t M, N;
  int32_t ldc;
  int32_t cblk;
};
static_assert(sizeof(TileDesc) == 40, "TileDesc layout");

// Generalised transpose of one block: out(j0..jr) = in(P-permuted index).
struct PermDesc {
  int64_t in_off, out_off;
  int64_t n;            // elements
  int32_t rank;
  int32_t conj;
  int64_t out_dims[8];
  int64_t in_stride[8]; // stride in the input of output leg k
  int32_t fast_in_leg;  // output leg with input stride 1 (tiled blocks)
  int32_t pad_;
};

// A strided view of one operand block in place of the permuted copy that
// permute_to makes (Source/QSpace.hh:2824-2866) when the contracted legs of
// an operand are not contiguous: element (line, k) of the operand as the
// GEMM reads it -- line = row of op(A) / column of op(B), k = depth -- sits at
// block offset  sum_i l_i lstr[i] + sum_t k_t kstr[t],  line = sum_i l_i
// prod_{i'<i} ldim[i'] (first leg fastest), likewise k.  nl = 0: no view.
// The kernels read the offsets from tables built on the host once per
// operand block: ltab[line] = sum_i l_i lstr[i], ktab[k] likewise (device
// pointers; the host fills them in after the tables are uploaded).
constexpr int VIEW_LEGS = 4;
struct OperandView {
  int32_t nl, nk;
  int32_t ldim[VIEW_LEGS], kdim[VIEW_LEGS];
  int64_t lstr[VIEW_LEGS], kstr[VIEW_LEGS];
  const int64_t *ltab, *ktab;
};

// One 32 x 32 tile of a tiled block: tile (ti, tj) of (output leg 0,
// output leg fast_in_leg) at linear index `rest` of the other legs.
struct PermTile {
  int64_t desc;
  int64_t rest;
  int32_t ti, tj;
};

// ------------------------------------------------------- kernel launchers
// qs_permute.cu: tiles through shared memory (ntiles items) and output-order
// lines (nchunks chunks of chunk_elems elements); either list may be empty
void launch_permute(Ctx *ctx, const PermDesc *d_desc, const int64_t *d_chunk_blk,
                    const int64_t *d_chunk_start, int64_t nchunks, const PermTile *d_tiles, int64_t ntiles,
                    const double *in, double *out, int is_complex, int chunk_elems);

// qs_gemm_f64.cu -- plain FP64 grouped GEMM (deterministic: one CTA owns an
// output tile, pairs summed in order)
void launch_gemm_f64(Ctx *ctx, const PairDesc *d_pairs, const TileDesc *d_tiles,
                     int64_t ntiles, const double *A, const double *B, double *C,
                     int is_complex);
int gemm_f64_tile_m();
int gemm_f64_tile_n();

// qs_permute.cu -- per-block "all zero" test for SkipZeroData, and the
// real -> complex widening of an operand arena
void launch_block_nonzero(Ctx *ctx, const int64_t *d_offs, const int64_t *d_sizes,
                          int64_t nblk, const double *data, int is_complex,
                          int *d_flags);
void launch_widen(Ctx *ctx, const double *in, double *out, int64_t n);
// dst block b += f * src block b (element offsets / sizes; es = 1 real, 2
// complex; a real source into a complex destination adds to the real parts)
void launch_block_axpy(Ctx *ctx, const int64_t *d_soff, const int64_t *d_doff, const int64_t *d_size, int64_t nb,
                       int64_t max_size, const double *src, double *dst, double f, int es_src, int es_dst);
// copies `bytes` from mapped page-locked host memory to device memory with a kernel
void launch_stage_copy(Ctx *ctx, const void *src, void *dst, size_t bytes);

// Contexts alive in this process (qs_capi.cpp).  Objects that outlive their
// context (device tensors, plans) release their memory without its stream.
void ctx_register(const Ctx *c);
void ctx_unregister(const Ctx *c);
bool ctx_alive(const Ctx *c);

// qs_linalg.cu
void destroy_solver(Ctx *ctx);

// ------------------------------------------------------ small utilities
template <class T>
T *dev_alloc(Ctx *ctx, size_t n) {
  void *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMallocAsync(&p, n * sizeof(T), ctx->stream);
  if (e != cudaSuccess)
    fail(e == cudaErrorMemoryAllocation ? QS_ERR_OOM : QS_ERR_CUDA,
         "cudaMallocAsync(%zu bytes): %s", n * sizeof(T), cudaGetErrorString(e));
  return static_cast<T *>(p);
}
void dev_free(Ctx *ctx, void *p);

template <class T>
T *dev_upload(Ctx *ctx, const std::vector<T> &v) {
  T *p = dev_alloc<T>(ctx, v.size());
  if (!v.empty()) ctx->stage_upload(p, v.data(), v.size() * sizeof(T));
  return p;
}

}  // namespace qs

// C-ABI context object: one device, one stream, one memory pool.
struct qs_ctx {
  qs::Ctx c;
};

// Exception-to-status translation at every C-ABI entry point.
#define QS_API_BEGIN try {
#define QS_API_END                                \
  }                                               \
  catch (const qs::Error &e) {                    \
    qs::set_last_error(e.what());                 \
    return e.code;                                \
  }                                               \
  catch (const std::bad_alloc &) {                \
    qs::set_last_error("host allocation failed"); \
    return QS_ERR_OOM;                            \
  }                                               \
  catch (const std::exception &e) {               \
    qs::set_last_error(e.what());                 \
    return QS_ERR_INTERNAL;                       \
  }                                               \
  return QS_OK;
