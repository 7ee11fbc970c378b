// Split-precision grouped block GEMM on the sm_103a tensor cores.
//
// Method (error-free digit slicing in the spirit of Ozaki, Ogita, Oishi and
// Rump, Numer. Algorithms 59 (2012), adapted to BF16 operands with exact FP32
// accumulation):
//
//  * Every output block gets one power-of-two scale per row of op(A) and per
//    column of op(B), taken over all block pairs that feed it
//    (E_i = max exponent of row i, F_j likewise).  Rows/columns are then
//    |x| < 2^E.
//  * Each scaled FP64 entry is rounded to the integer N = round(x 2^(bS-E))
//    and cut into S balanced signed digits of b bits,
//    N = sum_t d_t 2^(b(S-1-t)), |d_0| <= 2^b, |d_t| <= 2^(b-1).
//    The digits are small integers, exact in BF16.  The cut uses integer
//    operations on the FP64 bit pattern only (GB300's FP64 pipe is narrow).
//  * The product of the two digit expansions is
//      sum_k x_ik y_kj = 2^(E_i+F_j-2b) sum_g 2^(-bg) acc_g,
//      acc_g = sum_k sum_{t+u=g} d_t(ik) d'_u(kj),   g = 0..S-1
//    (the triangular part; terms with t+u >= S are below the target).  b is
//    chosen so that |acc_g| < 2^24 for every partial sum: all tensor-core
//    accumulations in FP32 are then exact integer arithmetic.  When the summed
//    depth of a block exceeds that bound, the K loop is cut into chunks whose
//    accumulators are drained and added in FP64.
//  * The S digit tiles of B are laid side by side along N, so one
//    tcgen05.mma with A-digit t and N = (S-t)*64 produces all products
//    d_t * d'_u (u = 0..S-1-t) at once and drops each into the TMEM columns of
//    accumulator group g = t+u (column offset 64*g).  S(S+1)/2 digit
//    products therefore take about S + S/2 wide MMA instructions per K step.
//  * The epilogue reads the S accumulators from TMEM, combines them with a
//    double-FP32 Horner sum (exact until the final rounding to FP64), scales
//    by 2^(E_i+F_j-2b) and the CG factor, and writes (or, for later chunks,
//    adds) the FP64 result.  One CTA owns one 128x64 output tile and sums the
//    block pairs in plan order: deterministic, no atomics.
//
// Data movement: a slicing kernel writes the digits of every pair operand once
// into an HBM arena, pre-tiled in the tcgen05 K-major, no-swizzle core-matrix
// layout (8 rows x 16 bytes per core matrix); the GEMM kernel then moves
// whole digit tiles with 1-D TMA bulk copies (cp.async.bulk + mbarrier
// transaction counts) into a multi-stage shared-memory ring.  Warp roles:
// warp 0 = TMA producer, warp 1 = TMEM owner and MMA issuer, warps 2..5 =
// epilogue (one TMEM lane quarter each).  Every mbarrier wait is bounded; on
// timeout the kernel records an error code, stops issuing work, waits a
// bounded time for what is in flight, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "qs_internal.h"
#include "qs_split.h"

namespace qs {

namespace {

constexpr int TMS = 128;          // output tile rows (MMA M)
constexpr int TNS = 64;           // output tile cols (per digit group)
constexpr int TKS = 32;           // K block per pipeline stage
constexpr int A_DIGIT_BYTES = TMS * TKS * 2;  // 8 KB
constexpr int B_DIGIT_BYTES = TNS * TKS * 2;  // 4 KB
constexpr int EMPTY_EXP = -30000;
constexpr int SMEM_HDR = 1024;
constexpr int SMEM_LIMIT = 227 * 1024;
constexpr uint32_t WAIT_LIMIT = 1u << 22;  // bounded mbarrier polls (seconds)

struct SplitPair {
  int64_t a_off, b_off;    // element offsets of op(A)/op(B) storage
  int64_t as_off, bs_off;  // byte offsets of this pair's digit tiles
  int32_t M, N, K;         // logical (complex or real) sizes
  int32_t lda, ldb, trans;
  int32_t Mr, Kr;          // real rows of op(A~) and real depth
  int32_t MT, NT, KB;      // tile counts
  int32_t eoff, foff;      // exponent array offsets of the output block
  int32_t e_afac;          // exponent added by a folded CG factor
  double afac_fold;        // factor folded into A's digits (1: epilogue)
};

struct SplitTile {
  int64_t c_off;           // double offset of the output block
  int32_t p0, p1;
  int32_t mt, nt;
  int32_t Mr, N, ldc;
  int32_t eoff, foff;
  int32_t nchunk;          // drains of the accumulators
  double afac;             // epilogue factor
};

// ------------------------------------------------------------ bit helpers
__device__ __forceinline__ int exp_key(double x) {
  const long long b = __double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7ff);
  return ((b << 1) != 0) ? max(be, 1) : 0;
}

// Balanced digits of N = round(x * 2^(b*S - E)); |x| < 2^E is guaranteed by
// construction of E.  Integer operations only.
template <int S>
__device__ __forceinline__ void make_digits(double x, int E, int b, int (&d)[S]) {
  const long long bits = __double_as_longlong(x);
  int be = (int)((bits >> 52) & 0x7ff);
  long long mant = bits & 0xFFFFFFFFFFFFFLL;
  if (be == 0) be = 1; else mant |= (1LL << 52);
  long long N = 0;
  if (mant != 0) {
    const int shift = be - 1075 + b * S - E;
    if (shift >= 0) N = mant << min(shift, 62);
    else if (shift > -62) N = (mant + (1LL << (-shift - 1))) >> (-shift);
    if (bits < 0) N = -N;
  }
  const long long half = 1LL << (b - 1), mask = (1LL << b) - 1;
#pragma unroll
  for (int t = S - 1; t >= 1; --t) {
    const long long r = ((N + half) & mask) - half;
    d[t] = (int)r;
    N = (N - r) >> b;
  }
  d[0] = (int)N;
}

__device__ __forceinline__ uint32_t pack_bf16(int lo, int hi) {
  __nv_bfloat162 h = __floats2bfloat162_rn((float)lo, (float)hi);
  return *reinterpret_cast<uint32_t *>(&h);
}

// --------------------------------------------------------- exponent passes
// Row exponents of op(A~) (per output block, max over its pairs).
template <bool CPLX>
__global__ void __launch_bounds__(256)
exp_rows_kernel(const SplitPair *__restrict__ pairs, const int2 *__restrict__ tasks,
                const double *__restrict__ A, int *__restrict__ E) {
  const int2 tk = tasks[blockIdx.x];
  const SplitPair P = pairs[tk.x];
  const int m = tk.y + threadIdx.x;
  if (m >= P.M) return;
  const bool ta = P.trans & 1;
  int key = 0;
  for (int k = 0; k < P.K; ++k) {
    const int64_t idx = ta ? (int64_t)k + (int64_t)m * P.lda : (int64_t)m + (int64_t)k * P.lda;
    if (CPLX) {
      const double2 v = reinterpret_cast<const double2 *>(A)[P.a_off + idx];
      key = max(key, max(exp_key(v.x), exp_key(v.y)));
    } else {
      key = max(key, exp_key(A[P.a_off + idx]));
    }
  }
  if (!key) return;
  const int e = key - 1022 + P.e_afac;
  if (CPLX) {
    atomicMax(&E[P.eoff + 2 * m], e);
    atomicMax(&E[P.eoff + 2 * m + 1], e);
  } else {
    atomicMax(&E[P.eoff + m], e);
  }
}

// Column exponents of op(B~).
template <bool CPLX>
__global__ void __launch_bounds__(256)
exp_cols_kernel(const SplitPair *__restrict__ pairs, const int2 *__restrict__ tasks,
                const double *__restrict__ B, int *__restrict__ F) {
  const int2 tk = tasks[blockIdx.x];
  const SplitPair P = pairs[tk.x];
  const int n = tk.y + threadIdx.x;
  if (n >= P.N) return;
  const bool tb = P.trans & 2;
  int key = 0;
  for (int k = 0; k < P.K; ++k) {
    const int64_t idx = tb ? (int64_t)n + (int64_t)k * P.ldb : (int64_t)k + (int64_t)n * P.ldb;
    if (CPLX) {
      const double2 v = reinterpret_cast<const double2 *>(B)[P.b_off + idx];
      key = max(key, max(exp_key(v.x), exp_key(v.y)));
    } else {
      key = max(key, exp_key(B[P.b_off + idx]));
    }
  }
  if (key) atomicMax(&F[P.foff + n], key - 1022);
}

__global__ void fill_int_kernel(int *p, int64_t n, int v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// ------------------------------------------------------------ slicing
// A~ digit tile (mt, kb): 128 rows x 32 k, core matrix (row group g, k core c)
// at byte ((g*4 + c)*128), row r%8 at +16*(r%8), k%8 at +2*(k%8).
template <bool CPLX, int S>
__global__ void __launch_bounds__(256)
slice_a_kernel(const SplitPair *__restrict__ pairs, const int4 *__restrict__ tasks,
               const double *__restrict__ A, const int *__restrict__ E,
               uint8_t *__restrict__ arena, int b) {
  const int4 tk = tasks[blockIdx.x];  // (pair, mt, kb, -)
  const SplitPair P = pairs[tk.x];
  const int mt = tk.y, kb = tk.z;
  const bool ta = P.trans & 1, ca = P.trans & 4;
  uint8_t *tile = arena + P.as_off + ((int64_t)(mt * P.KB + kb) * S) * A_DIGIT_BYTES;
  for (int w = threadIdx.x; w < TMS * (TKS / 8); w += blockDim.x) {
    const int r = w % TMS, q = w / TMS;
    const int rr = mt * TMS + r;
    const bool rv = rr < P.Mr;
    const int Ei = rv ? E[P.eoff + rr] : 0;
    uint32_t pk[S][4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      int dd[2][S];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int kk = kb * TKS + q * 8 + e + h;
        double v = 0.0;
        if (rv && kk < P.Kr) {
          if (CPLX) {
            const int m = rr >> 1, rho = rr & 1, k = kk >> 1, kap = kk & 1;
            const double2 a = reinterpret_cast<const double2 *>(A)[
                P.a_off + (ta ? (int64_t)k + (int64_t)m * P.lda : (int64_t)m + (int64_t)k * P.lda)];
            const double ai = ca ? -a.y : a.y;
            v = rho == 0 ? (kap == 0 ? a.x : -ai) : (kap == 0 ? ai : a.x);
          } else {
            v = A[P.a_off + (ta ? (int64_t)kk + (int64_t)rr * P.lda : (int64_t)rr + (int64_t)kk * P.lda)];
          }
          if (P.afac_fold != 1.0) v *= P.afac_fold;
        }
        make_digits<S>(v, Ei, b, dd[h]);
      }
#pragma unroll
      for (int t = 0; t < S; ++t) pk[t][e >> 1] = pack_bf16(dd[0][t], dd[1][t]);
    }
    uint8_t *dst = tile + ((r >> 3) * 4 + q) * 128 + (r & 7) * 16;
#pragma unroll
    for (int t = 0; t < S; ++t)
      *reinterpret_cast<uint4 *>(dst + t * A_DIGIT_BYTES) = make_uint4(pk[t][0], pk[t][1], pk[t][2], pk[t][3]);
  }
}

// B~ digit tile (nt, kb): 64 columns x 32 k, same core-matrix layout with the
// column index in the role of the row.
template <bool CPLX, int S>
__global__ void __launch_bounds__(256)
slice_b_kernel(const SplitPair *__restrict__ pairs, const int4 *__restrict__ tasks,
               const double *__restrict__ B, const int *__restrict__ F,
               uint8_t *__restrict__ arena, int b) {
  const int4 tk = tasks[blockIdx.x];
  const SplitPair P = pairs[tk.x];
  const int nt = tk.y, kb = tk.z;
  const bool tb = P.trans & 2, cb = P.trans & 8;
  uint8_t *tile = arena + P.bs_off + ((int64_t)(nt * P.KB + kb) * S) * B_DIGIT_BYTES;
  for (int w = threadIdx.x; w < TNS * (TKS / 8); w += blockDim.x) {
    const int c = w % TNS, q = w / TNS;
    const int n = nt * TNS + c;
    const bool nv = n < P.N;
    const int Fj = nv ? F[P.foff + n] : 0;
    uint32_t pk[S][4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      int dd[2][S];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int kk = kb * TKS + q * 8 + e + h;
        double v = 0.0;
        if (nv && kk < P.Kr) {
          if (CPLX) {
            const int k = kk >> 1, kap = kk & 1;
            const double2 x = reinterpret_cast<const double2 *>(B)[
                P.b_off + (tb ? (int64_t)n + (int64_t)k * P.ldb : (int64_t)k + (int64_t)n * P.ldb)];
            v = kap ? (cb ? -x.y : x.y) : x.x;
          } else {
            v = B[P.b_off + (tb ? (int64_t)n + (int64_t)kk * P.ldb : (int64_t)kk + (int64_t)n * P.ldb)];
          }
        }
        make_digits<S>(v, Fj, b, dd[h]);
      }
#pragma unroll
      for (int t = 0; t < S; ++t) pk[t][e >> 1] = pack_bf16(dd[0][t], dd[1][t]);
    }
    uint8_t *dst = tile + ((c >> 3) * 4 + q) * 128 + (c & 7) * 16;
#pragma unroll
    for (int t = 0; t < S; ++t)
      *reinterpret_cast<uint4 *>(dst + t * B_DIGIT_BYTES) = make_uint4(pk[t][0], pk[t][1], pk[t][2], pk[t][3]);
  }
}

// ------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: returns false (and raises the CTA abort flag and the global
// error word) when the barrier phase did not complete in time, or when
// another role already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *err, int code) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
  }
  *abort_flag = 1;
  atomicExch(err, code);
  return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// SWIZZLE_NONE K-major shared-memory matrix descriptor: start address, LBO =
// byte distance between core matrices adjacent in K, SBO = between core
// matrices adjacent in M/N, descriptor version 1 (bits 46-47).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// kind::f16 instruction descriptor: D=F32, A=B=BF16, both K-major, N, M=128.
__host__ __device__ constexpr uint32_t make_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TMS >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Exact double-FP32 helpers for the recombination.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Chunking rule shared by the host and the MMA issuer: a new chunk starts
// when adding the next K block would push the summed (real) depth of the
// current chunk above kchunk.
__device__ __forceinline__ int kblock_depth(int Kr, int kb) { return min(TKS, Kr - kb * TKS); }

// ------------------------------------------------------------ GEMM kernel
template <int S>
__global__ void __launch_bounds__(192, 1)
gemm_split_kernel(const SplitTile *__restrict__ tiles, const SplitPair *__restrict__ pairs,
                  const uint8_t *__restrict__ arena, const int *__restrict__ E,
                  const int *__restrict__ F, double *__restrict__ C, int b, int nstages,
                  int kchunk, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);       // [8]
  uint64_t *empty = full + 8;                                 // [8]
  uint64_t *acc_full = full + 16;
  uint64_t *acc_empty = full + 17;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 512);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + 516);
  uint8_t *stages = smem + SMEM_HDR;
  constexpr uint32_t A_BYTES = S * A_DIGIT_BYTES, B_BYTES = S * B_DIGIT_BYTES;
  constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr uint32_t NCOLS = (S * TNS <= 256) ? 256 : 512;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const SplitTile T = tiles[blockIdx.x];

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 4);  // one arrive per epilogue warp
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------ TMA producer
      int it = 0;
      bool ok = true;
      for (int p = T.p0; p < T.p1 && ok; ++p) {
        const SplitPair &P = pairs[p];
        const int KB = P.KB;
        const uint8_t *a_src = arena + P.as_off + (int64_t)T.mt * KB * A_BYTES;
        const uint8_t *b_src = arena + P.bs_off + (int64_t)T.nt * KB * B_BYTES;
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int st = it % nstages;
          const uint32_t ph = (uint32_t)((it / nstages) & 1);
          if (!mbar_wait(&empty[st], ph ^ 1u, abort_flag, err, 1)) { ok = false; break; }
          uint8_t *sa = stages + (size_t)st * STAGE_BYTES;
          mbar_expect_tx(&full[st], STAGE_BYTES);
          bulk_g2s(sa, a_src + (int64_t)kb * A_BYTES, A_BYTES, &full[st]);
          bulk_g2s(sa + A_BYTES, b_src + (int64_t)kb * B_BYTES, B_BYTES, &full[st]);
        }
      }
      // Wait (bounded) until every stage issued has landed, so that no bulk
      // copy is still writing shared memory when the CTA exits.
      const int issued = it;
      for (int j = max(0, issued - nstages); j < issued; ++j) {
        const int st = j % nstages;
        const uint32_t ph = (uint32_t)((j / nstages) & 1);
        for (uint32_t i = 0; i < WAIT_LIMIT && !mbar_try_wait(&full[st], ph); ++i) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------ MMA issuer
      uint32_t idesc[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) idesc[j] = make_idesc(TNS * (j + 1));
      int it = 0, chunk = 0, depth = 0;
      bool fresh = true, ok = true;
      for (int p = T.p0; p < T.p1 && ok; ++p) {
        const int KB = pairs[p].KB, Kr = pairs[p].Kr;
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int dk = max(kblock_depth(Kr, kb), 0);
          if (!fresh && depth + dk > kchunk) {
            // drain: hand the accumulators to the epilogue, wait until read
            umma_commit(acc_full);
            if (!mbar_wait(acc_empty, (uint32_t)(chunk & 1), abort_flag, err, 2)) { ok = false; break; }
            tc_fence_after();
            ++chunk;
            fresh = true;
            depth = 0;
          }
          depth += dk;
          const int st = it % nstages;
          const uint32_t ph = (uint32_t)((it / nstages) & 1);
          if (!mbar_wait(&full[st], ph, abort_flag, err, 3)) { ok = false; break; }
          tc_fence_after();
          const uint32_t a0 = smem_u32(stages + (size_t)st * STAGE_BYTES);
          const uint32_t b0 = a0 + A_BYTES;
#pragma unroll
          for (int ks = 0; ks < TKS / 16; ++ks) {
#pragma unroll
            for (int t = 0; t < S; ++t) {
#pragma unroll
              for (int u0 = 0; u0 < S - t; u0 += 4) {
                const int nu = min(4, S - t - u0);
                const uint64_t ad = make_desc(a0 + t * A_DIGIT_BYTES + ks * 256, 128, 512);
                const uint64_t bd = make_desc(b0 + u0 * B_DIGIT_BYTES + ks * 256, 128, 512);
                const uint32_t acc = (fresh && ks == 0 && t == 0) ? 0u : 1u;
                umma_bf16(tmem + (uint32_t)((t + u0) * TNS), ad, bd, idesc[nu - 1], acc);
              }
            }
          }
          fresh = false;
          umma_commit(&empty[st]);
        }
      }
      umma_commit(acc_full);
      // make sure every MMA issued has completed before TMEM is released
      if (ok) {
        // the epilogue's final acc_empty arrive follows its last TMEM read
        mbar_wait(acc_empty, (uint32_t)(chunk & 1), abort_flag, err, 4);
      } else {
        for (uint32_t i = 0; i < WAIT_LIMIT && !mbar_try_wait(acc_full, (uint32_t)(chunk & 1)); ++i) {
        }
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2..5)
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int i_glob = T.mt * TMS + row;
    const bool rv = i_glob < T.Mr;
    const int Ei = rv ? E[T.eoff + i_glob] : 0;
    const float sb = ldexpf(1.0f, -b);
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    for (int ch = 0; ch < T.nchunk; ++ch) {
      // one lane polls; the warp proceeds together (tcgen05.ld is .aligned)
      int ok = 1;
      if (lane == 0) ok = mbar_wait(acc_full, (uint32_t)(ch & 1), abort_flag, err, 5) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      tc_fence_after();
#pragma unroll 1
      for (int c0 = 0; c0 < TNS; c0 += 8) {
        float acc[S][8];
#pragma unroll
        for (int g = 0; g < S; ++g) tmem_ld8(lane_base + (uint32_t)(g * TNS + c0), acc[g]);
        tmem_wait_ld();
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const int j = T.nt * TNS + c0 + cc;
          if (!rv || j >= T.N) continue;
          // Horner sum of 2^(-b g) acc_g in double-FP32 (hi, lo)
          float hi = acc[S - 1][cc], lo = 0.0f;
#pragma unroll
          for (int g = S - 2; g >= 0; --g) {
            hi *= sb;
            lo *= sb;
            float s, e;
            two_sum(hi, acc[g][cc], s, e);
            lo += e;
            const float h2 = s + lo;
            lo = lo - (h2 - s);
            hi = h2;
          }
          double v = (double)hi + (double)lo;
          const int ex = Ei + F[T.foff + j] - 2 * b;
          v = ldexp(v, ex) * T.afac;
          double *dst = C + T.c_off + (int64_t)i_glob + (int64_t)j * T.ldc;
          if (ch == 0) *dst = v;
          else *dst += v;
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
  }
}

template <int S>
size_t smem_bytes(int nstages) {
  return SMEM_HDR + (size_t)nstages * S * (A_DIGIT_BYTES + B_DIGIT_BYTES);
}

template <int S>
int pick_stages() {
  const size_t per = (size_t)S * (A_DIGIT_BYTES + B_DIGIT_BYTES);
  int n = (int)((SMEM_LIMIT - SMEM_HDR) / per);
  return std::max(1, std::min(n, 4));
}

template <int S>
void launch_split_s(Ctx *ctx, bool cplx, const SplitPair *d_pairs, const int2 *d_rt, int nrt,
                    const int2 *d_ct, int nct, const int4 *d_at, int nat, const int4 *d_bt, int nbt,
                    const SplitTile *d_tiles, int ntiles, const double *A, const double *B, double *C,
                    int *dE, int64_t nE, int *dF, int64_t nF, uint8_t *arena, int b, int kchunk) {
  cudaStream_t st = ctx->stream;
  const int fg = (int)std::min<int64_t>(std::max<int64_t>((nE + nF + 255) / 256, 1), 4096);
  ctx->mark(0);
  fill_int_kernel<<<fg, 256, 0, st>>>(dE, nE, EMPTY_EXP);
  QS_LAUNCHED(ctx);
  fill_int_kernel<<<fg, 256, 0, st>>>(dF, nF, EMPTY_EXP);
  QS_LAUNCHED(ctx);
  if (cplx) {
    if (nrt) { exp_rows_kernel<true><<<nrt, 256, 0, st>>>(d_pairs, d_rt, A, dE); QS_LAUNCHED(ctx); }
    if (nct) { exp_cols_kernel<true><<<nct, 256, 0, st>>>(d_pairs, d_ct, B, dF); QS_LAUNCHED(ctx); }
    if (nat) { slice_a_kernel<true, S><<<nat, 256, 0, st>>>(d_pairs, d_at, A, dE, arena, b); QS_LAUNCHED(ctx); }
    if (nbt) { slice_b_kernel<true, S><<<nbt, 256, 0, st>>>(d_pairs, d_bt, B, dF, arena, b); QS_LAUNCHED(ctx); }
  } else {
    if (nrt) { exp_rows_kernel<false><<<nrt, 256, 0, st>>>(d_pairs, d_rt, A, dE); QS_LAUNCHED(ctx); }
    if (nct) { exp_cols_kernel<false><<<nct, 256, 0, st>>>(d_pairs, d_ct, B, dF); QS_LAUNCHED(ctx); }
    if (nat) { slice_a_kernel<false, S><<<nat, 256, 0, st>>>(d_pairs, d_at, A, dE, arena, b); QS_LAUNCHED(ctx); }
    if (nbt) { slice_b_kernel<false, S><<<nbt, 256, 0, st>>>(d_pairs, d_bt, B, dF, arena, b); QS_LAUNCHED(ctx); }
  }
  const int nst = pick_stages<S>();
  const size_t sm = smem_bytes<S>(nst);
  QS_CUDA(cudaFuncSetAttribute(gemm_split_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  ctx->mark(1);
  gemm_split_kernel<S><<<ntiles, 192, sm, st>>>(d_tiles, d_pairs, arena, dE, dF, C, b, nst, kchunk, ctx->d_err);
  QS_LAUNCHED(ctx);
  ctx->mark(2);
}

}  // namespace

// ---------------------------------------------------------------- host side
DigitPlan choose_digits(int64_t kreal, double tol, int forced_slices) {
  (void)kreal;
  if (!(tol > 0)) tol = 1e-12;
  // bits of precision wanted: the tolerance plus a margin for the growth of
  // the error with the summed depth relative to |C|.
  const int need = (int)std::ceil(-std::log2(tol)) + 8;
  DigitPlan best{0, 0, 0};
  double best_cost = 1e300;
  for (int b = 8; b >= 5; --b) {
    int S = forced_slices > 0 ? forced_slices : (need - 1 + b - 1) / b;
    S = std::max(S, 2);
    if (S > 8) continue;
    // largest summed depth that keeps every accumulator exact
    const double grow = std::max(1.0, 1.0 + (S - 2) / 4.0);
    const double kchunk = std::floor(16777216.0 / (std::ldexp(1.0, 2 * b) * grow));
    if (kchunk < TKS) continue;
    // cost model: digit products per K step, plus a drain per chunk
    const double cost = S * (S + 1) / 2.0 * (1.0 + 24.0 / kchunk);
    if (cost < best_cost) {
      best_cost = cost;
      best.bits = b;
      best.nslices = S;
      best.err_bound = (S + 2) * std::ldexp(1.0, -b * S);
    }
  }
  if (!best.nslices) fail(QS_ERR_NUMERIC, "no digit plan for tol=%g, slices=%d", tol, forced_slices);
  return best;
}

static int kchunk_of(int b, int S) {
  const double grow = std::max(1.0, 1.0 + (S - 2) / 4.0);
  const double kc = std::floor(16777216.0 / (std::ldexp(1.0, 2 * b) * grow));
  return (int)std::min(kc, 1.0e9);
}

SplitResult run_split(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                      const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                      const std::vector<int64_t> &c_off, const double *A, const double *B, double *C,
                      bool cplx, int forced_slices, double tol, const std::vector<int32_t> *blk_ldc) {
  SplitResult res;
  const int64_t nb = (int64_t)blk_M.size();
  const int cm = cplx ? 2 : 1;
  int64_t kmax = 0;
  for (int64_t g = 0; g < nb; ++g) {
    int64_t ks = 0;
    for (int64_t p = grp[g]; p < grp[g + 1]; ++p) ks += (int64_t)pairs[p].K * cm;
    kmax = std::max(kmax, ks);
  }
  DigitPlan dp = choose_digits(kmax, tol, forced_slices);
  const int S = dp.nslices, b = dp.bits;
  const int kchunk = kchunk_of(b, S);
  res.nslices = S;
  res.bits = b;
  res.err_bound = dp.err_bound;

  // per-pair digit geometry and arena offsets
  std::vector<SplitPair> sp(pairs.size());
  std::vector<int64_t> eoff(nb), foff(nb);
  int64_t nE = 0, nF = 0;
  for (int64_t g = 0; g < nb; ++g) {
    eoff[g] = nE;
    foff[g] = nF;
    nE += (int64_t)blk_M[g] * cm;
    nF += blk_N[g];
  }
  if (nE > INT32_MAX || nF > INT32_MAX) fail(QS_ERR_SHAPE, "split: exponent arrays too large");
  int64_t arena = 0;
  std::vector<int2> rt, ct;
  std::vector<int4> at, bt;
  std::vector<SplitTile> tiles;
  for (int64_t g = 0; g < nb; ++g) {
    // one CG factor for the whole block goes into the epilogue; otherwise
    // each pair's factor is folded into its A digits
    bool same = true;
    for (int64_t p = grp[g]; p < grp[g + 1]; ++p) same &= (pairs[p].afac == pairs[grp[g]].afac);
    int64_t depth_blk = 0;
    for (int64_t p = grp[g]; p < grp[g + 1]; ++p) {
      const PairDesc &d = pairs[p];
      SplitPair &s = sp[p];
      s.a_off = d.a_off;
      s.b_off = d.b_off;
      s.M = d.M;
      s.N = d.N;
      s.K = d.K;
      s.lda = d.lda;
      s.ldb = d.ldb;
      s.trans = d.trans;
      s.Mr = d.M * cm;
      s.Kr = d.K * cm;
      s.MT = (s.Mr + TMS - 1) / TMS;
      s.NT = (s.N + TNS - 1) / TNS;
      s.KB = std::max(1, (s.Kr + TKS - 1) / TKS);
      s.eoff = (int32_t)eoff[g];
      s.foff = (int32_t)foff[g];
      if (same) {
        s.afac_fold = 1.0;
        s.e_afac = 0;
      } else {
        s.afac_fold = d.afac;
        int e = 0;
        std::frexp(d.afac, &e);
        s.e_afac = d.afac != 0.0 ? e : 0;
      }
      s.as_off = arena;
      arena += (int64_t)s.MT * s.KB * S * A_DIGIT_BYTES;
      s.bs_off = arena;
      arena += (int64_t)s.NT * s.KB * S * B_DIGIT_BYTES;
      for (int m0 = 0; m0 < d.M; m0 += 256) rt.push_back(make_int2((int)p, m0));
      for (int n0 = 0; n0 < d.N; n0 += 256) ct.push_back(make_int2((int)p, n0));
      for (int mt = 0; mt < s.MT; ++mt)
        for (int kb = 0; kb < s.KB; ++kb) at.push_back(make_int4((int)p, mt, kb, 0));
      for (int nt = 0; nt < s.NT; ++nt)
        for (int kb = 0; kb < s.KB; ++kb) bt.push_back(make_int4((int)p, nt, kb, 0));
      depth_blk += s.Kr;
    }
    // number of accumulator drains of this block's tiles (same rule as the
    // MMA issuer: per K block of depth min(32, Kr - 32 kb))
    int nchunk = 1, depth = 0;
    bool fresh = true;
    for (int64_t p = grp[g]; p < grp[g + 1]; ++p)
      for (int kb = 0; kb < sp[p].KB; ++kb) {
        const int dk = std::max(std::min(TKS, sp[p].Kr - kb * TKS), 0);
        if (!fresh && depth + dk > kchunk) { ++nchunk; depth = 0; fresh = true; }
        depth += dk;
        fresh = false;
      }
    const int MT = (blk_M[g] * cm + TMS - 1) / TMS, NT = (blk_N[g] + TNS - 1) / TNS;
    for (int nt = 0; nt < NT; ++nt)
      for (int mt = 0; mt < MT; ++mt) {
        SplitTile t{};
        t.c_off = c_off[g] * cm;
        t.p0 = (int32_t)grp[g];
        t.p1 = (int32_t)grp[g + 1];
        t.mt = mt;
        t.nt = nt;
        t.Mr = blk_M[g] * cm;
        t.N = blk_N[g];
        t.ldc = blk_ldc ? (*blk_ldc)[g] * cm : std::max(t.Mr, 1);
        t.eoff = (int32_t)eoff[g];
        t.foff = (int32_t)foff[g];
        t.nchunk = nchunk;
        t.afac = same ? pairs[grp[g]].afac : 1.0;
        tiles.push_back(t);
      }
  }
  // Longest tiles first (by summed depth): the tail of the launch is short.
  std::stable_sort(tiles.begin(), tiles.end(), [&](const SplitTile &x, const SplitTile &y) {
    int64_t kx = 0, ky = 0;
    for (int p = x.p0; p < x.p1; ++p) kx += sp[p].KB;
    for (int p = y.p0; p < y.p1; ++p) ky += sp[p].KB;
    return kx > ky;
  });
  if (tiles.empty()) return res;
  if (tiles.size() > 0x7fffffff || at.size() > 0x7fffffff || bt.size() > 0x7fffffff)
    fail(QS_ERR_SHAPE, "split: launch too large");
  res.slice_bytes = arena;
  res.ntiles = (int64_t)tiles.size();

  // device buffers: one allocation for the digit arena (pooled scratch)
  uint8_t *d_arena = static_cast<uint8_t *>(ctx->ensure_scratch((size_t)std::max<int64_t>(arena, 256)));
  SplitPair *d_pairs = dev_upload(ctx, sp);
  int2 *d_rt = dev_upload(ctx, rt);
  int2 *d_ct = dev_upload(ctx, ct);
  int4 *d_at = dev_upload(ctx, at);
  int4 *d_bt = dev_upload(ctx, bt);
  SplitTile *d_tiles = dev_upload(ctx, tiles);
  int *dE = dev_alloc<int>(ctx, (size_t)nE);
  int *dF = dev_alloc<int>(ctx, (size_t)nF);
  switch (S) {
#define QS_CASE(SS)                                                                                      \
  case SS:                                                                                               \
    launch_split_s<SS>(ctx, cplx, d_pairs, d_rt, (int)rt.size(), d_ct, (int)ct.size(), d_at, (int)at.size(), \
                       d_bt, (int)bt.size(), d_tiles, (int)tiles.size(), A, B, C, dE, nE, dF, nF, d_arena, b, \
                       kchunk);                                                                          \
    break;
    QS_CASE(2)
    QS_CASE(3)
    QS_CASE(4)
    QS_CASE(5)
    QS_CASE(6)
    QS_CASE(7)
    QS_CASE(8)
#undef QS_CASE
    default:
      fail(QS_ERR_INTERNAL, "split: unsupported digit count %d", S);
  }
  dev_free(ctx, d_pairs);
  dev_free(ctx, d_rt);
  dev_free(ctx, d_ct);
  dev_free(ctx, d_at);
  dev_free(ctx, d_bt);
  dev_free(ctx, d_tiles);
  dev_free(ctx, dE);
  dev_free(ctx, dF);
  return res;
}

}  // namespace qs
