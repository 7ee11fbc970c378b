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
//    accumulators are drained and added exactly (int64).
//  * The S digit tiles of B are laid side by side along N, so one
//    tcgen05.mma with A-digit t and N = (S-t)*32 produces all products
//    d_t * d'_u (u = 0..S-1-t) at once and drops each into the TMEM columns of
//    accumulator group g = t+u (column offset 32*g).  S(S+1)/2 digit
//    products therefore take about S + S/2 wide MMA instructions per K step.
//  * The CG factor of each pair is folded into A's digits with an exact
//    integer product (53 x 53 bits) before rounding, so pairs with different
//    factors share the accumulators.
//  * The epilogue reads the S accumulators from TMEM, combines them in int64
//    fixed point, and assembles the FP64 result with integer bit operations
//    (scale 2^(E_i+F_j-2b), round to nearest even): no FP64 instruction, as
//    the FP64 pipe of GB300 is narrow.  Partial sums of later accumulator
//    chunks are added exactly as int64 in the output slot.  One CTA owns one
//    128x32 output tile at a time and sums the block pairs in plan order:
//    deterministic, no atomics.
//
// Data movement: a slicing kernel writes the digits of every pair operand once
// into an HBM arena, pre-tiled in the tcgen05 K-major, no-swizzle core-matrix
// layout (8 rows x 16 bytes per core matrix); the GEMM kernel then moves
// whole digit tiles with 1-D TMA bulk copies (cp.async.bulk + mbarrier
// transaction counts) into a multi-stage shared-memory ring.  Warp roles:
// warp 0 = TMA producer, warp 1 = TMEM owner and MMA issuer, the other
// warps = epilogue (EPI_WARPS / 4 per TMEM lane quarter).  Every mbarrier wait is bounded; on
// timeout the kernel records an error code, stops issuing work, waits a
// bounded time for what is in flight, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <memory>
#include <numeric>
#include <type_traits>

#include "qs_internal.h"
#include "qs_split.h"
#include "qs_xcache.h"

namespace qs {

namespace {

constexpr int TMS = 128;          // output tile rows (MMA M)
constexpr int TNS = 32;           // output tile cols (per digit group)
constexpr int TKS = 32;           // K block per pipeline stage (two MMA K steps)
constexpr int KCM = TKS / 8;      // core matrices along K in a digit tile
constexpr int A_DIGIT_BYTES = TMS * TKS * 2;  // 8 KB
constexpr int B_DIGIT_BYTES = TNS * TKS * 2;  // 2 KB
constexpr int MAX_STAGES = 8;
constexpr int EMPTY_EXP = -30000;
constexpr int SMEM_HDR = 2048;   // barriers, TMEM slot, abort flag; tile-descriptor slots at 1024
constexpr int SMEM_LIMIT = 227 * 1024;
constexpr uint32_t WAIT_LIMIT = 1u << 22;  // bounded mbarrier polls (seconds)
constexpr int EPI_WARPS = 16;     // epilogue warps (4 per TMEM lane quarter)
constexpr int GEMM_THREADS = 64 + 32 * EPI_WARPS;
constexpr int TILE_SLOTS = 1024;  // shared-memory offset of the epilogue warps' descriptor slots

struct SplitPair {
  int64_t a_off, b_off;    // element offsets of op(A)/op(B) storage
  int64_t as_off, bs_off;  // byte offsets of this pair's digit tiles
  int32_t M, N, K;         // logical (complex or real) sizes
  int32_t lda, ldb, trans;
  int32_t Mr, Kr;          // real rows of op(A~) and real depth
  int32_t MT, NT, KB;      // tile counts
  int32_t eoff, foff;      // exponent array offsets of the output block
  int32_t e_afac;          // exponent added by the CG factor (|afac| < 2^e)
  int32_t fe, fneg;        // CG factor folded into A's digits: fm 2^fe, sign
  uint64_t fm;             // (fm = 0: factor 1)
  int32_t swap;            // block computed as C^T = op(B)^T op(A)^T: the A role reads the B arena
  // Real form of a complex block.  dupb = 0: A~ (2M x 2K) rows 2m, 2m+1 =
  // (Re, -Im), (Im, Re) of row m of op(A), B~ (2K x N) rows 2k, 2k+1 = (Re, Im)
  // of op(B), C~ (2M x N) rows = (Re, Im) of C.  dupb = 1: A' (M x 2K) columns
  // 2k, 2k+1 = (Re, Im) of op(A), B' (2K x 2N) columns 2n = (Re; -Im) and
  // 2n+1 = (Im; Re) of column n of op(B), C' (M x 2N) columns = (Re, Im) of C.
  int32_t dupb;
  int32_t Nr;              // real columns of op(B~)
  int32_t pad_;
};

struct SplitTile {
  int64_t c_off;           // double offset of the output block (first member: 8-byte aligned)
  int32_t p0, p1;
  int32_t mt, nt;
  int32_t Mr, N, ldc;
  int32_t eoff, foff;
  int32_t nchunk;          // drains of the accumulators
  int32_t rshift;          // bits dropped below the lowest group (int64 headroom)
  // output address of tile row r, column j (doubles from c_off):
  // (r >> rsplit) * rs + (r & rsplit) + (j >> csplit) * ldc + (j & csplit),
  // splits = rsplit | csplit << 1; rsplit = 1 for a complex block computed
  // transposed in the A-duplicated form (its rows interleave Re/Im of C's
  // columns), csplit = 1 for one in the B-duplicated form, not transposed
  // (its columns interleave Re/Im of C's columns)
  int32_t rs, splits;
};
constexpr int TILE_WORDS = (int)(sizeof(SplitTile) / 4);
static_assert(sizeof(SplitTile) % 8 == 0 && TILE_WORDS <= 16, "tile descriptor fits one 64-byte slot");

// ------------------------------------------------------------ bit helpers
__device__ __forceinline__ int exp_key(double x) {
  const long long b = __double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7ff);
  return ((b << 1) != 0) ? max(be, 1) : 0;
}

// A factor f (CG coefficient) as an exact integer mantissa and exponent,
// f = fm * 2^fe; fm = 0 means "no factor" (f = 1); fe = -100000 means f = 0.
struct Factor {
  unsigned long long fm;
  int fe;
  bool neg;
};

__host__ __device__ inline Factor make_factor(double f) {
  Factor r{0ull, 0, false};
  if (f == 1.0) return r;
  unsigned long long bits;
  memcpy(&bits, &f, 8);
  int be = (int)((bits >> 52) & 0x7ff);
  unsigned long long m = bits & 0xFFFFFFFFFFFFFull;
  if (be == 0) be = 1; else m |= (1ull << 52);
  r.fm = m ? m : 0ull;
  r.fe = be - 1075;
  r.neg = (bits >> 63) != 0;
  if (!m) { r.fm = 0; r.fe = 0; r.neg = false; r.fe = -100000; }  // f == 0
  return r;
}

// N = round(x f 2^(b*S - E)); |x f| < 2^E is guaranteed by construction of
// E, so |N| <= 2^(bS) (b*S <= 62).  Integer operations only.
__device__ __forceinline__ long long scaled_int(double x, int E, int bS, const Factor &F) {
  const long long bits = __double_as_longlong(x);
  int be = (int)((bits >> 52) & 0x7ff);
  unsigned long long mant = bits & 0xFFFFFFFFFFFFFull;
  if (be == 0) be = 1; else mant |= (1ull << 52);
  long long N = 0;
  bool neg = bits < 0;
  if (mant != 0 && F.fe > -100000) {
    if (F.fm == 0) {
      // N = round(mant * 2^shift)
      const int shift = be - 1075 + bS - E;
      if (shift >= 0) N = (long long)(mant << min(shift, 62));
      else if (shift > -62) N = (long long)((mant + (1ull << (-shift - 1))) >> (-shift));
    } else {
      // product with the factor's mantissa: the upper 64 bits of
      // (mant 2^11) (fm 2^11), i.e. mant fm 2^-42 truncated (relative error
      // < 2^-63, far below the 2^-(bS) of the digits), then the rounding shift
      // (|x f| < 2^E holds by construction of E)
      const unsigned long long P = __umul64hi(mant << 11, F.fm << 11);
      const int shift = be - 1075 + F.fe + 42 + bS - E;
      if (shift >= 0) N = (long long)(P << min(shift, 62));
      else if (shift > -64) N = (long long)((P >> (-shift - 1)) + 1 >> 1);
      neg ^= F.neg;
    }
    if (neg) N = -N;
  }
  return N;
}

// Balanced base-2^B digits of N as floats (exact small integers):
//   N = sum_t d_t 2^(B(S-1-t)),  d_t in [-2^(B-1), 2^(B-1)) for t >= 1,
//   |d_0| <= 2^B.
// With H = sum_{t>=1} 2^(B-1) 2^(B(S-1-t)), the low B(S-1) bits of M = N + H
// are the base-2^B digits d_t + 2^(B-1), and d_0 = floor(M / 2^(B(S-1))).
// Each digit is a funnel shift, one logic op (mask | 2^23 exponent) and one
// FP32 subtraction; all values are exact in BF16 (at most 8 significant bits).
template <int S, int B>
__device__ __forceinline__ void digits_f(long long N, float (&d)[S]) {
  constexpr long long HALF = 1LL << (B - 1);
  constexpr unsigned MASK = (1u << B) - 1;
  long long H = 0;
#pragma unroll
  for (int t = 1; t < S; ++t) H = (H << B) + HALF;
  const long long M = N + H;
  const unsigned lo = (unsigned)M, hi = (unsigned)((unsigned long long)M >> 32);
#pragma unroll
  for (int t = 1; t < S; ++t) {
    const int sh = B * (S - 1 - t);
    const unsigned w = sh >= 32 ? (hi >> (sh - 32)) : (sh == 0 ? lo : __funnelshift_r(lo, hi, sh));
    d[t] = __int_as_float((int)((w & MASK) | 0x4B000000u)) - (8388608.0f + (float)HALF);
  }
  const int d0 = (int)(M >> (B * (S - 1)));
  d[0] = __int_as_float(0x4B400000 + d0) - 12582912.0f;
}

// Two BF16 values packed as (lo, hi) halves of a 32-bit word.
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// L2 eviction priorities of the strip kernels (createpolicy, PTX ISA 7.4+):
// the first read of an operand line is kept (evict_last) for the re-read of
// phase 2, which is its last use (evict_first), and the digit stores stream
// through (evict_first), so that they do not push the operand lines out.
__device__ __forceinline__ uint64_t l2_policy_keep() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_stream() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ double2 ld_pol(const double2 *a, uint64_t pol) {
  double2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ double ld_pol(const double *a, uint64_t pol) {
  double v;
  asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_pol(uint8_t *a, uint4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.b32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(a), "r"(v.x), "r"(v.y), "r"(v.z),
               "r"(v.w), "l"(pol)
               : "memory");
}

// Element (line, k) of a pair's operand in the role being sliced: plain
// (lda/ldb, trans) addressing, or the offset tables of the operand's strided
// view when the contraction reads a permuted operand in place.
struct OpAddr {
  int64_t ls, ks;             // plain: line * ls + k * ks
  const int64_t *lt, *kt;     // or the view's tables (nullptr: plain)
  bool kunit;                 // unit depth stride (neighbouring k adjacent)
  __device__ __forceinline__ int64_t line(int64_t m) const { return lt ? lt[m] : m * ls; }
  __device__ __forceinline__ int64_t depth(int64_t k) const { return kt ? kt[k] : k * ks; }
};
// A role: lines are rows of op(A) (contiguous along k when transposed); B
// role: lines are columns of op(B) (contiguous along k when not transposed).
__device__ __forceinline__ OpAddr view_addr(const OperandView *views, int p, int64_t ls, int64_t ks) {
  if (views && views[p].nl > 0) {
    const OperandView &v = views[p];
    return OpAddr{0, 0, v.ltab, v.ktab, v.nk > 0 && v.kstr[0] == 1};
  }
  return OpAddr{ls, ks, nullptr, nullptr, ks == 1};
}
__device__ __forceinline__ OpAddr addr_a(const SplitPair &P, const OperandView *views, int p) {
  const bool ta = P.trans & 1;
  return view_addr(views, p, ta ? (int64_t)P.lda : 1, ta ? 1 : (int64_t)P.lda);
}
__device__ __forceinline__ OpAddr addr_b(const SplitPair &P, const OperandView *views, int p) {
  const bool tb = P.trans & 2;
  return view_addr(views, p, tb ? 1 : (int64_t)P.ldb, tb ? (int64_t)P.ldb : 1);
}

// ---------------------------------------------- exponents and slicing, fused
// One CTA per strip of STRIP real lines of one output block: rows of op(A~)
// (A role) or columns of op(B~) (B role), over every pair of the block and
// its whole depth.
//  Phase 1: the exponent of each line of the strip -- the largest exponent
//    key over all pairs and all k (both parts of a complex element), plus the
//    pair's CG-factor exponent for the A role -- kept in shared memory and
//    written to E / F for the epilogue (every line belongs to one strip, so
//    plain stores).  A line of zeros keeps EMPTY_EXP.
//  Phase 2: the digits of the strip's lines for every pair and k-block,
//    written into the pre-tiled digit arena.  It re-reads what phase 1 has
//    just read: a strip holds at most STRIP lines of the block's depth, so
//    the re-read is mostly served from L2 and the FP64 operands cross HBM
//    once.
// A complex block in the A-duplicated form turns each row m of op(A) into
// the real rows 2m, 2m+1 of A~ (rows (Re, -Im) and (Im, Re) along k) and
// each column of op(B) into one column of B~ (rows 2k, 2k+1 = (Re, Im));
// in the B-duplicated form row m of op(A) is one row of A' ((Re, Im) along
// k) and column n of op(B) the columns 2n, 2n+1 of B' ((Re; -Im), (Im; Re)).
constexpr int STRIP = 16;          // real lines per strip (two core-matrix groups)
constexpr int STRIP_THREADS = 128;

// Phase 1 for the lines l0 .. l0+nl-1 of op(X) (X = A role: rows, line m at
// m + k*ld (contig: k + m*ld); X = B role: columns, line n at k + n*ld
// (contig) or n + k*ld), max over the pairs p0..p1-1 into smax[line].
template <bool CPLX, bool ROLE_B>
__device__ __forceinline__ void strip_maxima(const SplitPair *__restrict__ pairs, const OperandView *views, int p0,
                                             int p1, int l0, int nl, const double *__restrict__ Aarena,
                                             const double *__restrict__ Barena, int *smax) {
  if (threadIdx.x < STRIP) smax[threadIdx.x] = EMPTY_EXP;
  __syncthreads();
  for (int p = p0; p < p1; ++p) {
    const SplitPair &P = pairs[p];
    // a swapped pair's roles read the other arena
    const double *__restrict__ X = (ROLE_B != (P.swap != 0)) ? Barena : Aarena;
    const int64_t off = ROLE_B ? P.b_off : P.a_off;
    const OpAddr ad = ROLE_B ? addr_b(P, views, p) : addr_a(P, views, p);
    // lines contiguous along k (unit depth stride): neighbouring lanes take
    // neighbouring k of one line; else neighbouring lines
    const bool contig = ad.kunit;
    constexpr int NPH = STRIP_THREADS / STRIP;
    const int line = contig ? threadIdx.x / NPH : threadIdx.x % STRIP;
    const int ph = contig ? threadIdx.x % NPH : threadIdx.x / STRIP;
    int key = 0;
    if (line < nl) {
      const uint64_t keep = l2_policy_keep();
      const int64_t base = off + ad.line(l0 + line);
      int k = ph;
      for (; k + 3 * NPH < P.K; k += 4 * NPH) {
        const int64_t o0 = base + ad.depth(k), o1 = base + ad.depth(k + NPH), o2 = base + ad.depth(k + 2 * NPH),
                      o3 = base + ad.depth(k + 3 * NPH);
        if (CPLX) {
          const double2 *x = reinterpret_cast<const double2 *>(X);
          const double2 v0 = ld_pol(x + o0, keep), v1 = ld_pol(x + o1, keep), v2 = ld_pol(x + o2, keep),
                        v3 = ld_pol(x + o3, keep);
          key = max(key, max(max(max(exp_key(v0.x), exp_key(v0.y)), max(exp_key(v1.x), exp_key(v1.y))),
                             max(max(exp_key(v2.x), exp_key(v2.y)), max(exp_key(v3.x), exp_key(v3.y)))));
        } else {
          key = max(key, max(max(exp_key(ld_pol(X + o0, keep)), exp_key(ld_pol(X + o1, keep))),
                             max(exp_key(ld_pol(X + o2, keep)), exp_key(ld_pol(X + o3, keep)))));
        }
      }
      for (; k < P.K; k += NPH) {
        const int64_t o = base + ad.depth(k);
        if (CPLX) {
          const double2 v = ld_pol(reinterpret_cast<const double2 *>(X) + o, keep);
          key = max(key, max(exp_key(v.x), exp_key(v.y)));
        } else {
          key = max(key, exp_key(ld_pol(X + o, keep)));
        }
      }
    }
    if (key) atomicMax(&smax[line], key - 1022 + (ROLE_B ? 0 : P.e_afac));
  }
  __syncthreads();
}

// A role.  Task = (first pair, end pair, first real row r0 of the strip).
template <bool CPLX, int S, int B>
__device__ __forceinline__ void strip_a(const SplitPair *__restrict__ pairs, const OperandView *views, int4 tk,
                                        const double *__restrict__ Aarena, const double *__restrict__ Barena,
                                        int *__restrict__ E, uint8_t *__restrict__ arena) {
  __shared__ int smax[STRIP];
  const int p0 = tk.x, p1 = tk.y, r0 = tk.z;
  const SplitPair &Q = pairs[p0];
  const bool dup = CPLX && Q.dupb == 0;  // two real rows per row of op(A)
  const int l0 = dup ? r0 / 2 : r0;
  const int nl = min(dup ? STRIP / 2 : STRIP, Q.M - l0);
  strip_maxima<CPLX, false>(pairs, views, p0, p1, l0, nl, Aarena, Barena, smax);
  if (threadIdx.x < nl) {
    const int e = smax[threadIdx.x];
    if (dup) {
      E[Q.eoff + 2 * (l0 + threadIdx.x)] = e;
      E[Q.eoff + 2 * (l0 + threadIdx.x) + 1] = e;
    } else {
      E[Q.eoff + l0 + threadIdx.x] = e;
    }
  }
  const int mt = r0 / TMS, rl = r0 % TMS;
  const uint64_t last = l2_policy_stream();  // last use of operand lines; digit stores
  for (int p = p0; p < p1; ++p) {
    const SplitPair &P = pairs[p];
    const double *__restrict__ A = P.swap ? Barena : Aarena;
    const bool ca = P.trans & 4;
    const OpAddr ad = addr_a(P, views, p);
    const Factor Fa{P.fm, P.fe, P.fneg != 0};
    uint8_t *tiles = arena + P.as_off + (int64_t)mt * P.KB * S * A_DIGIT_BYTES;
    if (dup) {
      // item = one row of op(A) (real rows 2m, 2m+1) x 4 complex k
      const int items = (STRIP / 2) * KCM * P.KB;
      for (int w = threadIdx.x; w < items; w += blockDim.x) {
        const int kb = w / ((STRIP / 2) * KCM), i = w % ((STRIP / 2) * KCM);
        const int ml = i % (STRIP / 2), q = i / (STRIP / 2);
        if (ml >= nl) continue;  // rows past the block feed discarded outputs only: not written
        const int64_t lo = P.a_off + ad.line(l0 + ml);
        const int Ei = smax[ml];
        double2 a[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = (kb * TKS + q * 8) / 2 + j;
          a[j] = make_double2(0.0, 0.0);
          if (k < P.K) a[j] = ld_pol(reinterpret_cast<const double2 *>(A) + lo + ad.depth(k), last);
        }
        uint32_t p0w[S][4], p1w[S][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float dr[S], di[S];
          digits_f<S, B>(scaled_int(a[j].x, Ei, B * S, Fa), dr);
          digits_f<S, B>(scaled_int(ca ? -a[j].y : a[j].y, Ei, B * S, Fa), di);
#pragma unroll
          for (int t = 0; t < S; ++t) {
            p0w[t][j] = pack2(dr[t], -di[t]);  // ( re, -im )
            p1w[t][j] = pack2(di[t], dr[t]);   // ( im,  re )
          }
        }
        const int rr0 = rl + 2 * ml, rr1 = rr0 + 1;
        uint8_t *tile = tiles + (int64_t)kb * S * A_DIGIT_BYTES;
        uint8_t *d0 = tile + ((rr0 >> 3) * KCM + q) * 128 + (rr0 & 7) * 16;
        uint8_t *d1 = tile + ((rr1 >> 3) * KCM + q) * 128 + (rr1 & 7) * 16;
#pragma unroll
        for (int t = 0; t < S; ++t) {
          st_pol(d0 + t * A_DIGIT_BYTES, make_uint4(p0w[t][0], p0w[t][1], p0w[t][2], p0w[t][3]), last);
          st_pol(d1 + t * A_DIGIT_BYTES, make_uint4(p1w[t][0], p1w[t][1], p1w[t][2], p1w[t][3]), last);
        }
      }
    } else {
      // item = one real row x 8 real k (4 complex k of the B-duplicated form)
      const int items = STRIP * KCM * P.KB;
      for (int w = threadIdx.x; w < items; w += blockDim.x) {
        const int kb = w / (STRIP * KCM), i = w % (STRIP * KCM);
        const int rloc = i % STRIP, q = i / STRIP;
        if (rloc >= nl) continue;
        const int64_t lo = P.a_off + ad.line(l0 + rloc);
        const int Ei = smax[rloc];
        uint32_t pk[S][4];
        if constexpr (CPLX) {
          double2 a[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int k = (kb * TKS + q * 8) / 2 + j;
            a[j] = make_double2(0.0, 0.0);
            if (k < P.K) a[j] = ld_pol(reinterpret_cast<const double2 *>(A) + lo + ad.depth(k), last);
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            float dr[S], di[S];
            digits_f<S, B>(scaled_int(a[j].x, Ei, B * S, Fa), dr);
            digits_f<S, B>(scaled_int(ca ? -a[j].y : a[j].y, Ei, B * S, Fa), di);
#pragma unroll
            for (int t = 0; t < S; ++t) pk[t][j] = pack2(dr[t], di[t]);
          }
        } else {
          double v[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            const int kk = kb * TKS + q * 8 + e;
            v[e] = 0.0;
            if (kk < P.Kr) v[e] = ld_pol(A + lo + ad.depth(kk), last);
          }
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            float d0[S], d1[S];
            digits_f<S, B>(scaled_int(v[e], Ei, B * S, Fa), d0);
            digits_f<S, B>(scaled_int(v[e + 1], Ei, B * S, Fa), d1);
#pragma unroll
            for (int t = 0; t < S; ++t) pk[t][e >> 1] = pack2(d0[t], d1[t]);
          }
        }
        const int rr = rl + rloc;
        uint8_t *dst = tiles + (int64_t)kb * S * A_DIGIT_BYTES + ((rr >> 3) * KCM + q) * 128 + (rr & 7) * 16;
#pragma unroll
        for (int t = 0; t < S; ++t)
          st_pol(dst + t * A_DIGIT_BYTES, make_uint4(pk[t][0], pk[t][1], pk[t][2], pk[t][3]), last);
      }
    }
  }
}

// B role.  Task = (first pair, end pair, first real column c0 of the strip).
template <bool CPLX, int S, int B>
__device__ __forceinline__ void strip_b(const SplitPair *__restrict__ pairs, const OperandView *views, int4 tk,
                                        const double *__restrict__ Aarena, const double *__restrict__ Barena,
                                        int *__restrict__ F, uint8_t *__restrict__ arena) {
  __shared__ int smax[STRIP];
  const int p0 = tk.x, p1 = tk.y, c0 = tk.z;
  const SplitPair &Q = pairs[p0];
  const bool dup = CPLX && Q.dupb != 0;  // two real columns per column of op(B)
  const int l0 = dup ? c0 / 2 : c0;
  const int nl = min(dup ? STRIP / 2 : STRIP, Q.N - l0);
  strip_maxima<CPLX, true>(pairs, views, p0, p1, l0, nl, Aarena, Barena, smax);
  if (threadIdx.x < nl) {
    const int e = smax[threadIdx.x];
    if (dup) {
      F[Q.foff + 2 * (l0 + threadIdx.x)] = e;
      F[Q.foff + 2 * (l0 + threadIdx.x) + 1] = e;
    } else {
      F[Q.foff + l0 + threadIdx.x] = e;
    }
  }
  const int nt = c0 / TNS, cl = c0 % TNS;
  const int ncols = dup ? 2 * nl : nl;  // real columns of this strip inside the block
  const Factor F1{0ull, 0, false};
  const uint64_t last = l2_policy_stream();  // last use of operand lines; digit stores
  for (int p = p0; p < p1; ++p) {
    const SplitPair &P = pairs[p];
    const double *__restrict__ Bm = P.swap ? Aarena : Barena;
    const bool cb = P.trans & 8;
    const OpAddr ad = addr_b(P, views, p);
    uint8_t *tiles = arena + P.bs_off + (int64_t)nt * P.KB * S * B_DIGIT_BYTES;
    // item = one real column x 8 real k
    const int items = STRIP * KCM * P.KB;
    for (int w = threadIdx.x; w < items; w += blockDim.x) {
      const int kb = w / (STRIP * KCM), i = w % (STRIP * KCM);
      const int cloc = i % STRIP, q = i / STRIP;
      if (cloc >= ncols) continue;  // columns past the block feed discarded outputs only
      const int c = cl + cloc;
      const int Fj = smax[dup ? cloc >> 1 : cloc];
      uint32_t pk[S][4];
      if constexpr (CPLX) {
        const int64_t lo = P.b_off + ad.line(dup ? l0 + (cloc >> 1) : l0 + cloc);
        double2 x[4];
        // B~ (A-duplicated form): rows 2k, 2k+1 = (Re, Im) of element k; B'
        // (B-duplicated form): the same 4 complex k per 8 real rows
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = (kb * TKS + q * 8) / 2 + j;
          x[j] = make_double2(0.0, 0.0);
          if (k < P.K) x[j] = ld_pol(reinterpret_cast<const double2 *>(Bm) + lo + ad.depth(k), last);
        }
        const bool odd = dup && (cloc & 1);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float dr[S], di[S];
          digits_f<S, B>(scaled_int(x[j].x, Fj, B * S, F1), dr);
          digits_f<S, B>(scaled_int(cb ? -x[j].y : x[j].y, Fj, B * S, F1), di);
#pragma unroll
          for (int t = 0; t < S; ++t)
            pk[t][j] = dup ? (odd ? pack2(di[t], dr[t]) : pack2(dr[t], -di[t])) : pack2(dr[t], di[t]);
        }
      } else {
        const int64_t lo = P.b_off + ad.line(l0 + cloc);
        double v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int kk = kb * TKS + q * 8 + e;
          v[e] = 0.0;
          if (kk < P.Kr) v[e] = ld_pol(Bm + lo + ad.depth(kk), last);
        }
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          float d0[S], d1[S];
          digits_f<S, B>(scaled_int(v[e], Fj, B * S, F1), d0);
          digits_f<S, B>(scaled_int(v[e + 1], Fj, B * S, F1), d1);
#pragma unroll
          for (int t = 0; t < S; ++t) pk[t][e >> 1] = pack2(d0[t], d1[t]);
        }
      }
      uint8_t *dst = tiles + (int64_t)kb * S * B_DIGIT_BYTES + ((c >> 3) * KCM + q) * 128 + (c & 7) * 16;
#pragma unroll
      for (int t = 0; t < S; ++t)
        st_pol(dst + t * B_DIGIT_BYTES, make_uint4(pk[t][0], pk[t][1], pk[t][2], pk[t][3]), last);
    }
  }
}

// VIEWS = false: no pair of the launch reads its operand through a view, and
// the view addressing is compiled out
template <bool CPLX, int S, bool VIEWS>
__global__ void __launch_bounds__(STRIP_THREADS)
strip_a_kernel(const SplitPair *__restrict__ pairs, const OperandView *__restrict__ views_in,
               const int4 *__restrict__ tasks, const double *__restrict__ A, const double *__restrict__ B,
               int *__restrict__ E, uint8_t *__restrict__ arena, int b) {
  const OperandView *views = VIEWS ? views_in : nullptr;
  const int4 tk = tasks[blockIdx.x];
  switch (b) {  // the host admits b = 5..8 only
    case 5: strip_a<CPLX, S, 5>(pairs, views, tk, A, B, E, arena); break;
    case 6: strip_a<CPLX, S, 6>(pairs, views, tk, A, B, E, arena); break;
    case 7: strip_a<CPLX, S, 7>(pairs, views, tk, A, B, E, arena); break;
    default: strip_a<CPLX, S, 8>(pairs, views, tk, A, B, E, arena); break;
  }
}

// VIEWS = false: no pair of the launch reads its operand through a view, and
// the view addressing is compiled out
template <bool CPLX, int S, bool VIEWS>
__global__ void __launch_bounds__(STRIP_THREADS)
strip_b_kernel(const SplitPair *__restrict__ pairs, const OperandView *__restrict__ views_in,
               const int4 *__restrict__ tasks, const double *__restrict__ A, const double *__restrict__ B,
               int *__restrict__ F, uint8_t *__restrict__ arena, int b) {
  const OperandView *views = VIEWS ? views_in : nullptr;
  const int4 tk = tasks[blockIdx.x];
  switch (b) {
    case 5: strip_b<CPLX, S, 5>(pairs, views, tk, A, B, F, arena); break;
    case 6: strip_b<CPLX, S, 6>(pairs, views, tk, A, B, F, arena); break;
    case 7: strip_b<CPLX, S, 7>(pairs, views, tk, A, B, F, arena); break;
    default: strip_b<CPLX, S, 8>(pairs, views, tk, A, B, F, arena); break;
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
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Recombination without the FP64 pipe.  The S accumulators hold exact
// integers (|acc_g| <= 2^24); their weighted sum
//   V = sum_g acc_g 2^(b(S-1-g) - r)
// is formed in 64-bit fixed point (r low bits of the smallest groups are
// rounded away so that V and the sum over accumulator chunks keep headroom),
// then turned into an FP64 value V * 2^scale by integer bit assembly (round
// to nearest even).
// Wrapping 32 x 32 -> 64-bit multiply-add: acc + (int64)a * m (mod 2^64).
__device__ __forceinline__ unsigned long long mad_wide(int a, int m, unsigned long long acc) {
  unsigned long long d;
  asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(m), "l"(acc));
  return d;
}

// How accumulator group g enters the fixed-point sum V = sum_g acc_g 2^sh_g
// (sh_g = b(S-1-g) - r): sh >= 32 adds acc * 2^(sh-32) to the high 32-bit
// word, 0 <= sh <= 30 adds acc * 2^sh to the low 64-bit word, sh < 0 adds
// acc / 2^-sh rounded.  All words wrap; V itself fits in int64, so
// V = hi * 2^32 + lo (mod 2^64) is exact.

// V * 2^scale: one int64 -> FP64 conversion (round to nearest even) and an
// exponent add.  Integer-only assemblies (64-bit or 32-bit words, exactly
// rounded, measured on GB300) made the launch slower: on short tiles the
// epilogue is the bottleneck and its cost follows its instruction count.
__device__ __forceinline__ double fixed_to_double(long long V, int scale) {
  if (V == 0) return 0.0;
  const double d = __ll2double_rn(V);
  const long long bits = __double_as_longlong(d);
  const int e = (int)((bits >> 52) & 0x7ff) + scale;
  if (e <= 0 || e >= 2047) return ldexp(d, scale);
  return __longlong_as_double(bits + ((long long)scale << 52));
}

// Folds accumulator groups G0..G0+NG-1 of one set (this thread's TMEM lane,
// 8 columns from cbase) into the fixed-point words: group g enters with shift
// sh = b(S-1-g) - rsh, >= 32 into the high word Vh, 0..30 into the low word
// Vl (the host keeps sh off 31), < 0 rounded down by -sh bits; exactly one
// form applies to a group (uniform branch).
template <int S, int G0, int NG>
__device__ __forceinline__ void fold_groups(uint32_t set_base, int cbase, int b, int rsh,
                                            unsigned long long (&Vl)[8], unsigned int (&Vh)[8]) {
  float acc[NG][8];
#pragma unroll
  for (int g = 0; g < NG; ++g) tmem_ld8(set_base + (uint32_t)((G0 + g) * TNS + cbase), acc[g]);
  tmem_wait_ld();
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const int sh = b * (S - 1 - (G0 + g)) - rsh;
    if (sh >= 32) {
      const unsigned m = 1u << (sh - 32);
#pragma unroll
      for (int c = 0; c < 8; ++c) Vh[c] += (unsigned int)__float2int_rn(acc[g][c]) * m;
    } else if (sh >= 0) {
#pragma unroll
      for (int c = 0; c < 8; ++c) Vl[c] = mad_wide(__float2int_rn(acc[g][c]), 1 << sh, Vl[c]);
    } else {
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int a = __float2int_rn(acc[g][c]);
        Vl[c] = mad_wide((a + (1 << (-sh - 1))) >> -sh, 1, Vl[c]);
      }
    }
  }
}

// Chunking rule shared by the host and the MMA issuer: a new chunk starts
// when adding the next K block would push the summed (real) depth of the
// current chunk above kchunk.
__device__ __forceinline__ int kblock_depth(int Kr, int kb) { return min(TKS, Kr - kb * TKS); }

// ------------------------------------------------------------ GEMM kernel
// Persistent: one CTA per SM walks tiles r*G + c (snake order over the
// depth-sorted tile list so every CTA gets a similar mix).  The three roles
// step through the same sequence; the TMA ring and the accumulator hand-off
// run continuously across tile boundaries.  TMEM holds two accumulator sets
// (S groups x 32 columns each): the epilogue drains one while the MMA issuer
// fills the other.
__device__ __forceinline__ int tile_of(int r, int c, int G) { return r * G + ((r & 1) ? (G - 1 - c) : c); }

template <int S>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
gemm_split_kernel(const SplitTile *__restrict__ tiles, int ntiles, const SplitPair *__restrict__ pairs,
                  const uint8_t *__restrict__ arena, const int *__restrict__ E,
                  const int *__restrict__ F, double *__restrict__ C, int b, int nstages,
                  int kchunk, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);       // [MAX_STAGES]
  uint64_t *empty = full + MAX_STAGES;                        // [MAX_STAGES]
  uint64_t *acc_full = full + 2 * MAX_STAGES;                 // [2]
  uint64_t *acc_empty = acc_full + 2;                         // [2]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 512);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + 516);
  uint8_t *stages = smem + SMEM_HDR;
  constexpr uint32_t A_BYTES = S * A_DIGIT_BYTES, B_BYTES = S * B_DIGIT_BYTES;
  constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr uint32_t SET_COLS = S * TNS;  // columns of one accumulator set
  constexpr uint32_t NCOLS = (2 * SET_COLS <= 256) ? 256 : 512;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = gridDim.x, cta = blockIdx.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&acc_full[s], 1);
      mbar_init(&acc_empty[s], EPI_WARPS);  // one arrive per epilogue warp
    }
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
      int it = 0, st = 0;  // stage it % nstages, its phase bit ph
      uint32_t ph = 0;
      bool ok = true;
      for (int r = 0; ok; ++r) {
        const int ti = tile_of(r, cta, G);
        if (ti >= ntiles) break;
        const SplitTile &T = tiles[ti];
        for (int p = T.p0; p < T.p1 && ok; ++p) {
          const SplitPair &P = pairs[p];
          const int KB = P.KB;
          const uint8_t *a_src = arena + P.as_off + (int64_t)T.mt * KB * A_BYTES;
          const uint8_t *b_src = arena + P.bs_off + (int64_t)T.nt * KB * B_BYTES;
          for (int kb = 0; kb < KB; ++kb, ++it) {
            if (!mbar_wait(&empty[st], ph ^ 1u, abort_flag, err, 1)) { ok = false; break; }
            uint8_t *sa = stages + (size_t)st * STAGE_BYTES;
            mbar_expect_tx(&full[st], STAGE_BYTES);
            bulk_g2s(sa, a_src + (int64_t)kb * A_BYTES, A_BYTES, &full[st]);
            bulk_g2s(sa + A_BYTES, b_src + (int64_t)kb * B_BYTES, B_BYTES, &full[st]);
            if (++st == nstages) {
              st = 0;
              ph ^= 1u;
            }
          }
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
      // one instruction per A digit t: N = (S - t) * 32 columns of B digits
      uint32_t idesc[S];
#pragma unroll
      for (int j = 0; j < S; ++j) idesc[j] = make_idesc(TNS * (j + 1));
      int it = 0, u = 0;  // u: accumulator uses (chunks) handed to the epilogue
      int st = 0;         // stage it % nstages, its phase bit ph
      uint32_t ph = 0;
      // shared-memory descriptors of stage 0; stage st adds st * STAGE_BYTES
      // to the start address field (addresses stay below 2^18, so the 14-bit
      // field never carries)
      const uint64_t desc0 = make_desc(smem_u32(stages), 128, KCM * 128);
      bool ok = true;
      // before filling set u & 1 for use u >= 2, wait until use u - 2 is read
      auto acquire = [&](int uu) -> bool {
        if (uu >= 2) {
          if (!mbar_wait(&acc_empty[uu & 1], (uint32_t)(((uu >> 1) - 1) & 1), abort_flag, err, 2)) return false;
          tc_fence_after();
        }
        return true;
      };
      for (int r = 0; ok; ++r) {
        const int ti = tile_of(r, cta, G);
        if (ti >= ntiles) break;
        const SplitTile &T = tiles[ti];
        int depth = 0;
        bool fresh = true;
        if (!acquire(u)) { ok = false; break; }
        // the sizes of the next pair are loaded one pair ahead, so that the
        // global-load latency stays off the issue path
        const int p1 = T.p1;
        int KBn = pairs[T.p0].KB, Krn = pairs[T.p0].Kr;
        for (int p = T.p0; p < p1 && ok; ++p) {
          const int KB = KBn, Kr = Krn;
          if (p + 1 < p1) {
            KBn = pairs[p + 1].KB;
            Krn = pairs[p + 1].Kr;
          }
          for (int kb = 0; kb < KB; ++kb, ++it) {
            const int dk = max(kblock_depth(Kr, kb), 0);
            if (!fresh && depth + dk > kchunk) {
              // this chunk is done: hand the set to the epilogue, go on in
              // the other set
              umma_commit(&acc_full[u & 1]);
              ++u;
              if (!acquire(u)) { ok = false; break; }
              fresh = true;
              depth = 0;
            }
            depth += dk;
            if (!mbar_wait(&full[st], ph, abort_flag, err, 3)) { ok = false; break; }
            tc_fence_after();
            const uint64_t dst0 = desc0 + (uint64_t)((st * STAGE_BYTES) >> 4);
            const uint32_t dset = tmem + (uint32_t)((u & 1) * SET_COLS);
#pragma unroll
            for (int ks = 0; ks < TKS / 16; ++ks) {
#pragma unroll
              for (int t = 0; t < S; ++t) {
                const uint64_t ad = dst0 + (uint64_t)((t * A_DIGIT_BYTES + ks * 256) >> 4);
                const uint64_t bd = dst0 + (uint64_t)((A_BYTES + ks * 256) >> 4);
                const uint32_t acc = (fresh && ks == 0 && t == 0) ? 0u : 1u;
                umma_bf16(dset + (uint32_t)(t * TNS), ad, bd, idesc[S - 1 - t], acc);
              }
            }
            fresh = false;
            umma_commit(&empty[st]);
            if (++st == nstages) {
              st = 0;
              ph ^= 1u;
            }
          }
        }
        if (!ok) break;
        umma_commit(&acc_full[u & 1]);
        ++u;
      }
      // every MMA must have completed before TMEM is released: wait until the
      // epilogue has read the last two uses
      if (ok) {
        for (int uu = max(0, u - 2); uu < u; ++uu)
          mbar_wait(&acc_empty[uu & 1], (uint32_t)((uu >> 1) & 1), abort_flag, err, 4);
      } else {
        umma_commit(&acc_full[u & 1]);
        for (uint32_t i = 0; i < WAIT_LIMIT && !mbar_try_wait(&acc_full[u & 1], (uint32_t)((u >> 1) & 1)); ++i) {
        }
      }
    }
  } else {
    // ------------------------------------------- epilogue (warps 2..)
    // warp w reads TMEM lane quarter w % 4; each run of four warps covers
    // all quarters for CW consecutive columns of the tile.
    const int q = warp & 3;
    constexpr int CW = TNS * 4 / EPI_WARPS;
    static_assert(CW == 8, "the drain reads 8 columns per thread and group");
    const int cbase = ((warp - 2) >> 2) * CW;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    const int scale_b = -b * (S + 1);
    int u = 0;
    bool ok = true;
    // The next tile's descriptor is fetched one tile ahead (one word per
    // lane) and handed over through this warp's shared-memory slot, so that
    // its global-load latency hides behind the current tile: short tiles are
    // bound by the epilogue.
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + TILE_SLOTS + (warp - 2) * 64);
    int ti = tile_of(0, cta, G);
    uint32_t tw = (ti < ntiles && lane < TILE_WORDS) ? reinterpret_cast<const uint32_t *>(tiles + ti)[lane] : 0u;
    for (int r = 0; ok; ++r) {
      if (ti >= ntiles) break;
      __syncwarp();  // every lane is done with the previous descriptor
      if (lane < TILE_WORDS) tslot[lane] = tw;
      __syncwarp();
      // fields are read from the slot where used (no registers held)
      const SplitTile &T = *reinterpret_cast<const SplitTile *>(tslot);
      ti = tile_of(r + 1, cta, G);
      tw = (ti < ntiles && lane < TILE_WORDS) ? reinterpret_cast<const uint32_t *>(tiles + ti)[lane] : 0u;
      const int i_glob = T.mt * TMS + q * 32 + lane;
      const bool rv = i_glob < T.Mr;
      // the row exponent is fetched now so that its load latency hides behind
      // the accumulation; the column exponents (broadcast loads) are read at
      // the stores, which keeps the drain's registers below the 96 a thread
      // of this launch has
      const int j0 = T.nt * TNS + cbase;
      const int Ei = rv ? E[T.eoff + i_glob] : 0;
      const int rsh = T.rshift;
      unsigned long long Vl[CW];
      unsigned int Vh[CW];
#pragma unroll
      for (int jj = 0; jj < CW; ++jj) {
        Vl[jj] = 0;
        Vh[jj] = 0;
      }
      for (int ch = 0; ch < T.nchunk; ++ch, ++u) {
        // one lane polls; the warp proceeds together (tcgen05.ld is .aligned)
        int w = 1;
        if (lane == 0) w = mbar_wait(&acc_full[u & 1], (uint32_t)((u >> 1) & 1), abort_flag, err, 5) ? 1 : 0;
        w = __shfl_sync(0xffffffffu, w, 0);
        if (!w) { ok = false; break; }
        tc_fence_after();
        const uint32_t set_base = lane_base + (uint32_t)((u & 1) * SET_COLS);
        // the groups' columns are in flight together (one wait per batch of up
        // to six): the drain is bound by TMEM load latency otherwise
        if constexpr (S <= 6) {
          fold_groups<S, 0, S>(set_base, cbase, b, rsh, Vl, Vh);
        } else {
          fold_groups<S, 0, 4>(set_base, cbase, b, rsh, Vl, Vh);
          fold_groups<S, 4, S - 4>(set_base, cbase, b, rsh, Vl, Vh);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[u & 1]);
      }
      if (!ok) break;
      if (rv) {
        const int rsplit = T.splits & 1, csplit = T.splits >> 1;
        double *crow = C + T.c_off + (int64_t)(i_glob >> rsplit) * T.rs + (i_glob & rsplit);
#pragma unroll
        for (int jj = 0; jj < CW; ++jj) {
          const int j = j0 + jj;
          if (j < T.N) {
            const long long V = (long long)(((unsigned long long)Vh[jj] << 32) + Vl[jj]);
            crow[(int64_t)(j >> csplit) * T.ldc + (j & csplit)] =
                fixed_to_double(V, Ei + F[T.foff + j] + rsh + scale_b);
          }
        }
      }
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
  return std::max(1, std::min(n, MAX_STAGES));
}

template <int S>
void launch_split_s(Ctx *ctx, bool cplx, const SplitPair *d_pairs, const OperandView *d_va, const OperandView *d_vb,
                    const int4 *d_sa, int nsa, const int4 *d_sb, int nsb, const SplitTile *d_tiles, int ntiles,
                    const double *A, const double *B, double *C, int *dE, int *dF, uint8_t *arena, int b,
                    int kchunk, int *err, bool may_fork) {
  if (b < 5 || b > 8 || b * S > 62) fail(QS_ERR_INTERNAL, "split: unsupported digit plan b=%d S=%d", b, S);
  cudaStream_t st = ctx->stream;
  ctx->mark(0);
  // the two roles' strips are independent: the B role runs on the
  // context's second stream beside the A role, so that neither launch's
  // last partial wave leaves SMs idle; the GEMM waits for both (not on the
  // allocation-free path, which creates no stream)
  const bool fork = may_fork && nsa && nsb;
  cudaStream_t sb = st;
  if (fork) {
    ctx->ensure_aux();
    QS_CUDA(cudaEventRecord(ctx->aux_fork, st));
    QS_CUDA(cudaStreamWaitEvent(ctx->aux, ctx->aux_fork, 0));
    sb = ctx->aux;
  }
  auto strips = [&](auto cx) {
    constexpr bool CX = decltype(cx)::value;
    if (nsb) {
      if (d_vb) strip_b_kernel<CX, S, true><<<nsb, STRIP_THREADS, 0, sb>>>(d_pairs, d_vb, d_sb, A, B, dF, arena, b);
      else strip_b_kernel<CX, S, false><<<nsb, STRIP_THREADS, 0, sb>>>(d_pairs, nullptr, d_sb, A, B, dF, arena, b);
      QS_LAUNCHED(ctx);
    }
    if (nsa) {
      if (d_va) strip_a_kernel<CX, S, true><<<nsa, STRIP_THREADS, 0, st>>>(d_pairs, d_va, d_sa, A, B, dE, arena, b);
      else strip_a_kernel<CX, S, false><<<nsa, STRIP_THREADS, 0, st>>>(d_pairs, nullptr, d_sa, A, B, dE, arena, b);
      QS_LAUNCHED(ctx);
    }
  };
  if (cplx) strips(std::true_type{});
  else strips(std::false_type{});
  if (fork) {
    QS_CUDA(cudaEventRecord(ctx->aux_join, ctx->aux));
    QS_CUDA(cudaStreamWaitEvent(st, ctx->aux_join, 0));
  }
  const int nst = pick_stages<S>();
  const size_t sm = smem_bytes<S>(nst);
  QS_CUDA(cudaFuncSetAttribute(gemm_split_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  ctx->mark(1);
  const int grid = std::min(ntiles, std::max(ctx->num_sms, 1));
  gemm_split_kernel<S><<<grid, GEMM_THREADS, sm, st>>>(d_tiles, ntiles, d_pairs, arena, dE, dF, C, b, nst, kchunk,
                                              err);
  QS_LAUNCHED(ctx);
  ctx->mark(2);
}

}  // namespace


// ---------------------------------------------------------------- host side
// Largest summed (real) depth that keeps every accumulator group exact:
// |sum_{t+u=g} d_t d'_u| <= 2^(2b) (1 + max(0, g-1)/4) per term.
static int kchunk_of(int b, int S) {
  const double grow = std::max(1.0, 1.0 + (S - 2) / 4.0);
  const double kc = std::floor(16777216.0 / (std::ldexp(1.0, 2 * b) * grow));
  return (int)std::min(kc, 1.0e9);
}

// Accumulator drains of one output block: a new chunk starts when the next K
// block would push the chunk's summed depth above kchunk (the MMA issuer
// applies the same rule).
static int chunks_of(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1, int cm, int kchunk) {
  int nchunk = 1, depth = 0;
  bool fresh = true;
  for (int64_t p = p0; p < p1; ++p) {
    const int Kr = pairs[p].K * cm;
    const int KB = std::max(1, (Kr + TKS - 1) / TKS);
    for (int kb = 0; kb < KB; ++kb) {
      const int dk = std::max(std::min(TKS, Kr - kb * TKS), 0);
      if (!fresh && depth + dk > kchunk) { ++nchunk; depth = 0; fresh = true; }
      depth += dk;
      fresh = false;
    }
  }
  return nchunk;
}

// Digit plan: the (bits, digits) pair that reaches the wanted precision at
// the lowest modelled cost over the actual tiles -- tensor work grows as
// S(S+1)/2 per K block, and each accumulator drain costs about as much as
// DRAIN_UNITS single-digit K blocks (small: with two accumulator sets the
// drain overlaps the next chunk's products).  QS_SPLIT_DRAIN_UNITS and
// QS_SPLIT_BITS override the model for tuning.
static double drain_units() {
  const char *e = std::getenv("QS_SPLIT_DRAIN_UNITS");
  return e ? std::atof(e) : 12.0;
}

DigitPlan choose_digits_for(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                            const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N, int cm,
                            double tol, int forced_slices, int forced_bits) {
  if (!(tol > 0)) tol = 1e-12;
  // bits of precision wanted: the tolerance plus a margin for the growth of
  // the error with the summed depth relative to |C|.
  const int need = (int)std::ceil(-std::log2(tol)) + 8;
  DigitPlan best{0, 0, 0};
  double best_cost = 1e300;
  const int64_t nb = (int64_t)blk_M.size();
  const double DRAIN_UNITS = drain_units();
  const char *fb = std::getenv("QS_SPLIT_BITS");
  int bhi = fb ? std::atoi(fb) : 8, blo = fb ? std::atoi(fb) : 5;
  if (forced_bits > 0) bhi = blo = forced_bits;
  for (int b = bhi; b >= blo; --b) {
    int S = forced_slices > 0 ? forced_slices : (need - 1 + b - 1) / b;
    S = std::max(S, 2);
    if (S > 8 || b * S > 62) continue;
    const int kchunk = kchunk_of(b, S);
    if (kchunk < TKS) continue;
    double cost = 0;
    for (int64_t g = 0; g < nb; ++g) {
      const double tiles = double((blk_M[g] * cm + TMS - 1) / TMS) * double((blk_N[g] + TNS - 1) / TNS);
      double kbs = 0;
      for (int64_t p = grp[g]; p < grp[g + 1]; ++p) kbs += std::max(1, (pairs[p].K * cm + TKS - 1) / TKS);
      cost += tiles * (S * (S + 1) / 2.0 * kbs + DRAIN_UNITS * chunks_of(pairs, grp[g], grp[g + 1], cm, kchunk));
    }
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

DigitPlan choose_digits(int64_t kreal, double tol, int forced_slices) {
  std::vector<PairDesc> one(1);
  one[0].M = TMS;
  one[0].N = TNS;
  one[0].K = (int32_t)std::max<int64_t>(kreal, 1);
  return choose_digits_for(one, {0, 1}, {TMS}, {TNS}, 1, tol, forced_slices);
}

// Host-side work lists of one planned split product.
struct SplitWork {
  int S = 0, b = 0, kchunk = 0;
  int64_t nE = 0, nF = 0, arena = 0;
  std::vector<SplitPair> sp;
  // strips of STRIP real lines: (first pair, end pair, first line, 0) of the
  // A role (rows of op(A~)) and of the B role (columns of op(B~))
  std::vector<int4> sa, sb;
  std::vector<SplitTile> tiles;
  // strided views of the A and B roles per pair (empty: none)
  std::vector<OperandView> va, vb;
};

// Their device copies, the exponent arrays and the digit arena.
struct SplitDev {
  SplitPair *pairs = nullptr;
  int4 *sa = nullptr, *sb = nullptr;
  SplitTile *tiles = nullptr;
  OperandView *va = nullptr, *vb = nullptr;
  int *E = nullptr, *F = nullptr;
  uint8_t *arena = nullptr;
};

// Host half of the split path: digit plan, per-pair digit geometry and arena
// offsets, and the device work lists (exponent lines, slicing tiles, output
// tiles in launch order).
// Layout of each output block: computed as C or as C^T = op(B)^T op(A)^T,
// and for complex blocks with the real form duplicating A (A~ is 2M x 2K) or
// B (B' is 2K x 2N; see SplitPair), whichever is estimated cheapest (a layout
// other than the plain one must be at least 3 % cheaper).  The estimate per
// k-block of the block's pairs, in bytes of slicing traffic: 26900 per
// 128 x 32 output tile (GEMM), plus the digit bytes the slicing writes for
// the A role (128-row tiles, 48 KB at six digits) and for the B role
// (32-column tiles, 12 KB, weighted 0.86) -- fitted to GB300 timings of the
// split GEMM (5.65 ns per tile and k-block) and of the slicing kernels (0.21
// and 0.18 ps per byte).  A swapped pair exchanges the roles and storage of
// its operands: A' = op(B)^T reads B's storage (transposed unless op(B) was),
// B' = op(A)^T reads A's, with the conjugation flags exchanged; the tiles
// store C^T transposed.  Returns per block bit 0 = swapped, bit 1 = B
// duplicated.
static std::vector<uint8_t> orient_blocks(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                                          std::vector<int32_t> &bM, std::vector<int32_t> &bN, int cm,
                                          std::vector<PairDesc> &tp) {
  const int64_t nb = (int64_t)bM.size();
  std::vector<uint8_t> mode(nb, 0);
  bool any = false;
  // rows of the A role and columns of the B role, real form
  auto cost = [&](int64_t rows, int64_t cols) {
    const double mt = double((rows + TMS - 1) / TMS), nt = double((cols + TNS - 1) / TNS);
    return 26900.0 * mt * nt + 49152.0 * mt + 10530.0 * nt;
  };
  for (int64_t g = 0; g < nb; ++g) {
    const int64_t m = bM[g], n = bN[g];
    double c[4] = {cost(m * cm, n), cost(n * cm, m), 1e300, 1e300};
    if (cm == 2) {
      c[2] = cost(m, 2 * n);
      c[3] = cost(n, 2 * m);
    }
    int best = 0;
    for (int o = 1; o < 4; ++o)
      if (c[o] < c[best]) best = o;
    if (c[best] >= 0.97 * c[0]) best = 0;
    // bit 0: swapped (layouts 1 and 3), bit 1: B duplicated (layouts 2 and 3)
    mode[g] = (uint8_t)(((best & 1) ? 1 : 0) | (best >= 2 ? 2 : 0));
    if (mode[g] & 1) any = true;
  }
  if (!any) return mode;
  tp = pairs;
  for (int64_t g = 0; g < nb; ++g) {
    if (!(mode[g] & 1)) continue;
    std::swap(bM[g], bN[g]);
    for (int64_t p = grp[g]; p < grp[g + 1]; ++p) {
      PairDesc &d = tp[p];
      const int t = d.trans;
      std::swap(d.M, d.N);
      std::swap(d.a_off, d.b_off);
      std::swap(d.lda, d.ldb);
      d.trans = ((t & 2) ? 0 : 1) | ((t & 1) ? 0 : 2) | ((t & 8) ? 4 : 0) | ((t & 4) ? 8 : 0);
    }
  }
  return mode;
}

static SplitResult plan_split(const std::vector<PairDesc> &pairs_in, const std::vector<int64_t> &grp,
                              const std::vector<int32_t> &blk_M_in, const std::vector<int32_t> &blk_N_in,
                              const std::vector<int64_t> &c_off, bool cplx, int forced_slices, double tol,
                              const std::vector<int32_t> *blk_ldc, SplitWork &w, int forced_bits = 0,
                              const std::vector<OperandView> *va = nullptr,
                              const std::vector<OperandView> *vb = nullptr) {
  SplitResult res;
  const int64_t nb = (int64_t)blk_M_in.size();
  const int cm = cplx ? 2 : 1;
  std::vector<int32_t> blk_M = blk_M_in, blk_N = blk_N_in;
  std::vector<PairDesc> swapped_pairs;
  const std::vector<uint8_t> mode = orient_blocks(pairs_in, grp, blk_M, blk_N, cm, swapped_pairs);
  const std::vector<PairDesc> &pairs = swapped_pairs.empty() ? pairs_in : swapped_pairs;
  // strided operand views follow their operands into the roles: a block
  // computed as C^T reads op(B)^T in the A role and op(A)^T in the B role,
  // whose lines are B's columns resp. A's rows -- the same views, exchanged
  if ((va && !va->empty()) || (vb && !vb->empty())) {
    const OperandView none{};
    w.va.assign(pairs.size(), none);
    w.vb.assign(pairs.size(), none);
    for (int64_t g = 0; g < nb; ++g)
      for (int64_t p = grp[g]; p < grp[g + 1]; ++p) {
        const OperandView x = (va && !va->empty()) ? (*va)[p] : none, y = (vb && !vb->empty()) ? (*vb)[p] : none;
        if (mode[g] & 1) {
          w.va[p] = y;
          w.vb[p] = x;
        } else {
          w.va[p] = x;
          w.vb[p] = y;
        }
      }
  }
  DigitPlan dp = choose_digits_for(pairs, grp, blk_M, blk_N, cm, tol, forced_slices, forced_bits);
  const int S = dp.nslices, b = dp.bits;
  const int kchunk = kchunk_of(b, S);
  w.S = S;
  w.b = b;
  w.kchunk = kchunk;
  res.nslices = S;
  res.bits = b;
  res.err_bound = dp.err_bound;

  // per-pair digit geometry and arena offsets
  std::vector<SplitPair> &sp = w.sp;
  sp.resize(pairs.size());
  std::vector<int64_t> eoff(nb), foff(nb);
  int64_t &nE = w.nE, &nF = w.nF;
  nE = nF = 0;
  // real rows of the A role and real columns of the B role per block
  std::vector<int64_t> rows_r(nb), cols_r(nb);
  for (int64_t g = 0; g < nb; ++g) {
    const bool dupb = mode[g] & 2;
    rows_r[g] = (int64_t)blk_M[g] * (dupb ? 1 : cm);
    cols_r[g] = (int64_t)blk_N[g] * (dupb ? 2 : 1);
    eoff[g] = nE;
    foff[g] = nF;
    nE += rows_r[g];
    nF += cols_r[g];
  }
  if (nE > INT32_MAX || nF > INT32_MAX) fail(QS_ERR_SHAPE, "split: exponent arrays too large");
  int64_t &arena = w.arena;
  arena = 0;
  std::vector<int4> &sa = w.sa, &sb = w.sb;
  std::vector<SplitTile> &tiles = w.tiles;
  for (int64_t g = 0; g < nb; ++g) {
    // every pair's CG factor is folded into its A digits (exact integer
    // product), so the pairs of a block share the accumulators
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
      s.dupb = (mode[g] & 2) ? 1 : 0;
      s.Mr = d.M * (s.dupb ? 1 : cm);
      s.Nr = d.N * (s.dupb ? 2 : 1);
      s.Kr = d.K * cm;
      s.MT = (s.Mr + TMS - 1) / TMS;
      s.NT = (s.Nr + TNS - 1) / TNS;
      s.KB = std::max(1, (s.Kr + TKS - 1) / TKS);
      s.eoff = (int32_t)eoff[g];
      s.foff = (int32_t)foff[g];
      const Factor f = make_factor(d.afac);
      s.fm = f.fm;
      s.fe = f.fe;
      s.fneg = f.neg ? 1 : 0;
      int e = 0;
      if (d.afac != 1.0 && d.afac != 0.0) std::frexp(d.afac, &e);
      s.e_afac = e;
      s.swap = mode[g] & 1;
      s.as_off = arena;
      arena += (int64_t)s.MT * s.KB * S * A_DIGIT_BYTES;
      s.bs_off = arena;
      arena += (int64_t)s.NT * s.KB * S * B_DIGIT_BYTES;
    }
    // exponent + slicing strips over all pairs of the block
    if (grp[g + 1] > grp[g]) {
      for (int64_t r0 = 0; r0 < rows_r[g]; r0 += STRIP)
        sa.push_back(make_int4((int)grp[g], (int)grp[g + 1], (int)r0, 0));
      for (int64_t c0 = 0; c0 < cols_r[g]; c0 += STRIP)
        sb.push_back(make_int4((int)grp[g], (int)grp[g + 1], (int)c0, 0));
    }
    const int nchunk = chunks_of(pairs, grp[g], grp[g + 1], cm, kchunk);
    // int64 headroom of the fixed-point sum over all chunks:
    // nchunk * 2^(24.2 + b(S-1) - r) < 2^63
    int lg = 0;
    while ((1 << lg) < nchunk) ++lg;
    int rshift = std::max(0, 25 + b * (S - 1) + lg - 63);
    // the epilogue adds each group with a shift of at most 30 into its low
    // 64-bit word or of at least 32 into its high 32-bit word: no group may
    // land exactly on bit 31
    for (int t = 0; t < S; ++t)
      if (b * (S - 1 - t) - rshift == 31) ++rshift;
    const int MT = (int)((rows_r[g] + TMS - 1) / TMS), NT = (int)((cols_r[g] + TNS - 1) / TNS);
    for (int nt = 0; nt < NT; ++nt)
      for (int mt = 0; mt < MT; ++mt) {
        SplitTile t{};
        t.c_off = c_off[g] * cm;
        t.p0 = (int32_t)grp[g];
        t.p1 = (int32_t)grp[g + 1];
        t.mt = mt;
        t.nt = nt;
        t.Mr = (int32_t)rows_r[g];
        t.N = (int32_t)cols_r[g];
        // column stride of C in its elements, in the caller's orientation
        const int64_t ldc0 = blk_ldc ? (*blk_ldc)[g] : std::max(blk_M_in[g], 1);
        const bool swp = mode[g] & 1, dupb = mode[g] & 2;
        if (!swp && !dupb) {
          t.ldc = (int32_t)(ldc0 * cm);
          t.rs = 1;
          t.splits = 0;
        } else if (!dupb && cm == 1) {
          t.ldc = 1;
          t.rs = (int32_t)ldc0;
          t.splits = 0;
        } else if (!dupb) {
          t.ldc = 2;
          t.rs = (int32_t)(2 * ldc0);
          t.splits = 1;
        } else if (!swp) {
          // C' = M x 2N: row m at 2m, column j at (j/2) of C's columns, part j%2
          t.rs = 2;
          t.ldc = (int32_t)(2 * ldc0);
          t.splits = 2;
        } else {
          // C'^T = N x 2M: row n at column n of C, column j = element j of the
          // interleaved (Re, Im) column
          t.rs = (int32_t)(2 * ldc0);
          t.ldc = 1;
          t.splits = 0;
        }
        t.eoff = (int32_t)eoff[g];
        t.foff = (int32_t)foff[g];
        t.nchunk = nchunk;
        t.rshift = rshift;
        tiles.push_back(t);
      }
  }
  // Longest tiles first (by summed depth): the tail of the launch is short.
  // The depth is a property of the tile's block: summed once per block, then
  // a stable sort of the tiles by it.
  {
    std::vector<int64_t> depth(tiles.size());
    for (size_t t = 0; t < tiles.size(); ++t) {
      if (t > 0 && tiles[t].p0 == tiles[t - 1].p0 && tiles[t].p1 == tiles[t - 1].p1) {
        depth[t] = depth[t - 1];
        continue;
      }
      int64_t k = 0;
      for (int p = tiles[t].p0; p < tiles[t].p1; ++p) k += sp[p].KB;
      depth[t] = k;
    }
    std::vector<int64_t> order(tiles.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return depth[x] > depth[y]; });
    std::vector<SplitTile> sorted(tiles.size());
    for (size_t t = 0; t < tiles.size(); ++t) sorted[t] = tiles[order[t]];
    tiles.swap(sorted);
  }
  if (tiles.empty()) return res;
  if (tiles.size() > 0x7fffffff || sa.size() > 0x7fffffff || sb.size() > 0x7fffffff)
    fail(QS_ERR_SHAPE, "split: launch too large");
  res.slice_bytes = arena;
  res.ntiles = (int64_t)tiles.size();

  return res;
}

// Device half: launches the exponent, slicing and GEMM kernels of a planned
// split product on the context's stream, with every work list, exponent
// array and the digit arena already on the device.
static void launch_split(Ctx *ctx, const SplitWork &w, bool cplx, const SplitDev &d, const double *A,
                         const double *B, double *C, int *err, bool may_fork = true) {
  switch (w.S) {
#define QS_CASE(SS)                                                                                      \
  case SS:                                                                                               \
    launch_split_s<SS>(ctx, cplx, d.pairs, d.va, d.vb, d.sa, (int)w.sa.size(), d.sb, (int)w.sb.size(),    \
                       d.tiles, (int)w.tiles.size(), A, B, C, d.E, d.F, d.arena, w.b, w.kchunk, err,     \
                       may_fork);                                                                        \
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
      fail(QS_ERR_INTERNAL, "split: unsupported digit count %d", w.S);
  }
}

static SplitResult run_split_lists(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                                   const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                                   const std::vector<int64_t> &c_off, const double *A, const double *B, double *C,
                                   bool cplx, int forced_slices, double tol, const std::vector<int32_t> *blk_ldc,
                                   int forced_bits, const std::vector<OperandView> *va,
                                   const std::vector<OperandView> *vb);

// Shallow output blocks (summed depth <= SHALLOW_K) are computed directly in
// FP64 (run_shallow); deep ones (few tiles, a very deep sum) are cut along
// their depth into parts computed as blocks of their own in a temporary
// buffer and summed in part order (split_deep).  Both decisions depend on the
// block alone, and the digit plan is the one of the list as given, so a
// block gives the same bits whatever else is in the launch.  Blocks with a
// pair read through a view run as they are.
SplitResult run_split(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                      const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                      const std::vector<int64_t> &c_off, const double *A, const double *B, double *C,
                      bool cplx, int forced_slices, double tol, const std::vector<int32_t> *blk_ldc,
                      int forced_bits, const std::vector<OperandView> *va,
                      const std::vector<OperandView> *vb) {
  const size_t nb = blk_M.size();
  const int64_t eb = cplx ? 16 : 8;
  // blocks with a pair read through a view stay as they are
  std::vector<char> keep;
  if (va || vb) {
    keep.assign(nb, 0);
    for (size_t g = 0; g < nb; ++g)
      for (int64_t p = grp[g]; p < grp[g + 1]; ++p)
        if ((va && (*va)[p].nl > 0) || (vb && (*vb)[p].nl > 0)) keep[g] = 1;
  }
  std::vector<char> shallow(nb, 0), rest(nb, 1);
  std::vector<int64_t> shallow_ids;
  for (size_t g = 0; g < nb; ++g)
    if (!(keep.size() && keep[g]) && is_shallow(pairs, grp[g], grp[g + 1]) &&
        shallow_direct_wins(pairs, grp[g], grp[g + 1], blk_M[g], blk_N[g], cplx)) {
      shallow[g] = 1;
      rest[g] = 0;
      shallow_ids.push_back((int64_t)g);
    }
  if (!shallow_ids.empty()) {
    const DigitPlan dp = choose_digits_for(pairs, grp, blk_M, blk_N, cplx ? 2 : 1, tol, forced_slices, forced_bits);
    run_shallow(ctx, pairs, grp, blk_M, blk_N, c_off, blk_ldc, shallow_ids, A, B, C, cplx);
    SplitResult res;
    res.nslices = dp.nslices;
    res.bits = dp.bits;
    res.err_bound = dp.err_bound;
    if (shallow_ids.size() == nb) return res;
    const BlockList R = select_blocks(pairs, grp, blk_M, blk_N, c_off, blk_ldc, rest);
    std::vector<OperandView> va2, vb2;
    for (int32_t q : R.src) {
      if (va) va2.push_back((*va)[q]);
      if (vb) vb2.push_back((*vb)[q]);
    }
    SplitResult r2 = run_split(ctx, R.pairs, R.grp, R.bM, R.bN, R.coff, A, B, C, cplx, dp.nslices, tol, &R.bldc,
                               dp.bits, va ? &va2 : nullptr, vb ? &vb2 : nullptr);
    return r2.nslices ? r2 : res;
  }
  DeepSplit ds;
  if (reinterpret_cast<uintptr_t>(C) % eb == 0 &&
      split_deep(pairs, grp, blk_M, blk_N, c_off, blk_ldc, ds, keep.empty() ? nullptr : &keep)) {
    const DigitPlan dp = choose_digits_for(pairs, grp, blk_M, blk_N, cplx ? 2 : 1, tol, forced_slices, forced_bits);
    double *T = dev_alloc<double>(ctx, (size_t)std::max<int64_t>(ds.temp_elems, 1) * (cplx ? 2 : 1));
    DeepReduce *d_red = nullptr;
    // the views follow their pairs (pairs of cut blocks have none)
    std::vector<OperandView> va2, vb2;
    for (int32_t q : ds.src) {
      if (va) va2.push_back((*va)[q]);
      if (vb) vb2.push_back((*vb)[q]);
    }
    try {
      ds.place((int64_t)(reinterpret_cast<intptr_t>(T) - reinterpret_cast<intptr_t>(C)) / eb);
      d_red = dev_upload(ctx, ds.red);
      // parts with a few outputs: one CTA per output element in FP64
      // (run_dot; the tiles would compute 4096 outputs for each); the rest
      // through the split path
      std::vector<char> sel(ds.bM.size(), 1);
      std::vector<int64_t> small;
      for (size_t g = 0; g < ds.bM.size(); ++g)
        if (ds.part[g] && (int64_t)ds.bM[g] * ds.bN[g] <= DOT_OUTPUTS) {
          sel[g] = 0;
          small.push_back((int64_t)g);
        }
      run_dot(ctx, ds.pairs, ds.grp, ds.bM, ds.bN, ds.coff, &ds.bldc, small, A, B, C, cplx);
      SplitResult res;
      res.nslices = dp.nslices;
      res.bits = dp.bits;
      res.err_bound = dp.err_bound;
      if (small.size() < ds.bM.size()) {
        const BlockList R = select_blocks(ds.pairs, ds.grp, ds.bM, ds.bN, ds.coff, &ds.bldc, sel);
        std::vector<OperandView> va3, vb3;
        for (int32_t q : R.src) {
          if (va) va3.push_back(va2[q]);
          if (vb) vb3.push_back(vb2[q]);
        }
        res = run_split_lists(ctx, R.pairs, R.grp, R.bM, R.bN, R.coff, A, B, C, cplx, dp.nslices, tol, &R.bldc,
                              dp.bits, va ? &va3 : nullptr, vb ? &vb3 : nullptr);
      }
      launch_reduce_parts(ctx, d_red, (int64_t)ds.red.size(), T, C, cplx);
      dev_free(ctx, d_red);
      dev_free(ctx, T);
      return res;
    } catch (...) {
      cudaStreamSynchronize(ctx->stream);
      if (d_red) dev_free(ctx, d_red);
      dev_free(ctx, T);
      throw;
    }
  }
  return run_split_lists(ctx, pairs, grp, blk_M, blk_N, c_off, A, B, C, cplx, forced_slices, tol, blk_ldc,
                         forced_bits, va, vb);
}

static SplitResult run_split_lists(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                                   const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                                   const std::vector<int64_t> &c_off, const double *A, const double *B, double *C,
                                   bool cplx, int forced_slices, double tol, const std::vector<int32_t> *blk_ldc,
                                   int forced_bits, const std::vector<OperandView> *va,
                                   const std::vector<OperandView> *vb) {
  SplitWork w;
  SplitResult res = plan_split(pairs, grp, blk_M, blk_N, c_off, cplx, forced_slices, tol, blk_ldc, w, forced_bits,
                               va, vb);
  if (w.tiles.empty()) return res;
  // device buffers: one allocation for the digit arena (pooled scratch)
  SplitDev d;
  d.arena = static_cast<uint8_t *>(ctx->ensure_scratch((size_t)std::max<int64_t>(w.arena, 256)));
  d.pairs = dev_upload(ctx, w.sp);
  d.sa = dev_upload(ctx, w.sa);
  d.sb = dev_upload(ctx, w.sb);
  d.tiles = dev_upload(ctx, w.tiles);
  if (!w.va.empty()) {
    d.va = dev_upload(ctx, w.va);
    d.vb = dev_upload(ctx, w.vb);
  }
  d.E = dev_alloc<int>(ctx, (size_t)w.nE);
  d.F = dev_alloc<int>(ctx, (size_t)w.nF);
  launch_split(ctx, w, cplx, d, A, B, C, ctx->d_err);
  dev_free(ctx, d.pairs);
  dev_free(ctx, d.sa);
  dev_free(ctx, d.sb);
  if (d.va) dev_free(ctx, d.va);
  if (d.vb) dev_free(ctx, d.vb);
  dev_free(ctx, d.tiles);
  dev_free(ctx, d.E);
  dev_free(ctx, d.F);
  return res;
}

SplitResult run_split_static(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                             const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                             const std::vector<int64_t> &c_off, const double *A, const double *B, double *C,
                             bool cplx, int forced_slices, double tol, const std::vector<int32_t> *blk_ldc,
                             uint8_t *scratch, size_t cap, int *err) {
  SplitWork w;
  SplitResult res = plan_split(pairs, grp, blk_M, blk_N, c_off, cplx, forced_slices, tol, blk_ldc, w);
  if (w.tiles.empty()) return res;
  size_t used = 0;
  auto take = [&](size_t bytes) {
    const size_t o = used;
    used += (std::max<size_t>(bytes, 1) + 255) / 256 * 256;
    return o;
  };
  const size_t o_pairs = take(w.sp.size() * sizeof(SplitPair));
  const size_t o_sa = take(w.sa.size() * sizeof(int4)), o_sb = take(w.sb.size() * sizeof(int4));
  const size_t o_tiles = take(w.tiles.size() * sizeof(SplitTile));
  const size_t o_E = take((size_t)w.nE * sizeof(int)), o_F = take((size_t)w.nF * sizeof(int));
  const size_t o_arena = take((size_t)w.arena);
  if (used > cap)
    fail(QS_ERR_OOM, "split (static scratch): this pair list needs %zu bytes of scratch (%lld of them "
         "BF16 digits), more than the %zu available", used, (long long)w.arena, cap);
  SplitDev d;
  d.pairs = reinterpret_cast<SplitPair *>(scratch + o_pairs);
  d.sa = reinterpret_cast<int4 *>(scratch + o_sa);
  d.sb = reinterpret_cast<int4 *>(scratch + o_sb);
  d.tiles = reinterpret_cast<SplitTile *>(scratch + o_tiles);
  d.E = reinterpret_cast<int *>(scratch + o_E);
  d.F = reinterpret_cast<int *>(scratch + o_F);
  d.arena = scratch + o_arena;
  auto put = [&](void *dst, const void *src, size_t bytes) {
    if (bytes) QS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  };
  put(d.pairs, w.sp.data(), w.sp.size() * sizeof(SplitPair));
  put(d.sa, w.sa.data(), w.sa.size() * sizeof(int4));
  put(d.sb, w.sb.data(), w.sb.size() * sizeof(int4));
  put(d.tiles, w.tiles.data(), w.tiles.size() * sizeof(SplitTile));
  launch_split(ctx, w, cplx, d, A, B, C, err, false);
  // the work lists are copied from pageable host memory, which the GPU may
  // read when the copies execute rather than when they are queued: keep them
  // alive until then
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  return res;
}

// Digit widths b whose plan meets `tol` (with `forced_slices` digits when
// that is set): the candidates an autotuner times.
std::vector<int> split_candidate_bits(double tol, int forced_slices) {
  if (!(tol > 0)) tol = 1e-12;
  const int need = (int)std::ceil(-std::log2(tol)) + 8;
  std::vector<int> out;
  for (int b = 8; b >= 5; --b) {
    int S = forced_slices > 0 ? forced_slices : (need - 1 + b - 1) / b;
    S = std::max(S, 2);
    if (S > 8 || b * S > 62 || kchunk_of(b, S) < TKS) continue;
    out.push_back(b);
  }
  return out;
}

// A planned split product that can be launched many times: its work lists,
// exponent arrays and digit arena are plain device allocations owned by the
// handle, so their addresses stay fixed (a CUDA graph can replay the launch).
struct SplitPlanHandle {
  SplitWork w;
  SplitDev d;
  bool cplx = false;
  SplitResult res;
  std::vector<void *> owned;
};

SplitPlanHandle *split_plan_create(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                                   const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                                   const std::vector<int64_t> &c_off, const std::vector<int32_t> &blk_ldc,
                                   bool cplx, int forced_slices, double tol, int bits, SplitResult *res) {
  std::unique_ptr<SplitPlanHandle> h(new SplitPlanHandle);
  h->cplx = cplx;
  h->res = plan_split(pairs, grp, blk_M, blk_N, c_off, cplx, forced_slices, tol, &blk_ldc, h->w, bits);
  if (res) *res = h->res;
  if (h->w.tiles.empty()) return h.release();
  try {
    auto own = [&](size_t bytes) -> void * {
      void *p = nullptr;
      cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
      if (e != cudaSuccess)
        fail(e == cudaErrorMemoryAllocation ? QS_ERR_OOM : QS_ERR_CUDA, "split plan: cudaMalloc(%zu): %s", bytes,
             cudaGetErrorString(e));
      h->owned.push_back(p);
      return p;
    };
    auto put = [&](const auto &v) {
      using T = typename std::decay_t<decltype(v)>::value_type;
      T *p = static_cast<T *>(own(v.size() * sizeof(T)));
      if (!v.empty()) QS_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
      return p;
    };
    SplitDev &d = h->d;
    d.pairs = put(h->w.sp);
    d.sa = put(h->w.sa);
    d.sb = put(h->w.sb);
    d.tiles = put(h->w.tiles);
    d.E = static_cast<int *>(own((size_t)h->w.nE * sizeof(int)));
    d.F = static_cast<int *>(own((size_t)h->w.nF * sizeof(int)));
    d.arena = static_cast<uint8_t *>(own((size_t)h->w.arena));
  } catch (...) {
    for (void *p : h->owned) cudaFree(p);
    throw;
  }
  return h.release();
}

void split_plan_launch(Ctx *ctx, SplitPlanHandle *h, const double *A, const double *B, double *C) {
  if (!h->w.tiles.empty()) launch_split(ctx, h->w, h->cplx, h->d, A, B, C, ctx->d_err);
}

// The caller makes sure no launch of the handle is still running.
void split_plan_destroy(SplitPlanHandle *h) {
  if (!h) return;
  for (void *p : h->owned) cudaFree(p);
  delete h;
}

}  // namespace qs
