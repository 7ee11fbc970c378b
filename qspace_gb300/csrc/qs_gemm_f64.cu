// Plain FP64 grouped block GEMM: the drop-in numerical path.
//
// Replaces the per-pair dgemm/zgemm of contractDATA_group (Source/
// QSpace_aux.cc:27-355 -> wbarray::contract Source/wbarray.cc:3389-3500 ->
// DZGEMM Source/wbarray_blas.cc:121-213).  One CTA owns one 64x64 tile of one
// output block and sums all block pairs of that block in plan order, so the
// result is deterministic and needs no atomics.  The K loop stages 64xKC
// panels of op(A) and KCx64 panels of op(B) in shared memory (coalesced
// loads in either storage order); each thread accumulates a 4x4 sub-tile in
// registers with FP64 FMAs (GB300's FP64 rate, not memory, bounds this path).
#include <type_traits>

#include "qs_internal.h"

namespace qs {

namespace {
constexpr int TM = 64, TN = 64;

template <bool CPLX>
struct Elem;
template <>
struct Elem<false> {
  using T = double;
  static constexpr int KC = 16;
  __device__ static T zero() { return 0.0; }
  __device__ static T load(const double *p, int64_t i, bool /*conj*/, double f) { return p[i] * f; }
  __device__ static void fma(T &c, T a, T b) { c = ::fma(a, b, c); }
  __device__ static void store(double *p, int64_t i, T v) { p[i] = v; }
};
template <>
struct Elem<true> {
  using T = double2;
  static constexpr int KC = 8;
  __device__ static T zero() { return make_double2(0.0, 0.0); }
  __device__ static T load(const double *p, int64_t i, bool conj, double f) {
    double2 v = reinterpret_cast<const double2 *>(p)[i];
    return make_double2(v.x * f, (conj ? -v.y : v.y) * f);
  }
  __device__ static void fma(T &c, T a, T b) {
    c.x = ::fma(a.x, b.x, c.x);
    c.x = ::fma(-a.y, b.y, c.x);
    c.y = ::fma(a.x, b.y, c.y);
    c.y = ::fma(a.y, b.x, c.y);
  }
  __device__ static void store(double *p, int64_t i, T v) { reinterpret_cast<double2 *>(p)[i] = v; }
};

// One staged K panel into the accumulators, for the NI x NJ leading 16 x 16
// groups of the tile and the first kn of its KC steps (CTA-uniform bounds).
template <class E, int NI, int NJ, int KC>
__device__ __forceinline__ void panel_fma(typename E::T (&acc)[4][4], const typename E::T (*As)[TM + 1],
                                          const typename E::T (*Bs)[TN + 1], int tx, int ty, int kn) {
  using T = typename E::T;
#pragma unroll
  for (int kk = 0; kk < KC; ++kk) {
    if (kk < kn) {
      T a[NI], b[NJ];
#pragma unroll
      for (int i = 0; i < NI; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < NJ; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < NI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j) E::fma(acc[i][j], a[i], b[j]);
    }
  }
}

template <bool CPLX>
__global__ void __launch_bounds__(256)
gemm_f64_kernel(const PairDesc *__restrict__ pairs, const TileDesc *__restrict__ tiles,
                const double *__restrict__ A, const double *__restrict__ B, double *__restrict__ C) {
  using E = Elem<CPLX>;
  using T = typename E::T;
  constexpr int KC = E::KC;
  __shared__ T As[KC][TM + 1];
  __shared__ T Bs[KC][TN + 1];

  const TileDesc t = tiles[blockIdx.x];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int shape = (min(4, (t.M - t.m0 + 15) / 16) - 1) * 4 + (min(4, (t.N - t.n0 + 15) / 16) - 1);

  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = E::zero();

  for (int p = t.p0; p < t.p1; ++p) {
    const PairDesc pd = pairs[p];
    const bool ta = pd.trans & 1, tb = pd.trans & 2;
    const bool ca = pd.trans & 4, cb = pd.trans & 8;
    for (int k0 = 0; k0 < pd.K; k0 += KC) {
      // op(A)(m,k): stored M x K (m fastest) or K x M (k fastest)
#pragma unroll
      for (int e = tid; e < TM * KC; e += 256) {
        int mm, kk;
        if (ta) { kk = e % KC; mm = e / KC; }
        else    { mm = e % TM; kk = e / TM; }
        const int m = t.m0 + mm, k = k0 + kk;
        T v = E::zero();
        if (m < pd.M && k < pd.K)
          v = E::load(A, pd.a_off + (ta ? (int64_t)k + (int64_t)m * pd.lda
                                        : (int64_t)m + (int64_t)k * pd.lda), ca, pd.afac);
        As[kk][mm] = v;
      }
      // op(B)(k,n): stored K x N (k fastest) or N x K (n fastest)
#pragma unroll
      for (int e = tid; e < TN * KC; e += 256) {
        int nn, kk;
        if (tb) { nn = e % TN; kk = e / TN; }
        else    { kk = e % KC; nn = e / KC; }
        const int n = t.n0 + nn, k = k0 + kk;
        T v = E::zero();
        if (n < pd.N && k < pd.K)
          v = E::load(B, pd.b_off + (tb ? (int64_t)n + (int64_t)k * pd.ldb
                                        : (int64_t)k + (int64_t)n * pd.ldb), cb, 1.0);
        Bs[kk][nn] = v;
      }
      __syncthreads();
      // only the 16-row / 16-column groups of the tile that hold outputs
      // of the block, and only the pair's own K steps: the FP64 pipe bounds
      // this kernel, so the padding a 64 x 64 tile carries on small blocks
      // would cost as much as real work
      const int kn = min(KC, pd.K - k0);
      switch (shape) {
        case 0: panel_fma<E, 1, 1, KC>(acc, As, Bs, tx, ty, kn); break;
        case 1: panel_fma<E, 1, 2, KC>(acc, As, Bs, tx, ty, kn); break;
        case 2: panel_fma<E, 1, 3, KC>(acc, As, Bs, tx, ty, kn); break;
        case 3: panel_fma<E, 1, 4, KC>(acc, As, Bs, tx, ty, kn); break;
        case 4: panel_fma<E, 2, 1, KC>(acc, As, Bs, tx, ty, kn); break;
        case 5: panel_fma<E, 2, 2, KC>(acc, As, Bs, tx, ty, kn); break;
        case 6: panel_fma<E, 2, 3, KC>(acc, As, Bs, tx, ty, kn); break;
        case 7: panel_fma<E, 2, 4, KC>(acc, As, Bs, tx, ty, kn); break;
        case 8: panel_fma<E, 3, 1, KC>(acc, As, Bs, tx, ty, kn); break;
        case 9: panel_fma<E, 3, 2, KC>(acc, As, Bs, tx, ty, kn); break;
        case 10: panel_fma<E, 3, 3, KC>(acc, As, Bs, tx, ty, kn); break;
        case 11: panel_fma<E, 3, 4, KC>(acc, As, Bs, tx, ty, kn); break;
        case 12: panel_fma<E, 4, 1, KC>(acc, As, Bs, tx, ty, kn); break;
        case 13: panel_fma<E, 4, 2, KC>(acc, As, Bs, tx, ty, kn); break;
        case 14: panel_fma<E, 4, 3, KC>(acc, As, Bs, tx, ty, kn); break;
        default: panel_fma<E, 4, 4, KC>(acc, As, Bs, tx, ty, kn); break;
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int n = t.n0 + ty + 16 * j;
    if (n >= t.N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int m = t.m0 + tx + 16 * i;
      if (m < t.M) E::store(C, t.c_off + (int64_t)m + (int64_t)n * t.ldc, acc[i][j]);
    }
  }
}
}  // namespace

int gemm_f64_tile_m() { return TM; }
int gemm_f64_tile_n() { return TN; }

void launch_gemm_f64(Ctx *ctx, const PairDesc *d_pairs, const TileDesc *d_tiles,
                     int64_t ntiles, const double *A, const double *B, double *C,
                     int is_complex) {
  if (ntiles <= 0) return;
  if (ntiles > 0x7fffffff) fail(QS_ERR_SHAPE, "gemm_f64: too many tiles");
  ctx->mark(0);
  ctx->mark(1);
  if (is_complex)
    gemm_f64_kernel<true><<<(unsigned)ntiles, 256, 0, ctx->stream>>>(d_pairs, d_tiles, A, B, C);
  else
    gemm_f64_kernel<false><<<(unsigned)ntiles, 256, 0, ctx->stream>>>(d_pairs, d_tiles, A, B, C);
  QS_LAUNCHED(ctx);
  ctx->mark(2);
}

}  // namespace qs
