// Generalised transpose of many blocks (the device counterpart of
// wbperm_helper::permute, Source/wbarray.cc:4453-4600, which QSpace runs per
// block from permute_to / Permute, Source/QSpace.hh:2670-2866).
//
// The host first drops legs of size 1 and merges legs that stay adjacent in
// both orders, so every block is described by its fewest legs.  Two kernels
// then cover all blocks of a call:
//  * permute_tile_kernel -- blocks whose output-fastest leg is not the
//    input-fastest one and where both of those legs span >= 8 elements: a
//    64 x 32 tile of (output-fastest, input-fastest) moves through shared
//    memory, read with lanes along the input's unit stride and written with
//    lanes along the output's, so both sides are full coalesced lines
//    (complex elements are single 16-byte accesses; eight loads in flight
//    per thread).  One CTA per tile; the remaining legs' offsets are decoded
//    once per CTA.
//  * permute_lines_kernel -- every other block (the fastest leg kept in
//    place: contiguous runs on both sides; or short legs): each thread walks
//    output elements in order, four loads in flight; its multi-index
//    advances by the mixed-radix digits of the CTA stride, so the inner loop
//    has no division.  A block that is one contiguous run is a plain copy.
#include <algorithm>

#include "qs_internal.h"

namespace qs {

template <bool CPLX>
struct PermElem {
  using T = double;
};
template <>
struct PermElem<true> {
  using T = double2;
};

__device__ __forceinline__ double perm_conj(double v, int) { return v; }
__device__ __forceinline__ double2 perm_conj(double2 v, int c) { return make_double2(v.x, c ? -v.y : v.y); }

constexpr int PT = 32;       // tile edge along the input's unit-stride leg
constexpr int PTI = 64;      // tile edge along the output's unit-stride leg
constexpr int PT_ROWS = 8;   // warps per tile CTA

template <bool CPLX>
__global__ void __launch_bounds__(PT * PT_ROWS)
permute_tile_kernel(const PermDesc *__restrict__ desc, const PermTile *__restrict__ tiles,
                    const double *__restrict__ in_, double *__restrict__ out_) {
  using T = typename PermElem<CPLX>::T;
  __shared__ T tile[PTI][PT + 1];
  const PermTile w = tiles[blockIdx.x];
  const PermDesc &d = desc[w.desc];
  const T *in = reinterpret_cast<const T *>(in_) + d.in_off;
  T *out = reinterpret_cast<T *>(out_) + d.out_off;
  const int b = d.fast_in_leg;  // output leg that is the input's unit-stride leg
  const int64_t n0 = d.out_dims[0], nb = d.out_dims[b];
  // offsets of the other legs (decoded once per CTA)
  int64_t rem = w.rest, ioff = 0, ooff = 0, ostride = 1, ob = 1;
  for (int k = 0; k < d.rank; ++k) {
    if (k == b) ob = ostride;
    if (k != 0 && k != b) {
      const int64_t j = rem % d.out_dims[k];
      rem /= d.out_dims[k];
      ioff += j * d.in_stride[k];
      ooff += j * ostride;
    }
    ostride *= d.out_dims[k];
  }
  const int64_t s0 = d.in_stride[0];
  const int64_t i0 = (int64_t)w.ti * PTI, j0 = (int64_t)w.tj * PT;
  const int lane = threadIdx.x, row = threadIdx.y;
  // read: lanes along the input's unit-stride leg (output leg b); all eight
  // loads of a thread are issued before the first use
  if (j0 + lane < nb) {
    T v[PTI / PT_ROWS];
#pragma unroll
    for (int u = 0; u < PTI / PT_ROWS; ++u) {
      const int r = row + u * PT_ROWS;
      if (i0 + r < n0) v[u] = in[ioff + (i0 + r) * s0 + j0 + lane];
    }
#pragma unroll
    for (int u = 0; u < PTI / PT_ROWS; ++u) tile[row + u * PT_ROWS][lane] = v[u];
  }
  __syncthreads();
  // write: lanes along the output's unit-stride leg 0, two 32-wide halves
#pragma unroll
  for (int h = 0; h < PTI / PT; ++h) {
    const int il = h * PT + lane;
    if (i0 + il < n0) {
#pragma unroll
      for (int r = row; r < PT; r += PT_ROWS)
        if (j0 + r < nb) out[ooff + (j0 + r) * ob + i0 + il] = perm_conj(tile[il][r], d.conj);
    }
  }
}

template <bool CPLX>
__global__ void __launch_bounds__(256)
permute_lines_kernel(const PermDesc *__restrict__ desc, const int64_t *__restrict__ chunk_blk,
                     const int64_t *__restrict__ chunk_start, int chunk_elems,
                     const double *__restrict__ in_, double *__restrict__ out_) {
  using T = typename PermElem<CPLX>::T;
  constexpr int U = 4;  // elements in flight per thread
  const int64_t c = blockIdx.x;
  const PermDesc &d = desc[chunk_blk[c]];
  const T *in = reinterpret_cast<const T *>(in_) + d.in_off;
  T *out = reinterpret_cast<T *>(out_) + d.out_off;
  const int64_t s0 = chunk_start[c];
  const int64_t s1 = min(d.n, s0 + (int64_t)chunk_elems);
  const int r = d.rank;
  int64_t e = s0 + threadIdx.x;
  if (e >= s1) return;
  if (r == 1 && d.in_stride[0] == 1) {
    // one contiguous run: a plain copy
    for (; e < s1; e += (int64_t)U * blockDim.x) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (e + u * blockDim.x < s1) v[u] = in[e + u * blockDim.x];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (e + u * blockDim.x < s1) out[e + u * blockDim.x] = perm_conj(v[u], d.conj);
    }
    return;
  }
  // multi-index of e and the mixed-radix digits of the step blockDim.x
  int64_t j[8], step[8], src = 0;
  {
    int64_t rem = e, st = blockDim.x;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < r) {
        const int64_t dk = d.out_dims[k];
        j[k] = rem % dk;
        rem /= dk;
        step[k] = st % dk;
        st /= dk;
        src += j[k] * d.in_stride[k];
      } else {
        j[k] = step[k] = 0;
      }
    }
  }
  while (e < s1) {
    // source offsets of the next U elements of this thread, then their loads
    int64_t srcs[U];
    int n = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (e + (int64_t)u * blockDim.x < s1) {
        srcs[u] = src;
        n = u + 1;
        // j += step with carries: every digit of the step is below its radix
        int carry = 0;
        src = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (k < r) {
            int64_t v = j[k] + step[k] + carry;
            carry = v >= d.out_dims[k];
            if (carry) v -= d.out_dims[k];
            j[k] = v;
            src += v * d.in_stride[k];
          }
        }
      }
    }
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (u < n) v[u] = in[srcs[u]];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (u < n) out[e + (int64_t)u * blockDim.x] = perm_conj(v[u], d.conj);
    e += (int64_t)U * blockDim.x;
  }
}

void launch_permute(Ctx *ctx, const PermDesc *d_desc, const int64_t *d_chunk_blk,
                    const int64_t *d_chunk_start, int64_t nchunks, const PermTile *d_tiles, int64_t ntiles,
                    const double *in, double *out, int is_complex, int chunk_elems) {
  if (nchunks > 0x7fffffff || ntiles > 0x7fffffff) fail(QS_ERR_SHAPE, "permute: too many work items");
  if (ntiles > 0) {
    const dim3 blk(PT, PT_ROWS);
    if (is_complex)
      permute_tile_kernel<true><<<(unsigned)ntiles, blk, 0, ctx->stream>>>(d_desc, d_tiles, in, out);
    else
      permute_tile_kernel<false><<<(unsigned)ntiles, blk, 0, ctx->stream>>>(d_desc, d_tiles, in, out);
    QS_LAUNCHED(ctx);
  }
  if (nchunks > 0) {
    if (is_complex)
      permute_lines_kernel<true><<<(unsigned)nchunks, 256, 0, ctx->stream>>>(d_desc, d_chunk_blk, d_chunk_start,
                                                                             chunk_elems, in, out);
    else
      permute_lines_kernel<false><<<(unsigned)nchunks, 256, 0, ctx->stream>>>(d_desc, d_chunk_blk, d_chunk_start,
                                                                              chunk_elems, in, out);
    QS_LAUNCHED(ctx);
  }
}

// Real -> complex widening of an arena (operands of mixed real/complex
// contractions are promoted, as the reference contracts QSpace<double> with
// QSpace<wbcomplex> into QSpace<wbcomplex>).
__global__ void widen_kernel(const double *__restrict__ in, double2 *__restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_double2(in[i], 0.0);
}

void launch_widen(Ctx *ctx, const double *in, double *out, int64_t n) {
  if (n <= 0) return;
  int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8);
  widen_kernel<<<grid, 256, 0, ctx->stream>>>(in, reinterpret_cast<double2 *>(out), n);
  QS_LAUNCHED(ctx);
}

// dst block b += f * src block b over block lists (element offsets and
// sizes); a real source added into a complex destination lands on the real
// parts.  Blocks of one launch must not share destination elements.
__global__ void block_axpy_kernel(const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                                  const int64_t *__restrict__ size, const double *__restrict__ src,
                                  double *__restrict__ dst, double f, int es_src, int es_dst) {
  const int64_t b = blockIdx.y;
  const int64_t n = size[b];
  const double *s = src + soff[b] * es_src;
  double *d = dst + doff[b] * es_dst;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * es_src; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = es_src == es_dst ? i : i * es_dst;  // real into complex: every other double
    d[e] = fma(f, s[i], d[e]);
  }
}

void launch_block_axpy(Ctx *ctx, const int64_t *d_soff, const int64_t *d_doff, const int64_t *d_size, int64_t nb,
                       int64_t max_size, const double *src, double *dst, double f, int es_src, int es_dst) {
  if (nb <= 0) return;
  if (nb > 65535) fail(QS_ERR_SHAPE, "block_axpy: %lld blocks in one launch", (long long)nb);
  const unsigned gx = (unsigned)std::min<int64_t>((std::max<int64_t>(max_size, 1) * es_src + 255) / 256, 1024);
  block_axpy_kernel<<<dim3(gx, (unsigned)nb), 256, 0, ctx->stream>>>(d_soff, d_doff, d_size, src, dst, f, es_src,
                                                                      es_dst);
  QS_LAUNCHED(ctx);
}

// Per-block nonzero test (SkipZeroData with eps = 0, Source/QSpace.cc:
// 3201-3269): flags[b] = 1 when any element of block b differs from zero.
__global__ void block_nonzero_kernel(const int64_t *__restrict__ offs,
                                     const int64_t *__restrict__ sizes, const double *__restrict__ data,
                                     int cplx, int *__restrict__ flags) {
  const int64_t b = blockIdx.x;
  const int64_t n = sizes[b] * (cplx ? 2 : 1);
  const double *p = data + offs[b] * (cplx ? 2 : 1);
  int nz = 0;
  for (int64_t i = threadIdx.x; i < n && !nz; i += blockDim.x) nz |= (p[i] != 0.0);
  nz = __syncthreads_or(nz);
  if (threadIdx.x == 0) flags[b] = nz;
}

void launch_block_nonzero(Ctx *ctx, const int64_t *d_offs, const int64_t *d_sizes,
                          int64_t nblk, const double *data, int is_complex, int *d_flags) {
  if (nblk <= 0) return;
  block_nonzero_kernel<<<(unsigned)nblk, 128, 0, ctx->stream>>>(d_offs, d_sizes, data,
                                                                 is_complex, d_flags);
  QS_LAUNCHED(ctx);
}

// Work-list upload from the page-locked staging ring: the SMs read the
// mapped host memory, so these small copies never queue on the copy engines
// behind bulk operand transfers.
__global__ void stage_copy_kernel(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, size_t bytes) {
  const size_t n16 = bytes / 16;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (size_t i = t0; i < n16; i += stride)
    reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(src)[i];
  const size_t t = n16 * 16 + t0;  // the last bytes % 16
  if (t < bytes) dst[t] = src[t];
}

void launch_stage_copy(Ctx *ctx, const void *src, void *dst, size_t bytes) {
  if (!bytes) return;
  const size_t n16 = std::max<size_t>(bytes / 16, 1);
  const int grid = (int)std::min<size_t>((n16 + 255) / 256, (size_t)std::max(ctx->num_sms, 1) * 4);
  stage_copy_kernel<<<grid, 256, 0, ctx->stream>>>(static_cast<const uint8_t *>(src), static_cast<uint8_t *>(dst),
                                                   bytes);
  QS_LAUNCHED(ctx);
}

}  // namespace qs
