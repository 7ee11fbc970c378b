// Generalised transpose of many blocks in one launch (the device counterpart
// of wbperm_helper::permute, Source/wbarray.cc:4453-4600, which QSpace runs
// per block from permute_to / Permute, Source/QSpace.hh:2670-2866).
//
// Work is cut into chunks of `chunk_elems` output elements; chunk c belongs to
// block chunk_blk[c] and starts at output element chunk_start[c].  Each CTA
// writes its chunk in output order (coalesced stores) and gathers the inputs
// through the permuted strides.  When the permutation keeps the first leg in
// place the gathers are unit-stride runs as well.
#include <algorithm>

#include "qs_internal.h"

namespace qs {

template <bool CPLX>
__global__ void __launch_bounds__(256)
permute_kernel(const PermDesc *__restrict__ desc, const int64_t *__restrict__ chunk_blk,
               const int64_t *__restrict__ chunk_start, int chunk_elems,
               const double *__restrict__ in, double *__restrict__ out) {
  const int64_t c = blockIdx.x;
  const PermDesc &d = desc[chunk_blk[c]];
  const int64_t s0 = chunk_start[c];
  const int64_t s1 = min(d.n, s0 + (int64_t)chunk_elems);
  const int r = d.rank;
  for (int64_t e = s0 + threadIdx.x; e < s1; e += blockDim.x) {
    int64_t rem = e, src = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < r) {
        const int64_t dk = d.out_dims[k];
        const int64_t j = rem % dk;
        rem /= dk;
        src += j * d.in_stride[k];
      }
    }
    if (CPLX) {
      const double2 v = reinterpret_cast<const double2 *>(in)[d.in_off + src];
      reinterpret_cast<double2 *>(out)[d.out_off + e] = make_double2(v.x, d.conj ? -v.y : v.y);
    } else {
      out[d.out_off + e] = in[d.in_off + src];
    }
  }
}

void launch_permute(Ctx *ctx, const PermDesc *d_desc, const int64_t *d_chunk_blk,
                    const int64_t *d_chunk_start, int64_t nchunks, const double *in,
                    double *out, int is_complex, int chunk_elems) {
  if (nchunks <= 0) return;
  if (nchunks > 0x7fffffff) fail(QS_ERR_SHAPE, "permute: too many chunks");
  dim3 grid((unsigned)nchunks);
  if (is_complex)
    permute_kernel<true><<<grid, 256, 0, ctx->stream>>>(d_desc, d_chunk_blk, d_chunk_start,
                                                        chunk_elems, in, out);
  else
    permute_kernel<false><<<grid, 256, 0, ctx->stream>>>(d_desc, d_chunk_blk, d_chunk_start,
                                                         chunk_elems, in, out);
  QS_LAUNCHED(ctx);
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
