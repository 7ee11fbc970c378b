// Deep output blocks of a grouped product: cut along the summed depth into
// parts that run as output blocks of their own, then summed in part order.
//
// The reference computes such a block with one zgemm per pair into the
// output block (Source/QSpace_aux.cc:27-355), each call parallel inside BLAS.
// The grouped kernels here parallelise over output tiles instead, one CTA per
// tile for the block's whole depth; a block with a handful of tiles and a
// sum of millions (the reduced density matrix or the overlap of tensors with
// large bonds) would keep a few SMs busy for the whole launch.  Cutting the
// depth into parts gives every part its own tiles; the parts' sum is formed
// by one kernel in a fixed order, so the result does not depend on how the
// work was scheduled.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "qs_internal.h"

namespace qs {

namespace {

// Depth of a part (elements of K, complex or real) and the number of tiles a
// block should reach.  A tile of 64 x 32 outputs is the unit of the estimate.
constexpr int64_t KPART = 4096;
constexpr int64_t TARGET_TILES = 256;

int64_t parts_of(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1, int32_t M, int32_t N) {
  int64_t depth = 0;
  for (int64_t p = p0; p < p1; ++p) depth += std::max<int32_t>(pairs[p].K, 0);
  if (depth < 2 * KPART) return 1;
  const int64_t tiles = std::max<int64_t>(1, ((int64_t)M + 63) / 64 * (((int64_t)N + 31) / 32));
  return std::max<int64_t>(1, std::min<int64_t>(depth / KPART, TARGET_TILES / tiles));
}

__global__ void reduce_parts_kernel(const DeepReduce *__restrict__ red, const double *__restrict__ T,
                                    double *__restrict__ C, int es) {
  const DeepReduce r = red[blockIdx.y];
  const int64_t n = (int64_t)r.M * r.N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * es; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = e / es, c = e % es;  // element, part of a complex value
    const int64_t i = x % r.M, j = x / r.M;
    const double *t = T + r.t_off * es + e;
    double s = 0.0;
    for (int q = 0; q < r.nparts; ++q) s += t[(int64_t)q * n * es];
    C[(r.c_off + i + j * (int64_t)r.ldc) * es + c] = s;
  }
}

}  // namespace

bool has_deep_blocks(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                     const std::vector<int32_t> &bM, const std::vector<int32_t> &bN) {
  for (size_t b = 0; b < bM.size(); ++b)
    if (parts_of(pairs, grp[b], grp[b + 1], bM[b], bN[b]) > 1) return true;
  return false;
}

bool split_deep(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                const std::vector<int32_t> &bM, const std::vector<int32_t> &bN,
                const std::vector<int64_t> &coff, const std::vector<int32_t> *bldc, DeepSplit &out,
                const std::vector<char> *keep) {
  auto cut = [&](size_t b) -> int64_t {
    if (keep && (*keep)[b]) return 1;
    return parts_of(pairs, grp[b], grp[b + 1], bM[b], bN[b]);
  };
  bool any = false;
  for (size_t b = 0; b < bM.size() && !any; ++b) any = cut(b) > 1;
  if (!any) return false;
  DeepSplit d;
  d.grp.push_back(0);
  for (size_t b = 0; b < bM.size(); ++b) {
    const int64_t p0 = grp[b], p1 = grp[b + 1];
    const int32_t M = bM[b], N = bN[b];
    const int32_t ldc = bldc ? (*bldc)[b] : std::max(M, 1);
    const int64_t np = cut(b);
    if (np <= 1) {
      for (int64_t p = p0; p < p1; ++p) {
        d.pairs.push_back(pairs[p]);
        d.src.push_back((int32_t)p);
      }
      d.grp.push_back((int64_t)d.pairs.size());
      d.bM.push_back(M);
      d.bN.push_back(N);
      d.bldc.push_back(ldc);
      d.coff.push_back(coff[b]);
      d.part.push_back(0);
      continue;
    }
    int64_t depth = 0;
    for (int64_t p = p0; p < p1; ++p) depth += std::max<int32_t>(pairs[p].K, 0);
    const int64_t mn = (int64_t)M * N;
    DeepReduce r{coff[b], d.temp_elems, M, N, ldc, (int32_t)np};
    d.red.push_back(r);
    // part q covers the summed depth [q D / np, (q + 1) D / np): the pairs'
    // K ranges are cut where the parts meet
    int64_t p = p0, k = 0;  // position: pair p, depth k inside it
    for (int64_t q = 0; q < np; ++q) {
      const int64_t end = (q + 1 == np) ? depth : depth * (q + 1) / np;
      int64_t at = depth * q / np;
      while (at < end && p < p1) {
        const PairDesc &s = pairs[p];
        const int64_t K = std::max<int32_t>(s.K, 0);
        const int64_t take = std::min(K - k, end - at);
        if (take > 0) {
          PairDesc t = s;
          const int64_t lda = s.lda, ldb = s.ldb;
          // op(A) columns k .. k+take: A not transposed is M x K (column k at
          // k lda), transposed it is stored K x M (row k at k); op(B) rows
          // likewise
          t.a_off = s.a_off + ((s.trans & 1) ? k : k * lda);
          t.b_off = s.b_off + ((s.trans & 2) ? k * ldb : k);
          t.K = (int32_t)take;
          d.pairs.push_back(t);
          d.src.push_back((int32_t)p);
        }
        k += take;
        at += take;
        if (k >= K) {
          ++p;
          k = 0;
        }
      }
      // pairs without depth contribute nothing; a part left without pairs
      // still gets one of them so that its block is written (zeros)
      if ((int64_t)d.pairs.size() == d.grp.back()) {
        PairDesc t = pairs[p0];
        t.K = 0;
        d.pairs.push_back(t);
        d.src.push_back((int32_t)p0);
      }
      d.grp.push_back((int64_t)d.pairs.size());
      d.bM.push_back(M);
      d.bN.push_back(N);
      d.bldc.push_back(std::max(M, 1));
      d.coff.push_back(r.t_off + q * mn);
      d.part.push_back(1);
    }
    d.temp_elems += np * mn;
  }
  out = std::move(d);
  return true;
}

void launch_reduce_parts(Ctx *ctx, const DeepReduce *d_red, int64_t nred, const double *T, double *C, bool cplx) {
  if (nred <= 0) return;
  if (nred > 65535) fail(QS_ERR_SHAPE, "too many deep output blocks in one launch");
  const int gx = std::max(1, std::min(64, (int)(1024 / std::max<int64_t>(nred, 1)) + 1));
  reduce_parts_kernel<<<dim3(gx, (unsigned)nred), 256, 0, ctx->stream>>>(d_red, T, C, cplx ? 2 : 1);
  QS_LAUNCHED(ctx);
}

}  // namespace qs
