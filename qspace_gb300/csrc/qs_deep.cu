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
#include <cmath>
#include <cstdint>
#include <vector>

#include "qs_internal.h"

namespace qs {

namespace {

// Depth of a part (elements of K, complex or real) and the parallel work a
// block should reach: output tiles (64 x 32 outputs as the unit of the
// estimate) for the products, and strips of 16 lines (each slicing its lines
// over the whole depth) for the digit preparation of the split path.
constexpr int64_t KPART = 4096;
constexpr int64_t TARGET_TILES = 256;
constexpr int64_t TARGET_STRIPS = 1024;

int64_t parts_of(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1, int32_t M, int32_t N) {
  int64_t depth = 0;
  for (int64_t p = p0; p < p1; ++p) depth += std::max<int32_t>(pairs[p].K, 0);
  if (depth < 2 * KPART) return 1;
  const int64_t tiles = std::max<int64_t>(1, ((int64_t)M + 63) / 64 * (((int64_t)N + 31) / 32));
  const int64_t strips = std::max<int64_t>(1, ((int64_t)M + N + 7) / 8);
  const int64_t want = std::max(TARGET_TILES / tiles, TARGET_STRIPS / strips);
  return std::max<int64_t>(1, std::min<int64_t>(depth / KPART, want));
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

// One thread per output element of a shallow block: C(i, j) = sum over the
// block's pairs, in order, of afac sum_k op(A)(i, k) op(B)(k, j).
struct ShallowTask {
  int64_t c_off;
  int32_t p0, p1, M, N, ldc, pad_;
  int64_t e0, e1;   // elements of this task (column-major over M x N)
};

template <bool CPLX>
__global__ void shallow_kernel(const ShallowTask *__restrict__ tasks, const PairDesc *__restrict__ pairs,
                               const double *__restrict__ A, const double *__restrict__ B, double *__restrict__ C) {
  const ShallowTask t = tasks[blockIdx.x];
  for (int64_t e = t.e0 + threadIdx.x; e < t.e1; e += blockDim.x) {
    const int64_t i = e % t.M, j = e / t.M;
    double re = 0.0, im = 0.0;
    for (int p = t.p0; p < t.p1; ++p) {
      const PairDesc P = pairs[p];
      const bool ta = P.trans & 1, tb = P.trans & 2, ca = P.trans & 4, cb = P.trans & 8;
      double sr = 0.0, si = 0.0;
      for (int k = 0; k < P.K; ++k) {
        const int64_t ia = P.a_off + (ta ? k + i * (int64_t)P.lda : i + k * (int64_t)P.lda);
        const int64_t ib = P.b_off + (tb ? j + k * (int64_t)P.ldb : k + j * (int64_t)P.ldb);
        if (CPLX) {
          const double ar = A[2 * ia], ai = ca ? -A[2 * ia + 1] : A[2 * ia + 1];
          const double br = B[2 * ib], bi = cb ? -B[2 * ib + 1] : B[2 * ib + 1];
          sr += ar * br - ai * bi;
          si += ar * bi + ai * br;
        } else {
          sr += A[ia] * B[ib];
        }
      }
      re += P.afac * sr;
      im += P.afac * si;
    }
    const int64_t o = t.c_off + i + j * (int64_t)t.ldc;
    if (CPLX) {
      C[2 * o] = re;
      C[2 * o + 1] = im;
    } else {
      C[o] = re;
    }
  }
}

// One CTA per output element of a small block: every thread sums its share
// of the block's (pair, k) terms in order, then a fixed tree reduces them.
struct DotTask {
  int64_t c_off;
  int32_t p0, p1, M, ldc, i, j;
};
constexpr int DOT_THREADS = 256;

template <bool CPLX>
__global__ void __launch_bounds__(DOT_THREADS)
dot_kernel(const DotTask *__restrict__ tasks, const PairDesc *__restrict__ pairs, const double *__restrict__ A,
           const double *__restrict__ B, double *__restrict__ C) {
  __shared__ double red[2][DOT_THREADS];
  const DotTask t = tasks[blockIdx.x];
  double re = 0.0, im = 0.0;
  for (int p = t.p0; p < t.p1; ++p) {
    const PairDesc P = pairs[p];
    const bool ta = P.trans & 1, tb = P.trans & 2, ca = P.trans & 4, cb = P.trans & 8;
    double sr = 0.0, si = 0.0;
    for (int k = threadIdx.x; k < P.K; k += DOT_THREADS) {
      const int64_t ia = P.a_off + (ta ? k + t.i * (int64_t)P.lda : t.i + k * (int64_t)P.lda);
      const int64_t ib = P.b_off + (tb ? t.j + k * (int64_t)P.ldb : k + t.j * (int64_t)P.ldb);
      if (CPLX) {
        const double ar = A[2 * ia], ai = ca ? -A[2 * ia + 1] : A[2 * ia + 1];
        const double br = B[2 * ib], bi = cb ? -B[2 * ib + 1] : B[2 * ib + 1];
        sr += ar * br - ai * bi;
        si += ar * bi + ai * br;
      } else {
        sr += A[ia] * B[ib];
      }
    }
    re += P.afac * sr;
    im += P.afac * si;
  }
  red[0][threadIdx.x] = re;
  red[1][threadIdx.x] = im;
  __syncthreads();
  for (int w = DOT_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int64_t o = t.c_off + t.i + t.j * (int64_t)t.ldc;
    if (CPLX) {
      C[2 * o] = red[0][0];
      C[2 * o + 1] = red[1][0];
    } else {
      C[o] = red[0][0];
    }
  }
}

}  // namespace

void run_dot(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
             const std::vector<int32_t> &bM, const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
             const std::vector<int32_t> *bldc, const std::vector<int64_t> &blocks, const double *A,
             const double *B, double *C, bool cplx) {
  std::vector<DotTask> tasks;
  for (int64_t b : blocks)
    for (int32_t j = 0; j < bN[b]; ++j)
      for (int32_t i = 0; i < bM[b]; ++i)
        tasks.push_back(DotTask{coff[b], (int32_t)grp[b], (int32_t)grp[b + 1], bM[b],
                                bldc ? (*bldc)[b] : std::max(bM[b], 1), i, j});
  if (tasks.empty()) return;
  if (tasks.size() > 0x7fffffff) fail(QS_ERR_SHAPE, "small-block products: too many outputs");
  DotTask *dt = dev_upload(ctx, tasks);
  PairDesc *dp = dev_upload(ctx, pairs);
  if (cplx) dot_kernel<true><<<(unsigned)tasks.size(), DOT_THREADS, 0, ctx->stream>>>(dt, dp, A, B, C);
  else dot_kernel<false><<<(unsigned)tasks.size(), DOT_THREADS, 0, ctx->stream>>>(dt, dp, A, B, C);
  dev_free(ctx, dt);
  dev_free(ctx, dp);
  QS_LAUNCHED(ctx);
}

bool is_shallow(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1) {
  int64_t depth = 0;
  for (int64_t p = p0; p < p1; ++p) depth += std::max<int32_t>(pairs[p].K, 0);
  return depth <= SHALLOW_K;
}

bool shallow_direct_wins(const std::vector<PairDesc> &pairs, int64_t p0, int64_t p1, int32_t M, int32_t N,
                         bool cplx) {
  int64_t depth = 0;
  for (int64_t p = p0; p < p1; ++p) depth += std::max<int32_t>(pairs[p].K, 0);
  const double m = M, n = N, cm = cplx ? 2.0 : 1.0;
  // direct: FP64 multiply-adds at ~1 TFLOP/s and the output written once
  const double direct = (cplx ? 8.0 : 2.0) * m * n * (double)depth / 1.0e12 + 8.0 * cm * m * n / 5.0e12;
  // tiled: 128 x 32 tiles of the real form, either orientation, ~3000 cycles
  // each (one k-block and the epilogue) spread over 152 SMs at 2 GHz
  auto tiles = [](double r, double c) { return std::ceil(r / 128.0) * std::ceil(c / 32.0); };
  const double t = std::min(tiles(cm * m, n), tiles(cm * n, m));
  const double tiled = t * 3000.0 / (152.0 * 2.0e9);
  return direct < tiled;
}

static std::vector<ShallowTask> shallow_tasks(const std::vector<int64_t> &grp, const std::vector<int32_t> &bM,
                                              const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
                                              const std::vector<int32_t> *bldc, const std::vector<int64_t> &blocks) {
  constexpr int64_t CHUNK = 8192;  // elements per CTA
  std::vector<ShallowTask> tasks;
  for (int64_t b : blocks) {
    const int64_t n = (int64_t)bM[b] * bN[b];
    for (int64_t e0 = 0; e0 < n; e0 += CHUNK) {
      ShallowTask t{};
      t.c_off = coff[b];
      t.p0 = (int32_t)grp[b];
      t.p1 = (int32_t)grp[b + 1];
      t.M = bM[b];
      t.N = bN[b];
      t.ldc = bldc ? (*bldc)[b] : std::max(bM[b], 1);
      t.e0 = e0;
      t.e1 = std::min(n, e0 + CHUNK);
      tasks.push_back(t);
    }
  }
  if (tasks.size() > 0x7fffffff) fail(QS_ERR_SHAPE, "shallow products: too many tasks");
  return tasks;
}

void run_shallow(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                 const std::vector<int32_t> &bM, const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
                 const std::vector<int32_t> *bldc, const std::vector<int64_t> &blocks, const double *A,
                 const double *B, double *C, bool cplx) {
  const std::vector<ShallowTask> tasks = shallow_tasks(grp, bM, bN, coff, bldc, blocks);
  if (tasks.empty()) return;
  ShallowTask *dt = dev_upload(ctx, tasks);
  PairDesc *dp = dev_upload(ctx, pairs);
  if (cplx) shallow_kernel<true><<<(unsigned)tasks.size(), 256, 0, ctx->stream>>>(dt, dp, A, B, C);
  else shallow_kernel<false><<<(unsigned)tasks.size(), 256, 0, ctx->stream>>>(dt, dp, A, B, C);
  // the work lists are released in stream order, also when the launch failed
  dev_free(ctx, dt);
  dev_free(ctx, dp);
  QS_LAUNCHED(ctx);
}

ShallowPlan shallow_prepare(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                            const std::vector<int32_t> &bM, const std::vector<int32_t> &bN,
                            const std::vector<int64_t> &coff, const std::vector<int32_t> *bldc,
                            const std::vector<int64_t> &blocks, bool cplx) {
  const std::vector<ShallowTask> tasks = shallow_tasks(grp, bM, bN, coff, bldc, blocks);
  ShallowPlan sp;
  sp.cplx = cplx;
  sp.ntasks = (int64_t)tasks.size();
  if (tasks.empty()) return sp;
  try {
    QS_CUDA(cudaMalloc(&sp.tasks, tasks.size() * sizeof(ShallowTask)));
    QS_CUDA(cudaMemcpy(sp.tasks, tasks.data(), tasks.size() * sizeof(ShallowTask), cudaMemcpyHostToDevice));
    QS_CUDA(cudaMalloc(&sp.pairs, std::max<size_t>(pairs.size(), 1) * sizeof(PairDesc)));
    if (!pairs.empty())
      QS_CUDA(cudaMemcpy(sp.pairs, pairs.data(), pairs.size() * sizeof(PairDesc), cudaMemcpyHostToDevice));
  } catch (...) {
    shallow_release(sp);
    throw;
  }
  return sp;
}

void shallow_launch(Ctx *ctx, const ShallowPlan &sp, const double *A, const double *B, double *C) {
  if (!sp.ntasks) return;
  const ShallowTask *dt = static_cast<const ShallowTask *>(sp.tasks);
  const PairDesc *dp = static_cast<const PairDesc *>(sp.pairs);
  if (sp.cplx) shallow_kernel<true><<<(unsigned)sp.ntasks, 256, 0, ctx->stream>>>(dt, dp, A, B, C);
  else shallow_kernel<false><<<(unsigned)sp.ntasks, 256, 0, ctx->stream>>>(dt, dp, A, B, C);
  QS_LAUNCHED(ctx);
}

void shallow_release(ShallowPlan &sp) {
  if (sp.tasks) cudaFree(sp.tasks);
  if (sp.pairs) cudaFree(sp.pairs);
  sp.tasks = sp.pairs = nullptr;
  sp.ntasks = 0;
}

BlockList select_blocks(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                        const std::vector<int32_t> &bM, const std::vector<int32_t> &bN,
                        const std::vector<int64_t> &coff, const std::vector<int32_t> *bldc,
                        const std::vector<char> &sel) {
  BlockList L;
  L.grp.push_back(0);
  for (size_t b = 0; b < bM.size(); ++b) {
    if (!sel[b]) continue;
    for (int64_t p = grp[b]; p < grp[b + 1]; ++p) {
      L.pairs.push_back(pairs[p]);
      L.src.push_back((int32_t)p);
    }
    L.grp.push_back((int64_t)L.pairs.size());
    L.bM.push_back(bM[b]);
    L.bN.push_back(bN[b]);
    L.bldc.push_back(bldc ? (*bldc)[b] : std::max(bM[b], 1));
    L.coff.push_back(coff[b]);
  }
  return L;
}

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
