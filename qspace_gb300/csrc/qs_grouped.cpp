// qs_grouped_gemm / qs_grouped_gemm_host: the per-output-block seam of the
// reference (Source/QSpace.cc:4375-4393 -> contractDATA_group, Source/
// QSpace_aux.cc:27-355) exposed directly: a list of block pairs with CG
// factors, grouped by output block, executed in one grouped launch.
#include <algorithm>
#include <cstring>
#include <memory>

#include "qs_internal.h"
#include "qs_plan.h"
#include "qs_split.h"

namespace qs {
void grouped_run(Ctx *ctx, const qs_pair_list *pl, const double *A, const double *B, double *C,
                 const qs_opts *opts, qs_stats *stats, int64_t a_elems, int64_t b_elems,
                 int64_t c_elems, uint8_t *static_scratch = nullptr, size_t static_cap = 0,
                 int *static_err = nullptr);
}

using namespace qs;

namespace qs {

// Validates the pair list, builds the device work lists and launches the
// FP64 or the split path.  When the element counts are known (host form),
// every access is checked against them.  With `static_scratch` the split
// path carves its device buffers from that scratch instead of allocating.
void grouped_run(Ctx *ctx, const qs_pair_list *pl, const double *A, const double *B, double *C,
                 const qs_opts *opts, qs_stats *stats, int64_t a_elems, int64_t b_elems,
                 int64_t c_elems, uint8_t *static_scratch, size_t static_cap, int *static_err) {
  if (!pl) fail(QS_ERR_ARG, "null pair list");
  const int64_t n = pl->npairs;
  if (n < 0) fail(QS_ERR_ARG, "negative pair count");
  if (stats) std::memset(stats, 0, sizeof *stats);
  if (n == 0) return;
  if (!pl->M || !pl->N || !pl->K || !pl->a_off || !pl->b_off || !pl->c_off || !pl->lda || !pl->ldb ||
      !pl->ldc || !pl->trans || !pl->afac || !pl->c_blk)
    fail(QS_ERR_ARG, "null array in pair list");
  const bool cplx = pl->is_complex != 0;
  const int64_t launches0 = ctx->launches;
  std::vector<PairDesc> pairs(n);
  std::vector<int64_t> grp{0};
  std::vector<int32_t> bM, bN, bldc;
  std::vector<int64_t> coff;
  double flops = 0, bytes = 0;
  for (int64_t p = 0; p < n; ++p) {
    const int32_t M = pl->M[p], N = pl->N[p], K = pl->K[p];
    if (M < 0 || N < 0 || K < 0) fail(QS_ERR_SHAPE, "pair %lld: negative size", (long long)p);
    const int t = pl->trans[p];
    const int32_t lda = pl->lda[p], ldb = pl->ldb[p], ldc = pl->ldc[p];
    const int64_t arows = (t & 1) ? K : M, acols = (t & 1) ? M : K;
    const int64_t brows = (t & 2) ? N : K, bcols = (t & 2) ? K : N;
    if (lda < std::max<int64_t>(arows, 1) || ldb < std::max<int64_t>(brows, 1) || ldc < std::max(M, 1))
      fail(QS_ERR_SHAPE, "pair %lld: leading dimension too small", (long long)p);
    if (a_elems >= 0) {
      const int64_t ea = pl->a_off[p] + (acols ? (acols - 1) * (int64_t)lda + arows : 0);
      const int64_t eb = pl->b_off[p] + (bcols ? (bcols - 1) * (int64_t)ldb + brows : 0);
      const int64_t ec = pl->c_off[p] + (N ? (N - 1) * (int64_t)ldc + M : 0);
      if (pl->a_off[p] < 0 || ea > a_elems || pl->b_off[p] < 0 || eb > b_elems || pl->c_off[p] < 0 ||
          ec > c_elems)
        fail(QS_ERR_SHAPE, "pair %lld: operand outside its buffer", (long long)p);
    }
    if (p > 0 && pl->c_blk[p] != pl->c_blk[p - 1]) {
      grp.push_back(p);
    }
    const bool newblk = (p == 0) || pl->c_blk[p] != pl->c_blk[p - 1];
    if (newblk) {
      bM.push_back(M);
      bN.push_back(N);
      bldc.push_back(ldc);
      coff.push_back(pl->c_off[p]);
    } else if (M != bM.back() || N != bN.back() || pl->c_off[p] != coff.back() || ldc != bldc.back()) {
      fail(QS_ERR_SHAPE, "pair %lld: pairs of one output block disagree on its shape", (long long)p);
    }
    PairDesc &d = pairs[p];
    d.a_off = pl->a_off[p];
    d.b_off = pl->b_off[p];
    d.M = M;
    d.N = N;
    d.K = K;
    d.lda = lda;
    d.ldb = ldb;
    d.trans = t & 15;
    if (!cplx) d.trans &= 3;
    d.afac = pl->afac[p];
    flops += (cplx ? 8.0 : 2.0) * double(M) * N * K;
    bytes += (cplx ? 16.0 : 8.0) * (double(M) * K + double(K) * N);
  }
  grp.push_back(n);
  // a block id must not reappear after its run ended (pairs of a block are
  // contiguous)
  {
    std::vector<int32_t> ids;
    for (size_t g = 0; g + 1 < grp.size(); ++g) ids.push_back(pl->c_blk[grp[g]]);
    std::sort(ids.begin(), ids.end());
    if (std::adjacent_find(ids.begin(), ids.end()) != ids.end())
      fail(QS_ERR_ARG, "pairs of one output block must be contiguous");
  }
  for (size_t g = 0; g < bM.size(); ++g) bytes += (cplx ? 16.0 : 8.0) * double(bM[g]) * bN[g];
  const int prec = opts ? opts->prec : QS_PREC_FP64;
  if (stats) {
    stats->flops = flops;
    stats->bytes = bytes;
    stats->npairs = n;
    stats->nblk_out = (int64_t)bM.size();
  }
  if (prec == QS_PREC_SPLIT) {
    const int ns = opts ? opts->nslices : 0;
    const double tol = opts && opts->tol > 0 ? opts->tol : 1e-12;
    SplitResult sr = static_scratch
                         ? run_split_static(ctx, pairs, grp, bM, bN, coff, A, B, C, cplx, ns, tol, &bldc,
                                            static_scratch, static_cap, static_err)
                         : run_split(ctx, pairs, grp, bM, bN, coff, A, B, C, cplx, ns, tol, &bldc);
    if (stats) {
      stats->nslices = sr.nslices;
      stats->digit_bits = sr.bits;
      stats->err_bound = sr.err_bound;
    }
  } else if (static_scratch) {
    fail(QS_ERR_ARG, "the static-scratch entry point runs the split path only");
  } else if (prec == QS_PREC_FP64) {
    std::vector<TileDesc> tiles = make_tiles(grp, bM, bN, coff, gemm_f64_tile_m(), gemm_f64_tile_n(), &bldc);
    PairDesc *dp = dev_upload(ctx, pairs);
    TileDesc *dt = dev_upload(ctx, tiles);
    launch_gemm_f64(ctx, dp, dt, (int64_t)tiles.size(), A, B, C, cplx ? 1 : 0);
    dev_free(ctx, dp);
    dev_free(ctx, dt);
  } else {
    fail(QS_ERR_ARG, "unknown precision mode %d", prec);
  }
  if (stats) stats->launches = (int32_t)(ctx->launches - launches0);
}

}  // namespace qs




extern "C" {

qs_status qs_grouped_gemm(qs_ctx *ctx, const qs_pair_list *pairs, const double *A, const double *B,
                          double *C, const qs_opts *opts, qs_stats *stats) {
  QS_API_BEGIN
  if (!ctx || !A || !B || !C) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  grouped_run(&ctx->c, pairs, A, B, C, opts, stats, -1, -1, -1);
  QS_API_END
}

qs_status qs_grouped_gemm_host(qs_ctx *ctx, const qs_pair_list *pairs, const double *A, int64_t a_elems,
                               const double *B, int64_t b_elems, double *C, int64_t c_elems,
                               const qs_opts *opts, qs_stats *stats) {
  QS_API_BEGIN
  if (!ctx || !A || !B || !C || !pairs) fail(QS_ERR_ARG, "null argument");
  if (a_elems < 0 || b_elems < 0 || c_elems < 0) fail(QS_ERR_ARG, "negative buffer size");
  Ctx *c = &ctx->c;
  QS_CUDA(cudaSetDevice(c->device));
  const int es = pairs->is_complex ? 2 : 1;
  double *dA = dev_alloc<double>(c, (size_t)a_elems * es);
  double *dB = dev_alloc<double>(c, (size_t)b_elems * es);
  double *dC = dev_alloc<double>(c, (size_t)c_elems * es);
  QS_CUDA(cudaMemcpyAsync(dA, A, (size_t)a_elems * es * 8, cudaMemcpyHostToDevice, c->stream));
  QS_CUDA(cudaMemcpyAsync(dB, B, (size_t)b_elems * es * 8, cudaMemcpyHostToDevice, c->stream));
  // elements of C outside every output block come back as zero
  QS_CUDA(cudaMemsetAsync(dC, 0, (size_t)c_elems * es * 8, c->stream));
  grouped_run(c, pairs, dA, dB, dC, opts, stats, a_elems, b_elems, c_elems);
  QS_CUDA(cudaMemcpyAsync(C, dC, (size_t)c_elems * es * 8, cudaMemcpyDeviceToHost, c->stream));
  QS_CUDA(cudaStreamSynchronize(c->stream));
  int kerr = 0;
  QS_CUDA(cudaMemcpy(&kerr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  dev_free(c, dA);
  dev_free(c, dB);
  dev_free(c, dC);
  if (kerr) {
    cudaMemset(c->d_err, 0, sizeof(int));
    fail(QS_ERR_TIMEOUT, "a bounded device wait ran out (code %d)", kerr);
  }
  QS_API_END
}

}  // extern "C"
