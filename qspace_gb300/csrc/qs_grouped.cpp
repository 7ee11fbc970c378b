// qs_grouped_gemm / qs_grouped_gemm_host: the per-output-block seam of the
// reference (Source/QSpace.cc:4375-4393 -> contractDATA_group, Source/
// QSpace_aux.cc:27-355) exposed directly: a list of block pairs with CG
// factors, grouped by output block, executed in one grouped launch.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "qs_internal.h"
#include "qs_plan.h"
#include "qs_split.h"
#include "qs_grouped.h"
#include "qs_xcache.h"

using namespace qs;

namespace qs {

// Validates the pair list.  When the element counts are known (host form),
// every access is checked against them.
GroupedPlan grouped_plan(const qs_pair_list *pl, int64_t a_elems, int64_t b_elems, int64_t c_elems) {
  if (!pl) fail(QS_ERR_ARG, "null pair list");
  const int64_t n = pl->npairs;
  if (n < 0) fail(QS_ERR_ARG, "negative pair count");
  GroupedPlan g;
  g.cplx = pl->is_complex != 0;
  g.grp.push_back(0);
  if (n == 0) return g;
  if (!pl->M || !pl->N || !pl->K || !pl->a_off || !pl->b_off || !pl->c_off || !pl->lda || !pl->ldb ||
      !pl->ldc || !pl->trans || !pl->afac || !pl->c_blk)
    fail(QS_ERR_ARG, "null array in pair list");
  const bool cplx = g.cplx;
  g.pairs.resize(n);
  g.a_end.resize(n);
  g.b_end.resize(n);
  for (int64_t p = 0; p < n; ++p) {
    const int32_t M = pl->M[p], N = pl->N[p], K = pl->K[p];
    if (M < 0 || N < 0 || K < 0) fail(QS_ERR_SHAPE, "pair %lld: negative size", (long long)p);
    const int t = pl->trans[p];
    const int32_t lda = pl->lda[p], ldb = pl->ldb[p], ldc = pl->ldc[p];
    const int64_t arows = (t & 1) ? K : M, acols = (t & 1) ? M : K;
    const int64_t brows = (t & 2) ? N : K, bcols = (t & 2) ? K : N;
    if (lda < std::max<int64_t>(arows, 1) || ldb < std::max<int64_t>(brows, 1) || ldc < std::max(M, 1))
      fail(QS_ERR_SHAPE, "pair %lld: leading dimension too small", (long long)p);
    const int64_t ea = pl->a_off[p] + (acols ? (acols - 1) * (int64_t)lda + arows : 0);
    const int64_t eb = pl->b_off[p] + (bcols ? (bcols - 1) * (int64_t)ldb + brows : 0);
    g.a_end[p] = ea;
    g.b_end[p] = eb;
    if (a_elems >= 0) {
      const int64_t ec = pl->c_off[p] + (N ? (N - 1) * (int64_t)ldc + M : 0);
      if (pl->a_off[p] < 0 || ea > a_elems || pl->b_off[p] < 0 || eb > b_elems || pl->c_off[p] < 0 ||
          ec > c_elems)
        fail(QS_ERR_SHAPE, "pair %lld: operand outside its buffer", (long long)p);
    }
    if (p > 0 && pl->c_blk[p] != pl->c_blk[p - 1]) {
      g.grp.push_back(p);
    }
    const bool newblk = (p == 0) || pl->c_blk[p] != pl->c_blk[p - 1];
    if (newblk) {
      g.bM.push_back(M);
      g.bN.push_back(N);
      g.bldc.push_back(ldc);
      g.coff.push_back(pl->c_off[p]);
    } else if (M != g.bM.back() || N != g.bN.back() || pl->c_off[p] != g.coff.back() || ldc != g.bldc.back()) {
      fail(QS_ERR_SHAPE, "pair %lld: pairs of one output block disagree on its shape", (long long)p);
    }
    PairDesc &d = g.pairs[p];
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
    g.flops += (cplx ? 8.0 : 2.0) * double(M) * N * K;
    g.bytes += (cplx ? 16.0 : 8.0) * (double(M) * K + double(K) * N);
  }
  g.grp.push_back(n);
  // a block id must not reappear after its run ended (pairs of a block are
  // contiguous)
  {
    std::vector<int32_t> ids;
    for (size_t b = 0; b + 1 < g.grp.size(); ++b) ids.push_back(pl->c_blk[g.grp[b]]);
    std::sort(ids.begin(), ids.end());
    if (std::adjacent_find(ids.begin(), ids.end()) != ids.end())
      fail(QS_ERR_ARG, "pairs of one output block must be contiguous");
  }
  for (size_t b = 0; b < g.bM.size(); ++b) g.bytes += (cplx ? 16.0 : 8.0) * double(g.bM[b]) * g.bN[b];
  return g;
}

void run_f64(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
             const std::vector<int32_t> &bM, const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
             const std::vector<int32_t> *bldc, const double *A, const double *B, double *C, bool cplx) {
  // shallow blocks directly (run_shallow), the rest through the tiles
  std::vector<char> rest(bM.size(), 1);
  std::vector<int64_t> ids;
  for (size_t b = 0; b < bM.size(); ++b)
    if (is_shallow(pairs, grp[b], grp[b + 1])) {
      rest[b] = 0;
      ids.push_back((int64_t)b);
    }
  if (!ids.empty()) {
    run_shallow(ctx, pairs, grp, bM, bN, coff, bldc, ids, A, B, C, cplx);
    if (ids.size() == bM.size()) return;
    const BlockList R = select_blocks(pairs, grp, bM, bN, coff, bldc, rest);
    run_f64(ctx, R.pairs, R.grp, R.bM, R.bN, R.coff, &R.bldc, A, B, C, cplx);
    return;
  }
  DeepSplit ds;
  const int64_t eb = cplx ? 16 : 8;
  const bool deep = reinterpret_cast<uintptr_t>(C) % eb == 0 && split_deep(pairs, grp, bM, bN, coff, bldc, ds);
  double *T = nullptr;
  PairDesc *dp = nullptr;
  TileDesc *dt = nullptr;
  DeepReduce *dr = nullptr;
  try {
    if (deep) {
      T = dev_alloc<double>(ctx, (size_t)std::max<int64_t>(ds.temp_elems, 1) * (cplx ? 2 : 1));
      ds.place((int64_t)(reinterpret_cast<intptr_t>(T) - reinterpret_cast<intptr_t>(C)) / eb);
    }
    const std::vector<PairDesc> &pp = deep ? ds.pairs : pairs;
    const std::vector<int64_t> &gg = deep ? ds.grp : grp, &cc = deep ? ds.coff : coff;
    const std::vector<int32_t> &mm = deep ? ds.bM : bM, &nn = deep ? ds.bN : bN;
    const std::vector<int32_t> *ll = deep ? &ds.bldc : bldc;
    // parts of deep blocks with a few outputs: one CTA per output element
    // (run_dot); the others through the 64 x 64 tiles
    std::vector<int64_t> small;
    std::vector<TileDesc> tiles;
    {
      std::vector<TileDesc> all = make_tiles(gg, mm, nn, cc, gemm_f64_tile_m(), gemm_f64_tile_n(), ll, &pp);
      std::vector<char> is_small(mm.size(), 0);
      for (size_t b = 0; b < mm.size(); ++b)
        if (deep && ds.part[b] && (int64_t)mm[b] * nn[b] <= DOT_OUTPUTS) {
          is_small[b] = 1;
          small.push_back((int64_t)b);
        }
      for (const TileDesc &t : all)
        if (!is_small[t.cblk]) tiles.push_back(t);
    }
    run_dot(ctx, pp, gg, mm, nn, cc, ll, small, A, B, C, cplx);
    dp = dev_upload(ctx, pp);
    dt = dev_upload(ctx, tiles);
    if (!tiles.empty()) launch_gemm_f64(ctx, dp, dt, (int64_t)tiles.size(), A, B, C, cplx ? 1 : 0);
    if (deep) {
      dr = dev_upload(ctx, ds.red);
      launch_reduce_parts(ctx, dr, (int64_t)ds.red.size(), T, C, cplx);
    }
  } catch (...) {
    cudaStreamSynchronize(ctx->stream);
    for (void *p : {(void *)T, (void *)dp, (void *)dt, (void *)dr})
      if (p) dev_free(ctx, p);
    throw;
  }
  for (void *p : {(void *)T, (void *)dp, (void *)dt, (void *)dr})
    if (p) dev_free(ctx, p);
}

// Launches the products of output blocks [b0, b1) of a plan (FP64 or split
// path).  With `static_scratch` the split path carves its device buffers from
// that scratch instead of allocating.
static void grouped_exec(Ctx *ctx, const GroupedPlan &g, size_t b0, size_t b1, const double *A,
                         const double *B, double *C, const qs_opts *opts, SplitResult *sr_out,
                         uint8_t *static_scratch, size_t static_cap, int *static_err) {
  if (b1 <= b0) return;
  const bool whole = b0 == 0 && b1 == g.bM.size();
  std::vector<PairDesc> sub_pairs;
  std::vector<int64_t> sub_grp, sub_coff;
  std::vector<int32_t> sub_M, sub_N, sub_ldc;
  if (!whole) {
    const int64_t p0 = g.grp[b0], p1 = g.grp[b1];
    sub_pairs.assign(g.pairs.begin() + p0, g.pairs.begin() + p1);
    for (size_t b = b0; b <= b1; ++b) sub_grp.push_back(g.grp[b] - p0);
    sub_M.assign(g.bM.begin() + b0, g.bM.begin() + b1);
    sub_N.assign(g.bN.begin() + b0, g.bN.begin() + b1);
    sub_ldc.assign(g.bldc.begin() + b0, g.bldc.begin() + b1);
    sub_coff.assign(g.coff.begin() + b0, g.coff.begin() + b1);
  }
  const std::vector<PairDesc> &pairs = whole ? g.pairs : sub_pairs;
  const std::vector<int64_t> &grp = whole ? g.grp : sub_grp;
  const std::vector<int32_t> &bM = whole ? g.bM : sub_M, &bN = whole ? g.bN : sub_N;
  const std::vector<int32_t> &bldc = whole ? g.bldc : sub_ldc;
  const std::vector<int64_t> &coff = whole ? g.coff : sub_coff;
  const int prec = opts ? opts->prec : QS_PREC_FP64;
  if (prec == QS_PREC_SPLIT) {
    const int ns = opts ? opts->nslices : 0;
    const double tol = opts && opts->tol > 0 ? opts->tol : 1e-12;
    SplitResult sr = static_scratch
                         ? run_split_static(ctx, pairs, grp, bM, bN, coff, A, B, C, g.cplx, ns, tol, &bldc,
                                            static_scratch, static_cap, static_err)
                         : run_split(ctx, pairs, grp, bM, bN, coff, A, B, C, g.cplx, ns, tol, &bldc, 0);
    if (sr_out && sr.err_bound >= sr_out->err_bound) *sr_out = sr;
  } else if (static_scratch) {
    fail(QS_ERR_ARG, "the static-scratch entry point runs the split path only");
  } else if (prec == QS_PREC_FP64) {
    run_f64(ctx, pairs, grp, bM, bN, coff, &bldc, A, B, C, g.cplx);
  } else {
    fail(QS_ERR_ARG, "unknown precision mode %d", prec);
  }
}

static void fill_stats(qs_stats *stats, const GroupedPlan &g, const SplitResult &sr, int64_t launches) {
  if (!stats) return;
  std::memset(stats, 0, sizeof *stats);
  stats->flops = g.flops;
  stats->bytes = g.bytes;
  stats->npairs = (int64_t)g.pairs.size();
  stats->nblk_out = (int64_t)g.bM.size();
  stats->nslices = sr.nslices;
  stats->digit_bits = sr.bits;
  stats->err_bound = sr.err_bound;
  stats->launches = (int32_t)launches;
}

// Validates the pair list, then launches the FP64 or the split path on all
// of it.
void grouped_run(Ctx *ctx, const qs_pair_list *pl, const double *A, const double *B, double *C,
                 const qs_opts *opts, qs_stats *stats, int64_t a_elems, int64_t b_elems,
                 int64_t c_elems, uint8_t *static_scratch, size_t static_cap, int *static_err) {
  if (stats) std::memset(stats, 0, sizeof *stats);
  GroupedPlan g = grouped_plan(pl, a_elems, b_elems, c_elems);
  if (g.pairs.empty()) return;
  const int64_t launches0 = ctx->launches;
  SplitResult sr;
  grouped_exec(ctx, g, 0, g.bM.size(), A, B, C, opts, &sr, static_scratch, static_cap, static_err);
  fill_stats(stats, g, sr, ctx->launches - launches0);
}

// Host-buffer form.  Large batches are cut at output-block boundaries into
// chunks of similar input size (the last few smaller); chunk i's operands are copied in on one copy
// stream while chunk i-1 computes on the context stream and earlier results
// are copied out on another, so the copies over the host link overlap the
// products.  Only the part of A and B not yet copied is sent per chunk (one
// past the highest element the chunk reads), and results go out per chunk as
// long as the chunks' output ranges are ordered; otherwise all of C goes out
// once at the end.  Elements of C outside every output block come back zero.
static void grouped_host(Ctx *c, const qs_pair_list *pl, const double *A, int64_t a_elems, const double *B,
                         int64_t b_elems, double *C, int64_t c_elems, const qs_opts *opts, qs_stats *stats) {
  GroupedPlan g = grouped_plan(pl, a_elems, b_elems, c_elems);
  if (stats) std::memset(stats, 0, sizeof *stats);
  const int es = g.cplx ? 2 : 1;
  const size_t eb = (size_t)es * 8;  // bytes per element
  const int64_t launches0 = c->launches;
  const size_t nb = g.bM.size();
  // chunk boundaries (in output blocks) by cumulative input bytes
  const double in_bytes = 8.0 * es * double(a_elems + b_elems);
  // QS_HOST_CHUNK_MB / QS_HOST_MAX_CHUNKS override the chunking for tuning
  const char *e_mb = std::getenv("QS_HOST_CHUNK_MB"), *e_max = std::getenv("QS_HOST_MAX_CHUNKS");
  const double chunk_bytes = (e_mb ? std::atof(e_mb) : 64.0) * (1 << 20);
  const double max_chunks = e_max ? std::atof(e_max) : 16.0;
  const int nchunk = (int)std::max<double>(1.0, std::min<double>(max_chunks, std::floor(in_bytes / chunk_bytes)));
  std::vector<size_t> cut{0};
  if (nb) {
    std::vector<double> w(nb, 0.0);
    double tot = 0;
    for (size_t b = 0; b < nb; ++b) {
      for (int64_t p = g.grp[b]; p < g.grp[b + 1]; ++p) {
        const PairDesc &d = g.pairs[p];
        w[b] += double(d.M) * d.K + double(d.K) * d.N;
      }
      tot += w[b];
    }
    // the last chunks shrink geometrically (weights 1/2, 1/4, ... of the
    // others; QS_HOST_TAPER of them, default 2): what remains after the last
    // copy in -- the last chunk's products and its copy out -- is short
    const char *e_tp = std::getenv("QS_HOST_TAPER");
    const int taper = std::min(std::max(e_tp ? std::atoi(e_tp) : 2, 0), std::max(nchunk - 2, 0));
    std::vector<double> frac(nchunk + 1, 0.0);
    for (int k = 0; k < nchunk; ++k) {
      const int t = k - (nchunk - taper) + 1;  // 1.. for the tapered chunks
      frac[k + 1] = frac[k] + (t > 0 ? std::ldexp(1.0, -t) : 1.0);
    }
    double acc = 0;
    for (size_t b = 0; b < nb; ++b) {
      acc += w[b];
      if (cut.size() < (size_t)nchunk && acc >= tot * frac[cut.size()] / frac[nchunk] && b + 1 < nb)
        cut.push_back(b + 1);
    }
  }
  cut.push_back(nb);
  const size_t nch = cut.size() - 1;
  // per chunk: highest A/B element read, output range
  std::vector<int64_t> ahi(nch, 0), bhi(nch, 0), clo(nch, INT64_MAX), chi(nch, 0);
  for (size_t k = 0; k < nch; ++k) {
    for (size_t b = cut[k]; b < cut[k + 1]; ++b) {
      for (int64_t p = g.grp[b]; p < g.grp[b + 1]; ++p) {
        ahi[k] = std::max(ahi[k], g.a_end[p]);
        bhi[k] = std::max(bhi[k], g.b_end[p]);
      }
      const int64_t lo = g.coff[b];
      const int64_t hi = lo + (g.bN[b] ? (int64_t)(g.bN[b] - 1) * g.bldc[b] + g.bM[b] : 0);
      clo[k] = std::min(clo[k], lo);
      chi[k] = std::max(chi[k], hi);
    }
  }
  bool ordered = true;
  for (size_t k = 1; k < nch; ++k)
    if (clo[k] < chi[k - 1]) ordered = false;

  double *dA = dev_alloc<double>(c, (size_t)a_elems * es);
  double *dB = dev_alloc<double>(c, (size_t)b_elems * es);
  double *dC = dev_alloc<double>(c, (size_t)c_elems * es);
  std::vector<cudaEvent_t> evs;
  auto event = [&]() {
    cudaEvent_t e;
    QS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    evs.push_back(e);
    return e;
  };
  SplitResult sr;
  try {
    c->ensure_copy_streams();
    // the copies in wait only for the allocations; the zero fill of C runs
    // meanwhile on the context stream, ahead of every product
    cudaEvent_t ready = event();
    QS_CUDA(cudaEventRecord(ready, c->stream));
    QS_CUDA(cudaStreamWaitEvent(c->h2d, ready, 0));
    QS_CUDA(cudaMemsetAsync(dC, 0, (size_t)c_elems * eb, c->stream));
    cudaEvent_t filled = event();
    QS_CUDA(cudaEventRecord(filled, c->stream));
    QS_CUDA(cudaStreamWaitEvent(c->d2h, filled, 0));
    // all copies in are queued first: the copy stream never waits for the
    // host to plan a chunk
    int64_t wa = 0, wb = 0, wc = 0;
    std::vector<cudaEvent_t> in(nch);
    for (size_t k = 0; k < nch; ++k) {
      if (ahi[k] > wa) {
        QS_CUDA(cudaMemcpyAsync(dA + wa * es, A + wa * es, (size_t)(ahi[k] - wa) * eb, cudaMemcpyHostToDevice, c->h2d));
        wa = ahi[k];
      }
      if (bhi[k] > wb) {
        QS_CUDA(cudaMemcpyAsync(dB + wb * es, B + wb * es, (size_t)(bhi[k] - wb) * eb, cudaMemcpyHostToDevice, c->h2d));
        wb = bhi[k];
      }
      in[k] = event();
      QS_CUDA(cudaEventRecord(in[k], c->h2d));
    }
    for (size_t k = 0; k < nch; ++k) {
      QS_CUDA(cudaStreamWaitEvent(c->stream, in[k], 0));
      grouped_exec(c, g, cut[k], cut[k + 1], dA, dB, dC, opts, &sr, nullptr, 0, nullptr);
      if (ordered && k + 1 < nch && chi[k] > wc) {
        cudaEvent_t done = event();
        QS_CUDA(cudaEventRecord(done, c->stream));
        QS_CUDA(cudaStreamWaitEvent(c->d2h, done, 0));
        QS_CUDA(cudaMemcpyAsync(C + wc * es, dC + wc * es, (size_t)(chi[k] - wc) * eb, cudaMemcpyDeviceToHost, c->d2h));
        wc = chi[k];
      }
    }
    cudaEvent_t done = event();
    QS_CUDA(cudaEventRecord(done, c->stream));
    QS_CUDA(cudaStreamWaitEvent(c->d2h, done, 0));
    if (c_elems > wc)
      QS_CUDA(cudaMemcpyAsync(C + wc * es, dC + wc * es, (size_t)(c_elems - wc) * eb, cudaMemcpyDeviceToHost, c->d2h));
    cudaEvent_t out = event();
    QS_CUDA(cudaEventRecord(out, c->d2h));
    QS_CUDA(cudaStreamWaitEvent(c->stream, out, 0));
    QS_CUDA(cudaStreamSynchronize(c->stream));
  } catch (...) {
    // nothing may still read or write the buffers when they are released
    if (c->h2d) cudaStreamSynchronize(c->h2d);
    if (c->d2h) cudaStreamSynchronize(c->d2h);
    cudaStreamSynchronize(c->stream);
    dev_free(c, dA);
    dev_free(c, dB);
    dev_free(c, dC);
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    throw;
  }
  for (cudaEvent_t e : evs) cudaEventDestroy(e);
  int kerr = 0;
  QS_CUDA(cudaMemcpy(&kerr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  dev_free(c, dA);
  dev_free(c, dB);
  dev_free(c, dC);
  if (kerr) {
    cudaMemset(c->d_err, 0, sizeof(int));
    fail(QS_ERR_TIMEOUT, "a bounded device wait ran out (code %d)", kerr);
  }
  fill_stats(stats, g, sr, c->launches - launches0);
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
  grouped_host(c, pairs, A, a_elems, B, b_elems, C, c_elems, opts, stats);
  QS_API_END
}

}  // extern "C"
