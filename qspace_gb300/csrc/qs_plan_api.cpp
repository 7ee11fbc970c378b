// Reusable grouped plans (qs_grouped_plan_*): a pair list is validated and
// planned once, its work lists and digit arena stay on the device, and its
// launch sequence is recorded as a CUDA graph that later runs replay.  On
// request the first run times every digit width that meets the tolerance and
// keeps the fastest (an autotuner over the actual batch); the choice is
// remembered per pair-list shape for the rest of the process.
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <unordered_map>

#include "qs_grouped.h"
#include "qs_internal.h"
#include "qs_plan.h"
#include "qs_split.h"

using namespace qs;

namespace {

std::mutex g_tune_mu;
std::unordered_map<uint64_t, int> g_tuned;  // pair-list signature -> digit width

uint64_t signature(const GroupedPlan &g, const qs_opts &o) {
  uint64_t h = 1469598103934665603ull;  // FNV-1a over the shapes
  auto mix = [&](uint64_t v) {
    h ^= v;
    h *= 1099511628211ull;
  };
  uint64_t tb;
  std::memcpy(&tb, &o.tol, sizeof tb);
  mix(g.cplx);
  mix((uint64_t)o.prec);
  mix((uint64_t)o.nslices);
  mix(tb);
  for (const PairDesc &d : g.pairs) {
    mix((uint64_t)d.M);
    mix((uint64_t)d.N);
    mix((uint64_t)d.K);
    mix((uint64_t)d.trans);
  }
  for (int64_t x : g.grp) mix((uint64_t)x);
  return h;
}

}  // namespace

struct qs_grouped_plan {
  Ctx *ctx = nullptr;
  GroupedPlan g;
  qs_opts o{};
  uint64_t sig = 0;
  SplitPlanHandle *split = nullptr;
  SplitResult sr;
  bool tune_pending = false;
  float tuned_ms = 0;
  PairDesc *d_pairs = nullptr;  // FP64 path
  TileDesc *d_tiles = nullptr;
  int64_t ntiles = 0;
  // shallow output blocks run directly (as in the one-shot calls); `main`
  // holds the other blocks (all of them when none is shallow)
  ShallowPlan shallow;
  GroupedPlan main;
  cudaGraphExec_t exec = nullptr;
  const double *gA = nullptr, *gB = nullptr;
  double *gC = nullptr;
  int64_t graph_launches = 0;  // kernels in the recorded graph
};

namespace {

void launch_direct(qs_grouped_plan *p, const double *A, const double *B, double *C) {
  shallow_launch(p->ctx, p->shallow, A, B, C);
  if (p->main.pairs.empty()) return;
  if (p->o.prec == QS_PREC_SPLIT)
    split_plan_launch(p->ctx, p->split, A, B, C);
  else
    launch_gemm_f64(p->ctx, p->d_pairs, p->d_tiles, p->ntiles, A, B, C, p->g.cplx ? 1 : 0);
}

SplitPlanHandle *make_split(qs_grouped_plan *p, int bits, SplitResult *r) {
  const GroupedPlan &g = p->main;
  int ns = p->o.nslices;
  if (!bits && p->shallow.ntasks) {
    // the digit plan of the whole list, as the one-shot call takes it
    const DigitPlan dp = choose_digits_for(p->g.pairs, p->g.grp, p->g.bM, p->g.bN, p->g.cplx ? 2 : 1, p->o.tol,
                                           p->o.nslices, 0);
    bits = dp.bits;
    ns = dp.nslices;
  }
  return split_plan_create(g.pairs, g.grp, g.bM, g.bN, g.coff, g.bldc, g.cplx, ns, p->o.tol, bits, r);
}

// Splits the plan's blocks into shallow ones (prepared for the direct
// kernel) and the others (`main`), with the one-shot calls' rule.
void split_shallow(qs_grouped_plan *p) {
  const GroupedPlan &g = p->g;
  std::vector<char> rest(g.bM.size(), 1);
  std::vector<int64_t> ids;
  const bool split = p->o.prec == QS_PREC_SPLIT;
  for (size_t b = 0; b < g.bM.size(); ++b)
    if (is_shallow(g.pairs, g.grp[b], g.grp[b + 1]) &&
        (!split || shallow_direct_wins(g.pairs, g.grp[b], g.grp[b + 1], g.bM[b], g.bN[b], g.cplx))) {
      rest[b] = 0;
      ids.push_back((int64_t)b);
    }
  if (ids.empty()) {
    p->main = g;
    return;
  }
  p->shallow = shallow_prepare(g.pairs, g.grp, g.bM, g.bN, g.coff, &g.bldc, ids, g.cplx);
  BlockList R = select_blocks(g.pairs, g.grp, g.bM, g.bN, g.coff, &g.bldc, rest);
  GroupedPlan &m = p->main;
  m.cplx = g.cplx;
  m.pairs = std::move(R.pairs);
  m.grp = std::move(R.grp);
  m.bM = std::move(R.bM);
  m.bN = std::move(R.bN);
  m.bldc = std::move(R.bldc);
  m.coff = std::move(R.coff);
}

// Times every feasible digit width on the caller's operands (one warm-up and
// two timed launches each) and keeps the fastest.  C holds a valid product
// afterwards (every candidate computes it).
void autotune(qs_grouped_plan *p, const double *A, const double *B, double *C) {
  Ctx *c = p->ctx;
  std::vector<int> bits = split_candidate_bits(p->o.tol, p->o.nslices);
  if (bits.empty()) fail(QS_ERR_NUMERIC, "no digit plan meets tol=%g", p->o.tol);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  QS_CUDA(cudaEventCreate(&e0));
  QS_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bbest = bits[0];
  for (int b : bits) {
    SplitPlanHandle *h = nullptr;
    float ms = 0;
    try {
      h = make_split(p, b, nullptr);
      split_plan_launch(c, h, A, B, C);
      QS_CUDA(cudaEventRecord(e0, c->stream));
      split_plan_launch(c, h, A, B, C);
      split_plan_launch(c, h, A, B, C);
      QS_CUDA(cudaEventRecord(e1, c->stream));
      QS_CUDA(cudaEventSynchronize(e1));
      QS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    } catch (...) {
      cudaStreamSynchronize(c->stream);
      split_plan_destroy(h);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    split_plan_destroy(h);
    if (ms < best) {
      best = ms;
      bbest = b;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[p->sig] = bbest;
  }
  p->tuned_ms = best / 2;
  p->split = make_split(p, bbest, &p->sr);
  p->tune_pending = false;
}

// Records the launch sequence for (A, B, C) as a graph (nothing runs) and
// installs it, updating the existing executable graph when possible.
void record_graph(qs_grouped_plan *p, const double *A, const double *B, double *C) {
  Ctx *c = p->ctx;
  const bool timing = c->timing;
  const int64_t l0 = c->launches;
  c->timing = false;
  cudaGraph_t gr = nullptr;
  c->ensure_aux();  // the launch forks onto the second stream: created outside the capture
  QS_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  try {
    launch_direct(p, A, B, C);
  } catch (...) {
    cudaStreamEndCapture(c->stream, &gr);
    if (gr) cudaGraphDestroy(gr);
    c->timing = timing;
    c->launches = l0;
    throw;
  }
  cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
  c->timing = timing;
  p->graph_launches = c->launches - l0;
  c->launches = l0;
  if (e != cudaSuccess) fail(QS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  if (p->exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(p->exec, gr, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(p->exec);
      p->exec = nullptr;
    }
  }
  if (!p->exec) {
    e = cudaGraphInstantiate(&p->exec, gr, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(gr);
      p->exec = nullptr;
      fail(QS_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e));
    }
  }
  cudaGraphDestroy(gr);
  p->gA = A;
  p->gB = B;
  p->gC = C;
}

}  // namespace

extern "C" {

qs_status qs_grouped_plan_create(qs_ctx *ctx, const qs_pair_list *pairs, const qs_opts *opts,
                                 qs_grouped_plan **out) {
  QS_API_BEGIN
  if (!ctx || !pairs || !out) fail(QS_ERR_ARG, "null argument");
  *out = nullptr;
  Ctx *c = &ctx->c;
  QS_CUDA(cudaSetDevice(c->device));
  std::unique_ptr<qs_grouped_plan> p(new qs_grouped_plan);
  p->ctx = c;
  p->o = opts ? *opts : qs_opts{QS_PREC_FP64, 0, 1e-12, 0};
  if (!(p->o.tol > 0)) p->o.tol = 1e-12;
  p->g = grouped_plan(pairs, -1, -1, -1);
  if (p->o.prec == QS_PREC_SPLIT || p->o.prec == QS_PREC_FP64) split_shallow(p.get());
  if (p->o.prec == QS_PREC_SPLIT) {
    p->sig = signature(p->g, p->o);
    int bits = 0;
    if (p->o.flags & QS_FLAG_AUTOTUNE) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tuned.find(p->sig);
      if (it == g_tuned.end())
        p->tune_pending = !p->main.pairs.empty();
      else
        bits = it->second;
    }
    if (!p->tune_pending && !p->main.pairs.empty()) p->split = make_split(p.get(), bits, &p->sr);
    if (p->main.pairs.empty()) {  // every block shallow: the digit plan is reported only
      const DigitPlan dp = choose_digits_for(p->g.pairs, p->g.grp, p->g.bM, p->g.bN, p->g.cplx ? 2 : 1, p->o.tol,
                                             p->o.nslices, 0);
      p->sr.nslices = dp.nslices;
      p->sr.bits = dp.bits;
      p->sr.err_bound = dp.err_bound;
    }
  } else if (p->o.prec == QS_PREC_FP64) {
    if (!p->main.pairs.empty()) {
      const GroupedPlan &m = p->main;
      std::vector<TileDesc> tiles =
          make_tiles(m.grp, m.bM, m.bN, m.coff, gemm_f64_tile_m(), gemm_f64_tile_n(), &m.bldc, &m.pairs);
      p->ntiles = (int64_t)tiles.size();
      QS_CUDA(cudaMalloc(&p->d_pairs, m.pairs.size() * sizeof(PairDesc)));
      QS_CUDA(cudaMemcpy(p->d_pairs, m.pairs.data(), m.pairs.size() * sizeof(PairDesc),
                         cudaMemcpyHostToDevice));
      QS_CUDA(cudaMalloc(&p->d_tiles, std::max<size_t>(tiles.size(), 1) * sizeof(TileDesc)));
      if (!tiles.empty())
        QS_CUDA(cudaMemcpy(p->d_tiles, tiles.data(), tiles.size() * sizeof(TileDesc), cudaMemcpyHostToDevice));
    }
  } else {
    fail(QS_ERR_ARG, "unknown precision mode %d", p->o.prec);
  }
  *out = p.release();
  QS_API_END
}

qs_status qs_grouped_plan_run(qs_grouped_plan *p, const double *A, const double *B, double *C,
                              qs_stats *stats) {
  QS_API_BEGIN
  if (!p || !A || !B || !C) fail(QS_ERR_ARG, "null argument");
  Ctx *c = p->ctx;
  QS_CUDA(cudaSetDevice(c->device));
  const int64_t l0 = c->launches;
  if (!p->g.pairs.empty()) {
    if (p->tune_pending) autotune(p, A, B, C);
    if (p->o.flags & QS_FLAG_NO_GRAPH) {
      launch_direct(p, A, B, C);
    } else if (p->exec && p->gA == A && p->gB == B && p->gC == C) {
      QS_CUDA(cudaGraphLaunch(p->exec, c->stream));
      c->launches += p->graph_launches;
    } else {
      // run directly now (kernel attributes and modules are set up outside
      // the capture), and record the graph for the next runs
      launch_direct(p, A, B, C);
      record_graph(p, A, B, C);
    }
  }
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->flops = p->g.flops;
    stats->bytes = p->g.bytes;
    stats->npairs = (int64_t)p->g.pairs.size();
    stats->nblk_out = (int64_t)p->g.bM.size();
    stats->nslices = p->sr.nslices;
    stats->digit_bits = p->sr.bits;
    stats->err_bound = p->sr.err_bound;
    stats->device_ms = p->tuned_ms;
    stats->launches = (int32_t)(c->launches - l0);
  }
  QS_API_END
}

void qs_grouped_plan_destroy(qs_grouped_plan *p) {
  if (!p) return;
  if (p->ctx && ctx_alive(p->ctx)) {  // else the context's stream is gone
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
  }
  if (p->exec) cudaGraphExecDestroy(p->exec);
  split_plan_destroy(p->split);
  shallow_release(p->shallow);
  if (p->d_pairs) cudaFree(p->d_pairs);
  if (p->d_tiles) cudaFree(p->d_tiles);
  delete p;
}

}  // extern "C"
