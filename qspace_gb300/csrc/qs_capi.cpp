// C-ABI entry points of libqsgpu (include/qsgpu.h): context, device tensors,
// contractQS / permuteQS drivers and the grouped block-product seam.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <mutex>
#include <new>
#include <numeric>

#include "qs_internal.h"
#include "qs_grouped.h"
#include "qs_xcache.h"
#include "qs_objects.h"
#include "qs_plan.h"
#include "qs_split.h"

namespace qs {
const std::string &last_error();
}  // namespace qs

using namespace qs;

namespace qs {

void dev_free(Ctx *ctx, void *p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

void *Ctx::ensure_scratch(size_t bytes) {
  if (bytes <= scratch_bytes) return scratch;
  if (scratch) QS_CUDA(cudaFreeAsync(scratch, stream));
  size_t nb = std::max(bytes, scratch_bytes * 3 / 2);
  scratch = nullptr;
  cudaError_t e = cudaMallocAsync(&scratch, nb, stream);
  if (e != cudaSuccess) {
    scratch_bytes = 0;
    fail(e == cudaErrorMemoryAllocation ? QS_ERR_OOM : QS_ERR_CUDA, "scratch allocation of %zu bytes: %s", nb,
         cudaGetErrorString(e));
  }
  scratch_bytes = nb;
  return scratch;
}

// Copies `bytes` from host memory to `dst` (device) on the context stream
// through the page-locked ring, read by a copy kernel (not a copy engine).
// A region of the ring is reused only after the copy that last read it has
// completed.
namespace {
std::mutex g_live_mu;
std::unordered_set<const Ctx *> g_live;
}  // namespace

void ctx_register(const Ctx *c) {
  std::lock_guard<std::mutex> lk(g_live_mu);
  g_live.insert(c);
}
void ctx_unregister(const Ctx *c) {
  std::lock_guard<std::mutex> lk(g_live_mu);
  g_live.erase(c);
}
bool ctx_alive(const Ctx *c) {
  std::lock_guard<std::mutex> lk(g_live_mu);
  return g_live.count(c) != 0;
}

void Ctx::stage_upload(void *dst, const void *src, size_t bytes) {
  if (!bytes) return;
  const int64_t n = (int64_t)((bytes + 255) & ~size_t(255));
  if ((size_t)n > stage_cap / 2) {
    // grow: wait for every staged copy, then replace the buffer
    QS_CUDA(cudaStreamSynchronize(stream));
    for (auto &m : stage_q) stage_ev.push_back(m.ev);
    stage_q.clear();
    if (stage_buf) cudaFreeHost(stage_buf);
    stage_buf = stage_dev = nullptr;
    stage_cap = 0;
    const size_t cap = std::max<size_t>({(size_t)n * 4, stage_cap * 2, (size_t)4 << 20});
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(&stage_buf), cap, cudaHostAllocMapped);
    if (e != cudaSuccess) {
      stage_buf = nullptr;
      fail(QS_ERR_OOM, "page-locked staging buffer of %zu bytes: %s", cap, cudaGetErrorString(e));
    }
    e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&stage_dev), stage_buf, 0);
    if (e != cudaSuccess) {
      cudaFreeHost(stage_buf);
      stage_buf = stage_dev = nullptr;
      fail(QS_ERR_CUDA, "staging buffer device address: %s", cudaGetErrorString(e));
    }
    stage_cap = cap;
    stage_head = 0;
  }
  const int64_t cap = (int64_t)stage_cap;
  int64_t h = stage_head;
  if (h % cap + n > cap) h += cap - h % cap;  // wrap to the start
  while (!stage_q.empty() && stage_q.front().start < h + n - cap) {
    QS_CUDA(cudaEventSynchronize(stage_q.front().ev));
    stage_ev.push_back(stage_q.front().ev);
    stage_q.pop_front();
  }
  std::memcpy(stage_buf + h % cap, src, bytes);
  launch_stage_copy(this, stage_dev + h % cap, dst, bytes);
  cudaEvent_t ev;
  if (stage_ev.empty()) {
    QS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  } else {
    ev = stage_ev.back();
    stage_ev.pop_back();
  }
  QS_CUDA(cudaEventRecord(ev, stream));
  stage_q.push_back({ev, h});
  stage_head = h + n;
}

void Ctx::destroy_staging() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto &m : stage_q) cudaEventDestroy(m.ev);
  for (auto e : stage_ev) cudaEventDestroy(e);
  stage_q.clear();
  stage_ev.clear();
  if (stage_buf) cudaFreeHost(stage_buf);
  stage_buf = stage_dev = nullptr;
  stage_cap = 0;
}

void Ctx::ensure_copy_streams() {
  if (!h2d) QS_CUDA(cudaStreamCreateWithFlags(&h2d, cudaStreamNonBlocking));
  if (!d2h) QS_CUDA(cudaStreamCreateWithFlags(&d2h, cudaStreamNonBlocking));
}

void Ctx::ensure_aux() {
  if (!aux) QS_CUDA(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
  if (!aux_fork) QS_CUDA(cudaEventCreateWithFlags(&aux_fork, cudaEventDisableTiming));
  if (!aux_join) QS_CUDA(cudaEventCreateWithFlags(&aux_join, cudaEventDisableTiming));
}

void Ctx::destroy_copy_streams() {
  if (h2d) cudaStreamDestroy(h2d);
  if (d2h) cudaStreamDestroy(d2h);
  h2d = d2h = nullptr;
  if (aux) {
    cudaStreamSynchronize(aux);
    cudaStreamDestroy(aux);
  }
  if (aux_fork) cudaEventDestroy(aux_fork);
  if (aux_join) cudaEventDestroy(aux_join);
  aux = nullptr;
  aux_fork = aux_join = nullptr;
}

// A block's permutation on its fewest legs: legs of size 1 dropped, and
// output legs k, k+1 merged where they are also adjacent (and in order) in
// the input.  The element order of input and output is unchanged.
static PermDesc reduce_perm(const PermDesc &d) {
  PermDesc r = d;
  int n = 0;
  for (int k = 0; k < d.rank; ++k) {
    if (d.out_dims[k] == 1) continue;
    if (n > 0 && r.in_stride[n - 1] * r.out_dims[n - 1] == d.in_stride[k]) {
      r.out_dims[n - 1] *= d.out_dims[k];
      continue;
    }
    r.out_dims[n] = d.out_dims[k];
    r.in_stride[n] = d.in_stride[k];
    ++n;
  }
  if (n == 0) {  // a single element
    r.out_dims[0] = 1;
    r.in_stride[0] = 1;
    n = 1;
  }
  for (int k = n; k < 8; ++k) {
    r.out_dims[k] = 1;
    r.in_stride[k] = 0;
  }
  r.rank = n;
  r.fast_in_leg = -1;
  for (int k = 0; k < n; ++k)
    if (r.in_stride[k] == 1) r.fast_in_leg = k;
  return r;
}

// Work lists of the permute kernels: blocks whose output-fastest leg differs
// from the input-fastest one, both spanning >= 8 elements, go through 64 x 32
// shared-memory tiles; the others through output-order lines.
static void run_permute(Ctx *ctx, const std::vector<PermDesc> &descs_in, const double *in, double *out,
                        bool cplx, bool timed = false) {
  if (descs_in.empty()) return;
  const int CH = 8192, TILE_I = 64, TILE_J = 32, MIN_EDGE = 8;
  std::vector<PermDesc> descs;
  descs.reserve(descs_in.size());
  std::vector<int64_t> cb, cs;
  std::vector<PermTile> tiles;
  for (size_t i = 0; i < descs_in.size(); ++i) {
    if (descs_in[i].n <= 0) continue;
    PermDesc d = reduce_perm(descs_in[i]);
    const int b = d.fast_in_leg;
    const int64_t di = (int64_t)descs.size();
    if (b > 0 && d.out_dims[0] >= MIN_EDGE && d.out_dims[b] >= MIN_EDGE) {
      const int64_t nt0 = (d.out_dims[0] + TILE_I - 1) / TILE_I, ntb = (d.out_dims[b] + TILE_J - 1) / TILE_J;
      const int64_t nrest = d.n / (d.out_dims[0] * d.out_dims[b]);
      for (int64_t rest = 0; rest < nrest; ++rest)
        for (int64_t tj = 0; tj < ntb; ++tj)
          for (int64_t ti = 0; ti < nt0; ++ti) tiles.push_back(PermTile{di, rest, (int32_t)ti, (int32_t)tj});
    } else {
      for (int64_t s0 = 0; s0 < d.n; s0 += CH) {
        cb.push_back(di);
        cs.push_back(s0);
      }
    }
    descs.push_back(d);
  }
  if (descs.empty()) return;
  PermDesc *dd = dev_upload(ctx, descs);
  int64_t *dcb = cb.empty() ? nullptr : dev_upload(ctx, cb);
  int64_t *dcs = cs.empty() ? nullptr : dev_upload(ctx, cs);
  PermTile *dt = tiles.empty() ? nullptr : dev_upload(ctx, tiles);
  if (timed) ctx->mark(0);
  launch_permute(ctx, dd, dcb, dcs, (int64_t)cb.size(), dt, (int64_t)tiles.size(), in, out, cplx ? 1 : 0, CH);
  if (timed) {
    ctx->mark(1);
    ctx->mark(2);
  }
  dev_free(ctx, dd);
  if (dcb) dev_free(ctx, dcb);
  if (dcs) dev_free(ctx, dcs);
  if (dt) dev_free(ctx, dt);
}

// Rank-2 exemption of SkipZeroData (Source/QSpace.cc:3225-3229): zero blocks
// of a rank-2 QSpace are kept when it is block diagonal in vector storage or
// hermitian (isHConj, Source/QSpace.cc:1719-1775 -> isSym_aux :1802-).
static bool rank2_keeps_zero_blocks(const QMeta &m, const std::vector<double> &h) {
  const int qd = m.qdim;
  // 'd' storage: labels equal on both legs, every block a vector
  bool dstore = true;
  for (int64_t i = 0; i < m.nblk && dstore; ++i) {
    if (rec_compare(m.qrow(i), m.qrow(i) + qd, qd) != 0) dstore = false;
    const int64_t *d = m.drow(i);
    if (d[0] != 1 && d[1] != 1) dstore = false;
  }
  if (dstore) return true;
  // hermitian: the label set is invariant under leg swap, labels unique,
  // and data(i) == data(j)^H within 1e-14 * max(1, |A|)
  const int64_t n = m.nblk;
  const int w = 2 * qd;
  std::vector<int32_t> R(n * w), R2(n * w);
  for (int64_t i = 0; i < n; ++i) {
    std::memcpy(&R[i * w], m.qrow(i), w * 4);
    std::memcpy(&R2[i * w], m.qrow(i) + qd, qd * 4);
    std::memcpy(&R2[i * w + qd], m.qrow(i), qd * 4);
  }
  auto sp = [&](const std::vector<int32_t> &X) {
    std::vector<int64_t> p(n);
    std::iota(p.begin(), p.end(), 0);
    std::stable_sort(p.begin(), p.end(), [&](int64_t a, int64_t b) { return rec_compare(&X[a * w], &X[b * w], w) < 0; });
    return p;
  };
  std::vector<int64_t> p1 = sp(R), p2 = sp(R2);
  for (int64_t i = 0; i < n; ++i)
    if (rec_compare(&R[p1[i] * w], &R2[p2[i] * w], w) != 0) return false;
  for (int64_t i = 1; i < n; ++i)
    if (rec_compare(&R[p1[i] * w], &R[p1[i - 1] * w], w) == 0) return false;
  const int es = m.cplx ? 2 : 1;
  double nrm2 = 0;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = 0; e < m.bsize(i) * es; ++e) nrm2 += h[m.offs[i] * es + e] * h[m.offs[i] * es + e];
  const double deps = std::max(std::sqrt(nrm2), 1.0) * 1e-14;
  std::vector<int64_t> ip2(n);
  for (int64_t i = 0; i < n; ++i) ip2[p2[i]] = i;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t j = p1[ip2[i]];
    if (j < i) continue;
    const int64_t *di = m.drow(i), *dj = m.drow(j);
    if (di[0] != dj[1] || di[1] != dj[0]) return false;
    for (int64_t r = 0; r < di[0]; ++r)
      for (int64_t c = 0; c < di[1]; ++c) {
        const int64_t a = m.offs[i] + r + c * di[0], b = m.offs[j] + c + r * dj[0];
        const double re = h[a * es] - h[b * es];
        const double im = m.cplx ? h[a * es + 1] + h[b * es + 1] : 0.0;
        if (std::fabs(re) > deps || std::fabs(im) > deps) return false;
      }
  }
  return true;
}

static std::unique_ptr<qs_tensor> empty_tensor(Ctx *ctx, int rank, int qdim, bool cplx) {
  auto T = std::make_unique<qs_tensor>();
  T->ctx = ctx;
  T->meta.rank = rank;
  T->meta.qdim = qdim;
  T->meta.cplx = cplx;
  return T;
}

// ------------------------------------------------------ contraction driver
// A contraction in flight: its plan, operands in the layout and element type
// the plan wants, and its output arena before zero-block removal.
struct Prepared {
  ContractPlan pl;
  bool cplx = false;
  const double *a2 = nullptr, *b2 = nullptr;
  double *dC = nullptr;
  std::vector<void *> tmp;
  std::unique_ptr<qs_tensor> done;  // set when no product is needed
  // per pair: strided views of operands read in place instead of permuted
  // (split path; empty when neither operand needed a permutation)
  std::vector<OperandView> va, vb;
};

// The view of block `blk` of m whose lines run over `line_legs` and whose
// depth runs over `k_legs` (first leg fastest): the element order of the
// permuted copy that permute_to would make, read in place.
static bool make_view(const QMeta &m, int64_t blk, const std::vector<int> &line_legs, const std::vector<int> &k_legs,
                      OperandView &v) {
  v = OperandView{};
  // legs of size 1 do not move anything; drop them
  std::vector<int> ll, kl;
  for (int k : line_legs)
    if (m.drow(blk)[k] != 1) ll.push_back(k);
  for (int k : k_legs)
    if (m.drow(blk)[k] != 1) kl.push_back(k);
  if ((int)ll.size() > VIEW_LEGS || (int)kl.size() > VIEW_LEGS) return false;
  int64_t stride[16];
  int64_t sacc = 1;
  for (int k = 0; k < m.rank && k < 16; ++k) {
    stride[k] = sacc;
    sacc *= m.drow(blk)[k];
  }
  v.nl = (int32_t)ll.size();
  v.nk = (int32_t)kl.size();
  for (int i = 0; i < v.nl; ++i) {
    v.ldim[i] = (int32_t)m.drow(blk)[ll[i]];
    v.lstr[i] = stride[ll[i]];
  }
  for (int i = 0; i < v.nk; ++i) {
    v.kdim[i] = (int32_t)m.drow(blk)[kl[i]];
    v.kstr[i] = stride[kl[i]];
  }
  if (v.nl == 0) {  // a single line: one leg of size 1 keeps the view active
    v.nl = 1;
    v.ldim[0] = 1;
    v.lstr[0] = 0;
  }
  return true;
}

// The offsets sum_i l_i str[i] of the n-leg index space dim (first leg
// fastest) appended to `tab` (one entry for n = 0).
static void append_offsets(int n, const int32_t *dim, const int64_t *str, std::vector<int64_t> &tab) {
  int64_t count = 1;
  for (int i = 0; i < n; ++i) count *= dim[i];
  int32_t idx[VIEW_LEGS] = {0, 0, 0, 0};
  int64_t off = 0;
  for (int64_t e = 0; e < count; ++e) {
    tab.push_back(off);
    for (int i = 0; i < n; ++i) {  // odometer step
      off += str[i];
      if (++idx[i] < dim[i]) break;
      off -= str[i] * dim[i];
      idx[i] = 0;
    }
  }
}

// Plan on the host, then widen/permute the operands as the plan wants and
// allocate the output (kernels on ctx->stream).
static void prepare(Ctx *ctx, Prepared &w, const QMeta &Am, const double *dA, const QMeta &Bm,
                    const double *dB, const char *ia, const char *ib, const int32_t *perm, int32_t nperm,
                    bool views = false) {
  w.pl = plan_contract(Am, ia, Bm, ib, perm, nperm);
  ContractPlan &pl = w.pl;
  const bool cplx = w.cplx = pl.C.cplx;
  if (pl.C.nblk == 0) {
    // no matching sectors: an empty QSpace that still carries the itags
    w.done = empty_tensor(ctx, 0, Am.qdim, cplx);
    for (int k = 0; k < (int)pl.C.itags.size(); ++k)
      w.done->meta.itags.push_back(pl.C.itags[pl.P.empty() ? k : pl.P[k]]);
    return;
  }
  const int es = cplx ? 2 : 1;
  // The split path reads a permuted operand in place through per-pair
  // strided views (lines over the kept legs, depth over the contracted legs
  // in pairing order, the order of permute_to's copy) when every block's legs
  // fit a view; the FP64 path reads the permuted copy.
  // Deep output blocks are cut along their depth (split_deep), which needs
  // plain operands: such contractions read permuted copies.
  bool deep = views && has_deep_blocks(pl.pairs, pl.grp, pl.blk_M, pl.blk_N);
  // likewise contractions whose blocks are all shallow (computed directly
  // from plain operands)
  if (views && !deep) {
    bool all_shallow = true;
    for (size_t b = 0; b + 1 < pl.grp.size() && all_shallow; ++b)
      all_shallow = is_shallow(pl.pairs, pl.grp[b], pl.grp[b + 1]) &&
                    shallow_direct_wins(pl.pairs, pl.grp[b], pl.grp[b + 1], pl.blk_M[b], pl.blk_N[b], w.cplx);
    deep = all_shallow;
  }
  // the views' offset tables, one pair of tables per operand block (every
  // pair reading the block shares them): all in one upload
  std::vector<int64_t> vtab;
  std::vector<std::pair<int64_t, int64_t>> toff_a, toff_b;  // per pair: (line, depth) table starts
  auto fused = [&](const QMeta &m, bool is_a, std::vector<OperandView> &out) -> bool {
    const OperandLayout &lay = is_a ? pl.la : pl.lb;
    if (!views || deep || !lay.permute) return false;
    const std::vector<int> &lines = is_a ? pl.ika : pl.ikb;
    const std::vector<int> &ks = is_a ? pl.ica.idx : pl.icb.idx;
    std::vector<OperandView> v(pl.pairs.size());
    std::vector<std::pair<int64_t, int64_t>> toff(pl.pairs.size());
    std::unordered_map<int64_t, size_t> first;  // block -> first pair that reads it
    const size_t tab0 = vtab.size();
    for (size_t p = 0; p < pl.pairs.size(); ++p) {
      const int64_t blk = is_a ? pl.pair_ia[p] : pl.pair_ib[p];
      auto it = first.find(blk);
      if (it != first.end()) {
        v[p] = v[it->second];
        toff[p] = toff[it->second];
        continue;
      }
      if (!make_view(m, blk, lines, ks, v[p])) {
        vtab.resize(tab0);
        return false;
      }
      toff[p] = {(int64_t)vtab.size(), 0};
      append_offsets(v[p].nl, v[p].ldim, v[p].lstr, vtab);
      toff[p].second = (int64_t)vtab.size();
      append_offsets(v[p].nk, v[p].kdim, v[p].kstr, vtab);
      first.emplace(blk, p);
    }
    out.swap(v);
    (is_a ? toff_a : toff_b).swap(toff);
    // the permuted copy would have been conjugated: conjugate on the fly.
    // XOR, not OR: the conjugation flag may be set as well (the auto-conj
    // rule of contract_getIdxSet, after permute_to flipped the copy's itags),
    // and the two conjugations then cancel, as they do for the copy
    if (lay.conj)
      for (PairDesc &d : pl.pairs) d.trans ^= is_a ? 4 : 8;
    return true;
  };
  const bool fa = fused(Am, true, w.va), fb = fused(Bm, false, w.vb);
  if (!vtab.empty()) {
    const int64_t *d_tab = dev_upload(ctx, vtab);
    w.tmp.push_back(const_cast<int64_t *>(d_tab));
    for (size_t p = 0; p < w.va.size(); ++p) {
      w.va[p].ltab = d_tab + toff_a[p].first;
      w.va[p].ktab = d_tab + toff_a[p].second;
    }
    for (size_t p = 0; p < w.vb.size(); ++p) {
      w.vb[p].ltab = d_tab + toff_b[p].first;
      w.vb[p].ktab = d_tab + toff_b[p].second;
    }
  }
  auto prep = [&](const QMeta &m, const double *d, const OperandLayout &lay, bool in_place) -> const double * {
    const double *cur = d;
    if (cplx && !m.cplx) {
      double *x = dev_alloc<double>(ctx, (size_t)m.nelem * 2);
      w.tmp.push_back(x);
      launch_widen(ctx, d, x, m.nelem);
      cur = x;
    }
    if (lay.permute && !in_place) {
      double *o = dev_alloc<double>(ctx, (size_t)m.nelem * es);
      w.tmp.push_back(o);
      std::vector<PermDesc> pd = make_perm_descs(m, lay.perm, lay.conj, m.offs);
      run_permute(ctx, pd, cur, o, cplx);
      cur = o;
    }
    return cur;
  };
  w.a2 = prep(Am, dA, pl.la, fa);
  w.b2 = prep(Bm, dB, pl.lb, fb);
  w.dC = dev_alloc<double>(ctx, (size_t)pl.C.nelem * es);
}

// All block products of a batch of prepared contractions of one element type
// in one grouped launch.  The operands and outputs of different
// contractions are separate arenas in the device's one address space:
// their element offsets are taken relative to the lowest address of each
// kind, so that one pair list addresses all of them.  forced_slices /
// forced_bits (0: none) fix the split path's digit plan.
static void run_products(Ctx *ctx, const std::vector<Prepared *> &batch, const qs_opts *opts, qs_stats *stats,
                         int forced_slices = 0, int forced_bits = 0) {
  if (batch.empty()) return;
  const bool cplx = batch[0]->cplx;
  const int64_t eb = cplx ? 16 : 8;
  const double *baseA = batch[0]->a2, *baseB = batch[0]->b2;
  double *baseC = batch[0]->dC;
  for (Prepared *w : batch) {
    if (w->cplx != cplx) fail(QS_ERR_INTERNAL, "batched products of mixed element types");
    baseA = std::min(baseA, w->a2);
    baseB = std::min(baseB, w->b2);
    baseC = std::min(baseC, w->dC);
  }
  auto rel = [&](const void *p, const void *base) {
    const int64_t d = (int64_t)((const char *)p - (const char *)base);
    if (d % eb) fail(QS_ERR_INTERNAL, "misaligned arena in a batched launch");
    return d / eb;
  };
  std::vector<PairDesc> pairs;
  std::vector<int64_t> grp{0}, c_off;
  std::vector<int32_t> bM, bN;
  std::vector<OperandView> va, vb;
  bool any_view = false;
  for (Prepared *w : batch) any_view = any_view || !w->va.empty() || !w->vb.empty();
  for (Prepared *w : batch) {
    const ContractPlan &pl = w->pl;
    const int64_t da = rel(w->a2, baseA), db = rel(w->b2, baseB), dc = rel(w->dC, baseC);
    for (size_t p = 0; p < pl.pairs.size(); ++p) {
      PairDesc d = pl.pairs[p];
      d.a_off += da;
      d.b_off += db;
      pairs.push_back(d);
      if (any_view) {
        va.push_back(w->va.empty() ? OperandView{} : w->va[p]);
        vb.push_back(w->vb.empty() ? OperandView{} : w->vb[p]);
      }
    }
    for (size_t b = 0; b + 1 < pl.grp.size(); ++b) grp.push_back(grp.back() + (pl.grp[b + 1] - pl.grp[b]));
    for (size_t b = 0; b < pl.blk_M.size(); ++b) {
      bM.push_back(pl.blk_M[b]);
      bN.push_back(pl.blk_N[b]);
      c_off.push_back(pl.C.offs[b] + dc);
    }
  }
  const int prec = opts ? opts->prec : QS_PREC_FP64;
  if (prec == QS_PREC_SPLIT) {
    SplitResult sr = run_split(ctx, pairs, grp, bM, bN, c_off, baseA, baseB, baseC, cplx,
                               forced_slices ? forced_slices : (opts ? opts->nslices : 0),
                               opts && opts->tol > 0 ? opts->tol : 1e-12, nullptr, forced_bits,
                               any_view ? &va : nullptr, any_view ? &vb : nullptr);
    if (stats) {
      stats->nslices = sr.nslices;
      stats->digit_bits = sr.bits;
      stats->err_bound = sr.err_bound;
    }
  } else if (prec == QS_PREC_FP64) {
    if (any_view) fail(QS_ERR_INTERNAL, "FP64 products of operands read through views");
    run_f64(ctx, pairs, grp, bM, bN, c_off, nullptr, baseA, baseB, baseC, cplx);
  } else {
    fail(QS_ERR_ARG, "unknown precision mode %d", prec);
  }
  for (Prepared *w : batch) {
    for (void *p : w->tmp) dev_free(ctx, p);
    w->tmp.clear();
  }
}

// SkipZeroData of every contraction of the batch (one test launch, one
// synchronisation), then the final Permute(P) and the result tensors.
static void finish(Ctx *ctx, const std::vector<Prepared *> &batch) {
  if (batch.empty()) return;
  std::vector<int64_t> offs, sizes;
  std::vector<int64_t> first(batch.size() + 1, 0);
  double *base = batch[0]->dC;
  for (Prepared *w : batch) base = std::min(base, w->dC);
  const int64_t eb = batch[0]->cplx ? 16 : 8;
  for (size_t r = 0; r < batch.size(); ++r) {
    const ContractPlan &pl = batch[r]->pl;
    const int64_t dc = (int64_t)((const char *)batch[r]->dC - (const char *)base) / eb;
    for (int64_t i = 0; i < pl.C.nblk; ++i) {
      offs.push_back(pl.C.offs[i] + dc);
      sizes.push_back(pl.C.bsize(i));
    }
    first[r + 1] = (int64_t)offs.size();
  }
  const int64_t nb = (int64_t)offs.size();
  int64_t *doff = dev_upload(ctx, offs), *dsz = dev_upload(ctx, sizes);
  int *dflag = dev_alloc<int>(ctx, nb);
  launch_block_nonzero(ctx, doff, dsz, nb, base, batch[0]->cplx ? 1 : 0, dflag);
  std::vector<int> flags(nb);
  int kerr = 0;
  QS_CUDA(cudaMemcpyAsync(flags.data(), dflag, nb * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaMemcpyAsync(&kerr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, doff);
  dev_free(ctx, dsz);
  dev_free(ctx, dflag);
  if (kerr) {
    QS_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    fail(QS_ERR_TIMEOUT, "a bounded device wait ran out (code %d)", kerr);
  }
  for (size_t r = 0; r < batch.size(); ++r) {
    Prepared &w = *batch[r];
    const ContractPlan &pl = w.pl;
    const bool cplx = w.cplx;
    const int es = cplx ? 2 : 1;
    const int64_t nbr = pl.C.nblk;
    std::vector<int64_t> keep;
    for (int64_t i = 0; i < nbr; ++i)
      if (flags[first[r] + i]) keep.push_back(i);
    if ((int64_t)keep.size() < nbr && pl.rc == 2) {
      std::vector<double> h((size_t)pl.C.nelem * es);
      QS_CUDA(cudaMemcpyAsync(h.data(), w.dC, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
      QS_CUDA(cudaStreamSynchronize(ctx->stream));
      if (rank2_keeps_zero_blocks(pl.C, h)) {
        keep.resize(nbr);
        std::iota(keep.begin(), keep.end(), 0);
      }
    }
    auto T = std::make_unique<qs_tensor>();
    T->ctx = ctx;
    QMeta &M = T->meta;
    M.rank = pl.rc;
    M.qdim = pl.C.qdim;
    // output itags, permuted like the legs (QSpace::Permute)
    if (!pl.C.itags.empty()) {
      if (pl.P.empty()) M.itags = pl.C.itags;
      else
        for (int k = 0; k < pl.rc; ++k) M.itags.push_back(pl.C.itags[pl.P[k]]);
    }
    M.cplx = cplx;
    M.nblk = (int64_t)keep.size();
    const int rk = pl.rc, qd = pl.C.qdim;
    if (keep.empty()) {
      dev_free(ctx, w.dC);
      w.dC = nullptr;
      M.rank = 0;
    } else if (pl.P.empty()) {
      for (int64_t i : keep) {
        M.q.insert(M.q.end(), pl.C.qrow(i), pl.C.qrow(i) + rk * qd);
        M.dims.insert(M.dims.end(), pl.C.drow(i), pl.C.drow(i) + rk);
        M.offs.push_back(pl.C.offs[i]);
      }
      M.nelem = pl.C.nelem;
      T->d = w.dC;
      w.dC = nullptr;
    } else {
      // Permute(P) of labels and data (Source/QSpace.hh:2670-2719); the block
      // order is not changed.
      std::vector<int64_t> noffs;
      int64_t ne = 0;
      for (int64_t i : keep) {
        for (int k = 0; k < rk; ++k) {
          const int32_t *src = pl.C.qrow(i) + pl.P[k] * qd;
          M.q.insert(M.q.end(), src, src + qd);
          M.dims.push_back(pl.C.drow(i)[pl.P[k]]);
        }
        noffs.push_back(ne);
        ne += pl.C.bsize(i);
      }
      M.offs = noffs;
      M.nelem = ne;
      double *dP = dev_alloc<double>(ctx, (size_t)ne * es);
      std::vector<PermDesc> pd = make_perm_descs(pl.C, pl.P, false, noffs, &keep);
      run_permute(ctx, pd, w.dC, dP, cplx);
      dev_free(ctx, w.dC);
      w.dC = nullptr;
      T->d = dP;
    }
    w.done = std::move(T);
  }
}

static void release(Ctx *ctx, Prepared &w) {
  for (void *p : w.tmp) dev_free(ctx, p);
  w.tmp.clear();
  if (w.dC) dev_free(ctx, w.dC);
  w.dC = nullptr;
}

// The device contraction driver shared by the host and device entry points.
std::unique_ptr<qs_tensor> contract_core(Ctx *ctx, const QMeta &Am, const double *dA,
                                                const QMeta &Bm, const double *dB, const char *ia,
                                                const char *ib, const int32_t *perm, int32_t nperm,
                                                const qs_opts *opts, qs_stats *stats) {
  const int64_t launches0 = ctx->launches;
  Prepared w;
  if (stats) std::memset(stats, 0, sizeof *stats);
  try {
    prepare(ctx, w, Am, dA, Bm, dB, ia, ib, perm, nperm, opts && opts->prec == QS_PREC_SPLIT);
    if (stats) {
      stats->flops = w.pl.flops;
      stats->bytes = w.pl.bytes;
      stats->npairs = (int64_t)w.pl.pairs.size();
    }
    if (!w.done) {
      std::vector<Prepared *> one{&w};
      run_products(ctx, one, opts, stats);
      finish(ctx, one);
    }
  } catch (...) {
    release(ctx, w);
    throw;
  }
  if (stats) {
    stats->nblk_out = w.done->meta.nblk;
    stats->launches = (int32_t)(ctx->launches - launches0);
  }
  return std::move(w.done);
}

// A batch of contractions: the block products of all of them run in one
// grouped launch per result element type and, on the split path, per digit
// plan -- each contraction keeps the plan it would get alone, so every
// result is bit-identical to the same contraction run alone.  out[r]
// receives contraction r's result.
void contract_batch_core(Ctx *ctx, int n, const QMeta *const *Am, const double *const *dA,
                         const QMeta *const *Bm, const double *const *dB, const char *const *ia,
                         const char *const *ib, const int32_t *const *perm, const int32_t *nperm,
                         const qs_opts *opts, std::vector<std::unique_ptr<qs_tensor>> &out) {
  std::vector<Prepared> ws(n);
  try {
    const bool split = opts && opts->prec == QS_PREC_SPLIT;
    for (int r = 0; r < n; ++r)
      prepare(ctx, ws[r], *Am[r], dA[r], *Bm[r], dB[r], ia[r], ib[r], perm ? perm[r] : nullptr,
              nperm ? nperm[r] : 0, split);
    std::vector<std::pair<int, int>> plan(n, {0, 0});  // (slices, bits)
    if (split)
      for (int r = 0; r < n; ++r)
        if (!ws[r].done) {
          const ContractPlan &pl = ws[r].pl;
          const DigitPlan dp = choose_digits_for(pl.pairs, pl.grp, pl.blk_M, pl.blk_N, ws[r].cplx ? 2 : 1,
                                                 opts->tol > 0 ? opts->tol : 1e-12, opts->nslices);
          plan[r] = {dp.nslices, dp.bits};
        }
    std::vector<char> ran(n, 0);
    for (int r = 0; r < n; ++r) {
      if (ws[r].done || ran[r]) continue;
      std::vector<Prepared *> batch;
      for (int q = r; q < n; ++q)
        if (!ws[q].done && !ran[q] && ws[q].cplx == ws[r].cplx && plan[q] == plan[r]) {
          batch.push_back(&ws[q]);
          ran[q] = 1;
        }
      run_products(ctx, batch, opts, nullptr, plan[r].first, plan[r].second);
      finish(ctx, batch);
    }
  } catch (...) {
    for (Prepared &w : ws) release(ctx, w);
    throw;
  }
  out.clear();
  for (Prepared &w : ws) out.push_back(std::move(w.done));
}

int64_t contract_footprint(const QMeta &Am, const QMeta &Bm, const char *ia, const char *ib,
                           const qs_opts *opts) {
  ContractPlan pl = plan_contract(Am, ia, Bm, ib, nullptr, 0);
  const int64_t es = pl.C.cplx ? 16 : 8;
  int64_t fp = pl.C.nelem * es * 2;  // result, and its permuted copy
  if (pl.la.permute || (pl.C.cplx && !Am.cplx)) fp += Am.nelem * es * 2;
  if (pl.lb.permute || (pl.C.cplx && !Bm.cplx)) fp += Bm.nelem * es * 2;
  if (opts && opts->prec == QS_PREC_SPLIT) {
    // at most 8 BF16 digits of every pair operand in the real form (2M x 2K
    // and 2K x N when complex), padded to 128 x 32 / 32 x 32 tiles
    const int64_t cm = pl.C.cplx ? 2 : 1;
    for (const PairDesc &d : pl.pairs) {
      const int64_t Kr = std::max<int64_t>(d.K * cm, 1);
      const int64_t rows = (d.M * cm + 127) / 128 * 128 + (d.N + 31) / 32 * 32;
      fp += rows * ((Kr + 31) / 32 * 32) * 2 * 8;
    }
  }
  return fp;
}

static std::unique_ptr<qs_tensor> upload(Ctx *ctx, const qs_qspace_view *v) {
  QMeta m = meta_from_view(v);
  auto T = std::make_unique<qs_tensor>();
  T->ctx = ctx;
  T->meta = m;
  const size_t n = (size_t)m.nelem * (m.cplx ? 2 : 1);
  T->d = dev_alloc<double>(ctx, n);
  if (n) {
    QS_CUDA(cudaMemcpyAsync(T->d, v->data, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    // the caller may release its host buffer when the call returns, and a copy
    // from pageable memory may still read it later (the GPU can read host
    // memory directly): wait until the copy has read it
    QS_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return T;
}

static qs_result *download(Ctx *ctx, const qs_tensor *T) {
  auto R = std::make_unique<qs_result>();
  const QMeta &m = T->meta;
  R->meta = m;
  const int es = m.cplx ? 2 : 1;
  std::vector<double> h((size_t)m.nelem * es);
  if (!h.empty()) {
    QS_CUDA(cudaMemcpyAsync(h.data(), T->d, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  int64_t ne = 0;
  for (int64_t i = 0; i < m.nblk; ++i) ne += m.bsize(i);
  R->data.resize((size_t)ne * es);
  R->meta.nelem = ne;
  int64_t o = 0;
  for (int64_t i = 0; i < m.nblk; ++i) {
    const int64_t s = m.bsize(i);
    if (s) std::memcpy(&R->data[o * es], &h[m.offs[i] * es], s * es * 8);
    R->meta.offs[i] = o;
    o += s;
  }
  return R.release();
}

}  // namespace qs

// ------------------------------------------------- itag chain contraction
// Legs of A and B that contract (Source/wbindex.cc:1512-1595, iTags::getCtr,
// with itag_::sameAs :989-1007): the same tag name with opposite directions,
// or with equal directions when exactly one of the two operands carries a
// conj flag.  When nothing matches that way the other polarity is used and
// A's conj flag is toggled (the reference does so after a warning).
static void itag_pairs(const QMeta &A, bool ca, const QMeta &B, bool cb, std::vector<int> &ia,
                       std::vector<int> &ib, bool &flipA) {
  const int ra = A.rank, rb = B.rank;
  if ((int)A.itags.size() != ra || (int)B.itags.size() != rb)
    fail(QS_ERR_LABEL, "itag contraction needs itags on every leg ('%s' <> '%s')", join_itags(A.itags).c_str(),
         join_itags(B.itags).c_str());
  auto name = [](const std::string &t) { return t.substr(0, t.find('*')); };
  auto dir = [](const std::string &t) { return t.find('*') != std::string::npos; };
  for (const std::string &t : A.itags)
    if (name(t).empty()) fail(QS_ERR_LABEL, "itag contraction needs non-empty itags");
  for (const std::string &t : B.itags)
    if (name(t).empty()) fail(QS_ERR_LABEL, "itag contraction needs non-empty itags");
  std::vector<int> ma(ra, 0), mb(rb, 0);
  int nc = 0, e = 0, it = 0;
  bool cflag = ca != cb;
  for (; it < 2; ++it) {
    const int q = cflag ? 1 : -1;
    for (int i = 0; i < ra; ++i)
      for (int j = 0; j < rb; ++j) {
        if (name(A.itags[i]) != name(B.itags[j])) continue;
        const int sgn = dir(A.itags[i]) != dir(B.itags[j]) ? -1 : 1;
        if (sgn != q) continue;
        if (!ma[i] && !mb[j]) {
          ma[i] = j + 1;
          mb[j] = i + 1;
          ++nc;
        } else {
          ++e;
        }
      }
    if (nc || e) break;
    cflag = !cflag;
  }
  if (e)
    fail(QS_ERR_LABEL, "itag contraction: non-unique itags ('%s' <> '%s')", join_itags(A.itags).c_str(),
         join_itags(B.itags).c_str());
  if (!nc)
    fail(QS_ERR_LABEL, "itag contraction: no matching itags ('%s' <> '%s')", join_itags(A.itags).c_str(),
         join_itags(B.itags).c_str());
  ia.clear();
  ib.clear();
  for (int i = 0; i < ra; ++i)
    if (ma[i]) {
      ia.push_back(i + 1);
      ib.push_back(ma[i]);
    }
  flipA = it == 1;
}

static std::string idx_string(const std::vector<int> &ix, bool conj) {
  std::string s = "[";
  for (int i : ix) s += std::to_string(i) + " ";
  s += "]";
  if (conj) s += "*";
  return s;
}

// Cell contraction {X_0, ..., X_{n-1}} (Source/contractQS.cc:634-808,
// contractQS_itags): right to left, C = X_{n-1}; C = X_k * C for k = n-2..0
// over the legs matched by itag; the permutation applies to the final result;
// an empty operand makes the result empty.
static std::unique_ptr<qs_tensor> contract_itags_core(Ctx *ctx, int n, const qs_tensor *const *T,
                                                      const int32_t *conj, const int32_t *perm, int32_t nperm,
                                                      const qs_opts *opts) {
  if (n < 2) fail(QS_ERR_ARG, "itag contraction needs at least two tensors");
  for (int k = 0; k < n; ++k)
    if (!T[k]) fail(QS_ERR_ARG, "null tensor %d", k);
  std::unique_ptr<qs_tensor> cur;
  const QMeta *Bm = &T[n - 1]->meta;
  const double *Bd = T[n - 1]->d;
  bool cb = conj && conj[n - 1];
  for (int k = n - 2; k >= 0; --k) {
    const qs_tensor *A = T[k];
    const bool ca = conj && conj[k];
    if (A->meta.nblk == 0 || Bm->nblk == 0) {
      auto E = std::make_unique<qs_tensor>();
      E->ctx = ctx;
      return E;
    }
    std::vector<int> ia, ib;
    bool flip = false;
    itag_pairs(A->meta, ca, *Bm, cb, ia, ib, flip);
    const std::string sa = idx_string(ia, ca != flip), sb = idx_string(ib, cb);
    auto C = contract_core(ctx, A->meta, A->d, *Bm, Bd, sa.c_str(), sb.c_str(), k == 0 ? perm : nullptr,
                           k == 0 ? nperm : 0, opts, nullptr);
    cur = std::move(C);
    Bm = &cur->meta;
    Bd = cur->d;
    cb = false;
  }
  return cur;
}

// ======================================================================= C-ABI
extern "C" {

const char *qs_last_error(void) { return qs::last_error().c_str(); }
const char *qs_version(void) { return "qsgpu 0.1 (sm_103a)"; }

qs_status qs_ctx_create(int device, qs_ctx **out) {
  QS_API_BEGIN
  if (!out) fail(QS_ERR_ARG, "null out");
  auto c = std::make_unique<qs_ctx>();
  c->c.device = device;
  QS_CUDA(cudaSetDevice(device));
  QS_CUDA(cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking));
  QS_CUDA(cudaDeviceGetAttribute(&c->c.num_sms, cudaDevAttrMultiProcessorCount, device));
  // keep freed stream-ordered memory cached in the pool between calls
  cudaMemPool_t pool;
  QS_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t thr = UINT64_MAX;
  QS_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  QS_CUDA(cudaMalloc(&c->c.d_err, 64));
  QS_CUDA(cudaMemset(c->c.d_err, 0, 64));
  ctx_register(&c->c);
  *out = c.release();
  QS_API_END
}

void qs_ctx_destroy(qs_ctx *ctx) {
  if (!ctx) return;
  ctx_unregister(&ctx->c);
  cudaSetDevice(ctx->c.device);
  xcache_orphan_all(&ctx->c);
  if (ctx->c.scratch) cudaFreeAsync(ctx->c.scratch, ctx->c.stream);
  destroy_solver(&ctx->c);
  cudaStreamSynchronize(ctx->c.stream);
  if (ctx->c.d_err) cudaFree(ctx->c.d_err);
  for (auto &e : ctx->c.ev)
    if (e) cudaEventDestroy(e);
  ctx->c.destroy_copy_streams();
  ctx->c.destroy_staging();
  cudaStreamDestroy(ctx->c.stream);
  delete ctx;
}

void *qs_ctx_stream(qs_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

qs_status qs_ctx_sync(qs_ctx *ctx) {
  QS_API_BEGIN
  if (!ctx) fail(QS_ERR_ARG, "null ctx");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  QS_CUDA(cudaStreamSynchronize(ctx->c.stream));
  // a bounded device wait that ran out in an asynchronous call is reported here
  int kerr = 0;
  QS_CUDA(cudaMemcpy(&kerr, ctx->c.d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (kerr) {
    QS_CUDA(cudaMemset(ctx->c.d_err, 0, sizeof(int)));
    fail(QS_ERR_TIMEOUT, "a bounded device wait ran out (code %d)", kerr);
  }
  QS_API_END
}

int64_t qs_ctx_launches(const qs_ctx *ctx) { return ctx ? ctx->c.launches : 0; }

qs_status qs_ctx_set_timing(qs_ctx *ctx, int32_t enable) {
  QS_API_BEGIN
  if (!ctx) fail(QS_ERR_ARG, "null ctx");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  for (auto &e : ctx->c.ev)
    if (!e) QS_CUDA(cudaEventCreate(&e));
  ctx->c.timing = enable != 0;
  ctx->c.ev_used = false;
  QS_API_END
}

qs_status qs_ctx_phase_ms(qs_ctx *ctx, double *prep_ms, double *gemm_ms) {
  QS_API_BEGIN
  if (!ctx) fail(QS_ERR_ARG, "null ctx");
  if (!ctx->c.ev_used) fail(QS_ERR_ARG, "no timed call on this context");
  QS_CUDA(cudaEventSynchronize(ctx->c.ev[2]));
  float a = 0, b = 0;
  QS_CUDA(cudaEventElapsedTime(&a, ctx->c.ev[0], ctx->c.ev[1]));
  QS_CUDA(cudaEventElapsedTime(&b, ctx->c.ev[1], ctx->c.ev[2]));
  if (prep_ms) *prep_ms = a;
  if (gemm_ms) *gemm_ms = b;
  QS_API_END
}

qs_status qs_contractQS(qs_ctx *ctx, const qs_qspace_view *A, const char *ia,
                        const qs_qspace_view *B, const char *ib, const int32_t *perm,
                        int32_t nperm, const qs_opts *opts, qs_result **C, qs_stats *stats) {
  QS_API_BEGIN
  if (!ctx || !C) fail(QS_ERR_ARG, "null argument");
  *C = nullptr;
  QS_CUDA(cudaSetDevice(ctx->c.device));
  auto tA = upload(&ctx->c, A);
  auto tB = upload(&ctx->c, B);
  auto tC = contract_core(&ctx->c, tA->meta, tA->d, tB->meta, tB->d, ia, ib, perm, nperm, opts, stats);
  *C = download(&ctx->c, tC.get());
  QS_API_END
}

qs_status qs_result_info(const qs_result *C, int32_t *rank, int32_t *qdim, int64_t *nblk,
                         int64_t *nelem, int32_t *is_complex) {
  QS_API_BEGIN
  if (!C) fail(QS_ERR_ARG, "null result");
  if (rank) *rank = C->meta.rank;
  if (qdim) *qdim = C->meta.qdim;
  if (nblk) *nblk = C->meta.nblk;
  if (nelem) *nelem = C->meta.nelem;
  if (is_complex) *is_complex = C->meta.cplx ? 1 : 0;
  QS_API_END
}

qs_status qs_result_copy(const qs_result *C, int32_t *q, int64_t *dims, int64_t *offs, double *data) {
  QS_API_BEGIN
  if (!C) fail(QS_ERR_ARG, "null result");
  const QMeta &m = C->meta;
  if (q && !m.q.empty()) std::memcpy(q, m.q.data(), m.q.size() * 4);
  if (dims && !m.dims.empty()) std::memcpy(dims, m.dims.data(), m.dims.size() * 8);
  if (offs && !m.offs.empty()) std::memcpy(offs, m.offs.data(), m.offs.size() * 8);
  if (data && !C->data.empty()) std::memcpy(data, C->data.data(), C->data.size() * 8);
  QS_API_END
}

void qs_result_free(qs_result *C) { delete C; }

qs_status qs_tensor_upload(qs_ctx *ctx, const qs_qspace_view *A, qs_tensor **out) {
  QS_API_BEGIN
  if (!ctx || !out) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  *out = upload(&ctx->c, A).release();
  QS_API_END
}

qs_status qs_tensor_info(const qs_tensor *T, int32_t *rank, int32_t *qdim, int64_t *nblk,
                         int64_t *nelem, int32_t *is_complex) {
  QS_API_BEGIN
  if (!T) fail(QS_ERR_ARG, "null tensor");
  int64_t ne = 0;
  for (int64_t i = 0; i < T->meta.nblk; ++i) ne += T->meta.bsize(i);
  if (rank) *rank = T->meta.rank;
  if (qdim) *qdim = T->meta.qdim;
  if (nblk) *nblk = T->meta.nblk;
  if (nelem) *nelem = ne;
  if (is_complex) *is_complex = T->meta.cplx ? 1 : 0;
  QS_API_END
}

qs_status qs_tensor_download(qs_ctx *ctx, const qs_tensor *T, int32_t *q, int64_t *dims,
                             int64_t *offs, double *data) {
  QS_API_BEGIN
  if (!ctx || !T) fail(QS_ERR_ARG, "null argument");
  std::unique_ptr<qs_result> R(download(&ctx->c, T));
  return qs_result_copy(R.get(), q, dims, offs, data);
  QS_API_END
}

// C = A + bfac B for device tensors (plusQS, Source/plusQS.cc:11-45 ->
// QSpace::plus_plain, Source/QSpace.cc:3593-3700): blocks of the union of both
// label sets in lexicographic order of their label records (getQOverlapU:
// cat + groupRecs), each the sum of the blocks present, then SkipZeroData
// with its rank-2 exemption.  Abelian QSpaces; an empty operand contributes
// nothing; itags from the operand that has them (both: they must agree).
static std::unique_ptr<qs_tensor> plus_core(Ctx *ctx, const qs_tensor *A, const qs_tensor *B, double bfac) {
  const QMeta &a = A->meta, &b = B->meta;
  const bool ea = a.nblk == 0, eb = b.nblk == 0;
  if (!ea && !eb && (a.rank != b.rank || a.qdim != b.qdim))
    fail(QS_ERR_SHAPE, "plusQS: QSpace mismatch (QDIM=%d/%d; r=%d/%d)", a.qdim, b.qdim, a.rank, b.rank);
  std::vector<std::string> tags = a.itags;
  if (tags.empty()) tags = b.itags;
  else if (!b.itags.empty() && b.itags != a.itags)
    fail(QS_ERR_LABEL, "plusQS: inconsistent itags %s <> %s", join_itags(a.itags).c_str(), join_itags(b.itags).c_str());
  const int rank = ea ? b.rank : a.rank, qd = ea ? b.qdim : a.qdim, w = rank * qd;
  const bool cplx = a.cplx || b.cplx;
  const int es = cplx ? 2 : 1;
  // union of the label records (A's first), sorted, equal records grouped
  struct Rec { const int32_t *q; int src; int64_t i; };
  std::vector<Rec> all;
  for (int64_t i = 0; i < a.nblk; ++i) all.push_back({a.qrow(i), 0, i});
  for (int64_t i = 0; i < b.nblk; ++i) all.push_back({b.qrow(i), 1, i});
  std::stable_sort(all.begin(), all.end(), [&](const Rec &x, const Rec &y) { return rec_compare(x.q, y.q, w) < 0; });
  auto T = std::make_unique<qs_tensor>();
  T->ctx = ctx;
  QMeta &M = T->meta;
  M.rank = rank;
  M.qdim = qd;
  M.cplx = cplx;
  M.itags = tags;
  std::vector<int64_t> sa, da, za, sb, db, zb;
  int64_t off = 0, mxa = 1, mxb = 1;
  for (size_t k = 0; k < all.size();) {
    size_t e = k + 1;
    while (e < all.size() && rec_compare(all[e].q, all[k].q, w) == 0) ++e;
    if (e - k > 2 || (e - k == 2 && all[k].src == all[k + 1].src))
      fail(QS_ERR_LABEL, "plusQS: non-unique block labels");
    const QMeta &m0 = all[k].src ? b : a;
    const int64_t *d0 = m0.drow(all[k].i);
    if (e - k == 2) {
      const QMeta &m1 = all[k + 1].src ? b : a;
      const int64_t *d1 = m1.drow(all[k + 1].i);
      for (int r = 0; r < rank; ++r)
        if (d0[r] != d1[r]) fail(QS_ERR_SHAPE, "plusQS: block dims differ on leg %d (%lld/%lld)", r + 1, (long long)d0[r], (long long)d1[r]);
    }
    M.q.insert(M.q.end(), all[k].q, all[k].q + w);
    M.dims.insert(M.dims.end(), d0, d0 + rank);
    M.offs.push_back(off);
    const int64_t sz = m0.bsize(all[k].i);
    for (size_t j = k; j < e; ++j) {
      const QMeta &mj = all[j].src ? b : a;
      (all[j].src ? sb : sa).push_back(mj.offs[all[j].i]);
      (all[j].src ? db : da).push_back(off);
      (all[j].src ? zb : za).push_back(sz);
      (all[j].src ? mxb : mxa) = std::max(all[j].src ? mxb : mxa, sz);
    }
    off += sz;
    k = e;
  }
  M.nblk = (int64_t)M.offs.size();
  M.nelem = off;
  T->d = dev_alloc<double>(ctx, (size_t)std::max<int64_t>(off, 1) * es);
  QS_CUDA(cudaMemsetAsync(T->d, 0, (size_t)std::max<int64_t>(off, 1) * es * 8, ctx->stream));
  auto add = [&](const std::vector<int64_t> &so, const std::vector<int64_t> &dof, const std::vector<int64_t> &sz,
                 int64_t mx, const qs_tensor *X, double f) {
    if (so.empty()) return;
    int64_t *d1 = dev_upload(ctx, so), *d2 = dev_upload(ctx, dof), *d3 = dev_upload(ctx, sz);
    for (int64_t c0 = 0; c0 < (int64_t)so.size(); c0 += 65535)
      launch_block_axpy(ctx, d1 + c0, d2 + c0, d3 + c0, std::min<int64_t>(65535, (int64_t)so.size() - c0), mx, X->d,
                        T->d, f, X->meta.cplx ? 2 : 1, es);
    dev_free(ctx, d1);
    dev_free(ctx, d2);
    dev_free(ctx, d3);
  };
  add(sa, da, za, mxa, A, 1.0);
  add(sb, db, zb, mxb, B, bfac);
  if (M.nblk == 0) return T;
  // SkipZeroData
  std::vector<int64_t> sizes(M.nblk);
  for (int64_t i = 0; i < M.nblk; ++i) sizes[i] = M.bsize(i);
  int64_t *doff = dev_upload(ctx, M.offs), *dsz = dev_upload(ctx, sizes);
  int *dflag = dev_alloc<int>(ctx, M.nblk);
  launch_block_nonzero(ctx, doff, dsz, M.nblk, T->d, cplx ? 1 : 0, dflag);
  std::vector<int> flags(M.nblk);
  QS_CUDA(cudaMemcpyAsync(flags.data(), dflag, M.nblk * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, doff);
  dev_free(ctx, dsz);
  dev_free(ctx, dflag);
  std::vector<int64_t> keep;
  for (int64_t i = 0; i < M.nblk; ++i)
    if (flags[i]) keep.push_back(i);
  if ((int64_t)keep.size() < M.nblk && rank == 2) {
    std::vector<double> h((size_t)M.nelem * es);
    QS_CUDA(cudaMemcpyAsync(h.data(), T->d, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QS_CUDA(cudaStreamSynchronize(ctx->stream));
    if (rank2_keeps_zero_blocks(M, h)) {
      keep.resize(M.nblk);
      std::iota(keep.begin(), keep.end(), 0);
    }
  }
  if ((int64_t)keep.size() < M.nblk) {
    QMeta K = M;
    K.q.clear();
    K.dims.clear();
    K.offs.clear();
    for (int64_t i : keep) {
      K.q.insert(K.q.end(), M.qrow(i), M.qrow(i) + w);
      K.dims.insert(K.dims.end(), M.drow(i), M.drow(i) + rank);
      K.offs.push_back(M.offs[i]);
    }
    K.nblk = (int64_t)keep.size();
    if (K.nblk == 0) K.rank = 0;  // all zero: an empty QSpace (as the contraction's)
    M = K;
  }
  return T;
}

qs_status qs_plus_dev(qs_ctx *ctx, const qs_tensor *A, const qs_tensor *B, double bfac, qs_tensor **C) {
  QS_API_BEGIN
  if (!ctx || !A || !B || !C) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  *C = plus_core(&ctx->c, A, B, bfac).release();
  QS_API_END
}

qs_status qs_tensor_meta(const qs_tensor *T, int32_t *q, int64_t *dims, int64_t *offs) {
  QS_API_BEGIN
  if (!T) fail(QS_ERR_ARG, "null tensor");
  const QMeta &m = T->meta;
  if (q && !m.q.empty()) std::memcpy(q, m.q.data(), m.q.size() * 4);
  if (dims && !m.dims.empty()) std::memcpy(dims, m.dims.data(), m.dims.size() * 8);
  if (offs && !m.offs.empty()) std::memcpy(offs, m.offs.data(), m.offs.size() * 8);
  QS_API_END
}

const double *qs_tensor_data(const qs_tensor *T) { return T ? T->d : nullptr; }

static void copy_tags(const std::vector<std::string> &t, char *buf, size_t len) {
  if (!buf || !len) fail(QS_ERR_ARG, "null buffer");
  const std::string s = join_itags(t);
  if (s.size() + 1 > len) fail(QS_ERR_ARG, "itag buffer too small (%zu bytes needed)", s.size() + 1);
  std::memcpy(buf, s.c_str(), s.size() + 1);
}

qs_status qs_tensor_itags(const qs_tensor *T, char *buf, size_t len) {
  QS_API_BEGIN
  if (!T) fail(QS_ERR_ARG, "null tensor");
  copy_tags(T->meta.itags, buf, len);
  QS_API_END
}

qs_status qs_result_itags(const qs_result *C, char *buf, size_t len) {
  QS_API_BEGIN
  if (!C) fail(QS_ERR_ARG, "null result");
  copy_tags(C->meta.itags, buf, len);
  QS_API_END
}

void qs_tensor_free(qs_tensor *T) { delete T; }

qs_status qs_contract_batch(qs_ctx *ctx, int32_t n, const qs_tensor *const *A, const char *const *ia,
                            const qs_tensor *const *B, const char *const *ib, const int32_t *const *perm,
                            const int32_t *nperm, const qs_opts *opts, qs_tensor **C) {
  QS_API_BEGIN
  if (!ctx || !A || !ia || !B || !ib || !C) fail(QS_ERR_ARG, "null argument");
  if (n < 0) fail(QS_ERR_ARG, "negative batch size");
  for (int r = 0; r < n; ++r) {
    C[r] = nullptr;
    if (!A[r] || !B[r] || !ia[r] || !ib[r]) fail(QS_ERR_ARG, "null operand %d", r);
  }
  QS_CUDA(cudaSetDevice(ctx->c.device));
  std::vector<const QMeta *> am(n), bm(n);
  std::vector<const double *> ad(n), bd(n);
  for (int r = 0; r < n; ++r) {
    am[r] = &A[r]->meta;
    bm[r] = &B[r]->meta;
    ad[r] = A[r]->d;
    bd[r] = B[r]->d;
  }
  std::vector<std::unique_ptr<qs_tensor>> out;
  contract_batch_core(&ctx->c, n, am.data(), ad.data(), bm.data(), bd.data(), ia, ib, perm, nperm, opts, out);
  for (int r = 0; r < n; ++r) C[r] = out[r].release();
  QS_API_END
}

qs_status qs_contract_itags(qs_ctx *ctx, int32_t n, const qs_tensor *const *T, const int32_t *conj,
                            const int32_t *perm, int32_t nperm, const qs_opts *opts, qs_tensor **C) {
  QS_API_BEGIN
  if (!ctx || !T || !C) fail(QS_ERR_ARG, "null argument");
  *C = nullptr;
  QS_CUDA(cudaSetDevice(ctx->c.device));
  *C = contract_itags_core(&ctx->c, n, T, conj, perm, nperm, opts).release();
  QS_API_END
}

qs_status qs_contract_dev(qs_ctx *ctx, const qs_tensor *A, const char *ia, const qs_tensor *B,
                          const char *ib, const int32_t *perm, int32_t nperm, const qs_opts *opts,
                          qs_tensor **C, qs_stats *stats) {
  QS_API_BEGIN
  if (!ctx || !A || !B || !C) fail(QS_ERR_ARG, "null argument");
  *C = nullptr;
  QS_CUDA(cudaSetDevice(ctx->c.device));
  *C = contract_core(&ctx->c, A->meta, A->d, B->meta, B->d, ia, ib, perm, nperm, opts, stats).release();
  QS_API_END
}

static std::unique_ptr<qs_tensor> permute_core(Ctx *ctx, const QMeta &m, const double *d,
                                               const int32_t *perm, int32_t nperm, int32_t conj) {
  std::vector<int> P = parse_perm(perm, nperm, m.rank);
  auto T = std::make_unique<qs_tensor>();
  T->ctx = ctx;
  QMeta &M = T->meta;
  M.rank = m.rank;
  M.qdim = m.qdim;
  M.nblk = m.nblk;
  M.cplx = m.cplx;
  // itags follow the legs; 'conj' flips them as it conjugates the data
  // (QSpace::permute / Conj, Source/QSpace.hh:2670-2790, 1372-1380)
  for (int k = 0; k < (int)m.itags.size() && !m.itags.empty(); ++k) {
    const std::string &t = m.itags[P.empty() ? k : P[k]];
    M.itags.push_back(conj ? conj_itag(t) : t);
  }
  const int r = m.rank, qd = m.qdim;
  int64_t ne = 0;
  for (int64_t i = 0; i < m.nblk; ++i) {
    for (int k = 0; k < r; ++k) {
      const int src = P.empty() ? k : P[k];
      M.q.insert(M.q.end(), m.qrow(i) + src * qd, m.qrow(i) + (src + 1) * qd);
      M.dims.push_back(m.drow(i)[src]);
    }
    M.offs.push_back(ne);
    ne += m.bsize(i);
  }
  M.nelem = ne;
  const int es = m.cplx ? 2 : 1;
  T->d = dev_alloc<double>(ctx, (size_t)std::max<int64_t>(ne, 1) * es);
  std::vector<PermDesc> pd = make_perm_descs(m, P, conj && m.cplx, M.offs);
  run_permute(ctx, pd, d, T->d, m.cplx, true);
  return T;
}

qs_status qs_permuteQS(qs_ctx *ctx, const qs_qspace_view *A, const int32_t *perm, int32_t nperm,
                       int32_t conj, qs_result **B) {
  QS_API_BEGIN
  if (!ctx || !B) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  auto tA = upload(&ctx->c, A);
  auto tB = permute_core(&ctx->c, tA->meta, tA->d, perm, nperm, conj);
  *B = download(&ctx->c, tB.get());
  QS_API_END
}

qs_status qs_permute_dev(qs_ctx *ctx, const qs_tensor *A, const int32_t *perm, int32_t nperm,
                         int32_t conj, qs_tensor **B) {
  QS_API_BEGIN
  if (!ctx || !A || !B) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  *B = permute_core(&ctx->c, A->meta, A->d, perm, nperm, conj).release();
  QS_API_END
}

}  // extern "C"
