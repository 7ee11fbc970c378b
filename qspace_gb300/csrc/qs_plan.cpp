// Host planner of block-sparse contractions.  See qs_plan.h.
#include "qs_plan.h"

#include <algorithm>
#include <cctype>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>

namespace qs {

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

void fail(qs_status code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw Error(code, buf);
}

// ------------------------------------------------------------------ QMeta
void QMeta::check(const char *what) const {
  if (rank < 0 || rank > 8) fail(QS_ERR_ARG, "%s: rank %d out of range (0..8)", what, rank);
  if (qdim < 0 || qdim > 16) fail(QS_ERR_ARG, "%s: qdim %d out of range", what, qdim);
  if (nblk < 0) fail(QS_ERR_ARG, "%s: negative block count", what);
  if ((int64_t)q.size() != nblk * rank * qdim || (int64_t)dims.size() != nblk * rank ||
      (int64_t)offs.size() != nblk)
    fail(QS_ERR_ARG, "%s: label/dim/offset arrays inconsistent with nblk", what);
  for (int64_t i = 0; i < nblk; ++i) {
    int64_t s = 1;
    for (int k = 0; k < rank; ++k) {
      int64_t d = dims[i * rank + k];
      if (d < 0 || d > (int64_t(1) << 31)) fail(QS_ERR_SHAPE, "%s: block %lld leg %d has dim %lld", what, (long long)i, k, (long long)d);
      s *= d;
      if (s > (int64_t(1) << 40)) fail(QS_ERR_SHAPE, "%s: block %lld too large", what, (long long)i);
    }
    if (offs[i] < 0 || offs[i] + s > nelem)
      fail(QS_ERR_SHAPE, "%s: block %lld [%lld,+%lld) outside the data arena (%lld)", what,
           (long long)i, (long long)offs[i], (long long)s, (long long)nelem);
  }
}

QMeta meta_from_view(const qs_qspace_view *v) {
  if (!v) fail(QS_ERR_ARG, "null QSpace view");
  QMeta m;
  m.rank = v->rank;
  m.qdim = v->qdim;
  m.nblk = v->nblk;
  m.cplx = v->is_complex != 0;
  if (m.rank < 0 || m.rank > 8) fail(QS_ERR_ARG, "rank %d out of range (0..8)", m.rank);
  if (m.nblk < 0) fail(QS_ERR_ARG, "negative block count");
  if (m.nblk && (!v->q || !v->dims || !v->offs)) fail(QS_ERR_ARG, "null label/dim/offset array");
  m.q.assign(v->q, v->q + m.nblk * m.rank * m.qdim);
  m.dims.assign(v->dims, v->dims + m.nblk * m.rank);
  m.offs.assign(v->offs, v->offs + m.nblk);
  int64_t ext = 0;
  for (int64_t i = 0; i < m.nblk; ++i) {
    int64_t s = 1;
    for (int k = 0; k < m.rank; ++k) s *= std::max<int64_t>(m.dims[i * m.rank + k], 0);
    ext = std::max(ext, m.offs[i] + s);
  }
  m.nelem = ext;
  m.check("QSpace");
  if (m.nblk && !v->data && ext > 0) fail(QS_ERR_ARG, "null data pointer");
  m.itags = parse_itags(v->itags);
  if (!m.itags.empty() && (int)m.itags.size() != m.rank)
    fail(QS_ERR_LABEL, "invalid number of itags (%zu/%d)", m.itags.size(), m.rank);
  return m;
}

std::vector<std::string> parse_itags(const char *s) {
  std::vector<std::string> t;
  if (!s || !*s) return t;
  std::string cur;
  for (const char *p = s;; ++p) {
    if (*p == ',' || *p == 0) {
      size_t a = cur.find_first_not_of(' '), b = cur.find_last_not_of(' ');
      t.push_back(a == std::string::npos ? std::string() : cur.substr(a, b - a + 1));
      cur.clear();
      if (*p == 0) break;
    } else {
      cur.push_back(*p);
    }
  }
  return t;
}

std::string join_itags(const std::vector<std::string> &t) {
  std::string s;
  for (size_t i = 0; i < t.size(); ++i) s += (i ? "," : "") + t[i];
  return s;
}

std::string conj_itag(const std::string &t) {
  if (!t.empty() && t.back() == '*') return t.substr(0, t.size() - 1);
  return t + "*";
}

// ------------------------------------------------------------ index strings
// Restates Wb::Str2Idx (Source/wbio.c) in compact mode: one run of
// alphanumerics without separators is read character by character, otherwise
// tokens separated by ',', ';' or blanks are integers; brackets optional.
static std::vector<int> str2idx(const std::string &s0) {
  std::string s = s0;
  size_t a = s.find_first_not_of(" \t\n");
  size_t b = s.find_last_not_of(" \t\n");
  if (a == std::string::npos) return {};
  s = s.substr(a, b - a + 1);
  if (!s.empty() && s.front() == '[') {
    if (s.back() != ']') fail(QS_ERR_ARG, "invalid index '%s'", s0.c_str());
    s = s.substr(1, s.size() - 2);
  }
  bool sep = false;
  for (char c : s)
    if (c == ',' || c == ';' || std::isspace((unsigned char)c)) sep = true;
  std::vector<int> out;
  if (!sep) {
    for (char c : s) {
      if (c >= '0' && c <= '9') out.push_back(c - '0');
      else if (c >= 'A' && c <= 'Z') out.push_back(c - 'A' + 10);
      else if (c >= 'a' && c <= 'z') out.push_back(c - 'a' + 36);
      else fail(QS_ERR_ARG, "invalid index '%s'", s0.c_str());
    }
    return out;
  }
  std::string tok;
  auto flush = [&]() {
    if (tok.empty()) return;
    char *end = nullptr;
    long x = strtol(tok.c_str(), &end, 0);
    if (!end || *end) fail(QS_ERR_ARG, "invalid index token '%s' in '%s'", tok.c_str(), s0.c_str());
    out.push_back((int)x);
    tok.clear();
  };
  for (char c : s) {
    if (c == ',' || c == ';' || std::isspace((unsigned char)c)) flush();
    else tok.push_back(c);
  }
  flush();
  return out;
}

// ctrIdx::init (Source/wbindex.cc:482-521): trailing '*' (counted mod 2)
// conjugates; 1-based; entries must be unique.
CtrIdx parse_ctr_idx(const char *s) {
  if (!s || !s[0]) fail(QS_ERR_ARG, "empty contraction index");
  std::string t(s);
  int nconj = 0;
  while (!t.empty()) {
    char c = t.back();
    if (c == '*') { ++nconj; t.pop_back(); }
    else if (std::isspace((unsigned char)c)) t.pop_back();
    else break;
  }
  if (!t.empty() && (t.back() == ',' || t.back() == ';')) t.pop_back();
  std::vector<int> v = str2idx(t);
  if (v.empty()) fail(QS_ERR_ARG, "empty contraction index '%s'", s);
  CtrIdx ic;
  ic.conj = (nconj % 2) != 0;
  for (int x : v) {
    if (x < 1) fail(QS_ERR_ARG, "contraction index must be 1-based ('%s')", s);
    ic.idx.push_back(x - 1);
  }
  std::vector<int> u = ic.idx;
  std::sort(u.begin(), u.end());
  if (std::adjacent_find(u.begin(), u.end()) != u.end())
    fail(QS_ERR_ARG, "invalid index set '%s'", s);
  return ic;
}

std::vector<int> parse_perm(const int32_t *perm, int32_t nperm, int r) {
  std::vector<int> P;
  if (!perm || nperm <= 0) return P;
  if (nperm > r) fail(QS_ERR_ARG, "invalid permutation (length %d > rank %d)", nperm, r);
  std::vector<int> seen(r, 0);
  for (int i = 0; i < nperm; ++i) {
    int x = perm[i] - 1;
    if (x < 0 || x >= nperm || seen[x]) fail(QS_ERR_ARG, "invalid permutation");
    seen[x] = 1;
    P.push_back(x);
  }
  for (int i = nperm; i < r; ++i) P.push_back(i);  // partial perm: rest in place
  bool ident = true;
  for (int i = 0; i < r; ++i) ident &= (P[i] == i);
  if (ident) P.clear();
  return P;
}

int rec_compare(const int32_t *a, const int32_t *b, int n) {
  for (int i = 0; i < n; ++i) {
    if (a[i] < b[i]) return -1;
    if (a[i] > b[i]) return +1;
  }
  return 0;
}

// ------------------------------------------------------------------ planner
static bool is_range(const std::vector<int> &v, int start) {
  for (size_t i = 0; i < v.size(); ++i)
    if (v[i] != start + (int)i) return false;
  return true;
}

ContractPlan plan_contract(const QMeta &A, const char *ia, const QMeta &B,
                           const char *ib, const int32_t *perm, int32_t nperm) {
  ContractPlan pl;
  pl.ica = parse_ctr_idx(ia);
  pl.icb = parse_ctr_idx(ib);
  const int ra = A.rank, rb = B.rank;
  if (A.qdim != B.qdim && A.nblk && B.nblk)
    fail(QS_ERR_LABEL, "incompatible objects (QDIM=%d/%d)", A.qdim, B.qdim);
  if (pl.ica.idx.size() != pl.icb.idx.size())
    fail(QS_ERR_ARG, "invalid contraction (%zu/%zu indices)", pl.ica.idx.size(), pl.icb.idx.size());
  for (int x : pl.ica.idx)
    if (x >= ra) fail(QS_ERR_ARG, "index out of bounds (%d/%d)", x + 1, ra);
  for (int x : pl.icb.idx)
    if (x >= rb) fail(QS_ERR_ARG, "index out of bounds (%d/%d)", x + 1, rb);
  const int nc = (int)pl.ica.idx.size();

  // Co-sort the contracted legs by the larger operand when neither list is
  // sorted (Source/QSpace.cc:4344-4349).
  auto sorted = [](const std::vector<int> &v) { return std::is_sorted(v.begin(), v.end()); };
  if (!sorted(pl.ica.idx) && !sorted(pl.icb.idx)) {
    const std::vector<int> &key = A.data_size() > B.data_size() ? pl.ica.idx : pl.icb.idx;
    std::vector<int> o(nc);
    std::iota(o.begin(), o.end(), 0);
    std::stable_sort(o.begin(), o.end(), [&](int x, int y) { return key[x] < key[y]; });
    std::vector<int> a2(nc), b2(nc);
    for (int i = 0; i < nc; ++i) { a2[i] = pl.ica.idx[o[i]]; b2[i] = pl.icb.idx[o[i]]; }
    pl.ica.idx = a2;
    pl.icb.idx = b2;
  }
  for (int k = 0; k < ra; ++k)
    if (std::find(pl.ica.idx.begin(), pl.ica.idx.end(), k) == pl.ica.idx.end()) pl.ika.push_back(k);
  for (int k = 0; k < rb; ++k)
    if (std::find(pl.icb.idx.begin(), pl.icb.idx.end(), k) == pl.icb.idx.end()) pl.ikb.push_back(k);
  pl.rc = (int)(pl.ika.size() + pl.ikb.size());
  pl.P = parse_perm(perm, nperm, pl.rc);

  // Operand layouts (permute_to, Source/QSpace.hh:2824-2866): A keeps its
  // contracted legs in front or at the end when they already sit there in
  // pairing order, else it is permuted to put them at the end; B likewise
  // with end/front preference reversed.
  if (is_range(pl.ica.idx, 0)) {
    pl.la.ctr_front = true;
  } else if (is_range(pl.ica.idx, ra - nc)) {
    pl.la.ctr_front = false;
  } else {
    pl.la.permute = true;
    pl.la.perm = pl.ika;
    pl.la.perm.insert(pl.la.perm.end(), pl.ica.idx.begin(), pl.ica.idx.end());
    pl.la.ctr_front = false;
  }
  if (is_range(pl.icb.idx, rb - nc)) {
    pl.lb.ctr_front = false;
  } else if (is_range(pl.icb.idx, 0)) {
    pl.lb.ctr_front = true;
  } else {
    pl.lb.permute = true;
    pl.lb.perm = pl.icb.idx;
    pl.lb.perm.insert(pl.lb.perm.end(), pl.ikb.begin(), pl.ikb.end());
    pl.lb.ctr_front = true;
  }

  // A permuted operand takes its conjugation into the permutation
  // (permute_to, Source/QSpace.hh:2855-2858, then QSpace::permute): the
  // permuted copy holds the conjugated data and conjugated itags, and the
  // flag itself is cleared.
  std::vector<std::string> tagA = A.itags, tagB = B.itags;
  if (pl.la.permute && pl.ica.conj) {
    pl.la.conj = A.cplx;
    for (auto &t : tagA) t = conj_itag(t);
    pl.ica.conj = false;
  }
  if (pl.lb.permute && pl.icb.conj) {
    pl.lb.conj = B.cplx;
    for (auto &t : tagB) t = conj_itag(t);
    pl.icb.conj = false;
  }

  // itags (contract_getIdxSet, Source/QSpace.cc:4230-4271, with
  // itag_::sameAs, Source/wbindex.cc:989-1005): contracted legs carry the
  // same name (an empty tag matches leniently) and all pairs agree on the
  // relative direction; if all point the same way and the conjugation flags
  // do not differ, A's flag is toggled (the reference warns).
  if (!tagA.empty() && !tagB.empty()) {
    int zflag = 0;
    for (int i = 0; i < nc; ++i) {
      const std::string &ta = tagA[pl.ica.idx[i]], &tb = tagB[pl.icb.idx[i]];
      const bool ca = !ta.empty() && ta.back() == '*', cb = !tb.empty() && tb.back() == '*';
      const std::string na = ca ? ta.substr(0, ta.size() - 1) : ta, nb = cb ? tb.substr(0, tb.size() - 1) : tb;
      int q = (na == nb || na.empty() || nb.empty()) ? 1 : 0;
      if (q && ca != cb) q = -1;
      if (zflag && q != zflag) q = 0;
      if (!zflag) zflag = q;
      if (!q) fail(QS_ERR_LABEL, "contract() itag mismatch %s <> %s @ i=%d", ta.c_str(), tb.c_str(), i + 1);
    }
    if (zflag > 0 && pl.ica.conj == pl.icb.conj) pl.ica.conj = !pl.ica.conj;
    for (int k : pl.ika) pl.C.itags.push_back(pl.ica.conj ? conj_itag(tagA[k]) : tagA[k]);
    for (int k : pl.ikb) pl.C.itags.push_back(pl.icb.conj ? conj_itag(tagB[k]) : tagB[k]);
  }

  pl.C.rank = pl.rc;
  pl.C.qdim = A.qdim;
  pl.C.cplx = A.cplx || B.cplx;
  if (A.nblk == 0 || B.nblk == 0) return pl;

  const int qd = A.qdim;
  const int wc = nc * qd;  // width of a contracted-label record
  // Contracted-label records (getQsub, Source/QSpace.hh:2316-2336).
  std::vector<int32_t> QAc(A.nblk * wc), QBc(B.nblk * wc);
  for (int64_t i = 0; i < A.nblk; ++i)
    for (int k = 0; k < nc; ++k)
      std::memcpy(&QAc[i * wc + k * qd], A.qrow(i) + pl.ica.idx[k] * qd, qd * sizeof(int32_t));
  for (int64_t i = 0; i < B.nblk; ++i)
    for (int k = 0; k < nc; ++k)
      std::memcpy(&QBc[i * wc + k * qd], B.qrow(i) + pl.icb.idx[k] * qd, qd * sizeof(int32_t));

  // matchIndex: sort both, merge, cross product of equal groups
  // (Source/wbMatrix.cc:2075-2102, Source/wbsort.cc:154-272).
  auto sort_perm = [&](const std::vector<int32_t> &R, int64_t n) {
    std::vector<int64_t> p(n);
    std::iota(p.begin(), p.end(), 0);
    std::stable_sort(p.begin(), p.end(), [&](int64_t x, int64_t y) {
      return rec_compare(&R[x * wc], &R[y * wc], wc) < 0;
    });
    return p;
  };
  std::vector<int64_t> pa = sort_perm(QAc, A.nblk), pb = sort_perm(QBc, B.nblk);
  std::vector<int32_t> Ia, Ib;
  for (int64_t x = 0, y = 0; x < A.nblk && y < B.nblk;) {
    int c = rec_compare(&QAc[pa[x] * wc], &QBc[pb[y] * wc], wc);
    if (c < 0) { ++x; continue; }
    if (c > 0) { ++y; continue; }
    int64_t x1 = x, y1 = y;
    while (x1 < A.nblk && rec_compare(&QAc[pa[x1] * wc], &QAc[pa[x] * wc], wc) == 0) ++x1;
    while (y1 < B.nblk && rec_compare(&QBc[pb[y1] * wc], &QBc[pb[y] * wc], wc) == 0) ++y1;
    for (int64_t i = x; i < x1; ++i)
      for (int64_t j = y; j < y1; ++j) {
        Ia.push_back((int32_t)pa[i]);
        Ib.push_back((int32_t)pb[j]);
      }
    x = x1;
    y = y1;
  }
  const int64_t np = (int64_t)Ia.size();
  if (np == 0) return pl;

  // Output records QC = [QAk(Ia) QBk(Ib)] (Source/QSpace.cc:4278), sorted
  // lexicographically and grouped (groupRecs, Source/wbMatrix.cc:1734-1792):
  // the sorted order is the output block order.
  const int nka = (int)pl.ika.size(), nkb = (int)pl.ikb.size();
  const int wq = pl.rc * qd;
  std::vector<int32_t> QC(np * wq);
  for (int64_t p = 0; p < np; ++p) {
    int32_t *r = &QC[p * wq];
    for (int k = 0; k < nka; ++k) std::memcpy(r + k * qd, A.qrow(Ia[p]) + pl.ika[k] * qd, qd * 4);
    for (int k = 0; k < nkb; ++k) std::memcpy(r + (nka + k) * qd, B.qrow(Ib[p]) + pl.ikb[k] * qd, qd * 4);
  }
  std::vector<int64_t> order(np);
  std::iota(order.begin(), order.end(), 0);
  if (wq > 0)
    std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
      return rec_compare(&QC[x * wq], &QC[y * wq], wq) < 0;
    });

  // Group, set shapes and per-pair descriptors.
  pl.grp.push_back(0);
  std::vector<int64_t> c_off;
  for (int64_t t = 0; t < np; ++t) {
    const int64_t p = order[t];
    const int32_t a = Ia[p], b = Ib[p];
    const int64_t *da = A.drow(a), *db = B.drow(b);
    int64_t K = 1, M = 1, N = 1;
    for (int k = 0; k < nc; ++k) {
      if (da[pl.ica.idx[k]] != db[pl.icb.idx[k]])
        fail(QS_ERR_SHAPE, "contracted dimension mismatch (A block %d leg %d: %lld, B block %d leg %d: %lld)",
             a + 1, pl.ica.idx[k] + 1, (long long)da[pl.ica.idx[k]], b + 1, pl.icb.idx[k] + 1,
             (long long)db[pl.icb.idx[k]]);
      K *= da[pl.ica.idx[k]];
    }
    for (int k : pl.ika) M *= da[k];
    for (int k : pl.ikb) N *= db[k];
    if (M > INT32_MAX || N > INT32_MAX || K > INT32_MAX) fail(QS_ERR_SHAPE, "block too large for the GEMM path");
    bool newblk = (t == 0) || (wq > 0 && rec_compare(&QC[order[t - 1] * wq], &QC[p * wq], wq) != 0);
    if (newblk) {
      if (t) pl.grp.push_back(t);
      const int64_t ib = (int64_t)pl.blk_M.size();
      pl.C.q.insert(pl.C.q.end(), &QC[p * wq], &QC[p * wq] + wq);
      for (int k : pl.ika) pl.C.dims.push_back(da[k]);
      for (int k : pl.ikb) pl.C.dims.push_back(db[k]);
      pl.C.offs.push_back(pl.C.nelem);
      c_off.push_back(pl.C.nelem);
      pl.C.nelem += M * N;
      pl.blk_M.push_back((int32_t)M);
      pl.blk_N.push_back((int32_t)N);
      (void)ib;
    } else {
      // all pairs of one output block must produce the same block shape
      const int64_t ib = (int64_t)pl.blk_M.size() - 1;
      const int64_t *dc = &pl.C.dims[ib * pl.rc];
      for (int k = 0; k < nka; ++k)
        if (dc[k] != da[pl.ika[k]]) fail(QS_ERR_SHAPE, "inconsistent output block dims (A block %d)", a + 1);
      for (int k = 0; k < nkb; ++k)
        if (dc[nka + k] != db[pl.ikb[k]]) fail(QS_ERR_SHAPE, "inconsistent output block dims (B block %d)", b + 1);
    }
    PairDesc d{};
    d.a_off = A.offs[a];
    d.b_off = B.offs[b];
    d.M = (int32_t)M;
    d.N = (int32_t)N;
    d.K = (int32_t)K;
    d.trans = 0;
    if (pl.la.ctr_front) { d.lda = (int32_t)std::max<int64_t>(K, 1); d.trans |= 1; }
    else d.lda = (int32_t)std::max<int64_t>(M, 1);
    if (pl.lb.ctr_front) d.ldb = (int32_t)std::max<int64_t>(K, 1);
    else { d.ldb = (int32_t)std::max<int64_t>(N, 1); d.trans |= 2; }
    if (pl.ica.conj && A.cplx) d.trans |= 4;
    if (pl.icb.conj && B.cplx) d.trans |= 8;
    d.afac = 1.0;
    pl.pairs.push_back(d);
    pl.pair_blk.push_back((int32_t)(pl.blk_M.size() - 1));
    pl.pair_ia.push_back(a);
    pl.pair_ib.push_back(b);
    pl.flops += (pl.C.cplx ? 8.0 : 2.0) * double(M) * double(N) * double(K);
  }
  pl.grp.push_back(np);
  pl.C.nblk = (int64_t)pl.blk_M.size();
  for (size_t g = 0; g + 1 < pl.grp.size(); ++g) {
    int64_t ks = 0;
    for (int64_t t = pl.grp[g]; t < pl.grp[g + 1]; ++t) ks += pl.pairs[t].K;
    pl.kmax = std::max(pl.kmax, ks);
  }
  const double es = pl.C.cplx ? 16.0 : 8.0;
  pl.bytes = es * double(A.data_size() + B.data_size() + pl.C.nelem);
  return pl;
}

std::vector<TileDesc> make_tiles(const std::vector<int64_t> &grp,
                                 const std::vector<int32_t> &blk_M,
                                 const std::vector<int32_t> &blk_N,
                                 const std::vector<int64_t> &c_off, int tm, int tn,
                                 const std::vector<int32_t> *blk_ldc, const std::vector<PairDesc> *pairs) {
  std::vector<TileDesc> tiles;
  const int64_t nb = (int64_t)blk_M.size();
  for (int64_t b = 0; b < nb; ++b) {
    const int32_t M = blk_M[b], N = blk_N[b];
    for (int32_t n0 = 0; n0 < N; n0 += tn)
      for (int32_t m0 = 0; m0 < M; m0 += tm) {
        TileDesc t{};
        t.c_off = c_off[b];
        t.p0 = (int32_t)grp[b];
        t.p1 = (int32_t)grp[b + 1];
        t.m0 = m0;
        t.n0 = n0;
        t.M = M;
        t.N = N;
        t.ldc = blk_ldc ? (*blk_ldc)[b] : std::max(M, 1);
        t.cblk = (int32_t)b;
        tiles.push_back(t);
      }
  }
  if (pairs && tiles.size() > 1) {
    std::vector<int64_t> depth(nb, 0);
    for (int64_t b = 0; b < nb; ++b)
      for (int64_t p = grp[b]; p < grp[b + 1]; ++p) depth[b] += std::max((*pairs)[p].K, 0);
    auto work = [&](const TileDesc &t) {
      const int64_t rows = std::min<int64_t>(tm, t.M - t.m0), cols = std::min<int64_t>(tn, t.N - t.n0);
      return depth[t.cblk] * ((rows + 15) / 16) * ((cols + 15) / 16);
    };
    std::vector<int64_t> key(tiles.size());
    for (size_t i = 0; i < tiles.size(); ++i) key[i] = work(tiles[i]);
    std::vector<size_t> ord(tiles.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return key[x] > key[y]; });
    std::vector<TileDesc> sorted(tiles.size());
    for (size_t i = 0; i < ord.size(); ++i) sorted[i] = tiles[ord[i]];
    tiles.swap(sorted);
  }
  return tiles;
}

std::vector<PermDesc> make_perm_descs(const QMeta &in, const std::vector<int> &perm,
                                      bool conj, const std::vector<int64_t> &out_offs,
                                      const std::vector<int64_t> *sel) {
  std::vector<PermDesc> v;
  const int r = in.rank;
  const int64_t n = sel ? (int64_t)sel->size() : in.nblk;
  for (int64_t t = 0; t < n; ++t) {
    const int64_t i = sel ? (*sel)[t] : t;
    PermDesc d{};
    d.in_off = in.offs[i];
    d.out_off = out_offs[t];
    d.rank = r;
    d.conj = conj ? 1 : 0;
    int64_t stride[8];
    int64_t s = 1;
    for (int k = 0; k < r; ++k) { stride[k] = s; s *= in.dims[i * r + k]; }
    d.n = s;
    for (int k = 0; k < r; ++k) {
      const int src = perm.empty() ? k : perm[k];
      d.out_dims[k] = in.dims[i * r + src];
      d.in_stride[k] = stride[src];
    }
    v.push_back(d);
  }
  return v;
}

}  // namespace qs
