// Host-side planner of a block-sparse contraction: label matching, output
// block order, block-pair enumeration and operand layouts.  Labels and block
// order are bit-exact with QSpace::contract (Source/QSpace.cc:4131-4420).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "qs_internal.h"

namespace qs {

// Labels and shapes of a block-sparse tensor (always host side).
struct QMeta {
  int rank = 0, qdim = 0;
  int64_t nblk = 0;
  std::vector<int32_t> q;     // nblk * rank * qdim
  std::vector<int64_t> dims;  // nblk * rank
  std::vector<int64_t> offs;  // nblk
  int64_t nelem = 0;          // extent of the data arena (elements)
  bool cplx = false;
  std::vector<std::string> itags;  // leg tags ("L", "R*"), empty: none

  const int32_t *qrow(int64_t i) const { return q.data() + i * rank * qdim; }
  const int64_t *drow(int64_t i) const { return dims.data() + i * rank; }
  int64_t bsize(int64_t i) const {
    int64_t s = 1;
    for (int k = 0; k < rank; ++k) s *= dims[i * rank + k];
    return s;
  }
  int64_t data_size() const {
    int64_t s = 0;
    for (int64_t i = 0; i < nblk; ++i) s += bsize(i);
    return s;
  }
  void check(const char *what) const;
};

QMeta meta_from_view(const qs_qspace_view *v);
std::vector<std::string> parse_itags(const char *s);
std::string join_itags(const std::vector<std::string> &t);
std::string conj_itag(const std::string &t);

// Contraction index: 0-based legs + conj flag.
struct CtrIdx {
  std::vector<int> idx;
  bool conj = false;
};
CtrIdx parse_ctr_idx(const char *s);
std::vector<int> parse_perm(const int32_t *perm, int32_t nperm, int r);

// Operand layout after the reference's permute_to (Source/QSpace.hh:2824-2866).
struct OperandLayout {
  bool permute = false;       // materialise a permuted copy first
  std::vector<int> perm;      // leg order of the permuted copy (0-based)
  bool ctr_front = false;     // contracted legs lead (else they trail)
  bool conj = false;          // the permuted copy is conjugated
};

struct ContractPlan {
  CtrIdx ica, icb;
  std::vector<int> ika, ikb;
  OperandLayout la, lb;
  int rc = 0;
  QMeta C;                     // output before zero-block removal/permutation
  std::vector<PairDesc> pairs; // grouped by output block, in summation order
  std::vector<int32_t> pair_blk;
  std::vector<int32_t> pair_ia, pair_ib;
  std::vector<int64_t> grp;    // nout + 1 pair ranges
  std::vector<int32_t> blk_M, blk_N;
  std::vector<int> P;          // final 0-based permutation (empty = none)
  double flops = 0, bytes = 0;
  int64_t kmax = 0;            // max summed depth over output blocks
};

ContractPlan plan_contract(const QMeta &A, const char *ia, const QMeta &B,
                           const char *ib, const int32_t *perm, int32_t nperm);

// Tiles of the grouped GEMM over the plan's output blocks; with `pairs`,
// ordered by estimated work, largest first (the summed depth of the block
// times the tile's 16 x 16 groups that hold outputs), so that the tail of
// the launch is made of short tiles.
std::vector<TileDesc> make_tiles(const std::vector<int64_t> &grp,
                                 const std::vector<int32_t> &blk_M,
                                 const std::vector<int32_t> &blk_N,
                                 const std::vector<int64_t> &c_off, int tm, int tn,
                                 const std::vector<int32_t> *blk_ldc = nullptr,
                                 const std::vector<PairDesc> *pairs = nullptr);

// Permutation descriptors: out block = permute(in block, perm) [+conj].
std::vector<PermDesc> make_perm_descs(const QMeta &in, const std::vector<int> &perm,
                                      bool conj, const std::vector<int64_t> &out_offs,
                                      const std::vector<int64_t> *sel = nullptr);

// Lexicographic comparison of int label rows (Wb::recCompare, lex=1,
// Source/gathered.hh:538-552).
int rec_compare(const int32_t *a, const int32_t *b, int n);

}  // namespace qs
