// Validated form of a qs_pair_list, shared by the one-shot grouped entry
// points (qs_grouped.cpp) and the reusable plans (qs_plan_api.cpp).
#pragma once

#include <cstdint>
#include <vector>

#include "qs_internal.h"

namespace qs {

// Device descriptors per pair, the output blocks (runs of equal c_blk) with
// their shapes, and per-pair element ranges of A and B.
struct GroupedPlan {
  bool cplx = false;
  std::vector<PairDesc> pairs;
  std::vector<int64_t> grp;  // pairs of block g: [grp[g], grp[g+1])
  std::vector<int32_t> bM, bN, bldc;
  std::vector<int64_t> coff;
  std::vector<int64_t> a_end, b_end;  // one past the last element a pair reads
  double flops = 0, bytes = 0;
};

// Validates the pair list.  When the element counts are known (>= 0), every
// access is checked against them.
GroupedPlan grouped_plan(const qs_pair_list *pl, int64_t a_elems, int64_t b_elems, int64_t c_elems);

// The plain FP64 grouped product of a list (64 x 64 tiles): shallow output
// blocks computed directly (run_shallow), deep ones cut along their depth and
// summed in part order (split_deep).
void run_f64(Ctx *ctx, const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
             const std::vector<int32_t> &bM, const std::vector<int32_t> &bN, const std::vector<int64_t> &coff,
             const std::vector<int32_t> *bldc, const double *A, const double *B, double *C, bool cplx);

// Validates the pair list, then launches the FP64 or the split path on all of
// it.
void grouped_run(Ctx *ctx, const qs_pair_list *pl, const double *A, const double *B, double *C,
                 const qs_opts *opts, qs_stats *stats, int64_t a_elems, int64_t b_elems,
                 int64_t c_elems, uint8_t *static_scratch = nullptr, size_t static_cap = 0,
                 int *static_err = nullptr);

}  // namespace qs
