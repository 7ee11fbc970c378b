// Split-precision grouped block GEMM (FP64 emulated with BF16 digits on the
// 5th-generation tensor cores).  See qs_gemm_split.cu for the method.
#pragma once

#include <cstdint>
#include <vector>

#include "qs_internal.h"

namespace qs {

struct SplitResult {
  int nslices = 0;
  int bits = 0;
  double err_bound = 0;
  int64_t slice_bytes = 0;
  int64_t ntiles = 0;
};

// Digit plan for a maximal accumulated depth `kreal` (real terms summed into
// one output element) and a target relative error.
struct DigitPlan {
  int bits;    // bits per digit (the leading digit carries bits+1)
  int nslices; // digits per operand
  double err_bound;
};
DigitPlan choose_digits(int64_t kreal, double tol, int forced_slices);
// The digit plan the split path picks for a grouped product (cm = 2 for
// complex), optionally with the digit count and/or width forced.
DigitPlan choose_digits_for(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                            const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N, int cm,
                            double tol, int forced_slices, int forced_bits = 0);

// With va / vb (one per pair; nl = 0 for none) the slicing reads op(A) /
// op(B) of a pair through its strided view instead of (lda, trans): a
// permuted operand needs no copy.
SplitResult run_split(Ctx *ctx, const std::vector<PairDesc> &pairs,
                      const std::vector<int64_t> &grp, const std::vector<int32_t> &blk_M,
                      const std::vector<int32_t> &blk_N, const std::vector<int64_t> &c_off,
                      const double *A, const double *B, double *C, bool cplx,
                      int forced_slices, double tol,
                      const std::vector<int32_t> *blk_ldc = nullptr, int forced_bits = 0,
                      const std::vector<OperandView> *va = nullptr,
                      const std::vector<OperandView> *vb = nullptr);

// The same product with every device buffer carved from caller-provided
// scratch (`cap` bytes, 256-byte aligned) instead of allocated; the bounded
// waits report to `err`.  A plan that does not fit is refused (QS_ERR_OOM)
// before anything is copied or launched.
SplitResult run_split_static(Ctx *ctx, const std::vector<PairDesc> &pairs,
                             const std::vector<int64_t> &grp, const std::vector<int32_t> &blk_M,
                             const std::vector<int32_t> &blk_N, const std::vector<int64_t> &c_off,
                             const double *A, const double *B, double *C, bool cplx,
                             int forced_slices, double tol, const std::vector<int32_t> *blk_ldc,
                             uint8_t *scratch, size_t cap, int *err);

// Reusable split plans (stable device addresses, for CUDA graph replay).
struct SplitPlanHandle;
std::vector<int> split_candidate_bits(double tol, int forced_slices);
// bits = 0: the cost model picks the digit width
SplitPlanHandle *split_plan_create(const std::vector<PairDesc> &pairs, const std::vector<int64_t> &grp,
                                   const std::vector<int32_t> &blk_M, const std::vector<int32_t> &blk_N,
                                   const std::vector<int64_t> &c_off, const std::vector<int32_t> &blk_ldc,
                                   bool cplx, int forced_slices, double tol, int bits, SplitResult *res);
void split_plan_launch(Ctx *ctx, SplitPlanHandle *h, const double *A, const double *B, double *C);
void split_plan_destroy(SplitPlanHandle *h);

}  // namespace qs
