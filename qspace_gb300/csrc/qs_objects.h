// C-ABI object definitions shared by the contraction driver (qs_capi.cpp)
// and the serving loop (qs_serve.cpp).
#pragma once

#include <memory>
#include <vector>

#include "qs_internal.h"
#include "qs_plan.h"

struct qs_tensor {
  qs::QMeta meta;
  double *d = nullptr;   // owned arena (stream-ordered allocation)
  qs::Ctx *ctx = nullptr;  // context whose stream frees the arena
  ~qs_tensor() {
    if (!d) return;
    if (ctx && qs::ctx_alive(ctx))
      cudaFreeAsync(d, ctx->stream);
    else
      cudaFree(d);  // the context is gone: device pool memory, freed synchronously
  }
};

struct qs_result {
  qs::QMeta meta;              // contiguous offsets
  std::vector<double> data;    // nelem (x2 when complex)
};

namespace qs {
// The device contraction driver: plan on the host, kernels on ctx->stream.
// Synchronises ctx->stream once (the data-dependent zero-block test).
std::unique_ptr<qs_tensor> contract_core(Ctx *ctx, const QMeta &Am, const double *dA, const QMeta &Bm,
                                         const double *dB, const char *ia, const char *ib,
                                         const int32_t *perm, int32_t nperm, const qs_opts *opts,
                                         qs_stats *stats);
// A batch of contractions whose block products share one grouped launch per
// element type (and digit plan); out[r] receives contraction r's result.
void contract_batch_core(Ctx *ctx, int n, const QMeta *const *Am, const double *const *dA,
                         const QMeta *const *Bm, const double *const *dB, const char *const *ia,
                         const char *const *ib, const int32_t *const *perm, const int32_t *nperm,
                         const qs_opts *opts, std::vector<std::unique_ptr<qs_tensor>> &out);
// Device bytes a contraction will hold while it runs (output, operand
// copies, digit arena): the admission footprint of the serving loop.
int64_t contract_footprint(const QMeta &Am, const QMeta &Bm, const char *ia, const char *ib,
                           const qs_opts *opts);
// eigQS of a device-resident rank-2 QSpace on ctx's stream: kept and
// discarded eigenvectors as new tensors, optional host copies of the
// eigenvalues / keep flags (sum of block sizes each), NK and Etrunc.
void eigqs_core(Ctx *ctx, const qs_tensor *H, int64_t nkeep, double etrunc, double deps,
                std::unique_ptr<qs_tensor> &AK, std::unique_ptr<qs_tensor> &AD, double *E, uint8_t *keep,
                int64_t *nkeep_out, double *etrunc_out);
// Device bytes eigqs_core holds while it runs (admission footprint).
int64_t eigqs_footprint(const QMeta &m);
}  // namespace qs
