// qs_xcache_*: the device-resident CG / X-symbol factor table, and
// qs_grouped_gemm_keyed: the grouped product with every pair's factor looked
// up on the device (probe rule and layout in qs_xcache.h).
//
// Inserts happen on the host (a mirror of the table, then one upload): they
// belong to warm-up, like the reference's first contractCGR call per key.
// Lookups run on the device: repeated contractions carry keys, and the
// looked-up factors (8 bytes per pair) come back to run the listed-factor
// product, so keyed and listed products are the same computation.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "qs_grouped.h"
#include "qs_internal.h"
#include "qs_xcache.h"

struct qs_xcache {
  qs::Ctx *ctx = nullptr;
  uint64_t cap = 0;
  int64_t count = 0;
  std::vector<uint64_t> hkeys;  // host mirror, 2 words per slot
  std::vector<double> hvals;
  uint64_t *dkeys = nullptr;
  double *dvals = nullptr;
};

namespace qs {

namespace {

__global__ void xcache_get_kernel(XView v, const uint64_t *__restrict__ keys, int64_t n, double *__restrict__ vals,
                                  int32_t *__restrict__ found) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x = 0.0;
    const bool f = xview_find(v, keys[2 * i], keys[2 * i + 1], &x);
    vals[i] = f ? x : 0.0;
    found[i] = f ? 1 : 0;
  }
}

int grid_for(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 4096); }

XView view_of(const qs_xcache *c) { return XView{c->dkeys, c->dvals, c->cap - 1}; }

// Replaces the device table with the host arrays.  Ordered on the context's
// stream (after every launch queued so far, which may still read the table)
// and waited for: a copy from pageable memory may return before its data
// has reached the device.
void upload(qs_xcache *c, const std::vector<uint64_t> &hk, const std::vector<double> &hv) {
  cudaStream_t st = c->ctx->stream;
  QS_CUDA(cudaMemcpyAsync(c->dkeys, hk.data(), hk.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
  QS_CUDA(cudaMemcpyAsync(c->dvals, hv.data(), hv.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  QS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

void xcache_orphan_all(Ctx *ctx) {
  cudaStreamSynchronize(ctx->stream);
  for (qs_xcache *c : ctx->tables) {
    cudaFree(c->dkeys);
    cudaFree(c->dvals);
    c->dkeys = nullptr;
    c->dvals = nullptr;
    c->ctx = nullptr;
  }
  ctx->tables.clear();
}

}  // namespace qs

using namespace qs;

extern "C" {

qs_status qs_xcache_create(qs_ctx *ctx, int64_t capacity, qs_xcache **out) {
  QS_API_BEGIN
  if (!ctx || !out) fail(QS_ERR_ARG, "null argument");
  *out = nullptr;
  if (capacity < 1 || capacity > (int64_t(1) << 30)) fail(QS_ERR_ARG, "factor table capacity %lld out of range",
                                                          (long long)capacity);
  QS_CUDA(cudaSetDevice(ctx->c.device));
  auto c = std::make_unique<qs_xcache>();
  c->ctx = &ctx->c;
  uint64_t cap = 16;
  // at most 3/4 full at the requested number of entries
  while (cap * 3 < (uint64_t)capacity * 4) cap <<= 1;
  c->cap = cap;
  c->hkeys.assign(2 * cap, XKEY_EMPTY);
  c->hvals.assign(cap, 0.0);
  cudaError_t e = cudaMalloc(&c->dkeys, 2 * cap * sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMalloc(&c->dvals, cap * sizeof(double));
  if (e != cudaSuccess) {
    if (c->dkeys) cudaFree(c->dkeys);
    fail(e == cudaErrorMemoryAllocation ? QS_ERR_OOM : QS_ERR_CUDA, "factor table: %s", cudaGetErrorString(e));
  }
  upload(c.get(), c->hkeys, c->hvals);
  ctx->c.tables.push_back(c.get());
  *out = c.release();
  QS_API_END
}

void qs_xcache_destroy(qs_xcache *c) {
  if (!c) return;
  if (Ctx *ctx = c->ctx) {  // else its context is gone and freed the memory
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);  // no launch may still read the table
    cudaFree(c->dkeys);
    cudaFree(c->dvals);
    auto &t = ctx->tables;
    t.erase(std::remove(t.begin(), t.end(), c), t.end());
  }
  delete c;
}

qs_status qs_xcache_put(qs_xcache *c, int64_t n, const uint64_t *keys, const double *vals) {
  QS_API_BEGIN
  if (!c || n < 0 || (n > 0 && (!keys || !vals))) fail(QS_ERR_ARG, "null argument");
  if (!c->ctx) fail(QS_ERR_ARG, "the table's context was destroyed");
  for (int64_t i = 0; i < n; ++i)
    if (keys[2 * i] == XKEY_EMPTY && keys[2 * i + 1] == XKEY_EMPTY)
      fail(QS_ERR_ARG, "key %lld is the reserved empty key", (long long)i);
  // insert into a copy of the mirror: a refused batch leaves the table as it was
  std::vector<uint64_t> hk = c->hkeys;
  std::vector<double> hv = c->hvals;
  int64_t count = c->count;
  const uint64_t mask = c->cap - 1;
  for (int64_t i = 0; i < n; ++i) {
    const uint64_t a = keys[2 * i], b = keys[2 * i + 1];
    uint64_t s = xkey_hash(a, b) & mask;
    while (!(hk[2 * s] == a && hk[2 * s + 1] == b) && !(hk[2 * s] == XKEY_EMPTY && hk[2 * s + 1] == XKEY_EMPTY))
      s = (s + 1) & mask;
    if (hk[2 * s] == XKEY_EMPTY && hk[2 * s + 1] == XKEY_EMPTY) {
      if ((uint64_t)(count + 1) * 4 > c->cap * 3)
        fail(QS_ERR_OOM, "factor table full (%lld entries, capacity %llu)", (long long)count,
             (unsigned long long)c->cap);
      hk[2 * s] = a;
      hk[2 * s + 1] = b;
      ++count;
    }
    hv[s] = vals[i];
  }
  QS_CUDA(cudaSetDevice(c->ctx->device));
  upload(c, hk, hv);
  c->hkeys.swap(hk);
  c->hvals.swap(hv);
  c->count = count;
  QS_API_END
}

qs_status qs_xcache_get(qs_xcache *c, int64_t n, const uint64_t *keys, double *vals, int32_t *found) {
  QS_API_BEGIN
  if (!c || n < 0 || (n > 0 && (!keys || !vals || !found))) fail(QS_ERR_ARG, "null argument");
  if (!c->ctx) fail(QS_ERR_ARG, "the table's context was destroyed");
  if (n == 0) return QS_OK;
  Ctx *ctx = c->ctx;
  QS_CUDA(cudaSetDevice(ctx->device));
  std::vector<uint64_t> k(keys, keys + 2 * n);
  uint64_t *dk = dev_upload(ctx, k);
  double *dv = dev_alloc<double>(ctx, (size_t)n);
  int32_t *df = dev_alloc<int32_t>(ctx, (size_t)n);
  xcache_get_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(view_of(c), dk, n, dv, df);
  QS_LAUNCHED(ctx);
  QS_CUDA(cudaMemcpyAsync(vals, dv, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaMemcpyAsync(found, df, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, dk);
  dev_free(ctx, dv);
  dev_free(ctx, df);
  QS_API_END
}

qs_status qs_xcache_count(const qs_xcache *c, int64_t *n) {
  QS_API_BEGIN
  if (!c || !n) fail(QS_ERR_ARG, "null argument");
  *n = c->count;
  QS_API_END
}

qs_status qs_grouped_gemm_keyed(qs_ctx *ctx, const qs_pair_list *pairs, const uint64_t *fkeys,
                                const qs_xcache *cache, const double *A, const double *B, double *C,
                                const qs_opts *opts, qs_stats *stats) {
  QS_API_BEGIN
  if (!ctx || !pairs || !fkeys || !cache || !A || !B || !C) fail(QS_ERR_ARG, "null argument");
  if (cache->ctx != &ctx->c) fail(QS_ERR_ARG, "the factor table belongs to another context");
  if (pairs->npairs < 0) fail(QS_ERR_ARG, "negative pair count");
  Ctx *c = &ctx->c;
  QS_CUDA(cudaSetDevice(c->device));
  const int64_t n = pairs->npairs;
  // the factors come from the table: a placeholder list satisfies the checks
  qs_pair_list pl = *pairs;
  std::vector<double> ones;
  if (!pl.afac) {
    ones.assign((size_t)std::max<int64_t>(n, 1), 1.0);
    pl.afac = ones.data();
  }
  // The factors are looked up on the device and come back to the host (8
  // bytes per pair); the product then runs with them as listed factors, so a
  // keyed product is the same computation as the listed one, whatever route
  // its blocks take (shallow, deep, tiled).
  std::vector<uint64_t> k(fkeys, fkeys + 2 * n);
  std::vector<double> vals((size_t)std::max<int64_t>(n, 1), 0.0);
  std::vector<int32_t> found((size_t)std::max<int64_t>(n, 1), 1);
  if (n) {
    uint64_t *dk = dev_upload(c, k);
    double *dv = dev_alloc<double>(c, (size_t)n);
    int32_t *df = dev_alloc<int32_t>(c, (size_t)n);
    try {
      const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
      xcache_get_kernel<<<grid, 256, 0, c->stream>>>(view_of(cache), dk, n, dv, df);
      QS_LAUNCHED(c);
      QS_CUDA(cudaMemcpyAsync(vals.data(), dv, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
      QS_CUDA(cudaMemcpyAsync(found.data(), df, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
      QS_CUDA(cudaStreamSynchronize(c->stream));
    } catch (...) {
      cudaStreamSynchronize(c->stream);
      dev_free(c, dk);
      dev_free(c, dv);
      dev_free(c, df);
      throw;
    }
    dev_free(c, dk);
    dev_free(c, dv);
    dev_free(c, df);
  }
  pl.afac = vals.data();
  grouped_run(c, &pl, A, B, C, opts, stats, -1, -1, -1);
  for (int64_t i = 0; i < n; ++i)
    if (!found[i]) fail(QS_ERR_ARG, "a pair's factor key is not in the table (its products used factor 0)");
  QS_API_END
}

}  // extern "C"
