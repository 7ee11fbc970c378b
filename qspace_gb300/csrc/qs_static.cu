// qs_grouped_gemm_split_static: the split-precision grouped GEMM for callers
// that must not allocate device memory while they run.  Every device buffer
// of the call -- work lists, exponent arrays, BF16 digit arena, error word --
// lives in one file-scope array per device and process; nothing is allocated.
#include <mutex>

#include "qs_grouped.h"
#include "qs_internal.h"

using namespace qs;

namespace {

// Bytes [0, 4) hold the error word of the bounded waits (must start at zero);
// the work lists and digits start at byte 256.
constexpr size_t HDR = 256;
static __device__ __align__(256) unsigned char g_scratch[QS_STATIC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
uint8_t *g_addr[MAX_DEVICES] = {};

// Address of this device's array; looked up once per device with that
// device current, when the error word is also cleared.
uint8_t *scratch_of(int device) {
  if (device < 0 || device >= MAX_DEVICES) fail(QS_ERR_ARG, "device %d out of range", device);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    QS_CUDA(cudaGetSymbolAddress(&p, g_scratch));
    QS_CUDA(cudaMemset(p, 0, HDR));
    g_addr[device] = static_cast<uint8_t *>(p);
  }
  return g_addr[device];
}

}  // namespace

extern "C" qs_status qs_grouped_gemm_split_static(qs_ctx *ctx, const qs_pair_list *pairs, const double *A,
                                                  const double *B, double *C, const qs_opts *opts,
                                                  qs_stats *stats) {
  QS_API_BEGIN
  if (!ctx || !pairs || !A || !B || !C) fail(QS_ERR_ARG, "null argument");
  qs_opts o{QS_PREC_SPLIT, 0, 1e-12, 0};
  if (opts) o = *opts;
  if (o.prec != QS_PREC_SPLIT) fail(QS_ERR_ARG, "qs_grouped_gemm_split_static runs the split path only");
  Ctx *c = &ctx->c;
  QS_CUDA(cudaSetDevice(c->device));
  uint8_t *base = scratch_of(c->device);
  int *err = reinterpret_cast<int *>(base);
  grouped_run(c, pairs, A, B, C, &o, stats, -1, -1, -1, base + HDR, QS_STATIC_SCRATCH_BYTES - HDR, err);
  int kerr = 0;
  QS_CUDA(cudaMemcpyAsync(&kerr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  QS_CUDA(cudaStreamSynchronize(c->stream));
  if (kerr) {
    QS_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    QS_CUDA(cudaStreamSynchronize(c->stream));
    fail(QS_ERR_TIMEOUT, "a bounded device wait ran out (code %d)", kerr);
  }
  QS_API_END
}
