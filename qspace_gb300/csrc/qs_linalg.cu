// FP64 block linear algebra: Hermitian eigendecomposition and SVD of every
// symmetry block, global truncation (markSet) and the Davidson double
// Gram-Schmidt re-orthogonalisation.
//
//  * qs_eig_blocks  -- the OpenMP loop of QSpace::EigenSymmetric
//    (Source/QSpace.cc:4789-4811) calling wbEigenS -> dsyevd / zheevd
//    (Source/wbarray_blas.cc:501-660).  Blocks up to 16 rows go through one
//    batched Jacobi call per distinct size (syevjBatched); larger blocks
//    through one batched solve per distinct size (XsyevBatched), spread over
//    concurrent solver lanes.
//  * qs_svd_blocks  -- SVD_Data::blockSVD (Source/mpsortho.cc:546-613) ->
//    wbSVD -> dgesdd (Source/wbarray_blas.cc:995-1090); Jacobi SVD (gesvdj).
//  * qs_mark_keep   -- markSet (Source/gathered.cc:1822-1990) on the host.
//  * qs_gs_reortho  -- RunDavidson's double classical Gram-Schmidt
//    (Source/david2SiteQS.cc:440-470): two passes of v -= V (V^T v), then
//    v /= |v|; FP64 dot/axpy kernels (memory bound).
#include <cusolverDn.h>

#include <cstdlib>
#include <exception>
#include <functional>
#include <thread>
#include <tuple>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <vector>

#include "qs_internal.h"
#include "qs_objects.h"

namespace qs {

#define QS_SOLVER(call)                                                                   \
  do {                                                                                    \
    cusolverStatus_t s_ = (call);                                                         \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                                    \
      ::qs::fail(QS_ERR_CUDA, "%s:%d %s -> cusolver status %d", __FILE__, __LINE__, #call, \
                 (int)s_);                                                                \
  } while (0)

cusolverDnHandle_t solver_of(Ctx *ctx) {
  if (!ctx->solver) {
    cusolverDnHandle_t h;
    QS_SOLVER(cusolverDnCreate(&h));
    ctx->solver = h;
  }
  cusolverDnHandle_t h = static_cast<cusolverDnHandle_t>(ctx->solver);
  QS_SOLVER(cusolverDnSetStream(h, ctx->stream));
  return h;
}

// Solver lanes: streams with their own cuSOLVER handles, driven from their
// own host threads, so that the decompositions of independent symmetry
// blocks run concurrently (the solver synchronises with its stream inside
// each call, and one medium-size call keeps only part of the GPU busy).
constexpr int NLANES = 8;
constexpr int64_t JACOBI_MAX = 16;     // largest block sent to the batched Jacobi solver
constexpr int64_t EIG_BUCKET = 64;     // larger blocks are padded to a multiple of this

// Estimated GB300 time (ms) of one solver call on nb real blocks of size n,
// fitted to measured XsyevBatched times (one block: 2.2, 5.6, 7.9, 11.8,
// 17.3, 22.7 ms at n = 64, 128, 256, 400, 550, 690; batches: a start-up
// term ~ n^1.57 plus ~ n^2.5 per block beyond two).  Only its ratios
// matter: it balances the work over the solver lanes.
static double eig_unit_ms(int64_t n, int64_t nb) {
  const double x = (double)n;
  if (nb <= 1) return 0.5 + 0.032 * x;
  return 0.00215 * std::pow(x, 1.565) + 2.7e-7 * std::pow(x, 2.5) * double(nb - 2);
}
struct SolverLanes {
  cudaStream_t st[NLANES] = {};
  cusolverDnHandle_t h[NLANES] = {};
  cudaEvent_t ev[NLANES] = {};
};

// Joins the lane threads on every path out of a scope: a throw between two
// thread launches must not destroy a joinable std::thread.
struct ThreadJoiner {
  std::vector<std::thread> &t;
  ~ThreadJoiner() {
    for (auto &x : t)
      if (x.joinable()) x.join();
  }
};

static SolverLanes *lanes_of(Ctx *ctx) {
  if (!ctx->solver_lanes) {
    auto L = new SolverLanes;
    ctx->solver_lanes = L;
    for (int i = 0; i < NLANES; ++i) {
      QS_CUDA(cudaStreamCreateWithFlags(&L->st[i], cudaStreamNonBlocking));
      QS_SOLVER(cusolverDnCreate(&L->h[i]));
      QS_SOLVER(cusolverDnSetStream(L->h[i], L->st[i]));
      QS_CUDA(cudaEventCreateWithFlags(&L->ev[i], cudaEventDisableTiming));
    }
  }
  return static_cast<SolverLanes *>(ctx->solver_lanes);
}

void destroy_solver(Ctx *ctx) {
  if (ctx->solver) cusolverDnDestroy(static_cast<cusolverDnHandle_t>(ctx->solver));
  ctx->solver = nullptr;
  if (ctx->solver_lanes) {
    auto L = static_cast<SolverLanes *>(ctx->solver_lanes);
    for (int i = 0; i < NLANES; ++i) {
      if (L->st[i]) cudaStreamSynchronize(L->st[i]);
      if (L->h[i]) cusolverDnDestroy(L->h[i]);
      if (L->ev[i]) cudaEventDestroy(L->ev[i]);
      if (L->st[i]) cudaStreamDestroy(L->st[i]);
    }
    delete L;
    ctx->solver_lanes = nullptr;
  }
}

namespace {

// dst[i] (+)= ..., block-strided gather/scatter helpers
__global__ void copy_blocks_kernel(const double *__restrict__ src, double *__restrict__ dst,
                                   const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                                   const int64_t *__restrict__ size, int es) {
  const int64_t b = blockIdx.y;
  const int64_t n = size[b] * es;
  const double *s = src + soff[b] * es;
  double *d = dst + doff[b] * es;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = s[i];
}

// V^T for an n x k column-major V (complex: conjugate transpose).
__global__ void transpose_kernel(const double *__restrict__ in, double *__restrict__ out, int64_t n,
                                 int64_t k, int cplx) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * k; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i % n, c = i / n;  // in(r, c)
    if (cplx) {
      const double2 v = reinterpret_cast<const double2 *>(in)[i];
      reinterpret_cast<double2 *>(out)[c + r * k] = make_double2(v.x, -v.y);
    } else {
      out[c + r * k] = in[i];
    }
  }
}

// Per staged eig block b (n[b] x n[b] at soff[b] in U): the value that pads
// it, 1.01 * |H|_F + 1, above every eigenvalue of the block (|lambda| <=
// |H|_2 <= |H|_F).  One CTA per block.
__global__ void pad_value_kernel(const double *__restrict__ U, const int64_t *__restrict__ soff,
                                 const int64_t *__restrict__ nn, int es, double *__restrict__ cval) {
  const int64_t b = blockIdx.x;
  const int64_t cnt = nn[b] * nn[b] * es;
  const double *src = U + soff[b] * es;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) acc = fma(src[i], src[i], acc);
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) cval[b] = 1.01 * sqrt(red[0]) + 1.0;
}

// Staging of eig blocks padded to a common size m: block b (n[b] x n[b] at
// soff[b] in U) becomes the leading part of an m x m matrix at doff[b] in
// the stage, the rest zero except cval[b] on the padded diagonal.  The
// padded matrix is block diagonal, so its first n eigenpairs are the
// block's, with eigenvectors exactly zero in the padded rows.
__global__ void pad_in_kernel(const double *__restrict__ U, double *__restrict__ stage,
                              const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                              const int64_t *__restrict__ nn, int64_t m, const double *__restrict__ cval,
                              int cplx) {
  const int64_t b = blockIdx.y, n = nn[b];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m * m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i % m, c = i / m;
    const bool in = r < n && c < n;
    const double d = (!in && r == c) ? cval[b] : 0.0;
    if (cplx) {
      const double2 v = in ? reinterpret_cast<const double2 *>(U)[soff[b] + r + c * n] : make_double2(d, 0.0);
      reinterpret_cast<double2 *>(stage)[doff[b] + i] = v;
    } else {
      stage[doff[b] + i] = in ? U[soff[b] + r + c * n] : d;
    }
  }
}

// The leading n x n eigenvectors of each padded m x m block back into U.
__global__ void pad_out_kernel(const double *__restrict__ stage, double *__restrict__ U,
                               const int64_t *__restrict__ doff, const int64_t *__restrict__ soff,
                               const int64_t *__restrict__ nn, int64_t m, int cplx) {
  const int64_t b = blockIdx.y, n = nn[b];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i % n, c = i / n;
    if (cplx)
      reinterpret_cast<double2 *>(U)[soff[b] + i] = reinterpret_cast<const double2 *>(stage)[doff[b] + r + c * m];
    else
      U[soff[b] + i] = stage[doff[b] + r + c * m];
  }
}

// c[j] = V(:,j)^T v, one CTA per (chunk, j) accumulated with atomics into
// FP64 partial sums per chunk (deterministic: chunks are reduced in order
// by the second kernel).
constexpr int GS_CHUNK = 8192;
__global__ void gs_dot_kernel(const double *__restrict__ V, const double *__restrict__ v, int64_t n,
                              double *__restrict__ part) {
  const int64_t c = blockIdx.x, j = blockIdx.y;
  const int64_t i0 = c * GS_CHUNK, i1 = min(n, i0 + GS_CHUNK);
  double s = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) s = fma(V[j * n + i], v[i], s);
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[j * gridDim.x + c] = red[0];
}

__global__ void gs_reduce_kernel(const double *__restrict__ part, int64_t nchunk, int64_t nv,
                                 double *__restrict__ coef) {
  const int64_t j = blockIdx.x;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int64_t c = 0; c < nchunk; ++c) s += part[j * nchunk + c];
    coef[j] = s;
  }
}

__global__ void gs_axpy_kernel(const double *__restrict__ V, double *__restrict__ v, int64_t n, int64_t nv,
                               const double *__restrict__ coef) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x = v[i];
    for (int64_t j = 0; j < nv; ++j) x = fma(-coef[j], V[j * n + i], x);
    v[i] = x;
  }
}

__global__ void scale_kernel(double *__restrict__ v, int64_t n, const double *__restrict__ nrm) {
  const double s = nrm[0] > 0 ? 1.0 / sqrt(nrm[0]) : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= s;
}

}  // namespace

// ------------------------------------------------------------- markSet
// Sorted global selection of the kept eigenvalues, restating markSet for the
// ascending direction (Source/gathered.cc:1822-2040) with eigQS's option
// handling (Source/eigQS.cc:55-100): deps > 0 averages near-degenerate
// levels (relative to the spectral width) and moves the cut to the largest
// weighted gap near Nkeep (b = -1, dmax = -1); otherwise the Nkeep lowest
// levels are kept, or those below E_min + Etrunc when Etrunc > 0.
// *nkeep_out is the reference's NK output: the number kept, except with
// Etrunc > 0 and deps = 0, where markSet leaves it at min(Nkeep, N) (only its
// gap-search branch writes the cut back); `keep` holds the kept states.
// With e_avg the levels after the degeneracy averaging go there, in E's
// order: markSet writes them back into the blocks' eigenvalue vectors, so
// eigQS reports averaged levels when deps > 0 (Source/gathered.cc:1851-1866).
void mark_keep_host(int64_t nblk, const int64_t *n, const double *E, int64_t nkeep_in, double etrunc,
                    double deps, uint8_t *keep, int64_t *nkeep_out, double *etrunc_out, double *e_avg) {
  int64_t N = 0;
  for (int64_t i = 0; i < nblk; ++i) N += n[i];
  std::fill(keep, keep + N, 0);
  if (nkeep_out) *nkeep_out = 0;
  if (etrunc_out) *etrunc_out = etrunc;
  if (N == 0) return;
  std::vector<double> e(E, E + N);
  std::vector<int64_t> P(N);
  std::iota(P.begin(), P.end(), 0);
  std::stable_sort(P.begin(), P.end(), [&](int64_t a, int64_t b) { return e[a] < e[b]; });
  std::vector<double> s(N);
  for (int64_t i = 0; i < N; ++i) s[i] = e[P[i]];
  const double b = deps > 0 ? -1.0 : 0.0;
  if (deps > 0) {
    const double eps = deps * std::fabs(s[N - 1] - s[0]);
    int64_t i0 = 0;
    for (int64_t i = 1; i <= N; ++i) {
      if (i == N || std::fabs(s[i] - s[i - 1]) > eps) {
        const int64_t d = i - i0;
        if (d > 1) {
          double avg = 0;
          for (int64_t j = i0; j < i; ++j) avg += s[j];
          avg /= (double)d;
          for (int64_t j = i0; j < i; ++j) s[j] = avg;
        }
        i0 = i;
      }
    }
  }
  if (e_avg)
    for (int64_t i = 0; i < N; ++i) e_avg[P[i]] = s[i];
  int64_t Nkeep = (nkeep_in < 0 || nkeep_in > N) ? N : nkeep_in;
  if (Nkeep == 0) return;
  if (Nkeep >= N && etrunc <= 0) {
    std::fill(keep, keep + N, 1);
    if (nkeep_out) *nkeep_out = N;
    return;
  }
  int64_t l;
  const int64_t Nkmin = 0;
  if (etrunc > 0) {
    const double x = etrunc + s[0];
    for (l = 1; l < N; ++l)
      if (s[l] >= x && l > Nkmin) break;
    if (l > Nkeep) l = Nkeep;
  } else {
    l = Nkeep;
  }
  if (l < N && l > 0 && b < 0) {
    const int64_t nx = std::max<int64_t>(16, l / 5);
    const double q = 10.0 / (-b * (double)nx);
    const int64_t NX = (int64_t)(5.0 / q);
    int64_t i = std::max<int64_t>(1, l - NX);
    const int64_t i2 = std::min<int64_t>(N, l + NX);
    int64_t imax = l;
    double xmax = 0;
    for (; i < i2; ++i) {
      const double t = q * (double)(i - l);
      const double x = std::exp(-t * t) * std::fabs(s[i] - s[i - 1]);
      if (x > xmax) { xmax = x; imax = i; }
    }
    if (i == N) {
      const double t = q * (double)(i - l);
      const double x = 0.1 * std::exp(-t * t) * std::fabs(s[N - 1] - s[0]);
      if (x > xmax) { xmax = x; imax = i; }
    }
    l = imax;
  }
  if (l >= N) l = N;
  for (int64_t i = 0; i < l; ++i) keep[P[i]] = 1;
  if (nkeep_out) *nkeep_out = (etrunc > 0 && !(deps > 0)) ? Nkeep : l;
  if (etrunc_out) *etrunc_out = (l < N) ? s[l] - s[0] : 0.0;
}

// ------------------------------------------------------ markSet on device
// The same truncation with the eigenvalues left on the device: the global
// stable ascending order comes from merging the blocks' ascending runs
// (ties keep the block order, as std::stable_sort over the global index
// does), the degeneracy averaging runs one thread per cluster with the host's
// summation order, and the first level above E_min + Etrunc is found on the
// device.  Only the values around the cut that the weighted-gap search
// reads (at most 2 NX + 1 of them) and s[0], s[N-1] travel to the host, which
// takes the remaining scalar decisions with the host code's arithmetic, so
// keep flags, NK and Etrunc are identical to mark_keep_host.

// Merges runs 2j and 2j+1 of (v, idx) (run r = [bnd[r], bnd[r+1])) into out.
__global__ void merge_runs_kernel(const double *__restrict__ v, const int64_t *__restrict__ ix,
                                  double *__restrict__ ov, int64_t *__restrict__ oix,
                                  const int64_t *__restrict__ bnd, int nruns, int64_t N) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nruns;  // run r with bnd[r] <= e < bnd[r+1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (bnd[mid] <= e) lo = mid; else hi = mid;
    }
    const int r = lo, p = r ^ 1;
    const double x = v[e];
    int64_t pos;
    if (p >= nruns) {
      pos = e;
    } else {
      const int64_t b0 = bnd[p], b1 = bnd[p + 1];
      int64_t a = b0, z = b1;
      if (r & 1) {  // second run: elements of the first run that are <= x go first
        while (a < z) { const int64_t m = (a + z) / 2; if (v[m] <= x) a = m + 1; else z = m; }
      } else {      // first run: elements of the second run that are < x go first
        while (a < z) { const int64_t m = (a + z) / 2; if (v[m] < x) a = m + 1; else z = m; }
      }
      const int64_t start = bnd[r & ~1];
      pos = start + (e - bnd[r]) + (a - b0);
    }
    ov[pos] = x;
    oix[pos] = ix[e];
  }
}

// flag = 1 when any of p[0..n) is not finite (NaN or infinite)
__global__ void nonfinite_kernel(const double *__restrict__ p, int64_t n, int *flag) {
  int bad = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(p[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

// Host check that a device array holds finite values only (one pass, one
// synchronisation).
bool all_finite(Ctx *ctx, const double *p, int64_t n) {
  if (n <= 0) return true;
  int *d = dev_alloc<int>(ctx, 1);
  int h = 0;
  QS_CUDA(cudaMemsetAsync(d, 0, sizeof(int), ctx->stream));
  const int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)std::max(ctx->num_sms, 1) * 8);
  nonfinite_kernel<<<grid, 256, 0, ctx->stream>>>(p, n, d);
  QS_LAUNCHED(ctx);
  QS_CUDA(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, d);
  return h == 0;
}

// flag = 1 + the first element index found out of ascending order inside a
// run of bnd (first run boundary 0, last N)
__global__ void runs_ascending_kernel(const double *__restrict__ v, const int64_t *__restrict__ bnd, int nruns,
                                      unsigned long long *flag) {
  for (int r = blockIdx.x; r < nruns; r += gridDim.x)
    for (int64_t i = bnd[r] + 1 + threadIdx.x; i < bnd[r + 1]; i += blockDim.x)
      if (v[i] < v[i - 1]) atomicMin(flag, (unsigned long long)i);
}

// Stable insertion sort of every run of (v, idx) by v.  Runs that a solver
// returned ascending up to rounding (degenerate levels a unit in the last
// place apart, in either order) take a few steps; the merged order is then
// the stable ascending order of all levels, whatever the input.
__global__ void sort_runs_kernel(double *__restrict__ v, int64_t *__restrict__ idx, const int64_t *__restrict__ bnd,
                                 int nruns) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nruns; r += gridDim.x * blockDim.x) {
    const int64_t a = bnd[r], b = bnd[r + 1];
    for (int64_t i = a + 1; i < b; ++i) {
      const double x = v[i];
      if (!(x < v[i - 1])) continue;
      const int64_t xi = idx[i];
      int64_t j = i;
      while (j > a && v[j - 1] > x) {
        v[j] = v[j - 1];
        idx[j] = idx[j - 1];
        --j;
      }
      v[j] = x;
      idx[j] = xi;
    }
  }
}

// The eigenvalues of every block made non-decreasing: a level below its
// predecessor by at most rel * max|E| of the block (rounding of degenerate
// levels) takes the predecessor's value, so that each block's lowest levels
// are its first eigenvectors.  A larger inversion is not rounding: 1 + its
// index goes to *bad and the level is left as it is.
__global__ void monotone_blocks_kernel(double *__restrict__ E, const int64_t *__restrict__ bnd, int nruns, double rel,
                                       unsigned long long *bad) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nruns; r += gridDim.x * blockDim.x) {
    const int64_t a = bnd[r], b = bnd[r + 1];
    if (b - a < 2) continue;
    const double tol = rel * fmax(fabs(E[a]), fabs(E[b - 1]));
    double m = E[a];
    for (int64_t i = a + 1; i < b; ++i) {
      const double x = E[i];
      if (x >= m) {
        m = x;
      } else if (m - x <= tol) {
        E[i] = m;
      } else {
        atomicMin(bad, (unsigned long long)i);
      }
    }
  }
}

// cnt[P[i]] += 1 for every i; afterwards any cnt != 1 marks a broken order
__global__ void count_targets_kernel(const int64_t *__restrict__ P, int64_t N, int *__restrict__ cnt,
                                     unsigned long long *bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = P[i];
    if (t < 0 || t >= N) atomicMin(bad, (unsigned long long)i);
    else atomicAdd(&cnt[t], 1);
  }
}
__global__ void check_counts_kernel(const int *__restrict__ cnt, int64_t N, unsigned long long *bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    if (cnt[i] != 1) atomicMin(bad, (unsigned long long)i);
}

__global__ void iota_kernel(int64_t *p, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = i;
}

// s (sorted) -> a: clusters of consecutive levels closer than
// eps = deps |s[N-1] - s[0]| replaced by their mean (summed in order);
__global__ void average_clusters_kernel(const double *__restrict__ s, double *__restrict__ a, int64_t N,
                                        double deps) {
  const double eps = deps * fabs(s[N - 1] - s[0]);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    if (!(deps > 0)) {
      a[i] = s[i];
      continue;
    }
    if (i > 0 && !(fabs(s[i] - s[i - 1]) > eps)) continue;  // not the first level of its cluster
    int64_t j = i + 1;
    while (j < N && !(fabs(s[j] - s[j - 1]) > eps)) ++j;
    const int64_t d = j - i;
    if (d > 1) {
      double avg = 0;
      for (int64_t t = i; t < j; ++t) avg += s[t];
      avg /= (double)d;
      for (int64_t t = i; t < j; ++t) a[t] = avg;
    } else {
      a[i] = s[i];
    }
  }
}

// the first l >= 1 with a[l] >= a[0] + etrunc (a ascending), by atomicMin
__global__ void first_above_kernel(const double *__restrict__ a, int64_t N, double etrunc,
                                   unsigned long long *lcut) {
  const double x = etrunc + a[0];
  for (int64_t l = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < N; l += (int64_t)gridDim.x * blockDim.x)
    if (a[l] >= x) atomicMin(lcut, (unsigned long long)l);
}

// out[P[i]] = v[i]: sorted levels back to block order
__global__ void scatter_levels_kernel(const int64_t *__restrict__ P, const double *__restrict__ v, int64_t N,
                                      double *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    out[P[i]] = v[i];
}

__global__ void scatter_keep_kernel(const int64_t *__restrict__ P, int64_t N, int64_t l, uint8_t *__restrict__ keep) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    keep[P[i]] = i < l ? 1 : 0;
}

// kept levels of each block (its lowest ones: a prefix of the block)
__global__ void count_kept_kernel(const uint8_t *__restrict__ keep, const int64_t *__restrict__ eoffs,
                                  const int64_t *__restrict__ n, int64_t nblk, int64_t *__restrict__ k) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nblk; b += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = 0;
    for (int64_t t = 0; t < n[b]; ++t) c += keep[eoffs[b] + t];
    k[b] = c;
  }
}

// Device counterpart of mark_keep_host: dE holds the ascending eigenvalues
// of block i at eoffs[i] (host arrays n, eoffs); d_keep (device, N bytes)
// receives the flags and kcount (host) the kept levels per block.
void mark_keep_dev(Ctx *ctx, int64_t nblk, const int64_t *n, const int64_t *eoffs, const double *dE,
                   int64_t nkeep_in, double etrunc, double deps, uint8_t *d_keep, std::vector<int64_t> &kcount,
                   int64_t *nkeep_out, double *etrunc_out, double *dE_avg) {
  int64_t N = 0;
  for (int64_t i = 0; i < nblk; ++i) N += n[i];
  kcount.assign((size_t)std::max<int64_t>(nblk, 0), 0);
  if (nkeep_out) *nkeep_out = 0;
  if (etrunc_out) *etrunc_out = etrunc;
  if (N == 0) return;
  cudaStream_t st = ctx->stream;
  const int grid = (int)std::min<int64_t>((N + 255) / 256, (int64_t)std::max(ctx->num_sms, 1) * 8);
  // the stable order needs comparable values: a NaN level is an error, as a
  // failed LAPACK call is for the reference
  if (!all_finite(ctx, dE, N)) fail(QS_ERR_NUMERIC, "markSet: non-finite eigenvalues");
  int64_t Nkeep = (nkeep_in < 0 || nkeep_in > N) ? N : nkeep_in;
  int64_t l = 0;
  std::vector<void *> tmp;
  auto alloc = [&](size_t bytes) {
    void *p = dev_alloc<uint8_t>(ctx, std::max<size_t>(bytes, 16));
    tmp.push_back(p);
    return p;
  };
  try {
    // markSet averages the degenerate clusters before it looks at Nkeep:
    // with dE_avg the averaged levels go back there (block order) even when
    // every level is kept
    const bool shortcut = Nkeep == 0 || (Nkeep >= N && etrunc <= 0);
    const bool avg_out = dE_avg && deps > 0;
    if (shortcut) {
      l = Nkeep == 0 ? 0 : N;
      QS_CUDA(cudaMemsetAsync(d_keep, l ? 1 : 0, (size_t)N, st));
    }
    if (!shortcut || avg_out) {
      // stable ascending order: log2(nblk) rounds of pairwise run merges
      double *v0 = static_cast<double *>(alloc(N * 8)), *v1 = static_cast<double *>(alloc(N * 8));
      int64_t *i0 = static_cast<int64_t *>(alloc(N * 8)), *i1 = static_cast<int64_t *>(alloc(N * 8));
      QS_CUDA(cudaMemcpyAsync(v0, dE, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
      iota_kernel<<<grid, 256, 0, st>>>(i0, N);
      QS_LAUNCHED(ctx);
      std::vector<int64_t> bnd;
      for (int64_t b = 0; b < nblk; ++b)
        if (n[b] > 0) bnd.push_back(eoffs[b]);
      bnd.push_back(N);
      // Host arrays reach the device through the context's page-locked
      // staging ring (dev_upload), never by a copy from pageable memory: such
      // a copy may read its source after the call returns, when the source
      // of an earlier round is already gone.
      auto upload = [&](const std::vector<int64_t> &h) {
        int64_t *d = dev_upload(ctx, h);
        tmp.push_back(d);
        return d;
      };
      int64_t *d_bnd = upload(bnd);
      unsigned long long *d_bad = static_cast<unsigned long long *>(alloc(8));
      const unsigned long long none = ~0ull;
      unsigned long long bad = none;
      // the merge needs every block's levels in ascending order: blocks that
      // are not (the caller's levels in any order, or a solver's degenerate
      // levels a rounding apart) are sorted first
      QS_CUDA(cudaMemsetAsync(d_bad, 0xFF, 8, st));
      const int nruns = (int)(bnd.size() - 1);
      runs_ascending_kernel<<<(int)std::min(nruns, 4096), 128, 0, st>>>(v0, d_bnd, nruns, d_bad);
      QS_LAUNCHED(ctx);
      QS_CUDA(cudaMemcpyAsync(&bad, d_bad, 8, cudaMemcpyDeviceToHost, st));
      QS_CUDA(cudaStreamSynchronize(st));
      if (bad != none) {
        sort_runs_kernel<<<(nruns + 127) / 128, 128, 0, st>>>(v0, i0, d_bnd, nruns);
        QS_LAUNCHED(ctx);
      }
      while (bnd.size() > 2) {
        if (bnd.size() - 1 > 0x7fffffff) fail(QS_ERR_SHAPE, "markSet: too many blocks");
        d_bnd = upload(bnd);
        merge_runs_kernel<<<grid, 256, 0, st>>>(v0, i0, v1, i1, d_bnd, (int)(bnd.size() - 1), N);
        QS_LAUNCHED(ctx);
        std::swap(v0, v1);
        std::swap(i0, i1);
        std::vector<int64_t> nb;
        for (size_t r = 0; r + 1 < bnd.size(); r += 2) nb.push_back(bnd[r]);
        nb.push_back(N);
        bnd.swap(nb);
      }
      // the merged order must be a permutation of 0..N-1
      {
        int *d_cnt = static_cast<int *>(alloc(N * 4));
        QS_CUDA(cudaMemsetAsync(d_cnt, 0, (size_t)N * 4, st));
        QS_CUDA(cudaMemsetAsync(d_bad, 0xFF, 8, st));
        count_targets_kernel<<<grid, 256, 0, st>>>(i0, N, d_cnt, d_bad);
        QS_LAUNCHED(ctx);
        check_counts_kernel<<<grid, 256, 0, st>>>(d_cnt, N, d_bad);
        QS_LAUNCHED(ctx);
        QS_CUDA(cudaMemcpyAsync(&bad, d_bad, 8, cudaMemcpyDeviceToHost, st));
        QS_CUDA(cudaStreamSynchronize(st));
        if (bad != none) fail(QS_ERR_INTERNAL, "markSet: merged order is not a permutation (at %llu)", bad);
      }
      // v0 = sorted levels, i0 = their global indices; averaged levels in v1
      const unsigned long long lN = (unsigned long long)N;
      unsigned long long *d_l = reinterpret_cast<unsigned long long *>(upload({(int64_t)N}));
      average_clusters_kernel<<<grid, 256, 0, st>>>(v0, v1, N, deps);
      QS_LAUNCHED(ctx);
      if (avg_out) {
        scatter_levels_kernel<<<grid, 256, 0, st>>>(i0, v1, N, dE_avg);
        QS_LAUNCHED(ctx);
      }
      if (!shortcut) {
        if (etrunc > 0) {
          first_above_kernel<<<grid, 256, 0, st>>>(v1, N, etrunc, d_l);
          QS_LAUNCHED(ctx);
        }
        double ends[2];
        unsigned long long lfirst = lN;
        QS_CUDA(cudaMemcpyAsync(&ends[0], v1, 8, cudaMemcpyDeviceToHost, st));
        QS_CUDA(cudaMemcpyAsync(&ends[1], v1 + N - 1, 8, cudaMemcpyDeviceToHost, st));
        QS_CUDA(cudaMemcpyAsync(&lfirst, d_l, 8, cudaMemcpyDeviceToHost, st));
        QS_CUDA(cudaStreamSynchronize(st));
        l = etrunc > 0 ? std::min<int64_t>((int64_t)lfirst, Nkeep) : Nkeep;
        if (l < N && l > 0 && deps > 0) {
          // weighted-gap search over the window around the cut (host arithmetic)
          const int64_t nx = std::max<int64_t>(16, l / 5);
          const double q = 10.0 / (double)nx;
          const int64_t NX = (int64_t)(5.0 / q);
          int64_t i = std::max<int64_t>(1, l - NX);
          const int64_t i2 = std::min<int64_t>(N, l + NX);
          std::vector<double> w((size_t)(i2 - i + 1));
          QS_CUDA(cudaMemcpyAsync(w.data(), v1 + (i - 1), w.size() * 8, cudaMemcpyDeviceToHost, st));
          QS_CUDA(cudaStreamSynchronize(st));
          const int64_t w0 = i - 1;
          int64_t imax = l;
          double xmax = 0;
          for (; i < i2; ++i) {
            const double t = q * (double)(i - l);
            const double x = std::exp(-t * t) * std::fabs(w[i - w0] - w[i - 1 - w0]);
            if (x > xmax) { xmax = x; imax = i; }
          }
          if (i == N) {
            const double t = q * (double)(i - l);
            const double x = 0.1 * std::exp(-t * t) * std::fabs(ends[1] - ends[0]);
            if (x > xmax) { xmax = x; imax = i; }
          }
          l = imax;
        }
        if (l >= N) l = N;
        scatter_keep_kernel<<<grid, 256, 0, st>>>(i0, N, l, d_keep);
        QS_LAUNCHED(ctx);
        if (etrunc_out) {
          double sl = 0;
          if (l < N) {
            QS_CUDA(cudaMemcpyAsync(&sl, v1 + l, 8, cudaMemcpyDeviceToHost, st));
            QS_CUDA(cudaStreamSynchronize(st));
          }
          *etrunc_out = (l < N) ? sl - ends[0] : 0.0;
        }
      }
    }
    int64_t *d_n = dev_upload(ctx, std::vector<int64_t>(n, n + nblk));
    tmp.push_back(d_n);
    int64_t *d_eo = dev_upload(ctx, std::vector<int64_t>(eoffs, eoffs + nblk));
    tmp.push_back(d_eo);
    int64_t *d_k = static_cast<int64_t *>(alloc(nblk * 8));
    count_kept_kernel<<<(int)std::min<int64_t>((nblk + 127) / 128, 1024), 128, 0, st>>>(d_keep, d_eo, d_n, nblk, d_k);
    QS_LAUNCHED(ctx);
    QS_CUDA(cudaMemcpyAsync(kcount.data(), d_k, nblk * 8, cudaMemcpyDeviceToHost, st));
    QS_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    cudaStreamSynchronize(st);
    for (void *p : tmp) dev_free(ctx, p);
    throw;
  }
  for (void *p : tmp) dev_free(ctx, p);
  if (nkeep_out) *nkeep_out = (etrunc > 0 && !(deps > 0)) ? Nkeep : l;
  if (etrunc_out && (Nkeep == 0 || (Nkeep >= N && etrunc <= 0))) *etrunc_out = etrunc;
}

// ------------------------------------------------------- svd truncation
// The truncation of svdQS: SVD_Data::dmrgTruncate (Source/mpsortho.cc:
// 616-700) with markSet in descending mode (Source/gathered.cc:1822-1880,
// 1964-1972, 2037-2090; no degeneracy averaging, no gap search).  All
// singular values are sorted ascending (stable); with stol > 0 the cut is the
// highest index l < N - Nkmin with S[l] <= stol; the states above the cut are
// kept, at most Nkeep of them (Nkeep < 0: all); the kept values are rescaled
// by sfac = sqrt(sum S^2 / (sum S^2 - discarded S^2)) so that the norm is
// preserved.
void svd_keep_host(int64_t nblk, const int64_t *k, const double *S, int64_t nkeep, int64_t nkmin, double stol,
                   uint8_t *keep, int64_t *nkeep_out, double *s2t_out, double *s2tot_out, double *sfac_out) {
  int64_t N = 0;
  for (int64_t i = 0; i < nblk; ++i) N += k[i];
  std::fill(keep, keep + N, 0);
  if (nkmin < 0) nkmin = 0;
  if (N > 0) {
    std::vector<int64_t> P(N);
    std::iota(P.begin(), P.end(), 0);
    std::stable_sort(P.begin(), P.end(), [&](int64_t a, int64_t b) { return S[a] < S[b]; });
    int64_t nk = nkeep < 0 ? N : nkeep;
    if (nk == 0) {
    } else if (nk >= N && stol <= 0) {
      std::fill(keep, keep + N, 1);
    } else {
      nk = std::min(nk, N);
      int64_t l;               // cut: keep sorted indices l+1 .. N-1
      bool all = false;
      if (stol > 0) {
        const int64_t lx = nkmin < N ? N - nkmin : 0;
        int64_t j = N - 1;
        for (; j >= 0; --j)
          if (S[P[j]] <= stol && j < lx) break;
        if (j < 0) {           // every value above stol (or protected by Nkmin)
          if (N > nk) l = N - 1 - nk;
          else all = true, l = -1;
        } else {
          l = (N - 1 - j > nk) ? N - 1 - nk : j;
        }
      } else {
        l = N - 1 - nk;
      }
      if (all || l < 0) std::fill(keep, keep + N, 1);
      else
        for (int64_t i = l + 1; i < N; ++i) keep[P[i]] = 1;
    }
  }
  double tot = 0, t2 = 0;
  int64_t nkept = 0;
  for (int64_t i = 0; i < N; ++i) {
    tot += S[i] * S[i];
    if (keep[i]) ++nkept; else t2 += S[i] * S[i];
  }
  if (nkeep_out) *nkeep_out = nkept;
  if (s2t_out) *s2t_out = t2;
  if (s2tot_out) *s2tot_out = tot;
  if (sfac_out) *sfac_out = (t2 > 0 && t2 < tot) ? std::sqrt(tot / (tot - t2)) : 1.0;
}

// -------------------------------------------------------------- eig blocks
void eig_blocks(Ctx *ctx, int64_t nblk, const int64_t *n, const int64_t *offs, const int64_t *eoffs,
                const double *H, double *E, double *U, bool cplx) {
  if (nblk <= 0) return;
  cusolverDnHandle_t h = solver_of(ctx);
  const int es = cplx ? 2 : 1;
  for (int64_t i = 0; i < nblk; ++i)
    if (n[i] < 0 || n[i] > INT32_MAX) fail(QS_ERR_SHAPE, "eig: block %lld has size %lld", (long long)i, (long long)n[i]);
  // U <- H (the solvers overwrite their input with the eigenvectors)
  {
    std::vector<int64_t> sz(nblk);
    int64_t mx = 1;
    for (int64_t i = 0; i < nblk; ++i) { sz[i] = n[i] * n[i]; mx = std::max(mx, sz[i]); }
    std::vector<int64_t> so(offs, offs + nblk);
    int64_t *d_so = dev_upload(ctx, so), *d_sz = dev_upload(ctx, sz);
    dim3 g((unsigned)std::min<int64_t>((mx * es + 255) / 256, 1024), (unsigned)nblk);
    if (nblk > 65535) fail(QS_ERR_SHAPE, "eig: too many blocks in one call");
    copy_blocks_kernel<<<g, 256, 0, ctx->stream>>>(H, U, d_so, d_so, d_sz, es);
    QS_LAUNCHED(ctx);
    dev_free(ctx, d_so);
    dev_free(ctx, d_sz);
  }
  // blocks up to JACOBI_MAX rows: one batched Jacobi call per size on the
  // context stream; larger blocks: one solver unit per distinct size (the
  // symmetry sectors of an NRG/DMRG step repeat sizes, e.g. q and -q)
  // Larger blocks are grouped by their size rounded up to a multiple of
  // EIG_BUCKET and padded to it (pad_in_kernel): fewer, larger batched
  // calls.  Measured on a 336-block NRG step: 188 ms by exact size, 176 /
  // 159 / 166 ms with buckets of 32 / 64 / 128.
  // (QS_EIG_BUCKET, 1..1024, overrides the bucket width)
  const char *eb = std::getenv("QS_EIG_BUCKET");
  const int64_t bucket = eb ? std::max<int64_t>(1, std::min<int64_t>(1024, std::atoll(eb))) : EIG_BUCKET;
  std::map<int64_t, std::vector<int64_t>> small, bysize;
  for (int64_t i = 0; i < nblk; ++i) {
    if (n[i] == 0) continue;
    if (n[i] <= JACOBI_MAX) small[n[i]].push_back(i);
    else bysize[(n[i] + bucket - 1) / bucket * bucket].push_back(i);
  }
  // units: (size, blocks); a unit is solved in place when its blocks follow
  // one another in U and E, otherwise through a staging copy
  struct Unit {
    int ni;
    int64_t first;     // index of its first block in `order` / the info array
    int nb;
    bool inplace;
  };
  std::vector<Unit> units;
  std::vector<int64_t> order;
  // One unit per size.  Splitting groups of large blocks into single-block
  // solves (faster alone: 22.7 ms for one n = 690 block against 60 ms for a
  // batch of two) was slower over a whole NRG step on eight lanes (218-233 ms
  // against 189 ms): concurrent single solves contend for the GPU, while the
  // batched algorithm's time per block keeps falling with the batch.
  for (auto &kv : bysize) {
    const int64_t ni = kv.first, bs = ni * ni;
    const auto &g = kv.second;
    Unit u{(int)ni, (int64_t)order.size(), (int)g.size(), true};
    for (size_t j = 0; j < g.size(); ++j) {
      if (n[g[j]] != ni || offs[g[j]] != offs[g[0]] + (int64_t)j * bs ||
          eoffs[g[j]] != eoffs[g[0]] + (int64_t)j * ni)
        u.inplace = false;
      order.push_back(g[j]);
    }
    units.push_back(u);
  }
  const int64_t nlarge = (int64_t)order.size();
  int *d_info = dev_alloc<int>(ctx, (size_t)std::max<int64_t>(nlarge, 1));
  QS_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int) * std::max<int64_t>(nlarge, 1), ctx->stream));
  // units spread over the solver lanes (largest first, each to the lane with
  // the least work so far), concurrent with the Jacobi calls on the context
  // stream
  std::vector<void *> bufs;      // device buffers released after the join
  std::vector<int> used;
  SolverLanes *L = nullptr;
  if (!units.empty()) {
    L = lanes_of(ctx);
    std::vector<int> uo(units.size());
    std::iota(uo.begin(), uo.end(), 0);
    auto cost = [&](int u) { return eig_unit_ms(units[u].ni, units[u].nb); };
    std::sort(uo.begin(), uo.end(), [&](int x, int y) { return cost(x) > cost(y); });
    // QS_EIG_LANES (1..8) overrides the number of concurrent lanes (eight
    // measured best for an NRG step on GB300: 189 ms, four 252 ms, twelve or
    // sixteen 237 ms)
    const char *el = std::getenv("QS_EIG_LANES");
    const int want = el ? std::max(1, std::min(NLANES, std::atoi(el))) : NLANES;
    const int nl = (int)std::min<size_t>(want, units.size());
    std::vector<std::vector<int>> part(nl);
    std::vector<double> load(nl, 0.0);
    for (int u : uo) {
      const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      part[l].push_back(u);
      load[l] += cost(u);
    }
    // per lane: device workspace, host workspace and staging area, sized for
    // its largest unit; gather/scatter tables for the staged units
    std::vector<cusolverDnParams_t> prm(nl, nullptr);
    std::vector<size_t> wdev(nl, 0), whost(nl, 0);
    const cudaDataType dtA = cplx ? CUDA_C_64F : CUDA_R_64F;
    std::vector<double *> work(nl, nullptr), stage(nl, nullptr), wstage(nl, nullptr);
    std::vector<std::vector<char>> hwork(nl);
    std::vector<int64_t> so, dof, sz, eo, ed, ez;  // per staged block: U/E offsets <-> staging offsets, sizes
    std::vector<int64_t> tab(units.size(), -1);    // first table row of a staged unit
    for (int l = 0; l < nl; ++l) {
      QS_SOLVER(cusolverDnCreateParams(&prm[l]));
      int64_t sa = 0, se = 0;
      for (int u : part[l]) {
        Unit &un = units[u];
        const int ni = un.ni;
        size_t wd = 0, wh = 0;
        QS_SOLVER(cusolverDnXsyevBatched_bufferSize(L->h[l], prm[l], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                                    ni, dtA, U, ni, CUDA_R_64F, E, dtA, &wd, &wh, un.nb));
        wdev[l] = std::max(wdev[l], wd);
        whost[l] = std::max(whost[l], wh);
        if (!un.inplace) {
          const int64_t bs = (int64_t)ni * ni;
          tab[u] = (int64_t)so.size();
          for (int j = 0; j < un.nb; ++j) {
            const int64_t i = order[un.first + j];
            so.push_back(offs[i]); dof.push_back(bs * j); sz.push_back(n[i]);
            eo.push_back(eoffs[i]); ed.push_back((int64_t)ni * j); ez.push_back(n[i]);
          }
          sa = std::max(sa, bs * un.nb);
          se = std::max(se, (int64_t)ni * un.nb);
        }
      }
      work[l] = dev_alloc<double>(ctx, (wdev[l] + 7) / 8 + 1);
      bufs.push_back(work[l]);
      hwork[l].resize(whost[l] + 16);
      if (sa) {
        stage[l] = dev_alloc<double>(ctx, (size_t)sa * es);
        wstage[l] = dev_alloc<double>(ctx, (size_t)se);
        bufs.push_back(stage[l]);
        bufs.push_back(wstage[l]);
      }
    }
    int64_t *d_tab = nullptr;
    if (!so.empty()) {
      std::vector<int64_t> t;
      for (auto *v : {&so, &dof, &sz, &eo, &ed, &ez}) t.insert(t.end(), v->begin(), v->end());
      d_tab = dev_upload(ctx, t);
      bufs.push_back(d_tab);
    }
    const int64_t nt = (int64_t)so.size();
    double *cval = nullptr;
    if (nt) {
      cval = dev_alloc<double>(ctx, (size_t)nt);
      bufs.push_back(cval);
      pad_value_kernel<<<(unsigned)nt, 256, 0, ctx->stream>>>(U, d_tab, d_tab + 2 * nt, es, cval);
      QS_LAUNCHED(ctx);
    }
    cudaEvent_t fork;
    QS_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    QS_CUDA(cudaEventRecord(fork, ctx->stream));
    // one host thread per lane: the solver synchronises with its stream
    // inside each call, so lanes driven from one thread would not overlap
    std::vector<std::thread> th;
    ThreadJoiner joiner{th};
    std::vector<std::exception_ptr> errs(nl);
    const int dev = ctx->device;
    int64_t nlaunch = 0;
    for (int l = 0; l < nl; ++l) {
      QS_CUDA(cudaStreamWaitEvent(L->st[l], fork, 0));
      used.push_back(l);
      for (int u : part[l]) nlaunch += units[u].inplace ? 1 : 4;
      th.emplace_back([&, l]() {
        try {
          QS_CUDA(cudaSetDevice(dev));
          for (int u : part[l]) {
            const Unit &un = units[u];
            const int ni = un.ni;
            int *info = d_info + un.first;
            const int64_t i0 = order[un.first];
            double *A = U + offs[i0] * es, *W = E + eoffs[i0];
            const int64_t bs = (int64_t)ni * ni;
            const int64_t *t = d_tab + (tab[u] < 0 ? 0 : tab[u]);
            dim3 g((unsigned)std::min<int64_t>((bs * es + 255) / 256, 256), (unsigned)un.nb);
            dim3 g2((unsigned)std::min<int64_t>((ni + 255) / 256, 4), (unsigned)un.nb);
            if (!un.inplace) {
              A = stage[l];
              W = wstage[l];
              pad_in_kernel<<<g, 256, 0, L->st[l]>>>(U, A, t, t + nt, t + 2 * nt, ni, cval + tab[u], cplx ? 1 : 0);
              QS_CUDA(cudaGetLastError());
            }
            QS_SOLVER(cusolverDnXsyevBatched(L->h[l], prm[l], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ni,
                                             dtA, A, ni, CUDA_R_64F, W, dtA, work[l], wdev[l],
                                             hwork[l].data(), whost[l], info, un.nb));
            if (!un.inplace) {
              pad_out_kernel<<<g, 256, 0, L->st[l]>>>(A, U, t + nt, t, t + 2 * nt, ni, cplx ? 1 : 0);
              QS_CUDA(cudaGetLastError());
              copy_blocks_kernel<<<g2, 256, 0, L->st[l]>>>(W, E, t + 4 * nt, t + 3 * nt, t + 5 * nt, 1);
              QS_CUDA(cudaGetLastError());
            }
          }
          QS_CUDA(cudaEventRecord(L->ev[l], L->st[l]));
        } catch (...) {
          errs[l] = std::current_exception();
        }
      });
    }
    ctx->launches += nlaunch;
    for (auto &t : th) t.join();
    cudaEventDestroy(fork);
    for (auto *p : prm)
      if (p) cusolverDnDestroyParams(p);
    for (auto &e : errs)
      if (e) {
        for (int l : used) cudaStreamSynchronize(L->st[l]);
        used.clear();
        for (void *p : bufs) dev_free(ctx, p);
        bufs.clear();
        dev_free(ctx, d_info);
        std::rethrow_exception(e);
      }
  }
  // rejoins the lanes on the context stream (also on the error path, so that
  // the workspaces are not released while a lane still uses them)
  auto join = [&]() {
    for (int l : used) cudaStreamWaitEvent(ctx->stream, L->ev[l], 0);
    used.clear();
    for (void *p : bufs) dev_free(ctx, p);
    bufs.clear();
  };
  try {
  // small blocks: batched Jacobi on contiguous copies
  if (!small.empty()) {
    syevjInfo_t params;
    QS_SOLVER(cusolverDnCreateSyevjInfo(&params));
    QS_SOLVER(cusolverDnXsyevjSetTolerance(params, 1e-15));
    QS_SOLVER(cusolverDnXsyevjSetMaxSweeps(params, 100));
    for (auto &kv : small) {
      const int ni = (int)kv.first;
      const int nb = (int)kv.second.size();
      const int64_t bs = (int64_t)ni * ni;
      double *Ab = dev_alloc<double>(ctx, (size_t)bs * nb * es);
      double *Wb = dev_alloc<double>(ctx, (size_t)ni * nb);
      int *ib = dev_alloc<int>(ctx, nb);
      std::vector<int64_t> so, dof, sz, eo, ed, es1;
      for (int j = 0; j < nb; ++j) {
        so.push_back(offs[kv.second[j]]);
        dof.push_back(bs * j);
        sz.push_back(bs);
        eo.push_back((int64_t)ni * j);
        ed.push_back(eoffs[kv.second[j]]);
        es1.push_back(ni);
      }
      int64_t *d_so = dev_upload(ctx, so), *d_do = dev_upload(ctx, dof), *d_sz = dev_upload(ctx, sz);
      dim3 g((unsigned)std::min<int64_t>((bs * es + 255) / 256, 64), (unsigned)nb);
      copy_blocks_kernel<<<g, 256, 0, ctx->stream>>>(U, Ab, d_so, d_do, d_sz, es);
      QS_LAUNCHED(ctx);
      int lwork = 0;
      if (cplx)
        QS_SOLVER(cusolverDnZheevjBatched_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ni,
                                                     reinterpret_cast<cuDoubleComplex *>(Ab), ni, Wb, &lwork,
                                                     params, nb));
      else
        QS_SOLVER(cusolverDnDsyevjBatched_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ni, Ab,
                                                     ni, Wb, &lwork, params, nb));
      double *work = dev_alloc<double>(ctx, (size_t)std::max(lwork, 1) * es);
      if (cplx)
        QS_SOLVER(cusolverDnZheevjBatched(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ni,
                                          reinterpret_cast<cuDoubleComplex *>(Ab), ni, Wb,
                                          reinterpret_cast<cuDoubleComplex *>(work), lwork, ib, params, nb));
      else
        QS_SOLVER(cusolverDnDsyevjBatched(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, ni, Ab, ni, Wb, work,
                                          lwork, ib, params, nb));
      ctx->launches++;
      // scatter vectors and values back
      copy_blocks_kernel<<<g, 256, 0, ctx->stream>>>(Ab, U, d_do, d_so, d_sz, es);
      QS_LAUNCHED(ctx);
      int64_t *d_eo = dev_upload(ctx, eo), *d_ed = dev_upload(ctx, ed), *d_es = dev_upload(ctx, es1);
      dim3 g2(1, (unsigned)nb);
      copy_blocks_kernel<<<g2, 64, 0, ctx->stream>>>(Wb, E, d_eo, d_ed, d_es, 1);
      QS_LAUNCHED(ctx);
      std::vector<int> hinfo(nb);
      QS_CUDA(cudaMemcpyAsync(hinfo.data(), ib, nb * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      QS_CUDA(cudaStreamSynchronize(ctx->stream));
      for (void *p : {(void *)Ab, (void *)Wb, (void *)ib, (void *)work, (void *)d_so, (void *)d_do, (void *)d_sz,
                      (void *)d_eo, (void *)d_ed, (void *)d_es})
        dev_free(ctx, p);
      for (int j = 0; j < nb; ++j) {
        if (hinfo[j] < 0) fail(QS_ERR_NUMERIC, "syevjBatched: argument error %d", hinfo[j]);
        if (hinfo[j] > 0)
          fail(QS_ERR_NUMERIC, "eig: block %lld (%d x %d) did not converge in the Jacobi solver (info %d)",
               (long long)kv.second[j], ni, ni, hinfo[j]);
      }
    }
    cusolverDnDestroySyevjInfo(params);
  }
  } catch (...) {
    join();
    dev_free(ctx, d_info);
    throw;
  }
  join();
  std::vector<int> info(std::max<int64_t>(nlarge, 1));
  QS_CUDA(cudaMemcpyAsync(info.data(), d_info, info.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, d_info);
  for (int64_t k = 0; k < nlarge; ++k)
    if (info[k] != 0)
      fail(QS_ERR_NUMERIC, "eig: block %lld did not converge (info %d)", (long long)order[k], info[k]);
}

// -------------------------------------------------------------- svd blocks
// Block SVDs, three solvers:
//  * a caller that bounds the Jacobi iteration (max_sweeps or tol given)
//    gets one Jacobi SVD (gesvdj) per block on the context's stream;
//  * otherwise blocks of at most 32 x 32 go, grouped by shape, to the
//    batched Jacobi solver (gesvdjBatched) on the context's stream,
//  * and the larger ones to the polar-decomposition SVD (Xgesvdp: QDWH
//    polar factor, then a Hermitian eigensolver), spread over the solver
//    lanes.  Measured on GB300 for one square FP64 block of n = 354 / 708 /
//    1416: gesvdj 198 / 577 / 1842 ms, Xgesvd 70 / 226 / 752 ms, Xgesvdp
//    33 / 82 / 268 ms (LAPACK's dgesdd on 16 Grace cores: 22 / 117 /
//    395 ms).  Xgesvdp wants M >= N: a wide block is decomposed as A^H.
// A block that does not converge fails the call with QS_ERR_NUMERIC, like
// the reference's wbSVD, which stops on a LAPACK info != 0
// (Source/wbarray_blas.cc:1040-1060).
constexpr int64_t SVD_BATCHED_MAX = 32;  // gesvdjBatched takes m, n <= 32

// V^T (conjugate transpose for complex) of nb blocks of n x k, block b read
// at soff[b], written at doff[b] (offsets in elements).
__global__ void transpose_blocks_kernel(const double *__restrict__ in, double *__restrict__ out,
                                        const int64_t *__restrict__ soff, const int64_t *__restrict__ doff,
                                        int64_t n, int64_t k, int cplx) {
  const int64_t b = blockIdx.y;
  const int es = cplx ? 2 : 1;
  const double *src = in + soff[b] * es;
  double *dst = out + doff[b] * es;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * k; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i % n, c = i / n;
    if (cplx) {
      const double2 v = reinterpret_cast<const double2 *>(src)[i];
      reinterpret_cast<double2 *>(dst)[c + r * k] = make_double2(v.x, -v.y);
    } else {
      dst[c + r * k] = src[i];
    }
  }
}

// Estimated GB300 time (ms) of one Xgesvdp call on an M x N block (M >= N),
// real: fitted to 33 / 82 / 268 ms at n = 354 / 708 / 1416 (complex about
// twice).  Only its ratios matter: it balances the blocks over the lanes.
static double svdp_ms(int64_t M, int64_t N) {
  return 5.0 + 2.2e-3 * std::pow((double)M * (double)N * (double)N, 0.55);
}

static void svd_batched(Ctx *ctx, const std::vector<int64_t> &ids, const int64_t *m, const int64_t *n,
                        const int64_t *offs, const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs,
                        const double *A, double *U, double *S, double *Vt, int cplx) {
  if (ids.empty()) return;
  const int64_t es = cplx ? 2 : 1;
  cusolverDnHandle_t h = solver_of(ctx);
  // (a group holds at most 32768 blocks: the copy kernels put one block per
  // grid row, and gridDim.y stops at 65535)
  std::map<std::tuple<int64_t, int64_t, int64_t>, std::vector<int64_t>> byshape;
  std::map<std::pair<int64_t, int64_t>, int64_t> seen;
  for (int64_t i : ids) {
    const int64_t c = seen[{m[i], n[i]}]++;
    byshape[{m[i], n[i], c / 32768}].push_back(i);
  }
  gesvdjInfo_t params;
  QS_SOLVER(cusolverDnCreateGesvdjInfo(&params));
  struct ParamsGuard {
    gesvdjInfo_t p;
    ~ParamsGuard() { cusolverDnDestroyGesvdjInfo(p); }
  } guard{params};
  QS_SOLVER(cusolverDnXgesvdjSetTolerance(params, 1e-15));
  QS_SOLVER(cusolverDnXgesvdjSetMaxSweeps(params, 100));
  for (auto &kv : byshape) {
    const int mi = (int)std::get<0>(kv.first), ni = (int)std::get<1>(kv.first), k = std::min(mi, ni);
    const int nb = (int)kv.second.size();
    // staging: A (m x n), U (m x m), V (n x n), S (k) per block, back to back
    std::vector<int64_t> so, ao, asz, uo, ud, usz, vo, vd, sso, sd, ssz;
    for (int j = 0; j < nb; ++j) {
      const int64_t i = kv.second[j];
      so.push_back(offs[i]); ao.push_back((int64_t)mi * ni * j); asz.push_back((int64_t)mi * ni);
      uo.push_back((int64_t)mi * mi * j); ud.push_back(uoffs[i]); usz.push_back((int64_t)mi * k);
      vo.push_back((int64_t)ni * ni * j); vd.push_back(voffs[i]);
      sso.push_back((int64_t)k * j); sd.push_back(soffs[i]); ssz.push_back(k);
    }
    std::vector<void *> bufs;
    auto take = [&](void *p) { bufs.push_back(p); return p; };
    try {
      double *Ab = (double *)take(dev_alloc<double>(ctx, (size_t)mi * ni * nb * es));
      double *Ub = (double *)take(dev_alloc<double>(ctx, (size_t)mi * mi * nb * es));
      double *Vb = (double *)take(dev_alloc<double>(ctx, (size_t)ni * ni * nb * es));
      double *Sb = (double *)take(dev_alloc<double>(ctx, (size_t)k * nb));
      int *ib = (int *)take(dev_alloc<int>(ctx, nb));
      int64_t *t_so = (int64_t *)take(dev_upload(ctx, so)), *t_ao = (int64_t *)take(dev_upload(ctx, ao));
      int64_t *t_asz = (int64_t *)take(dev_upload(ctx, asz)), *t_uo = (int64_t *)take(dev_upload(ctx, uo));
      int64_t *t_ud = (int64_t *)take(dev_upload(ctx, ud)), *t_usz = (int64_t *)take(dev_upload(ctx, usz));
      int64_t *t_vo = (int64_t *)take(dev_upload(ctx, vo)), *t_vd = (int64_t *)take(dev_upload(ctx, vd));
      int64_t *t_sso = (int64_t *)take(dev_upload(ctx, sso)), *t_sd = (int64_t *)take(dev_upload(ctx, sd));
      int64_t *t_ssz = (int64_t *)take(dev_upload(ctx, ssz));
      const dim3 ga((unsigned)std::min<int64_t>(((int64_t)mi * ni * es + 255) / 256, 16), (unsigned)nb);
      copy_blocks_kernel<<<ga, 256, 0, ctx->stream>>>(A, Ab, t_so, t_ao, t_asz, (int)es);
      QS_LAUNCHED(ctx);
      int lwork = 0;
      if (cplx)
        QS_SOLVER(cusolverDnZgesvdjBatched_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, mi, ni, (cuDoubleComplex *)Ab, mi,
                                                      Sb, (cuDoubleComplex *)Ub, mi, (cuDoubleComplex *)Vb, ni,
                                                      &lwork, params, nb));
      else
        QS_SOLVER(cusolverDnDgesvdjBatched_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, mi, ni, Ab, mi, Sb, Ub, mi, Vb,
                                                      ni, &lwork, params, nb));
      double *work = (double *)take(dev_alloc<double>(ctx, (size_t)std::max(lwork, 1) * es));
      if (cplx)
        QS_SOLVER(cusolverDnZgesvdjBatched(h, CUSOLVER_EIG_MODE_VECTOR, mi, ni, (cuDoubleComplex *)Ab, mi, Sb,
                                           (cuDoubleComplex *)Ub, mi, (cuDoubleComplex *)Vb, ni,
                                           (cuDoubleComplex *)work, lwork, ib, params, nb));
      else
        QS_SOLVER(cusolverDnDgesvdjBatched(h, CUSOLVER_EIG_MODE_VECTOR, mi, ni, Ab, mi, Sb, Ub, mi, Vb, ni, work,
                                           lwork, ib, params, nb));
      ctx->launches++;
      // the first k columns of U (contiguous m x k), the k values, V^H
      const dim3 gu((unsigned)std::min<int64_t>(((int64_t)mi * k * es + 255) / 256, 16), (unsigned)nb);
      copy_blocks_kernel<<<gu, 256, 0, ctx->stream>>>(Ub, U, t_uo, t_ud, t_usz, (int)es);
      QS_LAUNCHED(ctx);
      copy_blocks_kernel<<<dim3(1, (unsigned)nb), 64, 0, ctx->stream>>>(Sb, S, t_sso, t_sd, t_ssz, 1);
      QS_LAUNCHED(ctx);
      const dim3 gv((unsigned)std::min<int64_t>(((int64_t)ni * k + 255) / 256, 16), (unsigned)nb);
      transpose_blocks_kernel<<<gv, 256, 0, ctx->stream>>>(Vb, Vt, t_vo, t_vd, ni, k, cplx);
      QS_LAUNCHED(ctx);
      std::vector<int> hinfo(nb);
      QS_CUDA(cudaMemcpyAsync(hinfo.data(), ib, nb * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      QS_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int j = 0; j < nb; ++j) {
        if (hinfo[j] < 0) fail(QS_ERR_NUMERIC, "svd: block %lld argument error %d", (long long)kv.second[j], hinfo[j]);
        if (hinfo[j] > 0)
          fail(QS_ERR_NUMERIC, "svd: block %lld (%d x %d) did not converge in the batched Jacobi solver (info %d)",
               (long long)kv.second[j], mi, ni, hinfo[j]);
      }
    } catch (...) {
      cudaStreamSynchronize(ctx->stream);
      for (void *q : bufs) dev_free(ctx, q);
      throw;
    }
    for (void *q : bufs) dev_free(ctx, q);
  }
}

// The larger blocks: Xgesvdp, largest first onto the lane with the least
// estimated work, one host thread per lane (the solver synchronises with
// its stream inside each call).  `meanwhile` runs on the calling thread
// while the lanes work.
static void svd_polar_lanes(Ctx *ctx, const std::vector<int64_t> &ids, const int64_t *m, const int64_t *n,
                            const int64_t *offs, const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs,
                            const double *A, double *U, double *S, double *Vt, int cplx,
                            const std::function<void()> &meanwhile) {
  if (ids.empty()) {
    meanwhile();
    return;
  }
  const int64_t es = cplx ? 2 : 1;
  const cudaDataType dt = cplx ? CUDA_C_64F : CUDA_R_64F;
  SolverLanes *L = lanes_of(ctx);
  std::vector<int64_t> order(ids);
  auto cost = [&](int64_t i) { return svdp_ms(std::max(m[i], n[i]), std::min(m[i], n[i])); };
  std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return cost(x) > cost(y); });
  // QS_SVD_LANES (1..8) overrides the number of concurrent lanes
  const char *sl = std::getenv("QS_SVD_LANES");
  const int want = sl ? std::max(1, std::min(NLANES, std::atoi(sl))) : NLANES;
  const int nl = (int)std::min<size_t>(want, order.size());
  std::vector<std::vector<int64_t>> part(nl);
  std::vector<double> load(nl, 0.0);
  for (int64_t i : order) {
    const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    part[l].push_back(i);
    load[l] += cost(i);
  }
  // per lane: the solver's device and host workspaces, a staging copy of the
  // block (Xgesvdp overwrites its input) and the factor that is transposed
  std::vector<cusolverDnParams_t> prm(nl, nullptr);
  std::vector<size_t> wdev(nl, 0), whost(nl, 0);
  std::vector<double *> work(nl, nullptr), stage(nl, nullptr), tmp(nl, nullptr);
  std::vector<std::vector<char>> hwork(nl);
  std::vector<void *> bufs;
  int *d_info = nullptr;
  std::vector<int> used;
  auto release = [&]() {
    for (int l : used) cudaStreamSynchronize(L->st[l]);
    for (void *q : bufs) dev_free(ctx, q);
    bufs.clear();
    if (d_info) dev_free(ctx, d_info);
    d_info = nullptr;
    for (auto *q : prm)
      if (q) cusolverDnDestroyParams(q);
    prm.assign(nl, nullptr);
  };
  std::vector<double> err(order.size() + 1, 0.0);
  std::vector<int64_t> slot(order.size());
  try {
    int64_t ns = 0;
    for (int l = 0; l < nl; ++l) {
      QS_SOLVER(cusolverDnCreateParams(&prm[l]));
      int64_t sa = 0, st = 0;
      for (int64_t i : part[l]) {
        const int64_t M = std::max(m[i], n[i]), N = std::min(m[i], n[i]);
        size_t wd = 0, wh = 0;
        QS_SOLVER(cusolverDnXgesvdp_bufferSize(L->h[l], prm[l], CUSOLVER_EIG_MODE_VECTOR, 1, M, N, dt, A, M,
                                               CUDA_R_64F, S, dt, U, M, dt, Vt, N, dt, &wd, &wh));
        wdev[l] = std::max(wdev[l], wd);
        whost[l] = std::max(whost[l], wh);
        sa = std::max(sa, M * N);
        st = std::max(st, M * N);      // the transposed factor: N x N (tall) or M x N (wide)
        slot[ns++] = i;
      }
      work[l] = dev_alloc<double>(ctx, (wdev[l] + 7) / 8 + 1);
      bufs.push_back(work[l]);
      stage[l] = dev_alloc<double>(ctx, (size_t)sa * es);
      bufs.push_back(stage[l]);
      tmp[l] = dev_alloc<double>(ctx, (size_t)st * es);
      bufs.push_back(tmp[l]);
      hwork[l].resize(whost[l] + 16);
    }
    d_info = dev_alloc<int>(ctx, order.size());
    QS_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int) * order.size(), ctx->stream));
    cudaEvent_t fork;
    QS_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    QS_CUDA(cudaEventRecord(fork, ctx->stream));
    std::vector<std::thread> th;
    ThreadJoiner joiner{th};
    std::vector<std::exception_ptr> errs(nl);
    const int dev = ctx->device;
    int64_t base = 0;
    for (int l = 0; l < nl; ++l) {
      QS_CUDA(cudaStreamWaitEvent(L->st[l], fork, 0));
      used.push_back(l);
      th.emplace_back([&, l, base]() {
        try {
          QS_CUDA(cudaSetDevice(dev));
          cudaStream_t sl = L->st[l];
          for (size_t q = 0; q < part[l].size(); ++q) {
            const int64_t i = part[l][q];
            const int64_t mi = m[i], ni = n[i], k = std::min(mi, ni);
            const bool tall = mi >= ni;
            const int64_t M = tall ? mi : ni, N = tall ? ni : mi;
            const int64_t tot = mi * ni;
            const unsigned g = (unsigned)std::min<int64_t>((tot + 255) / 256, 1024);
            if (tall) {
              QS_CUDA(cudaMemcpyAsync(stage[l], A + offs[i] * es, (size_t)(tot * es) * 8, cudaMemcpyDeviceToDevice, sl));
            } else {
              transpose_kernel<<<g, 256, 0, sl>>>(A + offs[i] * es, stage[l], mi, ni, cplx);  // A^H
              QS_CUDA(cudaGetLastError());
            }
            // tall: U -> the output, V -> tmp; wide (A^H = U' S V'^H): V' -> U, U' -> tmp
            double *uo = tall ? U + uoffs[i] * es : tmp[l];
            double *vo = tall ? tmp[l] : U + uoffs[i] * es;
            double e = 0.0;
            QS_SOLVER(cusolverDnXgesvdp(L->h[l], prm[l], CUSOLVER_EIG_MODE_VECTOR, 1, M, N, dt, stage[l], M,
                                        CUDA_R_64F, S + soffs[i], dt, uo, M, dt, vo, N, dt, work[l], wdev[l],
                                        hwork[l].data(), whost[l], d_info + base + (int64_t)q, &e));
            err[base + q] = e;
            // Vt = (the factor in tmp)^H: n x k -> k x n
            transpose_kernel<<<(unsigned)std::min<int64_t>((ni * k + 255) / 256, 1024), 256, 0, sl>>>(
                tmp[l], Vt + voffs[i] * es, ni, k, cplx);
            QS_CUDA(cudaGetLastError());
          }
          QS_CUDA(cudaEventRecord(L->ev[l], sl));
        } catch (...) {
          errs[l] = std::current_exception();
        }
      });
      base += (int64_t)part[l].size();
    }
    std::exception_ptr mw;
    try {
      meanwhile();
    } catch (...) {
      mw = std::current_exception();
    }
    for (auto &t : th) t.join();
    if (mw) {
      cudaEventDestroy(fork);
      std::rethrow_exception(mw);
    }
    cudaEventDestroy(fork);
    for (size_t q = 0; q < order.size(); ++q) ctx->launches += (m[slot[q]] >= n[slot[q]] ? 2 : 3);
    for (auto &e : errs)
      if (e) std::rethrow_exception(e);
    for (int l : used) QS_CUDA(cudaStreamWaitEvent(ctx->stream, L->ev[l], 0));
    std::vector<int> info(order.size());
    QS_CUDA(cudaMemcpyAsync(info.data(), d_info, info.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QS_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t q = 0; q < order.size(); ++q) {
      const int64_t i = slot[q];
      if (info[q] != 0 || !std::isfinite(err[q]))
        fail(QS_ERR_NUMERIC, "svd: block %lld (%lld x %lld) failed in the polar-decomposition solver (info %d)",
             (long long)i, (long long)m[i], (long long)n[i], info[q]);
    }
  } catch (...) {
    release();
    throw;
  }
  release();
}

static void svd_jacobi_each(Ctx *ctx, int64_t nblk, const int64_t *m, const int64_t *n, const int64_t *offs,
                            const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs, const double *A,
                            double *U, double *S, double *Vt, int cplx, int max_sweeps, double tol);

void svd_blocks(Ctx *ctx, int64_t nblk, const int64_t *m, const int64_t *n, const int64_t *offs,
                const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs, const double *A, double *U,
                double *S, double *Vt, int cplx, int max_sweeps, double tol) {
  if (nblk <= 0) return;
  for (int64_t i = 0; i < nblk; ++i)
    if (m[i] < 0 || n[i] < 0 || m[i] > INT32_MAX || n[i] > INT32_MAX) fail(QS_ERR_SHAPE, "svd: bad block size");
  if (max_sweeps > 0 || tol > 0) {
    if (max_sweeps <= 0) max_sweeps = 100;
    if (!(tol > 0)) tol = 1e-15;
    svd_jacobi_each(ctx, nblk, m, n, offs, uoffs, soffs, voffs, A, U, S, Vt, cplx, max_sweeps, tol);
    return;
  }
  std::vector<int64_t> tiny, large;
  for (int64_t i = 0; i < nblk; ++i) {
    if (m[i] == 0 || n[i] == 0) continue;
    (m[i] <= SVD_BATCHED_MAX && n[i] <= SVD_BATCHED_MAX ? tiny : large).push_back(i);
  }
  // the batched Jacobi calls run on the context stream while the lanes
  // work; both write disjoint output slots
  svd_polar_lanes(ctx, large, m, n, offs, uoffs, soffs, voffs, A, U, S, Vt, cplx, [&]() {
    svd_batched(ctx, tiny, m, n, offs, uoffs, soffs, voffs, A, U, S, Vt, cplx);
  });
}

// One Jacobi SVD (gesvdj) per block on the context's stream with the
// caller's sweep limit and tolerance; the copy of the block, V and the
// solver workspace are allocated once for the largest block and reused.
static void svd_jacobi_each(Ctx *ctx, int64_t nblk, const int64_t *m, const int64_t *n, const int64_t *offs,
                            const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs, const double *A,
                            double *U, double *S, double *Vt, int cplx, int max_sweeps, double tol) {
  const int64_t es = cplx ? 2 : 1;  // doubles per element
  cusolverDnHandle_t h = solver_of(ctx);
  gesvdjInfo_t params;
  QS_SOLVER(cusolverDnCreateGesvdjInfo(&params));
  struct ParamsGuard {
    gesvdjInfo_t p;
    ~ParamsGuard() { cusolverDnDestroyGesvdjInfo(p); }
  } guard{params};
  QS_SOLVER(cusolverDnXgesvdjSetTolerance(params, tol));
  QS_SOLVER(cusolverDnXgesvdjSetMaxSweeps(params, max_sweeps));
  int64_t maxa = 0, maxv = 0;
  int lwork = 1;
  for (int64_t i = 0; i < nblk; ++i) {
    const int64_t mi = m[i], ni = n[i];
    if (mi < 0 || ni < 0 || mi > INT32_MAX || ni > INT32_MAX) fail(QS_ERR_SHAPE, "svd: bad block size");
    if (mi == 0 || ni == 0) continue;
    maxa = std::max(maxa, mi * ni);
    maxv = std::max(maxv, ni * std::min(mi, ni));
  }
  if (maxa == 0) return;
  double *a = dev_alloc<double>(ctx, (size_t)(maxa * es));
  double *v = dev_alloc<double>(ctx, (size_t)(maxv * es));
  int *d_info = dev_alloc<int>(ctx, (size_t)nblk);
  double *work = nullptr;
  try {
    // workspace for the largest need over the distinct block shapes
    std::vector<std::pair<int64_t, int64_t>> shapes;
    for (int64_t i = 0; i < nblk; ++i)
      if (m[i] > 0 && n[i] > 0) shapes.emplace_back(m[i], n[i]);
    std::sort(shapes.begin(), shapes.end());
    shapes.erase(std::unique(shapes.begin(), shapes.end()), shapes.end());
    for (auto &sh : shapes) {
      const int mi = (int)sh.first, ni = (int)sh.second;
      int lw = 0;
      if (cplx)
        QS_SOLVER(cusolverDnZgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, mi, ni, (cuDoubleComplex *)a, mi, S,
                                               (cuDoubleComplex *)U, mi, (cuDoubleComplex *)v, ni, &lw, params));
      else
        QS_SOLVER(cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, mi, ni, a, mi, S, U, mi, v, ni, &lw,
                                               params));
      lwork = std::max(lwork, lw);
    }
    work = dev_alloc<double>(ctx, (size_t)lwork * es);
    QS_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int) * nblk, ctx->stream));
    for (int64_t i = 0; i < nblk; ++i) {
      const int64_t mi = m[i], ni = n[i];
      if (mi == 0 || ni == 0) continue;
      const int64_t k = std::min(mi, ni);
      QS_CUDA(cudaMemcpyAsync(a, A + offs[i] * es, (size_t)(mi * ni * es) * 8, cudaMemcpyDeviceToDevice,
                              ctx->stream));
      if (cplx)
        QS_SOLVER(cusolverDnZgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)mi, (int)ni, (cuDoubleComplex *)a, (int)mi,
                                    S + soffs[i], (cuDoubleComplex *)(U + uoffs[i] * es), (int)mi,
                                    (cuDoubleComplex *)v, (int)ni, (cuDoubleComplex *)work, lwork, d_info + i,
                                    params));
      else
        QS_SOLVER(cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)mi, (int)ni, a, (int)mi, S + soffs[i],
                                    U + uoffs[i], (int)mi, v, (int)ni, work, lwork, d_info + i, params));
      ctx->launches++;
      const int64_t tot = ni * k;
      transpose_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 1024), 256, 0, ctx->stream>>>(
          v, Vt + voffs[i] * es, ni, k, cplx);
      QS_LAUNCHED(ctx);
    }
    std::vector<int> info(nblk);
    QS_CUDA(cudaMemcpyAsync(info.data(), d_info, nblk * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QS_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int64_t i = 0; i < nblk; ++i) {
      if (info[i] < 0) fail(QS_ERR_NUMERIC, "svd: block %lld argument error %d", (long long)i, info[i]);
      if (info[i] > 0)
        fail(QS_ERR_NUMERIC, "svd: block %lld (%lld x %lld) did not converge within %d sweeps (info %d)",
             (long long)i, (long long)m[i], (long long)n[i], max_sweeps, info[i]);
    }
  } catch (...) {
    cudaStreamSynchronize(ctx->stream);  // buffers may be in use by queued work
    dev_free(ctx, a);
    dev_free(ctx, v);
    dev_free(ctx, d_info);
    if (work) dev_free(ctx, work);
    throw;
  }
  dev_free(ctx, a);
  dev_free(ctx, v);
  dev_free(ctx, d_info);
  dev_free(ctx, work);
}

// ------------------------------------------------------------ Gram-Schmidt
void gs_reortho(Ctx *ctx, int64_t n, int64_t nv, const double *V, double *v, double *norm_out) {
  if (n <= 0) fail(QS_ERR_ARG, "gs_reortho: empty vector");
  if (nv < 0 || nv > 65535) fail(QS_ERR_ARG, "gs_reortho: bad basis size");
  const int64_t nch = (n + GS_CHUNK - 1) / GS_CHUNK;
  if (nch > 0x7fffffff) fail(QS_ERR_SHAPE, "gs_reortho: vector too long");
  double *part = dev_alloc<double>(ctx, (size_t)(nch * std::max<int64_t>(nv, 1)));
  double *coef = dev_alloc<double>(ctx, (size_t)std::max<int64_t>(nv, 1));
  const unsigned gax = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 16);
  for (int pass = 0; pass < 2 && nv > 0; ++pass) {
    gs_dot_kernel<<<dim3((unsigned)nch, (unsigned)nv), 256, 0, ctx->stream>>>(V, v, n, part);
    QS_LAUNCHED(ctx);
    gs_reduce_kernel<<<(unsigned)nv, 32, 0, ctx->stream>>>(part, nch, nv, coef);
    QS_LAUNCHED(ctx);
    gs_axpy_kernel<<<gax, 256, 0, ctx->stream>>>(V, v, n, nv, coef);
    QS_LAUNCHED(ctx);
  }
  // |v|^2 with the same chunked reduction (v against itself)
  gs_dot_kernel<<<dim3((unsigned)nch, 1), 256, 0, ctx->stream>>>(v, v, n, part);
  QS_LAUNCHED(ctx);
  gs_reduce_kernel<<<1, 32, 0, ctx->stream>>>(part, nch, 1, coef);
  QS_LAUNCHED(ctx);
  scale_kernel<<<gax, 256, 0, ctx->stream>>>(v, n, coef);
  QS_LAUNCHED(ctx);
  double nrm2 = 0;
  QS_CUDA(cudaMemcpyAsync(&nrm2, coef, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QS_CUDA(cudaStreamSynchronize(ctx->stream));
  if (norm_out) *norm_out = std::sqrt(nrm2);
  dev_free(ctx, part);
  dev_free(ctx, coef);
}

}  // namespace qs

using namespace qs;

extern "C" {

qs_status qs_eig_blocks(qs_ctx *ctx, int64_t nblk, const int64_t *n, const int64_t *offs, const int64_t *eoffs,
                        const double *H, double *E, double *U, int32_t is_complex) {
  QS_API_BEGIN
  if (!ctx || (nblk > 0 && (!n || !offs || !eoffs || !H || !E || !U))) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  eig_blocks(&ctx->c, nblk, n, offs, eoffs, H, E, U, is_complex != 0);
  QS_API_END
}

qs_status qs_mark_keep(int64_t nblk, const int64_t *n, const double *E, const double *qdim_w, int64_t nkeep,
                       double etrunc, double deps, uint8_t *keep, int64_t *nkeep_out, double *etrunc_out) {
  QS_API_BEGIN
  if (nblk < 0 || (nblk > 0 && (!n || !E || !keep))) fail(QS_ERR_ARG, "null argument");
  if (qdim_w) fail(QS_ERR_UNSUPPORTED, "multiplet weights: markSet counts every multiplet once; pass NULL");
  mark_keep_host(nblk, n, E, nkeep, etrunc, deps, keep, nkeep_out, etrunc_out, nullptr);
  QS_API_END
}

qs_status qs_average_levels(int64_t nblk, const int64_t *n, const double *E, double deps, double *E_out) {
  QS_API_BEGIN
  if (nblk < 0 || (nblk > 0 && (!n || !E || !E_out))) fail(QS_ERR_ARG, "null argument");
  int64_t N = 0;
  for (int64_t i = 0; i < nblk; ++i) {
    if (n[i] < 0) fail(QS_ERR_ARG, "negative block size");
    N += n[i];
  }
  if (N == 0) return QS_OK;
  std::vector<uint8_t> keep((size_t)N);
  mark_keep_host(nblk, n, E, -1, 0.0, deps, keep.data(), nullptr, nullptr, E_out);
  QS_API_END
}

// eigQS on a device-resident block-diagonal rank-2 QSpace (EigenSymmetric,
// Source/QSpace.cc:4673-4939, with markSet, Source/gathered.cc:1822-2040):
// block eig on the device, the global truncation on the host from the
// eigenvalues alone (a few bytes per state), and the kept / discarded
// eigenvectors gathered into device tensors AK / AD without leaving the
// device.  Every block's kept states are its lowest ones (markSet keeps a
// prefix of the ascending global order), i.e. its first k columns.
}  // extern "C"

namespace qs {
void eigqs_core(Ctx *c, const qs_tensor *H, int64_t nkeep, double etrunc, double deps,
                std::unique_ptr<qs_tensor> &AK, std::unique_ptr<qs_tensor> &AD, double *E, uint8_t *keep,
                int64_t *nkeep_out, double *etrunc_out) {
  const QMeta &m = H->meta;
  if (m.rank != 2) fail(QS_ERR_SHAPE, "eigQS: rank-2 QSpace required (got rank %d)", m.rank);
  const int64_t nb = m.nblk;
  std::vector<int64_t> n(nb), eoffs(nb);
  int64_t ntot = 0;
  for (int64_t i = 0; i < nb; ++i) {
    const int64_t *d = m.drow(i);
    if (d[0] != d[1]) fail(QS_ERR_SHAPE, "eigQS: block %lld is %lld x %lld, not square", (long long)i, (long long)d[0], (long long)d[1]);
    const int32_t *q = m.qrow(i);
    for (int j = 0; j < m.qdim; ++j)
      if (q[j] != q[m.qdim + j]) fail(QS_ERR_LABEL, "eigQS: block %lld is not on the diagonal", (long long)i);
    n[i] = d[0];
    eoffs[i] = ntot;
    ntot += d[0];
  }
  const int es = m.cplx ? 2 : 1;
  double *U = dev_alloc<double>(c, (size_t)std::max<int64_t>(m.nelem, 1) * es);
  double *dE = dev_alloc<double>(c, (size_t)std::max<int64_t>(ntot, 1));
  uint8_t *d_keep = nullptr;
  std::vector<double> hE((size_t)std::max<int64_t>(ntot, 1));
  std::vector<uint8_t> hk((size_t)std::max<int64_t>(ntot, 1));
  int64_t nk = 0;
  double et = 0;
  try {
    if (!all_finite(c, H->d, m.nelem * es)) fail(QS_ERR_NUMERIC, "eigQS: H holds non-finite entries");
    eig_blocks(c, nb, n.data(), m.offs.data(), eoffs.data(), H->d, dE, U, m.cplx);
    // each block's levels non-decreasing (solvers order degenerate levels
    // only up to rounding), so that its kept levels are its first columns
    if (ntot > 0) {
      std::vector<int64_t> bnd;
      for (int64_t i = 0; i < nb; ++i)
        if (n[i] > 0) bnd.push_back(eoffs[i]);
      bnd.push_back(ntot);
      int64_t *d_bnd = dev_upload(c, bnd);
      unsigned long long *d_bad = dev_alloc<unsigned long long>(c, 1);
      QS_CUDA(cudaMemsetAsync(d_bad, 0xFF, 8, c->stream));
      const int nruns = (int)(bnd.size() - 1);
      monotone_blocks_kernel<<<(nruns + 127) / 128, 128, 0, c->stream>>>(dE, d_bnd, nruns, 64 * DBL_EPSILON, d_bad);
      QS_LAUNCHED(c);
      unsigned long long bad = 0;
      QS_CUDA(cudaMemcpyAsync(&bad, d_bad, 8, cudaMemcpyDeviceToHost, c->stream));
      QS_CUDA(cudaStreamSynchronize(c->stream));
      dev_free(c, d_bnd);
      dev_free(c, d_bad);
      if (bad != ~0ull) fail(QS_ERR_NUMERIC, "eigQS: the solver returned level %llu below its predecessor", bad);
    }
    // markSet on the device: the eigenvalues stay there; the host gets the
    // kept count of every block (a prefix: its lowest levels)
    std::vector<int64_t> k;
    d_keep = dev_alloc<uint8_t>(c, (size_t)std::max<int64_t>(ntot, 1));
    mark_keep_dev(c, nb, n.data(), eoffs.data(), dE, nkeep, etrunc, deps, d_keep, k, &nk, &et, dE);
    for (int64_t i = 0; i < nb; ++i)
      if (k[i] < 0 || k[i] > n[i])
        fail(QS_ERR_INTERNAL, "eigQS: block %lld keeps %lld of %lld states", (long long)i, (long long)k[i],
             (long long)n[i]);
    if (E && ntot) QS_CUDA(cudaMemcpyAsync(hE.data(), dE, ntot * 8, cudaMemcpyDeviceToHost, c->stream));
    if (keep && ntot) QS_CUDA(cudaMemcpyAsync(hk.data(), d_keep, ntot, cudaMemcpyDeviceToHost, c->stream));
    auto part = [&](bool kept) {
      auto T = std::make_unique<qs_tensor>();
      T->ctx = c;
      QMeta &o = T->meta;
      o.rank = 2;
      o.qdim = m.qdim;
      o.cplx = m.cplx;
      o.itags = m.itags;
      std::vector<int64_t> so, dof, sz;
      int64_t off = 0;
      for (int64_t i = 0; i < nb; ++i) {
        const int64_t cols = kept ? k[i] : n[i] - k[i];
        if (cols == 0) continue;
        const int32_t *q = m.qrow(i);
        o.q.insert(o.q.end(), q, q + 2 * m.qdim);
        o.dims.push_back(n[i]);
        o.dims.push_back(cols);
        o.offs.push_back(off);
        so.push_back(m.offs[i] + (kept ? 0 : n[i] * k[i]));  // first or remaining columns
        dof.push_back(off);
        sz.push_back(n[i] * cols);
        off += n[i] * cols;
      }
      o.nblk = (int64_t)o.offs.size();
      o.nelem = off;
      T->d = dev_alloc<double>(c, (size_t)std::max<int64_t>(off, 1) * es);
      if (o.nblk) {
        int64_t mx = 1;
        for (int64_t v : sz) mx = std::max(mx, v);
        int64_t *d_so = dev_upload(c, so), *d_do = dev_upload(c, dof), *d_sz = dev_upload(c, sz);
        if (o.nblk > 65535) fail(QS_ERR_SHAPE, "eigQS: too many blocks in one call");
        dim3 g((unsigned)std::min<int64_t>((mx * es + 255) / 256, 1024), (unsigned)o.nblk);
        copy_blocks_kernel<<<g, 256, 0, c->stream>>>(U, T->d, d_so, d_do, d_sz, es);
        QS_LAUNCHED(c);
        dev_free(c, d_so);
        dev_free(c, d_do);
        dev_free(c, d_sz);
      }
      return T;
    };
    std::unique_ptr<qs_tensor> tk = part(true), td = part(false);
    QS_CUDA(cudaStreamSynchronize(c->stream));  // host copies of E / keep
    dev_free(c, U);
    dev_free(c, dE);
    dev_free(c, d_keep);
    U = dE = nullptr;
    d_keep = nullptr;
    if (E && ntot) std::memcpy(E, hE.data(), ntot * 8);
    if (keep && ntot) std::memcpy(keep, hk.data(), ntot);
    if (nkeep_out) *nkeep_out = nk;
    if (etrunc_out) *etrunc_out = et;
    AK = std::move(tk);
    AD = std::move(td);
  } catch (...) {
    cudaStreamSynchronize(c->stream);
    if (U) dev_free(c, U);
    if (dE) dev_free(c, dE);
    if (d_keep) dev_free(c, d_keep);
    throw;
  }
}

int64_t eigqs_footprint(const QMeta &m) {
  // eigenvectors, the kept and discarded copies, eigenvalues
  const int64_t es = m.cplx ? 16 : 8;
  int64_t ntot = 0;
  for (int64_t i = 0; i < m.nblk; ++i) ntot += m.drow(i)[0];
  return 2 * m.nelem * es + ntot * 8 + (64 << 20);
}
}  // namespace qs

extern "C" {

qs_status qs_eigQS_dev(qs_ctx *ctx, const qs_tensor *H, int64_t nkeep, double etrunc, double deps, qs_tensor **AK,
                       qs_tensor **AD, double *E, uint8_t *keep, int64_t *nkeep_out, double *etrunc_out) {
  QS_API_BEGIN
  if (!ctx || !H || !AK || !AD) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  std::unique_ptr<qs_tensor> tk, td;
  eigqs_core(&ctx->c, H, nkeep, etrunc, deps, tk, td, E, keep, nkeep_out, etrunc_out);
  *AK = tk.release();
  *AD = td.release();
  QS_API_END
}

qs_status qs_mark_keep_dev(qs_ctx *ctx, int64_t nblk, const int64_t *n, const double *E, int64_t nkeep,
                           double etrunc, double deps, uint8_t *keep, int64_t *nkeep_out, double *etrunc_out) {
  QS_API_BEGIN
  if (!ctx || nblk < 0 || (nblk > 0 && (!n || !E || !keep))) fail(QS_ERR_ARG, "null argument");
  std::vector<int64_t> eoffs((size_t)nblk);
  int64_t tot = 0;
  for (int64_t i = 0; i < nblk; ++i) {
    if (n[i] < 0) fail(QS_ERR_ARG, "negative block size");
    eoffs[i] = tot;
    tot += n[i];
  }
  QS_CUDA(cudaSetDevice(ctx->c.device));
  std::vector<int64_t> k;
  mark_keep_dev(&ctx->c, nblk, n, eoffs.data(), E, nkeep, etrunc, deps, keep, k, nkeep_out, etrunc_out, nullptr);
  QS_API_END
}

qs_status qs_svd_keep(int64_t nblk, const int64_t *k, const double *S, int64_t nkeep, int64_t nkmin, double stol,
                      uint8_t *keep, int64_t *nkeep_out, double *s2t_out, double *s2tot_out, double *sfac_out) {
  QS_API_BEGIN
  if (nblk < 0 || (nblk > 0 && (!k || !S || !keep))) fail(QS_ERR_ARG, "null argument");
  for (int64_t i = 0; i < nblk; ++i)
    if (k[i] < 0) fail(QS_ERR_ARG, "negative singular value count");
  svd_keep_host(nblk, k, S, nkeep, nkmin, stol, keep, nkeep_out, s2t_out, s2tot_out, sfac_out);
  QS_API_END
}

qs_status qs_svd_blocks(qs_ctx *ctx, int64_t nblk, const int64_t *m, const int64_t *n, const int64_t *offs,
                        const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs, const double *A, double *U,
                        double *S, double *Vt) {
  QS_API_BEGIN
  if (!ctx || (nblk > 0 && (!m || !n || !offs || !uoffs || !soffs || !voffs || !A || !U || !S || !Vt)))
    fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  svd_blocks(&ctx->c, nblk, m, n, offs, uoffs, soffs, voffs, A, U, S, Vt, 0, 0, 0.0);
  QS_API_END
}

qs_status qs_svd_blocks_ex(qs_ctx *ctx, int64_t nblk, const int64_t *m, const int64_t *n, const int64_t *offs,
                           const int64_t *uoffs, const int64_t *soffs, const int64_t *voffs, int32_t is_complex,
                           const double *A, double *U, double *S, double *Vt, int32_t max_sweeps, double tol) {
  QS_API_BEGIN
  if (!ctx || (nblk > 0 && (!m || !n || !offs || !uoffs || !soffs || !voffs || !A || !U || !S || !Vt)))
    fail(QS_ERR_ARG, "null argument");
  if (max_sweeps < 0) fail(QS_ERR_ARG, "svd: negative sweep limit");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  svd_blocks(&ctx->c, nblk, m, n, offs, uoffs, soffs, voffs, A, U, S, Vt, is_complex ? 1 : 0, max_sweeps, tol);
  QS_API_END
}

qs_status qs_gs_reortho(qs_ctx *ctx, int64_t n, int64_t nv, const double *V, double *v, double *norm_out) {
  QS_API_BEGIN
  if (!ctx || !v || (nv > 0 && !V)) fail(QS_ERR_ARG, "null argument");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  gs_reortho(&ctx->c, n, nv, V, v, norm_out);
  QS_API_END
}

}  // extern "C"
