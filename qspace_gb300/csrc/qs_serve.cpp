// Serving loop: continuous batching of contractions and block eigen-
// decompositions (eigQS) between device-resident tensors for many concurrent
// NRG / DMRG instances.  (The reference has no counterpart: its MEX calls
// run one at a time from MATLAB.)
//
//  * qs_server_submit enqueues a request (FIFO) and records an event on the
//    submitting context's stream, so the request sees every earlier write to
//    its operands; the results belong to that context (freed on its stream,
//    after its own later uses).  qs_server_submit_from names the submitting
//    context (one per client instance); qs_server_submit uses the server's.
//  * nslots worker threads each own a stream, a scratch arena and an error
//    word (a qs::Ctx).  A worker takes the head of the queue as soon as the
//    request's device footprint fits into the HBM budget next to the
//    requests already running, together with up to max_batch - 1 further
//    queued requests with the same options that also fit; the block
//    products of the whole batch run in one grouped launch.  Requests that
//    arrive while others are on the GPU are admitted as slots and memory
//    free up, and their kernels overlap on the device.  A request larger than the whole budget is
//    refused at submit time (QS_ERR_OOM).
//  * An eig request (qs_server_submit_eig) runs alone on a slot -- its block
//    eigensolver already spreads the blocks over concurrent solver lanes --
//    next to the contraction batches of the other slots.
//  * Results are identical alone and in the mix: every kernel is
//    deterministic (fixed reduction order) and requests share no buffers.
//  * qs_server_poll waits a bounded time; qs_server_cancel removes a
//    request that has not started.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>

#include "qs_objects.h"

using namespace qs;

namespace {

using clk = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  enum Kind { CONTRACT, EIG } kind = CONTRACT;
  const qs_tensor *A = nullptr, *B = nullptr;  // eig: A = H
  std::string ia, ib;
  std::vector<int32_t> perm;
  qs_opts opts{};
  bool has_opts = false;
  cudaEvent_t ready = nullptr;
  Ctx *owner = nullptr;            // context whose stream orders the request and frees its results
  int64_t footprint = 0;
  clk::time_point t_submit;
  enum State { QUEUED, RUNNING, DONE, FAILED, CANCELLED } state = QUEUED;
  qs_status status = QS_OK;
  std::string err;
  qs_tensor *C = nullptr;
  double latency_ms = 0;
  // eig requests: truncation options and results (C = kept eigenvectors)
  int64_t nkeep = -1;
  double etrunc = 0, deps = 0;
  qs_tensor *D = nullptr;         // discarded eigenvectors
  std::vector<double> E;          // eigenvalues, H's block order
  std::vector<uint8_t> keep;
  int64_t nk = 0;
  double et = 0;
};

}  // namespace

struct qs_server {
  qs_ctx *parent = nullptr;
  std::vector<std::unique_ptr<Ctx>> slots;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<int64_t, std::shared_ptr<Request>> reqs;
  int64_t next_ticket = 1;
  int64_t budget = 0, in_use = 0;
  bool stop = false;

  int max_batch = 16;

  static bool same_opts(const Request &a, const Request &b) {
    if (a.kind != Request::CONTRACT || b.kind != Request::CONTRACT) return false;  // eig requests run alone
    if (a.has_opts != b.has_opts) return false;
    if (!a.has_opts) return true;
    return a.opts.prec == b.opts.prec && a.opts.nslices == b.opts.nslices && a.opts.tol == b.opts.tol;
  }

  // Completes one request (under the lock).
  void complete(Request &r, qs_status st, const std::string &msg, qs_tensor *C) {
    in_use -= r.footprint;
    r.latency_ms = std::chrono::duration<double, std::milli>(clk::now() - r.t_submit).count();
    r.status = st;
    r.err = msg;
    r.C = C;
    r.state = st == QS_OK ? Request::DONE : Request::FAILED;
    if (r.ready) {
      cudaEventDestroy(r.ready);
      r.ready = nullptr;
    }
  }

  void worker(Ctx *slot) {
    cudaSetDevice(slot->device);
    for (;;) {
      std::vector<std::shared_ptr<Request>> batch;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] {
          return stop || (!queue.empty() && in_use + queue.front()->footprint <= budget);
        });
        if (stop) return;
        batch.push_back(queue.front());
        queue.pop_front();
        in_use += batch[0]->footprint;
        // continuous batching: queued requests with the same options that
        // fit next to it join the launch
        for (auto it = queue.begin(); it != queue.end() && (int)batch.size() < max_batch;) {
          if (same_opts(**it, *batch[0]) && in_use + (*it)->footprint <= budget) {
            in_use += (*it)->footprint;
            batch.push_back(*it);
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
        for (auto &r : batch) r->state = Request::RUNNING;
      }
      const int n = (int)batch.size();
      std::vector<qs_status> st(n, QS_OK);
      std::vector<std::string> msg(n);
      std::vector<qs_tensor *> C(n, nullptr);
      auto run_alone = [&](int k) {
        Request &r = *batch[k];
        try {
          auto T = contract_core(slot, r.A->meta, r.A->d, r.B->meta, r.B->d, r.ia.c_str(), r.ib.c_str(),
                                 r.perm.empty() ? nullptr : r.perm.data(), (int32_t)r.perm.size(),
                                 r.has_opts ? &r.opts : nullptr, nullptr);
          QS_CUDA(cudaStreamSynchronize(slot->stream));
          T->ctx = r.owner;  // the submitter frees the result on its context's stream
          C[k] = T.release();
        } catch (const Error &e) {
          st[k] = e.code;
          msg[k] = e.what();
        } catch (const std::exception &e) {
          st[k] = QS_ERR_INTERNAL;
          msg[k] = e.what();
        }
      };
      try {
        for (auto &r : batch)
          if (r->ready) QS_CUDA(cudaStreamWaitEvent(slot->stream, r->ready, 0));
        if (batch[0]->kind == Request::EIG) {
          Request &r = *batch[0];
          try {
            std::unique_ptr<qs_tensor> tk, td;
            int64_t ntot = 0;
            for (int64_t i = 0; i < r.A->meta.nblk; ++i) ntot += r.A->meta.drow(i)[0];
            r.E.assign((size_t)std::max<int64_t>(ntot, 1), 0.0);
            r.keep.assign((size_t)std::max<int64_t>(ntot, 1), 0);
            eigqs_core(slot, r.A, r.nkeep, r.etrunc, r.deps, tk, td, r.E.data(), r.keep.data(), &r.nk, &r.et);
            QS_CUDA(cudaStreamSynchronize(slot->stream));
            tk->ctx = r.owner;
            td->ctx = r.owner;
            C[0] = tk.release();
            r.D = td.release();
          } catch (const Error &e) {
            st[0] = e.code;
            msg[0] = e.what();
          } catch (const std::exception &e) {
            st[0] = QS_ERR_INTERNAL;
            msg[0] = e.what();
          }
        } else if (n == 1) {
          run_alone(0);
        } else {
          std::vector<const QMeta *> am(n), bm(n);
          std::vector<const double *> ad(n), bd(n);
          std::vector<const char *> ia(n), ib(n);
          std::vector<const int32_t *> pp(n);
          std::vector<int32_t> np(n);
          for (int k = 0; k < n; ++k) {
            const Request &r = *batch[k];
            am[k] = &r.A->meta;
            bm[k] = &r.B->meta;
            ad[k] = r.A->d;
            bd[k] = r.B->d;
            ia[k] = r.ia.c_str();
            ib[k] = r.ib.c_str();
            pp[k] = r.perm.empty() ? nullptr : r.perm.data();
            np[k] = (int32_t)r.perm.size();
          }
          std::vector<std::unique_ptr<qs_tensor>> out;
          try {
            contract_batch_core(slot, n, am.data(), ad.data(), bm.data(), bd.data(), ia.data(), ib.data(),
                                pp.data(), np.data(), batch[0]->has_opts ? &batch[0]->opts : nullptr, out);
            QS_CUDA(cudaStreamSynchronize(slot->stream));
            for (int k = 0; k < n; ++k) {
              out[k]->ctx = batch[k]->owner;
              C[k] = out[k].release();
            }
          } catch (...) {
            // a failed batch: each request again on its own, so that every
            // request gets its own status
            cudaStreamSynchronize(slot->stream);
            cudaGetLastError();
            for (int k = 0; k < n; ++k) run_alone(k);
          }
        }
      } catch (const Error &e) {
        for (int k = 0; k < n; ++k) {
          st[k] = e.code;
          msg[k] = e.what();
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        for (int k = 0; k < n; ++k) complete(*batch[k], st[k], msg[k], C[k]);
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

extern "C" {

qs_status qs_server_create(qs_ctx *ctx, const qs_server_cfg *cfg, qs_server **out) {
  QS_API_BEGIN
  if (!ctx || !cfg || !out) fail(QS_ERR_ARG, "null argument");
  if (cfg->nslots < 1 || cfg->nslots > 256) fail(QS_ERR_ARG, "nslots must be in 1..256");
  if (cfg->hbm_budget <= 0) fail(QS_ERR_ARG, "hbm_budget must be positive");
  QS_CUDA(cudaSetDevice(ctx->c.device));
  auto s = std::make_unique<qs_server>();
  s->parent = ctx;
  s->budget = cfg->hbm_budget;
  if (cfg->max_batch < 0 || cfg->max_batch > 1024) fail(QS_ERR_ARG, "max_batch must be in 0..1024");
  if (cfg->max_batch > 0) s->max_batch = cfg->max_batch;
  for (int i = 0; i < cfg->nslots; ++i) {
    auto c = std::make_unique<Ctx>();
    c->device = ctx->c.device;
    c->num_sms = ctx->c.num_sms;
    QS_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    QS_CUDA(cudaMalloc(&c->d_err, 64));
    QS_CUDA(cudaMemset(c->d_err, 0, 64));
    s->slots.push_back(std::move(c));
  }
  for (auto &c : s->slots) s->workers.emplace_back(&qs_server::worker, s.get(), c.get());
  *out = s.release();
  QS_API_END
}

void qs_server_destroy(qs_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  for (auto &kv : s->reqs) {
    if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    delete kv.second->C;  // results nobody collected
    delete kv.second->D;
  }
  for (auto &c : s->slots) {
    if (c->scratch) cudaFreeAsync(c->scratch, c->stream);
    cudaStreamSynchronize(c->stream);
    destroy_solver(c.get());
    cudaFree(c->d_err);
    c->destroy_copy_streams();
    c->destroy_staging();
    cudaStreamDestroy(c->stream);
  }
  delete s;
}

qs_status qs_server_submit(qs_server *s, const qs_tensor *A, const char *ia, const qs_tensor *B, const char *ib,
                           const int32_t *perm, int32_t nperm, const qs_opts *opts, int64_t *ticket) {
  return qs_server_submit_from(s, nullptr, A, ia, B, ib, perm, nperm, opts, ticket);
}

qs_status qs_server_submit_from(qs_server *s, qs_ctx *client, const qs_tensor *A, const char *ia,
                                const qs_tensor *B, const char *ib, const int32_t *perm, int32_t nperm,
                                const qs_opts *opts, int64_t *ticket) {
  QS_API_BEGIN
  if (!s || !A || !B || !ia || !ib || !ticket) fail(QS_ERR_ARG, "null argument");
  Ctx *owner = client ? &client->c : &s->parent->c;
  if (owner->device != s->parent->c.device) fail(QS_ERR_ARG, "the client context is on another device");
  // validate the request on the host now: a malformed request fails here,
  // not in a worker
  (void)parse_ctr_idx(ia);
  (void)parse_ctr_idx(ib);
  const int64_t fp = contract_footprint(A->meta, B->meta, ia, ib, opts);
  if (fp > s->budget)
    fail(QS_ERR_OOM, "admission refused: request needs %lld bytes, budget is %lld", (long long)fp,
         (long long)s->budget);
  auto r = std::make_shared<Request>();
  r->A = A;
  r->B = B;
  r->ia = ia;
  r->ib = ib;
  if (perm && nperm > 0) r->perm.assign(perm, perm + nperm);
  if (opts) {
    r->opts = *opts;
    r->has_opts = true;
  }
  r->footprint = fp;
  r->owner = owner;
  QS_CUDA(cudaSetDevice(s->parent->c.device));
  QS_CUDA(cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming));
  QS_CUDA(cudaEventRecord(r->ready, owner->stream));
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    r->t_submit = clk::now();
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  QS_API_END
}

qs_status qs_server_submit_eig(qs_server *s, const qs_tensor *H, int64_t nkeep, double etrunc, double deps,
                               int64_t *ticket) {
  return qs_server_submit_eig_from(s, nullptr, H, nkeep, etrunc, deps, ticket);
}

qs_status qs_server_submit_eig_from(qs_server *s, qs_ctx *client, const qs_tensor *H, int64_t nkeep,
                                    double etrunc, double deps, int64_t *ticket) {
  QS_API_BEGIN
  if (!s || !H || !ticket) fail(QS_ERR_ARG, "null argument");
  Ctx *owner = client ? &client->c : &s->parent->c;
  if (owner->device != s->parent->c.device) fail(QS_ERR_ARG, "the client context is on another device");
  if (H->meta.rank != 2) fail(QS_ERR_SHAPE, "eig request: rank-2 QSpace required (got rank %d)", H->meta.rank);
  const int64_t fp = eigqs_footprint(H->meta);
  if (fp > s->budget)
    fail(QS_ERR_OOM, "admission refused: request needs %lld bytes, budget is %lld", (long long)fp,
         (long long)s->budget);
  auto r = std::make_shared<Request>();
  r->kind = Request::EIG;
  r->A = H;
  r->nkeep = nkeep;
  r->etrunc = etrunc;
  r->deps = deps;
  r->footprint = fp;
  r->owner = owner;
  QS_CUDA(cudaSetDevice(s->parent->c.device));
  QS_CUDA(cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming));
  QS_CUDA(cudaEventRecord(r->ready, owner->stream));
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    r->t_submit = clk::now();
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  QS_API_END
}

qs_status qs_server_poll_eig(qs_server *s, int64_t ticket, int32_t timeout_ms, int32_t *done, qs_tensor **AK,
                             qs_tensor **AD, double *E, uint8_t *keep, int64_t *nkeep_out, double *etrunc_out,
                             double *latency_ms) {
  QS_API_BEGIN
  if (!s || !done) fail(QS_ERR_ARG, "null argument");
  *done = 0;
  if (AK) *AK = nullptr;
  if (AD) *AD = nullptr;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) fail(QS_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  std::shared_ptr<Request> r = it->second;
  if (r->kind != Request::EIG) fail(QS_ERR_ARG, "ticket %lld is not an eig request", (long long)ticket);
  auto finished = [&] { return r->state == Request::DONE || r->state == Request::FAILED || r->state == Request::CANCELLED; };
  if (!finished() && timeout_ms > 0) s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished);
  if (!finished()) return QS_OK;
  *done = 1;
  if (latency_ms) *latency_ms = r->latency_ms;
  s->reqs.erase(it);
  if (r->state == Request::CANCELLED) fail(QS_ERR_CANCELLED, "request %lld was cancelled", (long long)ticket);
  if (r->state == Request::FAILED) fail(r->status, "%s", r->err.c_str());
  int64_t ntot = 0;
  for (int64_t i = 0; i < r->A->meta.nblk; ++i) ntot += r->A->meta.drow(i)[0];
  if (E && ntot) std::memcpy(E, r->E.data(), (size_t)ntot * 8);
  if (keep && ntot) std::memcpy(keep, r->keep.data(), (size_t)ntot);
  if (nkeep_out) *nkeep_out = r->nk;
  if (etrunc_out) *etrunc_out = r->et;
  if (AK) *AK = r->C;
  else delete r->C;
  if (AD) *AD = r->D;
  else delete r->D;
  r->C = r->D = nullptr;
  QS_API_END
}

qs_status qs_server_poll(qs_server *s, int64_t ticket, int32_t timeout_ms, int32_t *done, qs_tensor **C,
                         double *latency_ms) {
  QS_API_BEGIN
  if (!s || !done) fail(QS_ERR_ARG, "null argument");
  *done = 0;
  if (C) *C = nullptr;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) fail(QS_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  std::shared_ptr<Request> r = it->second;
  if (r->kind != Request::CONTRACT)
    fail(QS_ERR_ARG, "ticket %lld is an eig request (qs_server_poll_eig)", (long long)ticket);
  auto finished = [&] { return r->state == Request::DONE || r->state == Request::FAILED || r->state == Request::CANCELLED; };
  if (!finished() && timeout_ms > 0) s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished);
  if (!finished()) return QS_OK;
  *done = 1;
  if (latency_ms) *latency_ms = r->latency_ms;
  s->reqs.erase(it);
  if (r->state == Request::CANCELLED) fail(QS_ERR_CANCELLED, "request %lld was cancelled", (long long)ticket);
  if (r->state == Request::FAILED) fail(r->status, "%s", r->err.c_str());
  if (C) *C = r->C;
  else delete r->C;
  r->C = nullptr;
  QS_API_END
}

qs_status qs_server_cancel(qs_server *s, int64_t ticket) {
  QS_API_BEGIN
  if (!s) fail(QS_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) fail(QS_ERR_ARG, "unknown ticket %lld", (long long)ticket);
  std::shared_ptr<Request> r = it->second;
  if (r->state != Request::QUEUED) fail(QS_ERR_ARG, "request %lld already started", (long long)ticket);
  for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
    if ((*q)->ticket == ticket) {
      s->queue.erase(q);
      break;
    }
  r->state = Request::CANCELLED;
  if (r->ready) {
    cudaEventDestroy(r->ready);
    r->ready = nullptr;
  }
  s->cv_done.notify_all();
  QS_API_END
}

}  // extern "C"
