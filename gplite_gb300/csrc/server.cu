// Request server: continuous batching of gp_fit (+ gp_pred) requests on one GPU.
//
// The reference fits one GP per R call (gp_fit, R/gp_fit.R:54-60, then
// gp_pred, R/gp_pred.R:88-122); this file serves many such calls as they
// arrive. Requests are copied on submit and admitted in arrival order while
// their device-memory estimate fits the HBM budget. Two kinds of lanes take
// admitted work:
//   * the batch lane: Gaussian full-method requests with one stationary term
//     and n <= batch_max_n. Whatever has gathered while the previous batch ran
//     becomes the next batch, solved by the batched pipeline (batched.cu) in one
//     launch sequence;
//   * worker lanes: everything else (Laplace / EP, FITC, compound kernels,
//     large n, predictions on resident models) through gpgp_fit / gpgp_pred,
//     one context (stream) per worker thread, so their kernels overlap.
// A model kept resident lives on the worker that fitted it; its predictions and
// its release are queued to that worker, behind the work already there.
#include <math.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "model.cuh"

namespace gpgp {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

enum ReqKind { REQ_FIT = 0, REQ_PREDICT = 1, REQ_RELEASE = 2 };

struct Req {
  int64_t id = 0;
  int kind = REQ_FIT;
  gpgp_kernel k{};
  gpgp_lik lik{};
  gpgp_method meth{};
  gpgp_approx ap{};
  std::vector<double> x, y, trials, offset, xt, inducing;
  int64_t n = 0, m = 0;
  int32_t d = 0;
  bool keep = false;
  int64_t model = -1;
  gpgp_model *target = nullptr;  // predict / release: the resident model
  double *mean = nullptr, *var = nullptr;
  int64_t bytes = 0;     // in-flight device memory estimate
  int64_t resident = 0;  // bytes that stay while the model is kept
  double work = 0;       // flop estimate (worker load balance)
  bool batchable = false;
  bool bad_input = false;  // NaN or Inf in x, y or xt: fails with GPGP_ENAN, never runs
  int worker = -1;
  bool done = false;
  Clock::time_point t_submit, t_admit, t_start, t_done;
  gpgp_request_result res{};
};

struct Worker {
  std::thread th;
  gpgp_ctx *ctx = nullptr;
  std::deque<Req *> q;
  double load = 0;  // flop estimate of the queued work
};

struct Resident {
  gpgp_model *model = nullptr;
  int worker = 0;
  int64_t bytes = 0;
};

bool is_stationary_single(const gpgp_kernel &k, int32_t d) {
  if (k.nterms != 1) return false;
  const gpgp_cf_term &t = k.term[0];
  if (t.kind != GPGP_CF_SEXP && t.kind != GPGP_CF_MATERN32 && t.kind != GPGP_CF_MATERN52) return false;
  if (t.periodic || t.normalize) return false;
  if (t.nvars != 0) {
    if (t.nvars != d) return false;
    for (int i = 0; i < d; ++i)
      if (t.vars[i] != i) return false;
  }
  return true;
}

}  // namespace
}  // namespace gpgp

using namespace gpgp;

struct gpgp_server {
  gpgp_server_opts o{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req *> pending;
  std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
  std::unordered_map<int64_t, Resident> models;
  std::vector<std::unique_ptr<Worker>> workers;
  std::thread batch_th;
  gpgp_ctx *bctx = nullptr;
  std::deque<Req *> batch_q;
  std::vector<std::unique_ptr<Req>> internal;  // release orders (no id)
  int64_t next_id = 1, next_model = 0;
  int64_t bytes_inflight = 0, bytes_resident = 0, bytes_peak = 0, budget = 0;
  int64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched_requests = 0, unfinished = 0;
  std::vector<double> lat;
  bool stop = false;
};

namespace {

// device bytes while the request runs, and while its model stays resident
void estimate(const gpgp_server *s, Req *r) {
  const double n = (double)r->n, m = (double)r->m;
  const bool mixed = s->o.precision == GPGP_PREC_MIXED;
  if (r->kind == REQ_PREDICT) {
    const double nn = (double)r->target->n;
    r->bytes = (int64_t)(8.0 * (2.0 * nn * std::min(m, 4096.0) + 64.0 * m + 4.0 * nn) + (1 << 20));
    r->work = 2.0 * nn * nn * m;
    return;
  }
  if (r->batchable) {
    r->bytes = (int64_t)batch_bytes_estimate(r->n, r->m, r->d, s->o.precision);
    r->work = n * n * n / 3.0 + n * n * m;
    return;
  }
  if (r->meth.kind == GPGP_METHOD_FITC) {
    const double M = (double)r->meth.num_inducing;
    r->bytes = (int64_t)(8.0 * (8.0 * n * M + 12.0 * M * M + 3.0 * m * M + 40.0 * n) + (4 << 20));
    r->resident = (int64_t)(8.0 * (5.0 * n * M + 8.0 * M * M + 20.0 * n));
    r->work = 4.0 * n * M * M;
    return;
  }
  const double iters = r->lik.kind == GPGP_LIK_GAUSSIAN ? 1.0 : 8.0;
  // n x 64 diagonal inverses; mixed adds two n x 256 four-slice panel operands
  // (the Cholesky's panel and its lookahead trailing update), 256 n doubles each
  r->bytes = (int64_t)(8.0 * ((mixed ? 5.0 : 3.0) * n * n + 2.0 * n * std::min(m, 4096.0) +
                              (mixed ? 576.0 : 64.0) * n + 20.0 * n) + (4 << 20));
  r->resident = (int64_t)(8.0 * (2.0 * n * n + 64.0 * n + 12.0 * n));
  r->work = iters * n * n * n / 3.0 + n * n * m;
}

void finish(gpgp_server *s, Req *r) {  // with s->mu held
  r->t_done = Clock::now();
  r->done = true;
  r->res.queue_ms = ms_between(r->t_submit, r->t_start);
  r->res.run_ms = ms_between(r->t_start, r->t_done);
  r->res.total_ms = ms_between(r->t_submit, r->t_done);
  s->bytes_inflight -= r->bytes;
  if (r->res.status == GPGP_OK || r->res.status == GPGP_ENOT_PD) {
    ++s->completed;
    s->lat.push_back(r->res.total_ms);
  } else {
    ++s->failed;
  }
  --s->unfinished;
}

void fail_now(gpgp_server *s, Req *r, gpgp_status st) {  // with s->mu held, never admitted
  r->t_start = Clock::now();
  r->bytes = 0;
  r->res.status = st;
  finish(s, r);
}

// admit pending requests in arrival order while they fit the budget; a later
// request may pass one that does not fit until that one has waited 100 ms
void try_admit(gpgp_server *s) {  // with s->mu held
  const Clock::time_point now = Clock::now();
  bool any = false;
  for (auto it = s->pending.begin(); it != s->pending.end();) {
    Req *r = *it;
    if (r->kind == REQ_PREDICT) {
      auto mit = s->models.find(r->model);
      if (mit == s->models.end()) {
        it = s->pending.erase(it);
        fail_now(s, r, GPGP_EINVAL);
        any = true;
        continue;
      }
    }
    const bool fits = s->bytes_inflight + s->bytes_resident + r->bytes <= s->budget;
    if (!fits) {
      if (s->bytes_inflight == 0) {  // only resident models stand in the way
        it = s->pending.erase(it);
        fail_now(s, r, GPGP_EOOM);
        any = true;
        continue;
      }
      if (ms_between(r->t_submit, now) > 100.0) break;
      ++it;
      continue;
    }
    it = s->pending.erase(it);
    r->t_admit = now;
    s->bytes_inflight += r->bytes;
    s->bytes_peak = std::max(s->bytes_peak, s->bytes_inflight + s->bytes_resident);
    if (r->kind == REQ_PREDICT) {
      const Resident &rs = s->models[r->model];
      r->target = rs.model;
      r->worker = rs.worker;
      s->workers[rs.worker]->q.push_back(r);
      s->workers[rs.worker]->load += r->work;
    } else if (r->batchable) {
      s->batch_q.push_back(r);
    } else {
      int best = 0;
      for (int w = 1; w < (int)s->workers.size(); ++w)
        if (s->workers[w]->load < s->workers[best]->load) best = w;
      r->worker = best;
      s->workers[best]->q.push_back(r);
      s->workers[best]->load += r->work;
    }
    any = true;
  }
  if (any) {
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
}

void run_request(gpgp_server *s, Worker &w, Req *r) {
  gpgp_status st = GPGP_OK;
  if (r->kind == REQ_RELEASE) {
    gpgp_model_free(r->target);
    return;
  }
  if (r->kind == REQ_PREDICT) {
    st = gpgp_pred(r->target, r->xt.data(), r->m, 0, r->mean, r->var);
    r->res.status = st;
    return;
  }
  gpgp_fit_opts op{};
  op.jitter = s->o.jitter;
  op.precision = s->o.precision;
  op.refine_iters = 2;
  if (r->meth.kind == GPGP_METHOD_FITC) r->meth.inducing = r->inducing.data();
  gpgp_model *model = nullptr;
  gpgp_fit_result fr{};
  st = gpgp_fit(w.ctx, &r->k, &r->lik, &r->meth, &r->ap, &op, r->x.data(), r->n, r->d, r->y.data(),
                r->trials.empty() ? nullptr : r->trials.data(), r->offset.empty() ? nullptr : r->offset.data(),
                &model, &fr);
  r->res.log_evidence = fr.log_evidence;
  r->res.converged = fr.converged;
  r->res.iters = fr.iters;
  r->res.precision_used = fr.precision_used;
  if (st == GPGP_OK && r->m > 0) st = gpgp_pred(model, r->xt.data(), r->m, 0, r->mean, r->var);
  r->res.status = st;
  if (st == GPGP_OK && r->keep) {
    std::lock_guard<std::mutex> lk(s->mu);
    const int64_t mid = s->next_model++;
    s->models[mid] = Resident{model, r->worker, r->resident};
    s->bytes_resident += r->resident;
    s->bytes_peak = std::max(s->bytes_peak, s->bytes_inflight + s->bytes_resident);
    r->res.model = mid;
  } else if (model) {
    gpgp_model_free(model);
  }
}

void worker_loop(gpgp_server *s, Worker *w) {
  cudaSetDevice(s->o.device);
  for (;;) {
    Req *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !w->q.empty(); });
      if (w->q.empty()) return;  // stop requested and nothing left
      r = w->q.front();
      w->q.pop_front();
      r->t_start = Clock::now();
    }
    run_request(s, *w, r);
    std::lock_guard<std::mutex> lk(s->mu);
    w->load -= r->work;
    if (r->kind != REQ_RELEASE) {
      finish(s, r);
    } else {
      for (auto it = s->internal.begin(); it != s->internal.end(); ++it)
        if (it->get() == r) {
          s->internal.erase(it);
          break;
        }
    }
    try_admit(s);
    s->cv_done.notify_all();
  }
}

void batch_loop(gpgp_server *s) {
  cudaSetDevice(s->o.device);
  for (;;) {
    std::vector<Req *> job;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->batch_q.empty(); });
      if (s->batch_q.empty()) return;
      while (!s->batch_q.empty() && (int)job.size() < s->o.batch_max) {
        job.push_back(s->batch_q.front());
        s->batch_q.pop_front();
      }
      const Clock::time_point now = Clock::now();
      for (Req *r : job) r->t_start = now;
    }
    std::vector<gpgp_batch_problem> probs(job.size());
    int64_t mtot = 0;
    for (size_t i = 0; i < job.size(); ++i) {
      const Req *r = job[i];
      gpgp_batch_problem &p = probs[i];
      p.n = (int32_t)r->n;
      p.d = r->d;
      p.m = (int32_t)r->m;
      p.kind = r->k.term[0].kind;
      p.lscale = r->k.term[0].lscale;
      p.magn = r->k.term[0].magn;
      p.sigma = r->lik.sigma;
      p.x = r->x.data();
      p.y = r->y.data();
      p.xt = r->m > 0 ? r->xt.data() : nullptr;
      mtot += r->m;
    }
    std::vector<double> lml(job.size()), mean(std::max<int64_t>(mtot, 1)), var(std::max<int64_t>(mtot, 1));
    const gpgp_status st = batch_solve_once(s->bctx, probs.data(), (int32_t)probs.size(), s->o.precision,
                                            s->o.jitter, lml.data(), mean.data(), var.data());
    int64_t off = 0;
    for (size_t i = 0; i < job.size(); ++i) {
      Req *r = job[i];
      if (st == GPGP_OK) {
        if (r->mean) std::memcpy(r->mean, mean.data() + off, r->m * sizeof(double));
        if (r->var) std::memcpy(r->var, var.data() + off, r->m * sizeof(double));
        r->res.log_evidence = lml[i];
        r->res.status = std::isinf(lml[i]) && lml[i] < 0 ? GPGP_ENOT_PD : GPGP_OK;
        r->res.converged = 1;
        r->res.iters = 1;
        r->res.precision_used = s->o.precision;
      } else {
        r->res.status = st;
      }
      off += r->m;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    ++s->batches;
    s->batched_requests += (int64_t)job.size();
    for (Req *r : job) finish(s, r);
    try_admit(s);
    s->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

gpgp_status gpgp_server_create(const gpgp_server_opts *opts, gpgp_server **out) {
  if (!opts || !out) return GPGP_EINVAL;
  *out = nullptr;
  if (opts->precision != GPGP_PREC_FP64 && opts->precision != GPGP_PREC_MIXED) return GPGP_EINVAL;
  std::unique_ptr<gpgp_server> s(new gpgp_server());
  s->o = *opts;
  if (s->o.workers <= 0) s->o.workers = 4;
  if (s->o.workers > 64) s->o.workers = 64;
  if (s->o.batch_max_n <= 0) s->o.batch_max_n = 1024;
  if (s->o.batch_max_n > 4096) s->o.batch_max_n = 4096;
  if (s->o.batch_max <= 0) s->o.batch_max = 4096;
  if (!(s->o.jitter > 0)) s->o.jitter = 1e-6;
  gpgp_status st = gpgp_create(&s->bctx, s->o.device);
  if (st != GPGP_OK) return st;
  if (s->o.hbm_budget > 0) {
    s->budget = s->o.hbm_budget;
  } else {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      (void)cudaGetLastError();
      gpgp_destroy(s->bctx);
      return GPGP_ECUDA;
    }
    s->budget = (int64_t)(0.8 * (double)fr);
  }
  for (int w = 0; w < s->o.workers; ++w) {
    std::unique_ptr<Worker> wk(new Worker());
    st = gpgp_create(&wk->ctx, s->o.device);
    if (st != GPGP_OK) {
      for (auto &x : s->workers) gpgp_destroy(x->ctx);
      gpgp_destroy(s->bctx);
      return st;
    }
    s->workers.push_back(std::move(wk));
  }
  gpgp_server *sp = s.get();
  for (auto &wk : s->workers) wk->th = std::thread(worker_loop, sp, wk.get());
  s->batch_th = std::thread(batch_loop, sp);
  *out = s.release();
  return GPGP_OK;
}

gpgp_status gpgp_server_submit(gpgp_server *s, const gpgp_request *q, int64_t *id) {
  if (!s || !q || !id) return GPGP_EINVAL;
  *id = -1;
  std::unique_ptr<Req> r(new Req());
  r->t_submit = Clock::now();
  r->res.model = -1;
  r->m = q->m;
  r->mean = q->mean;
  r->var = q->var;
  if (q->m < 0 || (q->m > 0 && (!q->xt || !q->mean))) return GPGP_EINVAL;
  if (q->model >= 0) {
    r->kind = REQ_PREDICT;
    r->model = q->model;
    std::lock_guard<std::mutex> lk(s->mu);
    auto mit = s->models.find(q->model);
    if (mit == s->models.end()) return GPGP_EINVAL;
    r->target = mit->second.model;
    r->d = r->target->d;
    r->xt.assign(q->xt, q->xt + q->m * r->d);
    estimate(s, r.get());
  } else {
    if (!q->kernel || !q->lik || !q->x || !q->y || q->n < 1 || q->d < 1) return GPGP_EINVAL;
    r->kind = REQ_FIT;
    r->k = *q->kernel;
    r->lik = *q->lik;
    if (q->method) {
      // the server keeps copies of full and FITC requests only (no random-feature draws)
      if (q->method->kind != GPGP_METHOD_FULL && q->method->kind != GPGP_METHOD_FITC) return GPGP_EUNSUPPORTED;
      r->meth = *q->method;
    } else {
      r->meth.kind = GPGP_METHOD_FULL;
    }
    if (q->approx) {
      r->ap = *q->approx;
    } else {
      r->ap.kind = GPGP_APPROX_LAPLACE;
      r->ap.maxiter = 30;
      r->ap.tol = 1e-4;
      r->ap.damping = 0.9;
      r->ap.damping_min = 0.1;
      r->ap.quad_order = 11;
    }
    r->n = q->n;
    r->d = q->d;
    r->keep = q->keep != 0;
    r->x.assign(q->x, q->x + q->n * q->d);
    r->y.assign(q->y, q->y + q->n);
    if (q->trials) r->trials.assign(q->trials, q->trials + q->n);
    if (q->offset) r->offset.assign(q->offset, q->offset + q->n);
    if (q->m > 0) r->xt.assign(q->xt, q->xt + q->m * q->d);
    if (r->meth.kind == GPGP_METHOD_FITC) {
      if (!r->meth.inducing || r->meth.num_inducing < 1) return GPGP_EINVAL;
      r->inducing.assign(r->meth.inducing, r->meth.inducing + (int64_t)r->meth.num_inducing * q->d);
    }
    bool finite = true;
    for (double v : r->x) finite = finite && std::isfinite(v);
    for (double v : r->y) finite = finite && std::isfinite(v);
    for (double v : r->xt) finite = finite && std::isfinite(v);
    r->bad_input = !finite;
    r->batchable = !r->keep && r->lik.kind == GPGP_LIK_GAUSSIAN && r->meth.kind == GPGP_METHOD_FULL &&
                   !q->trials && !q->offset && q->d <= 8 && q->n <= s->o.batch_max_n &&
                   is_stationary_single(r->k, q->d) && r->k.term[0].lscale > 0 && r->lik.sigma > 0;
    estimate(s, r.get());
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return GPGP_EBUSY;
  r->id = s->next_id++;
  *id = r->id;
  ++s->submitted;
  ++s->unfinished;
  Req *rp = r.get();
  s->reqs[r->id] = std::move(r);
  if (rp->bad_input || rp->bytes > s->budget) {
    fail_now(s, rp, rp->bad_input ? GPGP_ENAN : GPGP_EOOM);
    s->cv_done.notify_all();
    return GPGP_OK;
  }
  s->pending.push_back(rp);
  try_admit(s);
  return GPGP_OK;
}

gpgp_status gpgp_server_poll(gpgp_server *s, int64_t id, int32_t wait_ms, gpgp_request_result *res) {
  if (!s || !res) return GPGP_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return GPGP_EINVAL;
  Req *r = it->second.get();
  if (!r->done && wait_ms != 0) {
    if (wait_ms < 0)
      s->cv_done.wait(lk, [&] { return r->done; });
    else
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return r->done; });
  }
  if (!r->done) return GPGP_EBUSY;
  *res = r->res;
  res->lane = r->batchable ? 0 : 1;
  s->reqs.erase(it);
  return GPGP_OK;
}

gpgp_status gpgp_server_release(gpgp_server *s, int64_t model) {
  if (!s) return GPGP_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->models.find(model);
  if (it == s->models.end()) return GPGP_EINVAL;
  std::unique_ptr<Req> r(new Req());
  r->kind = REQ_RELEASE;
  r->target = it->second.model;
  r->worker = it->second.worker;
  s->bytes_resident -= it->second.bytes;
  s->models.erase(it);
  s->workers[r->worker]->q.push_back(r.get());
  s->internal.push_back(std::move(r));
  s->cv_work.notify_all();
  try_admit(s);
  return GPGP_OK;
}

gpgp_status gpgp_server_stats_get(gpgp_server *s, gpgp_server_stats *out) {
  if (!s || !out) return GPGP_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->pending = (int64_t)s->pending.size();
  out->inflight = s->unfinished - out->pending;
  out->batches = s->batches;
  out->batched_requests = s->batched_requests;
  out->bytes_inflight = s->bytes_inflight;
  out->bytes_resident = s->bytes_resident;
  out->bytes_peak = s->bytes_peak;
  out->budget = s->budget;
  if (!s->lat.empty()) {
    std::vector<double> v = s->lat;
    std::sort(v.begin(), v.end());
    auto q = [&](double p) { return v[(size_t)std::min<double>(v.size() - 1, std::floor(p * (v.size() - 1) + 0.5))]; };
    out->p50_ms = q(0.50);
    out->p99_ms = q(0.99);
    out->max_ms = v.back();
  }
  return GPGP_OK;
}

gpgp_status gpgp_server_destroy(gpgp_server *s) {
  if (!s) return GPGP_OK;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->unfinished == 0; });
    s->stop = true;
    s->cv_work.notify_all();
  }
  for (auto &w : s->workers) w->th.join();
  s->batch_th.join();
  cudaSetDevice(s->o.device);
  for (auto &m : s->models) gpgp_model_free(m.second.model);
  s->models.clear();
  for (auto &w : s->workers) gpgp_destroy(w->ctx);
  gpgp_destroy(s->bctx);
  delete s;
  return GPGP_OK;
}

}  // extern "C"
