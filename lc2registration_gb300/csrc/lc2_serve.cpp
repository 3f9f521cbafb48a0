// lc2_serve.cpp -- the request loop behind lc2_server_* (include/lc2.h).
//
// The reference registers one request per process (main.cu:728-801: parse,
// upload, optimise, export). Here a server keeps a FIFO of submitted
// registrations and a pool of max_active worker threads. A worker admits the
// request at the head of the queue when its device memory (lc2_context_bytes
// peak) fits what the running requests leave of the budget, then creates its
// context, uploads its images and runs lc2_register on it; the context's own
// stream lets the kernels of concurrent requests overlap on the GPU. Memory
// is returned and the next request admitted as each one completes
// (continuous admission, not a fixed batch). Admission is strictly in arrival
// order, so a large request is never starved by smaller ones behind it; on
// the GPU, small requests run on the most urgent stream priority.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lc2.h"

void lc2_set_error_message(const char* msg);

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

int fail(int code, const std::string& msg) {
  lc2_set_error_message(msg.c_str());
  return code;
}

struct Job {
  long long ticket = 0;
  lc2_request req{};
  std::vector<float> fixed, moving;
  size_t bytes = 0;
  enum { Queued, Running, Done } state = Queued;
  lc2_request_result res{};
  Clock::time_point t_submit, t_admit, t_done;
};

size_t image_voxels(const lc2_geometry& g, bool flat) {
  return (size_t)g.dim[0] * g.dim[1] * (flat ? 1 : g.dim[2]);
}

}  // namespace

struct lc2_server {
  lc2_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_admit;  // queue or budget changed
  std::condition_variable cv_done;   // a request completed
  std::deque<std::shared_ptr<Job>> queue;
  std::map<long long, std::shared_ptr<Job>> jobs;  // not yet returned by poll
  std::vector<std::thread> workers;
  bool stop = false;
  long long next_ticket = 1, admitted = 0;
  long long submitted = 0, completed = 0, failed = 0;
  int active = 0, peak_active = 0;
  size_t used = 0, peak = 0;
  std::vector<double> latencies;  // total_ms of completed requests
  Clock::time_point t0 = Clock::now();

  void run(Job& j) {
    lc2_registration reg = j.req.registration;
    lc2_registration_result out{};
    int st;
    if (reg.lc2_of_matrices) {
      st = lc2_register(nullptr, &reg, &out);
    } else {
      lc2_context* c = nullptr;
      lc2_config cfg = j.req.config;
      cfg.device = this->cfg.device;
      st = lc2_create(&cfg, &c);
      // small requests (virtual grid up to 2^20 voxels) on the most urgent
      // stream priority: their short launches are scheduled ahead of the
      // CTAs of large concurrent ones
      int vd[3] = {0, 0, 0};
      if (st == LC2_OK && lc2_virtual_dims(c, vd) == LC2_OK &&
          (long long)vd[0] * vd[1] * vd[2] <= (1LL << 20))
        st = lc2_set_option(c, LC2_OPTION_STREAM_PRIORITY, -1000);
      if (st == LC2_OK) st = lc2_set_images(c, j.fixed.data(), j.moving.data());
      if (st == LC2_OK) st = lc2_register(c, &reg, &out);
      std::string msg = st != LC2_OK ? lc2_last_error() : "";
      if (c) lc2_destroy(c);
      if (st != LC2_OK) lc2_set_error_message(msg.c_str());
    }
    j.res.status = st;
    j.res.result = out;
    if (st != LC2_OK) std::snprintf(j.res.message, sizeof(j.res.message), "%s", lc2_last_error());
  }

  void worker() {
    for (;;) {
      std::shared_ptr<Job> j;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_admit.wait(lk, [&] {
          return stop || (!queue.empty() && used + queue.front()->bytes <= cfg.hbm_budget_bytes);
        });
        if (stop) return;
        j = queue.front();
        queue.pop_front();
        used += j->bytes;
        peak = std::max(peak, used);
        ++active;
        peak_active = std::max(peak_active, active);
        j->state = Job::Running;
        j->t_admit = Clock::now();
        j->res.admission = admitted++;
      }
      cv_admit.notify_all();  // the next head may fit as well
      run(*j);
      {
        std::lock_guard<std::mutex> lk(mu);
        j->t_done = Clock::now();
        j->res.queue_ms = ms_between(j->t_submit, j->t_admit);
        j->res.run_ms = ms_between(j->t_admit, j->t_done);
        j->res.total_ms = ms_between(j->t_submit, j->t_done);
        j->res.device_bytes = j->bytes;
        j->state = Job::Done;
        j->fixed.clear();
        j->fixed.shrink_to_fit();
        j->moving.clear();
        j->moving.shrink_to_fit();
        used -= j->bytes;
        --active;
        if (j->res.status == LC2_OK) {
          ++completed;
          latencies.push_back(j->res.total_ms);
        } else {
          ++failed;
        }
      }
      cv_admit.notify_all();
      cv_done.notify_all();
    }
  }
};

extern "C" {

int lc2_server_create(const lc2_server_config* cfg, lc2_server** out) {
  if (!cfg || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (cfg->max_active < 0) return fail(LC2_ERR_INVALID_ARGUMENT, "max_active < 0");
  std::unique_ptr<lc2_server> s(new (std::nothrow) lc2_server());
  if (!s) return fail(LC2_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->cfg = *cfg;
  if (s->cfg.max_active == 0) s->cfg.max_active = 8;
  if (s->cfg.hbm_budget_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess)
      return fail(LC2_ERR_CUDA, std::string("server budget: ") + cudaGetErrorString(e));
    s->cfg.hbm_budget_bytes = (size_t)(0.8 * (double)free_b);
  }
  for (int i = 0; i < s->cfg.max_active; ++i) s->workers.emplace_back([p = s.get()] { p->worker(); });
  *out = s.release();
  return LC2_OK;
}

int lc2_server_submit(lc2_server* s, const lc2_request* req, long long* ticket) {
  if (!s || !req || !ticket) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  const lc2_config& cfg = req->config;
  size_t held = 0, peak = 0;
  int st = lc2_context_bytes(&cfg, &held, &peak);
  if (st != LC2_OK) return st;
  const bool host_objective = req->registration.lc2_of_matrices != nullptr;
  if (!host_objective && (!req->fixed || !req->moving))
    return fail(LC2_ERR_INVALID_ARGUMENT, "request without images");
  if (peak > s->cfg.hbm_budget_bytes)
    return fail(LC2_ERR_OUT_OF_MEMORY, "request needs " + std::to_string(peak) +
                                           " device bytes, the budget is " +
                                           std::to_string(s->cfg.hbm_budget_bytes));
  auto j = std::make_shared<Job>();
  j->req = *req;
  j->bytes = peak;
  if (!host_objective) {
    const bool flat = cfg.mode == LC2_MODE_2D;
    j->fixed.assign(req->fixed, req->fixed + image_voxels(cfg.fixed, flat));
    j->moving.assign(req->moving, req->moving + image_voxels(cfg.moving, flat));
  }
  j->req.fixed = nullptr;
  j->req.moving = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(LC2_ERR_NOT_READY, "server is shutting down");
    j->ticket = s->next_ticket++;
    j->t_submit = Clock::now();
    s->queue.push_back(j);
    s->jobs[j->ticket] = j;
    ++s->submitted;
    *ticket = j->ticket;
  }
  s->cv_admit.notify_all();
  return LC2_OK;
}

int lc2_server_poll(lc2_server* s, long long ticket, int wait_ms, lc2_request_result* out) {
  if (!s || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return fail(LC2_ERR_INVALID_ARGUMENT, "unknown or already returned ticket");
  std::shared_ptr<Job> j = it->second;
  auto done = [&] { return j->state == Job::Done; };
  if (wait_ms < 0)
    s->cv_done.wait(lk, done);
  else
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), done);
  if (!done()) return fail(LC2_ERR_NOT_READY, "request still queued or running");
  *out = j->res;
  s->jobs.erase(ticket);
  return LC2_OK;
}

int lc2_server_drain(lc2_server* s, int wait_ms) {
  if (!s) return fail(LC2_ERR_INVALID_ARGUMENT, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto idle = [&] { return s->queue.empty() && s->active == 0; };
  if (wait_ms < 0)
    s->cv_done.wait(lk, idle);
  else
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), idle);
  return idle() ? LC2_OK : fail(LC2_ERR_NOT_READY, "requests still queued or running");
}

int lc2_server_get_stats(lc2_server* s, lc2_server_stats* out) {
  if (!s || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->queued = (int)s->queue.size();
  out->active = s->active;
  out->peak_active = s->peak_active;
  out->budget_bytes = s->cfg.hbm_budget_bytes;
  out->bytes_in_use = s->used;
  out->peak_bytes = s->peak;
  out->elapsed_s = std::chrono::duration<double>(Clock::now() - s->t0).count();
  if (!s->latencies.empty()) {
    std::vector<double> v = s->latencies;
    std::sort(v.begin(), v.end());
    // nearest-rank percentiles
    auto pct = [&](double p) {
      size_t k = (size_t)std::ceil(p / 100.0 * (double)v.size());
      return v[std::min(v.size(), std::max<size_t>(k, 1)) - 1];
    };
    out->p50_ms = pct(50);
    out->p95_ms = pct(95);
    out->p99_ms = pct(99);
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / (double)v.size();
  }
  return LC2_OK;
}

int lc2_server_reset_stats(lc2_server* s) {
  if (!s) return fail(LC2_ERR_INVALID_ARGUMENT, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  s->latencies.clear();
  s->submitted = s->completed = s->failed = 0;
  s->peak = s->used;
  s->peak_active = s->active;
  s->t0 = Clock::now();
  return LC2_OK;
}

int lc2_server_destroy(lc2_server* s) {
  if (!s) return LC2_OK;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->queue.clear();  // queued requests are dropped
    s->cv_done.wait(lk, [&] { return s->active == 0; });
    s->stop = true;
  }
  s->cv_admit.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
  return LC2_OK;
}

}  // extern "C"
