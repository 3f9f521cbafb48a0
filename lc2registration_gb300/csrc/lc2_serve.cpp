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
  // stack requests: frames registered together on one shared moving volume
  bool is_stack = false;
  lc2_stack_request sreq{};
  std::vector<lc2_geometry> frame_geoms;
  std::vector<std::vector<float>> frame_images;
  std::vector<lc2_registration> frame_regs;
  std::vector<lc2_request_result> frame_res;
  size_t bytes = 0;
  enum { Queued, Running, Done } state = Queued;
  lc2_request_result res{};
  Clock::time_point t_submit, t_admit, t_done;
};

size_t image_voxels(const lc2_geometry& g, bool flat) {
  return (size_t)g.dim[0] * g.dim[1] * (flat ? 1 : g.dim[2]);
}

// Cross-request batching. Running requests of one mode, patch size and
// storage type form a group; each optimizer step (the batch of transforms
// lc2_register hands its objective) is queued in the group, and one thread --
// the first to find no launch in progress -- takes every queued step, waits
// up to the window for the steps of the group's other running requests,
// evaluates them all in one lc2_merger launch and hands each request its
// values. Steps that arrive during a launch go into the next one, so the
// group's requests advance in merged rounds without a fixed batch. A merged
// value equals the request's own lc2_evaluate_batch bit for bit, so every
// registration follows the path it would follow alone.
struct MergeStep {
  lc2_context* ctx = nullptr;
  int count = 0;
  const float* mats = nullptr;
  double* out = nullptr;
  int status = LC2_OK;
  std::string message;
  bool done = false;
};

struct MergeGroup {
  std::mutex mu;
  std::condition_variable cv;
  std::vector<MergeStep*> pending;
  bool launching = false;
  int members = 0;  // running requests of the group
  lc2_merger* merger = nullptr;
  long long launches = 0, steps = 0;
  std::chrono::microseconds window{200};

  int submit(MergeStep& step) {
    std::unique_lock<std::mutex> lk(mu);
    pending.push_back(&step);
    cv.notify_all();
    while (!step.done) {
      if (launching) {
        cv.wait(lk);
        continue;
      }
      launching = true;
      cv.wait_until(lk, Clock::now() + window, [&] { return (int)pending.size() >= members; });
      std::vector<MergeStep*> take;
      take.swap(pending);
      lk.unlock();
      std::vector<lc2_context*> ctxs;
      std::vector<int> counts;
      std::vector<float> mats;
      size_t total = 0;
      for (MergeStep* t : take) {
        ctxs.push_back(t->ctx);
        counts.push_back(t->count);
        total += (size_t)t->count;
      }
      for (MergeStep* t : take) {
        lc2_config c{};
        lc2_get_config(t->ctx, &c);
        const int f = c.mode == LC2_MODE_2D ? 9 : 16;
        mats.insert(mats.end(), t->mats, t->mats + (size_t)t->count * f);
      }
      std::vector<double> out(total);
      const int st = lc2_merger_evaluate(merger, (int)ctxs.size(), ctxs.data(), counts.data(),
                                         mats.data(), out.data());
      const std::string msg = st != LC2_OK ? lc2_last_error() : "";
      lk.lock();
      size_t k = 0;
      for (MergeStep* t : take) {
        if (st == LC2_OK) std::copy(out.begin() + k, out.begin() + k + t->count, t->out);
        k += (size_t)t->count;
        t->status = st;
        t->message = msg;
        t->done = true;
      }
      ++launches;
      steps += (long long)take.size();
      launching = false;
      cv.notify_all();
    }
    if (step.status != LC2_OK) lc2_set_error_message(step.message.c_str());
    return step.status;
  }
};

// lc2_register's objective for a merged request: its matrices (exact float
// values widened to double by the driver) go to the group as one step.
struct MergeClient {
  MergeGroup* group;
  lc2_context* ctx;
  std::vector<float> buf;
};

int merge_objective(void* user, int count, int dim, const double* m, double* f) {
  MergeClient* mc = static_cast<MergeClient*>(user);
  mc->buf.assign(m, m + (size_t)count * dim);
  MergeStep step;
  step.ctx = mc->ctx;
  step.count = count;
  step.mats = mc->buf.data();
  step.out = f;
  return mc->group->submit(step);
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

  // A stack request: the frames register concurrently on their own contexts
  // and streams (latency first), sharing one upload of the moving volume.
  void run_stack(Job& j) {
    const lc2_stack_request& q = j.sreq;
    const int n = (int)j.frame_geoms.size();
    j.frame_res.assign(n, lc2_request_result{});
    lc2_stack* st = nullptr;
    int status = lc2_stack_create(&q.moving, q.patch_size, q.storage, cfg.device, &st);
    // frames are small 2D grids: the most urgent stream priority, as small requests
    if (status == LC2_OK) status = lc2_stack_set_option(st, LC2_OPTION_STREAM_PRIORITY, -1000);
    if (status == LC2_OK) status = lc2_stack_set_option(st, LC2_OPTION_STACK_BATCHING, 0);
    if (status == LC2_OK) status = lc2_stack_set_moving(st, j.moving.data());
    std::vector<int> ids(n);
    for (int i = 0; i < n && status == LC2_OK; ++i)
      status = lc2_stack_add_frame(st, &j.frame_geoms[i], q.virtual_spacing,
                                   j.frame_images[i].data(), &ids[i]);
    for (int i = 0; i < n && status == LC2_OK; ++i) {
      lc2_context* fc = nullptr;
      status = lc2_stack_frame_context(st, ids[i], &fc);
      if (status == LC2_OK) status = lc2_set_option(fc, LC2_OPTION_STREAM_PRIORITY, -1000);
    }
    std::vector<lc2_registration_result> rr(n);
    std::vector<int> sts(n, status);
    if (status == LC2_OK)
      status = lc2_stack_register(st, n, ids.data(), j.frame_regs.data(), rr.data(), sts.data(),
                                  nullptr);
    const std::string msg = status != LC2_OK ? lc2_last_error() : "";
    if (st) lc2_stack_destroy(st);
    for (int i = 0; i < n; ++i) {
      j.frame_res[i].status = sts[i];
      j.frame_res[i].result = rr[i];
      if (sts[i] != LC2_OK)
        std::snprintf(j.frame_res[i].message, sizeof(j.frame_res[i].message), "%s", msg.c_str());
    }
    j.res.status = status;
    if (status != LC2_OK) std::snprintf(j.res.message, sizeof(j.res.message), "%s", msg.c_str());
  }

  void run(Job& j) {
    if (j.is_stack) {
      run_stack(j);
      return;
    }
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
      MergeGroup* g = nullptr;
      if (st == LC2_OK) g = merge_group(cfg);
      if (st == LC2_OK && g) {
        MergeClient mc{g, c, {}};
        lc2_registration merged = reg;
        merged.lc2_of_matrices = merge_objective;
        merged.user = &mc;
        {
          std::lock_guard<std::mutex> lk(g->mu);
          ++g->members;
        }
        st = lc2_register(nullptr, &merged, &out);
        {
          std::lock_guard<std::mutex> lk(g->mu);
          --g->members;
        }
        g->cv.notify_all();
      } else if (st == LC2_OK) {
        st = lc2_register(c, &reg, &out);
      }
      std::string msg = st != LC2_OK ? lc2_last_error() : "";
      if (c) lc2_destroy(c);
      if (st != LC2_OK) lc2_set_error_message(msg.c_str());
    }
    j.res.status = st;
    j.res.result = out;
    if (st != LC2_OK) std::snprintf(j.res.message, sizeof(j.res.message), "%s", lc2_last_error());
  }

  // The merge group of a request's configuration, or nullptr where its steps
  // are not merged (3D grids, HighResolutionModality Fixed, mutual
  // information, merging off).
  std::mutex merge_mu;
  std::map<long long, std::unique_ptr<MergeGroup>> groups;
  MergeGroup* merge_group(const lc2_config& c) {
    if (cfg.merge_window_us < 0 || c.mode == LC2_MODE_3D || !c.high_res_is_moving ||
        c.patch_size < 1)
      return nullptr;
    const long long key = ((long long)c.mode * 64 + c.patch_size) * 8 + c.storage;
    std::lock_guard<std::mutex> lk(merge_mu);
    auto& g = groups[key];
    if (!g) {
      std::unique_ptr<MergeGroup> ng(new MergeGroup());
      ng->window = std::chrono::microseconds(cfg.merge_window_us > 0 ? cfg.merge_window_us : 200);
      if (lc2_merger_create(cfg.device, &ng->merger) != LC2_OK) {
        groups.erase(key);
        return nullptr;
      }
      g = std::move(ng);
    }
    return g.get();
  }
  void merge_counts(long long* launches, long long* steps) {
    std::lock_guard<std::mutex> lk(merge_mu);
    *launches = *steps = 0;
    for (auto& kv : groups) {
      std::lock_guard<std::mutex> gl(kv.second->mu);
      *launches += kv.second->launches;
      *steps += kv.second->steps;
    }
  }
  ~lc2_server() {
    for (auto& kv : groups) lc2_merger_destroy(kv.second->merger);
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
        j->frame_images.clear();
        for (auto& r : j->frame_res) {
          r.queue_ms = j->res.queue_ms;
          r.run_ms = j->res.run_ms;
          r.total_ms = j->res.total_ms;
          r.device_bytes = j->bytes;
          r.admission = j->res.admission;
        }
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

static int enqueue_job(lc2_server* s, std::shared_ptr<Job> j, long long* ticket) {
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

int lc2_server_submit_stack(lc2_server* s, const lc2_stack_request* req, long long* ticket) {
  if (!s || !req || !ticket || !req->moving_image || req->frames < 1 || !req->frame_geoms ||
      !req->frame_images || !req->registrations)
    return fail(LC2_ERR_INVALID_ARGUMENT, "incomplete stack request");
  // device footprint: the moving volume once, each frame's own buffers
  size_t bytes = 0, held = 0, peak = 0;
  lc2_config fc{};
  fc.mode = LC2_MODE_2DTO3D;
  fc.moving = req->moving;
  fc.patch_size = req->patch_size;
  fc.high_res_is_moving = 1;
  fc.storage = req->storage;
  fc.max_batch = 1;
  for (int a = 0; a < 3; ++a) fc.virtual_spacing[a] = req->virtual_spacing[a];
  const size_t nm = (size_t)req->moving.dim[0] * req->moving.dim[1] * req->moving.dim[2];
  const size_t es = req->storage == LC2_STORE_F32 ? 4 : 2;
  for (int i = 0; i < req->frames; ++i) {
    fc.fixed = req->frame_geoms[i];
    int st = lc2_context_bytes(&fc, &held, &peak);
    if (st != LC2_OK) return st;
    bytes += held - nm * es;  // the frames share the stack's moving volume
  }
  bytes += nm * (es + sizeof(float));  // the volume and its upload staging
  if (bytes > s->cfg.hbm_budget_bytes)
    return fail(LC2_ERR_OUT_OF_MEMORY, "stack request needs " + std::to_string(bytes) +
                                           " device bytes, the budget is " +
                                           std::to_string(s->cfg.hbm_budget_bytes));
  auto j = std::make_shared<Job>();
  j->is_stack = true;
  j->sreq = *req;
  j->bytes = bytes;
  j->moving.assign(req->moving_image, req->moving_image + nm);
  for (int i = 0; i < req->frames; ++i) {
    const lc2_geometry& g = req->frame_geoms[i];
    j->frame_geoms.push_back(g);
    j->frame_images.emplace_back(req->frame_images[i],
                                 req->frame_images[i] + (size_t)g.dim[0] * g.dim[1] * g.dim[2]);
    j->frame_regs.push_back(req->registrations[i]);
  }
  j->sreq.moving_image = nullptr;
  j->sreq.frame_geoms = nullptr;
  j->sreq.frame_images = nullptr;
  j->sreq.registrations = nullptr;
  return enqueue_job(s, j, ticket);
}

int lc2_server_poll_stack(lc2_server* s, long long ticket, int wait_ms, lc2_request_result* out,
                          int frames) {
  if (!s || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return fail(LC2_ERR_INVALID_ARGUMENT, "unknown or already returned ticket");
  std::shared_ptr<Job> j = it->second;
  if (!j->is_stack || (int)j->frame_geoms.size() != frames)
    return fail(LC2_ERR_INVALID_ARGUMENT, "not a stack request of that many frames");
  auto done = [&] { return j->state == Job::Done; };
  if (wait_ms < 0)
    s->cv_done.wait(lk, done);
  else
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), done);
  if (!done()) return fail(LC2_ERR_NOT_READY, "request still queued or running");
  for (int i = 0; i < frames; ++i) out[i] = j->frame_res[i];
  s->jobs.erase(ticket);
  return LC2_OK;
}

int lc2_server_poll(lc2_server* s, long long ticket, int wait_ms, lc2_request_result* out) {
  if (!s || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return fail(LC2_ERR_INVALID_ARGUMENT, "unknown or already returned ticket");
  std::shared_ptr<Job> j = it->second;
  if (j->is_stack) return fail(LC2_ERR_INVALID_ARGUMENT, "a stack request: use lc2_server_poll_stack");
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
  s->merge_counts(&out->merged_launches, &out->merged_steps);
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
