// lc2_stack_reg.cpp -- registration of the frames of a 2D-to-3D stack, each
// frame with its own optimizer, with the evaluations of all frames batched
// into shared launches (lc2_stack_register, include/lc2.h).
//
// The reference registers one frame per run (Optimizers2DTo3D over
// Interpolator2DTo3D, src/Optimizers/optimizers.cu:1195-1640). Here every
// frame's registration (lc2_register) runs on its own host thread; its
// objective hands each optimizer step to a lock-step batcher: once every
// frame still registering has submitted its step, the last one to arrive
// launches all of them as one lc2_stack_evaluate call (one work-list launch,
// graph-replayed when the layout repeats) and hands the values back. A frame
// that finishes leaves the batcher, so the others never wait for it. With
// LC2_OPTION_STACK_BATCHING off, each thread instead registers its frame on
// the frame's own context and stream, independently of the others (lower
// latency when the GPU is shared). Stack values equal the frame's standalone
// values bit for bit and the optimizers are deterministic, so each frame's
// result equals lc2_register run on that frame alone either way.
#include <condition_variable>
#include <cstdio>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lc2.h"

void lc2_set_error_message(const char* msg);

namespace {

struct Batcher {
  lc2_stack* stack;
  std::mutex mu;
  std::condition_variable cv;
  struct Item {
    int frame;
    int count;
    const double* mats;  // count x 16 doubles
    double* out;
    bool done = false;
    int status = LC2_OK;
    std::string msg;
  };
  std::vector<Item*> pending;
  int clients;
  bool busy = false;
  long long launches = 0;

  Batcher(lc2_stack* s, int n) : stack(s), clients(n) {}

  // Runs the merged evaluation of `batch` (leader only, lock not held).
  void launch(std::vector<Item*>& batch) {
    size_t total = 0;
    for (Item* it : batch) total += (size_t)it->count;
    std::vector<int> ids;
    std::vector<float> mats;
    std::vector<double> vals(total);
    ids.reserve(total);
    mats.reserve(total * 16);
    for (Item* it : batch)
      for (int k = 0; k < it->count; ++k) {
        ids.push_back(it->frame);
        for (int i = 0; i < 16; ++i) mats.push_back((float)it->mats[(size_t)k * 16 + i]);
      }
    const int st = lc2_stack_evaluate(stack, (int)total, ids.data(), mats.data(), vals.data());
    const std::string msg = st == LC2_OK ? "" : lc2_last_error();
    size_t o = 0;
    for (Item* it : batch) {
      for (int k = 0; k < it->count; ++k) it->out[k] = vals[o + k];
      o += (size_t)it->count;
      it->status = st;
      it->msg = msg;
    }
    ++launches;
  }

  int evaluate(int frame, int count, const double* mats, double* out) {
    Item it;
    it.frame = frame;
    it.count = count;
    it.mats = mats;
    it.out = out;
    std::unique_lock<std::mutex> lk(mu);
    pending.push_back(&it);
    for (;;) {
      if (it.done) break;
      if (!busy && !pending.empty() && (int)pending.size() >= clients) {
        busy = true;
        std::vector<Item*> batch;
        batch.swap(pending);
        lk.unlock();
        launch(batch);
        lk.lock();
        for (Item* p : batch) p->done = true;
        busy = false;
        cv.notify_all();
        continue;
      }
      cv.wait(lk);
    }
    if (it.status != LC2_OK) lc2_set_error_message(it.msg.c_str());
    return it.status;
  }

  void leave() {
    std::lock_guard<std::mutex> lk(mu);
    --clients;
    cv.notify_all();  // the frames still waiting may now be complete
  }
};

struct Client {
  Batcher* b;
  int frame;
};

int objective(void* user, int count, int dim, const double* x, double* f) {
  Client* c = static_cast<Client*>(user);
  if (dim != 16) return LC2_ERR_INVALID_ARGUMENT;
  return c->b->evaluate(c->frame, count, x, f);
}

}  // namespace

extern "C" int lc2_stack_register(lc2_stack* s, int n, const int* frame_ids,
                                  const lc2_registration* regs, lc2_registration_result* results,
                                  int* statuses, long long* launches) {
  if (!s || n < 0 || (n > 0 && (!frame_ids || !regs || !results))) {
    lc2_set_error_message("lc2_stack_register: null argument or negative count");
    return LC2_ERR_INVALID_ARGUMENT;
  }
  if (n > 4096) {
    lc2_set_error_message("lc2_stack_register: at most 4096 registrations per call");
    return LC2_ERR_UNSUPPORTED;
  }
  const int nf = lc2_stack_frames(s);
  for (int i = 0; i < n; ++i) {
    if (frame_ids[i] < 0 || frame_ids[i] >= nf) {
      lc2_set_error_message("lc2_stack_register: frame id out of range");
      return LC2_ERR_INVALID_ARGUMENT;
    }
    if (regs[i].mode != LC2_MODE_2DTO3D) {
      lc2_set_error_message("lc2_stack_register: registrations of stack frames use LC2_MODE_2DTO3D");
      return LC2_ERR_INVALID_ARGUMENT;
    }
  }
  int batching = 1;
  lc2_stack_get_option(s, LC2_OPTION_STACK_BATCHING, &batching);
  std::vector<lc2_context*> ctx(n, nullptr);
  if (!batching) {
    std::vector<char> seen(nf, 0);
    for (int i = 0; i < n; ++i) {
      if (seen[frame_ids[i]]) {
        lc2_set_error_message("lc2_stack_register: frame ids must be distinct without batching");
        return LC2_ERR_INVALID_ARGUMENT;
      }
      seen[frame_ids[i]] = 1;
      lc2_stack_frame_context(s, frame_ids[i], &ctx[i]);
    }
  }
  Batcher b(s, n);
  std::vector<Client> clients(n);
  std::vector<int> st(n, LC2_OK);
  std::vector<std::string> msgs(n);
  std::vector<std::thread> threads;
  threads.reserve(n);
  for (int i = 0; i < n; ++i) {
    clients[i] = {&b, frame_ids[i]};
    threads.emplace_back([&, i] {
      lc2_registration r = regs[i];
      if (batching) {
        r.lc2_of_matrices = &objective;
        r.user = &clients[i];
        st[i] = lc2_register(nullptr, &r, &results[i]);
      } else {
        st[i] = lc2_register(ctx[i], &r, &results[i]);
      }
      if (st[i] != LC2_OK) msgs[i] = lc2_last_error();
      b.leave();
    });
  }
  for (auto& t : threads) t.join();
  if (launches) *launches = b.launches;
  int first = LC2_OK;
  for (int i = 0; i < n; ++i) {
    if (statuses) statuses[i] = st[i];
    if (st[i] != LC2_OK && first == LC2_OK) {
      first = st[i];
      lc2_set_error_message(msgs[i].c_str());
    }
  }
  return first;
}
