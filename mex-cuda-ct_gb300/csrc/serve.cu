// serve.cu -- continuous-batching request server (include/mexct_serve.h).
//
// Slots are worker threads with their own context (non-blocking stream and
// workspaces); a request runs entirely on its slot's stream, so requests on
// different slots overlap on the device.  Admission: a free slot takes the
// first queued request (in arrival order) whose footprint fits the HBM budget
// next to the running ones.  Solver buffers are stream-ordered allocations, so
// starting or finishing a request never synchronises the other slots.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mexct.h"
#include "../../include/mexct_serve.h"
#include "../../include/mexct_solver.h"
#include "api_internal.h"
#include "kernels.h"

using namespace mexct;
using Clock = std::chrono::steady_clock;

namespace {

struct Job {
  unsigned long long id = 0;
  mexct_request r{};
  std::vector<int32_t> picks;
  size_t bytes = 0;
  Clock::time_point t_submit, t_start, t_end;
  mexct_status result = MEXCT_OK;
  std::string err;
  bool done = false;
};

mexct_status run_job(Job& j, mexct_ctx* c) {
  const mexct_request& r = j.r;
  if (r.simulate_s > 0) {
    std::this_thread::sleep_for(std::chrono::duration<double>(r.simulate_s));
    return MEXCT_OK;
  }
  if (!c) return set_err(MEXCT_ERR_UNSUPPORTED, "server: host-only server runs simulated requests");
  if (r.kind == MEXCT_REQ_FDK)
    return mexct_fbp(c, r.pre, r.post, r.W, r.H, r.nP, r.angles, r.geom, r.sad, r.filter,
                     r.cutoff, r.q, r.recon);
  return osc_tv_recon_typed(c, r.pre, r.post, r.W, r.H, r.nP, r.angles, r.sad, r.geom,
                            r.n_iter, r.tv_const, r.n_sub_init, r.n_sub_final, r.p_val,
                            j.picks.data(), r.mu_type, r.recon, r.data_type);
}

}  // namespace

struct mexct_server {
  int device = 0;
  size_t budget = 0, in_use = 0, peak = 0;
  int running = 0, max_running = 0;
  long long submitted = 0, completed = 0, failed = 0, rejected = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::map<unsigned long long, std::unique_ptr<Job>> jobs;
  std::vector<std::thread> workers;
  std::vector<mexct_ctx*> ctxs;
  bool stop = false;
  unsigned long long next_id = 1;

  void worker(int slot) {
    if (device >= 0) cudaSetDevice(device);
    mexct_ctx* c = device >= 0 ? ctxs[slot] : nullptr;
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      Job* j = nullptr;
      for (auto it = queue.begin(); it != queue.end(); ++it) {
        if (in_use + (*it)->bytes <= budget) {
          j = *it;
          queue.erase(it);
          break;
        }
      }
      if (!j) {
        if (stop && queue.empty()) return;
        cv_work.wait(lk);
        continue;
      }
      in_use += j->bytes;
      peak = std::max(peak, in_use);
      ++running;
      max_running = std::max(max_running, running);
      j->t_start = Clock::now();
      lk.unlock();
      const mexct_status st = run_job(*j, c);
      std::string msg = st == MEXCT_OK ? std::string() : std::string(mexct_last_error());
      lk.lock();
      j->t_end = Clock::now();
      j->result = st;
      j->err = msg;
      j->done = true;
      in_use -= j->bytes;
      --running;
      if (st == MEXCT_OK) ++completed;
      else ++failed;
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

extern "C" {

size_t mexct_request_bytes(const mexct_request* r) {
  if (!r) return 0;
  const size_t N = (size_t)r->W * r->W * r->H, M = (size_t)r->W * r->H * r->nP;
  const size_t pad = (size_t)slab_pitch(r->W) * (r->W + 2) * (r->H + 2);
  if (r->kind == MEXCT_REQ_FDK) return 4 * (3 * M + N) + 4 * (size_t)r->nP * r->W + (1 << 20);
  const size_t ds = r->mu_type == MEXCT_F32 ? 4 : 2;
  // the largest subset's residual views: two views in the padded quad layout
  // (four values per texel) per view
  const int smin = std::max(1, std::min(r->n_sub_init, r->n_sub_final));
  const int nv = (r->nP + smin - 1) / smin;
  const size_t rs = r->data_type == MEXCT_F16 ? 2 : 4;
  const size_t quads = 2 * sino_pad_elems(r->W, r->H, nv) * 4 * rs;
  // staging (pre, post, recon) + solver (pre, post, residual views, mu,
  // mu_old, TV buffer, two padded copies).
  return 4 * (2 * M + N) + 4 * (2 * M) + quads + ds * (3 * N + 2 * pad) + (1 << 20);
}

mexct_status mexct_server_create(int device, int slots, size_t budget, mexct_server** out) {
  if (!out) return set_err(MEXCT_ERR_ARG, "server_create: out is NULL");
  *out = nullptr;
  if (slots <= 0 || slots > 64) return set_err(MEXCT_ERR_ARG, "server_create: slots %d", slots);
  if (budget == 0) return set_err(MEXCT_ERR_ARG, "server_create: zero HBM budget");
  std::unique_ptr<mexct_server> s(new mexct_server);
  s->device = device;
  s->budget = budget;
  for (int i = 0; device >= 0 && i < slots; ++i) {  // device -1: host-only (simulated)
    mexct_ctx* c = nullptr;
    mexct_status st = mexct_ctx_create(device, &c);
    if (st != MEXCT_OK) {
      for (mexct_ctx* x : s->ctxs) mexct_ctx_destroy(x);
      return st;
    }
    s->ctxs.push_back(c);
  }
  for (int i = 0; i < slots; ++i) s->workers.emplace_back([p = s.get(), i] { p->worker(i); });
  *out = s.release();
  return MEXCT_OK;
}

mexct_status mexct_server_submit(mexct_server* s, const mexct_request* r,
                                 unsigned long long* ticket) {
  if (!s || !r || !ticket) return set_err(MEXCT_ERR_ARG, "server_submit: NULL pointer");
  if (r->kind != MEXCT_REQ_FDK && r->kind != MEXCT_REQ_OSCTV)
    return set_err(MEXCT_ERR_ARG, "server_submit: unknown request kind %d", r->kind);
  if (r->simulate_s <= 0) {
    if (!r->angles || !r->pre || !r->post || !r->recon)
      return set_err(MEXCT_ERR_ARG, "server_submit: NULL array");
    if (r->W <= 0 || r->H <= 0 || r->nP <= 0 || r->geom < 0 || r->geom > 2)
      return set_err(MEXCT_ERR_ARG, "server_submit: bad dims / geometry");
    if (r->kind == MEXCT_REQ_OSCTV && (!r->first_picks || r->n_iter < 1))
      return set_err(MEXCT_ERR_ARG, "server_submit: OSC-TV needs n_iter >= 1 and first_picks");
  }
  std::unique_ptr<Job> j(new Job);
  j->r = *r;
  if (r->kind == MEXCT_REQ_OSCTV && r->first_picks && r->n_iter > 0)
    j->picks.assign(r->first_picks, r->first_picks + r->n_iter);
  j->bytes = mexct_request_bytes(r);
  j->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (j->bytes > s->budget) {
    ++s->rejected;
    return set_err(MEXCT_ERR_BUDGET, "server_submit: request needs %zu bytes, budget is %zu",
                   j->bytes, s->budget);
  }
  j->id = s->next_id++;
  *ticket = j->id;
  s->queue.push_back(j.get());
  s->jobs[j->id] = std::move(j);
  ++s->submitted;
  s->cv_work.notify_one();
  return MEXCT_OK;
}

mexct_status mexct_server_wait(mexct_server* s, unsigned long long ticket, double timeout_s,
                               mexct_status* result, double* queue_s, double* run_s,
                               double* total_s) {
  if (!s) return set_err(MEXCT_ERR_ARG, "server_wait: NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return set_err(MEXCT_ERR_ARG, "server_wait: unknown ticket %llu", ticket);
  Job* j = it->second.get();
  auto ready = [&] { return j->done; };
  if (timeout_s < 0) s->cv_done.wait(lk, ready);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
    return set_err(MEXCT_ERR_TIMEOUT, "server_wait: ticket %llu still running", ticket);
  if (result) *result = j->result;
  if (queue_s) *queue_s = std::chrono::duration<double>(j->t_start - j->t_submit).count();
  if (run_s) *run_s = std::chrono::duration<double>(j->t_end - j->t_start).count();
  if (total_s) *total_s = std::chrono::duration<double>(j->t_end - j->t_submit).count();
  if (j->result != MEXCT_OK) set_err(j->result, "%s", j->err.c_str());
  s->jobs.erase(it);
  return MEXCT_OK;
}

mexct_status mexct_server_stats_get(mexct_server* s, mexct_server_stats* out) {
  if (!s || !out) return set_err(MEXCT_ERR_ARG, "server_stats: NULL pointer");
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->rejected = s->rejected;
  out->bytes_in_use = s->in_use;
  out->peak_bytes = s->peak;
  out->budget = s->budget;
  out->max_concurrent = s->max_running;
  return MEXCT_OK;
}

mexct_status mexct_server_destroy(mexct_server* s) {
  if (!s) return MEXCT_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (std::thread& t : s->workers) t.join();
  for (mexct_ctx* c : s->ctxs) mexct_ctx_destroy(c);
  delete s;
  return MEXCT_OK;
}

}  // extern "C"
