// serve.cpp -- request loop over one resident basis (continuous batching).
//
// No counterpart in the reference, whose drivers compute one q-point per
// process run.  A server owns nslots contexts that share the parent's basis on
// the device (rpa_create_shared) and one worker thread per context.  Requests
// (chi0 or W solves of any q, local-field set and frequency grid) wait in a
// FIFO queue; the head request starts as soon as a worker is free and its
// device footprint fits next to the requests already running (a request
// larger than the whole budget runs alone).  Each context has its own stream,
// so the kernels of running requests overlap on the GPU, and a request that
// arrives while others run starts without waiting for them to finish.
// rpa_server_create_batched adds one batching worker with an rpa_batch: when
// it is free and the queue starts with W requests (charge mode, Sloss KK), it
// takes up to batch_q of them that fit the budget and runs them as one batch
// (per-request setup, then one CUDA graph with the grouped-tile S0 launches
// and every request's KK and Dyson); the slot workers keep serving the queue
// meanwhile, so requests of any kind still start as soon as any worker is free.

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rpa_gpu.h"

namespace {

using clock_type = std::chrono::steady_clock;

struct Job {
  rpa_request req;
  double footprint = 0;
  clock_type::time_point t_submit, t_start, t_end;
  bool done = false;
  int status = RPA_OK;
  std::string error;
};

double seconds(clock_type::time_point a, clock_type::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

}  // namespace

struct rpa_server {
  rpa_ctx* parent = nullptr;
  rpa_batch* batch = nullptr;  // the batching worker's batch (rpa_server_create_batched)
  int batch_q = 0;
  long long batched = 0;       // requests completed through the batch
  std::vector<rpa_ctx*> slots;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<long long> queue;
  std::unordered_map<long long, Job> jobs;
  long long next_id = 1;
  double budget = 0, in_use = 0;
  int running = 0;
  bool stop = false;
  std::string err;
  long long completed = 0;
  int nbnd = 0;
};

namespace {

// Device bytes a request holds while it runs: S0 and its double-float copy,
// chi0, the Dyson buffers (W requests) and the vertex rows of all transitions.
double footprint_of(const rpa_request& r, int nbnd) {
  const double ng2 = (double)r.nlf * r.nlf;
  const bool cplx = r.args.mode == RPA_MODE_CURRENT;
  const double rows = cplx ? 2.0 * r.args.no + 1 : (double)r.args.no;
  double b = rows * ng2 * (cplx ? 16.0 : 8.0) * 2.0 + (r.args.no - 1.0) * ng2 * 16.0;
  if (r.kind == RPA_REQ_W) b += 2.0 * (r.args.no - 1.0) * ng2 * 16.0;
  const double pairs = cplx ? (double)nbnd * nbnd : (double)r.args.nocc * (nbnd - r.args.nocc);
  b += (double)r.ntot * pairs * r.nlf * 8.0 * 3.0;
  return b;
}

int run_request(rpa_ctx* c, const rpa_request& r) {
  int rc = rpa_kmap(c, r.ntot, r.ktot, r.K1, r.R1, r.K2, r.R2, r.iG0);
  if (rc == RPA_OK) rc = rpa_set_q(c, r.q, r.nlf, r.ilf, r.parG);
  if (rc == RPA_OK) rc = rpa_chi0(c, &r.args, r.S0_out, r.Qeff_out);
  if (rc == RPA_OK) rc = rpa_kk(c, r.kk_variant, r.chi0_out);
  if (rc == RPA_OK && r.kind == RPA_REQ_W) rc = rpa_dyson(c, r.c0, r.eps, r.WT_out, nullptr, r.head_out);
  return rc;
}

void worker(rpa_server* s, int slot) {
  rpa_ctx* c = s->slots[slot];
  for (;;) {
    long long id;
    Job* job;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] {
        if (s->queue.empty()) return s->stop;
        const Job& head = s->jobs[s->queue.front()];
        return s->running == 0 || s->in_use + head.footprint <= s->budget;
      });
      if (s->queue.empty()) return;  // stop requested and nothing left
      id = s->queue.front();
      s->queue.pop_front();
      job = &s->jobs[id];
      s->in_use += job->footprint;
      ++s->running;
      job->t_start = clock_type::now();
    }
    const int rc = run_request(c, job->req);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      job->t_end = clock_type::now();
      job->status = rc;
      if (rc != RPA_OK) job->error = rpa_last_error(c);
      job->done = true;
      s->in_use -= job->footprint;
      --s->running;
      ++s->completed;
    }
    s->cv.notify_all();
  }
}

bool batchable(const rpa_request& r) {
  return r.kind == RPA_REQ_W && r.args.mode == RPA_MODE_CHARGE && r.kk_variant == RPA_KK_SLOSS_REAL &&
         !r.S0_out && !r.Qeff_out && !r.chi0_out;
}

void batch_worker(rpa_server* s) {
  std::vector<long long> ids;
  std::vector<rpa_request> reqs;
  std::vector<int> status;
  for (;;) {
    double fp = 0;
    ids.clear();
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // the oldest queued W request that fits next to the running ones
      auto first = [&]() -> std::deque<long long>::iterator {
        for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
          const Job& j = s->jobs[*it];
          if (batchable(j.req)) return (s->running == 0 || s->in_use + j.footprint <= s->budget) ? it : s->queue.end();
        }
        return s->queue.end();
      };
      s->cv.wait(lk, [&] { return s->stop || first() != s->queue.end(); });
      if (first() == s->queue.end()) return;  // stopping: the slot workers finish what is queued
      // up to batch_q W requests in arrival order (other kinds stay queued for
      // the slot workers), as long as they fit the budget
      for (auto it = first(); it != s->queue.end() && (int)ids.size() < s->batch_q;) {
        Job& j = s->jobs[*it];
        if (!batchable(j.req)) {
          ++it;
          continue;
        }
        if (!ids.empty() && s->in_use + fp + j.footprint > s->budget) break;
        ids.push_back(*it);
        fp += j.footprint;
        j.t_start = clock_type::now();
        it = s->queue.erase(it);
      }
      s->in_use += fp;
      ++s->running;
      reqs.clear();
      for (long long id : ids) reqs.push_back(s->jobs[id].req);
    }
    status.assign(ids.size(), RPA_OK);
    const int rc = rpa_batch_run(s->batch, (int)ids.size(), reqs.data(), status.data());
    {
      std::lock_guard<std::mutex> lk(s->mu);
      const auto now = clock_type::now();
      for (size_t i = 0; i < ids.size(); ++i) {
        Job& j = s->jobs[ids[i]];
        j.t_end = now;
        j.status = status[i] != RPA_OK ? status[i] : (rc != RPA_OK && rc != RPA_ESINGULAR ? rc : RPA_OK);
        if (j.status != RPA_OK) j.error = rpa_batch_last_error(s->batch);
        j.done = true;
      }
      s->in_use -= fp;
      --s->running;
      s->completed += (long long)ids.size();
      s->batched += (long long)ids.size();
    }
    s->cv.notify_all();
  }
}

}  // namespace

extern "C" {

int rpa_server_create_batched(rpa_server** out, rpa_ctx* parent, int nslots, double mem_bytes, int batch_q) {
  if (!out || batch_q < 1) return RPA_EINVAL;
  rpa_batch* b = nullptr;
  int rc = rpa_batch_create(&b, parent, batch_q);
  if (rc != RPA_OK) return rc;
  rc = rpa_server_create(out, parent, nslots, mem_bytes);
  if (rc != RPA_OK) {
    rpa_batch_destroy(b);
    return rc;
  }
  rpa_server* s = *out;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->batch = b;
    s->batch_q = batch_q;
  }
  s->workers.emplace_back(batch_worker, s);
  return RPA_OK;
}

int rpa_server_batched_count(const rpa_server* s, long long* n) {
  if (!s || !n) return RPA_EINVAL;
  *n = s->batched;
  return RPA_OK;
}

int rpa_server_create(rpa_server** out, rpa_ctx* parent, int nslots, double mem_bytes) {
  if (!out || !parent || nslots < 1 || nslots > 64 || !(mem_bytes > 0)) return RPA_EINVAL;
  *out = nullptr;
  rpa_server* s = new rpa_server();
  s->parent = parent;
  s->budget = mem_bytes;
  int info[4] = {0, 0, 0, 0};
  if (rpa_basis_info(parent, info) != RPA_OK || info[0] == 0) {
    delete s;
    return RPA_ESTATE;
  }
  s->nbnd = info[1];
  for (int i = 0; i < nslots; ++i) {
    rpa_ctx* c = nullptr;
    const int rc = rpa_create_shared(&c, parent, -1);
    if (rc != RPA_OK) {
      for (rpa_ctx* d : s->slots) rpa_destroy(d);
      delete s;
      return rc;
    }
    s->slots.push_back(c);
  }
  for (int i = 0; i < nslots; ++i) s->workers.emplace_back(worker, s, i);
  *out = s;
  return RPA_OK;
}

int rpa_server_submit(rpa_server* s, const rpa_request* req, long long* id) {
  if (!s || !req || !id) return RPA_EINVAL;
  if (req->kind != RPA_REQ_CHI0 && req->kind != RPA_REQ_W) return RPA_EINVAL;
  if (req->nlf < 1 || req->args.no < 3 || req->ntot < 1) return RPA_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return RPA_ESTATE;
  const long long k = s->next_id++;
  Job& j = s->jobs[k];
  j.req = *req;
  j.footprint = footprint_of(*req, s->nbnd);
  j.t_submit = clock_type::now();
  s->queue.push_back(k);
  *id = k;
  s->cv.notify_all();
  return RPA_OK;
}

int rpa_server_wait(rpa_server* s, long long id, double* times3) {
  if (!s) return RPA_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return RPA_EINVAL;
  // element references stay valid when submissions rehash the table; iterators do not
  const Job& j = it->second;
  s->cv.wait(lk, [&] { return j.done; });
  if (times3) {
    times3[0] = seconds(j.t_submit, j.t_end);
    times3[1] = seconds(j.t_submit, j.t_start);
    times3[2] = seconds(j.t_start, j.t_end);
  }
  const int rc = j.status;
  if (rc != RPA_OK) s->err = j.error;
  s->jobs.erase(id);
  return rc;
}

const char* rpa_server_last_error(const rpa_server* s) { return s ? s->err.c_str() : ""; }

int rpa_server_destroy(rpa_server* s) {
  if (!s) return RPA_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto& t : s->workers) t.join();
  int rc = RPA_OK;
  if (s->batch) rpa_batch_destroy(s->batch);
  for (rpa_ctx* c : s->slots) {
    const int r = rpa_destroy(c);
    if (r != RPA_OK) rc = r;
  }
  delete s;
  return rc;
}

}  // extern "C"
