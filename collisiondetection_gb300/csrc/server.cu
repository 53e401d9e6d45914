// Serving engine (include/ccd_gb300.h, ccd_server_*): continuous batching of
// collision queries on one device.  No counterpart in the reference, whose
// detection runs in the caller's thread; each request runs exactly the
// reference's per-step chain (the ccd_mesh_detect path).
//
// A server owns `slots` worker threads, each with its own context (streams
// and device buffers).  Requests wait in FIFO order and are admitted while
// the sum of their estimated device footprints stays within the memory
// budget (a request larger than the whole budget runs alone).  An admitted
// request keeps its mesh -- topology, positions, broad-phase and narrow-phase
// buffers -- resident on its worker for all of its steps; requests on
// different workers overlap on the device.
#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ccd_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// Estimated device bytes of one request: topology and positions, broad-phase
// buffers (slabs, tree, Morton keys, about 8 candidate face pairs per face and
// their stencil keys) and the narrow-phase rows and refinement scratch of its
// candidate stencils.
int64_t footprint(const ccd_request &r) {
  return (int64_t)4096 * r.nfaces + (int64_t)64 * r.nverts + ((int64_t)64 << 20);
}

struct Job {
  uint64_t ticket = 0;
  ccd_request req{};
  std::vector<int32_t> faces;   // copies: the caller's arrays may go away after submit
  std::vector<uint8_t> fixed;
  const double *frames = nullptr;  // the caller's, read until the request completes
  int64_t bytes = 0;
  Clock::time_point submitted, started, finished;
  bool done = false;
  int status = CCD_OK;
  std::string error;
  std::vector<int64_t> vf_hits, ee_hits, vf_off, ee_off;
  std::vector<int32_t> vf, ee;
  std::vector<double> vf_t, ee_t, step_ms;
};

}  // namespace

struct ccd_server {
  int device = 0;
  int64_t budget = 0;
  std::vector<ccd_context *> ctxs;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<Job>> queue;
  std::map<uint64_t, std::shared_ptr<Job>> jobs;
  uint64_t next_ticket = 1;
  int64_t in_use = 0;
  int running = 0;
  bool stop = false;
};

namespace {

int run_job(ccd_context *ctx, Job &j) {
  const ccd_request &r = j.req;
  ccd_mesh *m = nullptr;
  int rc = ccd_mesh_create(ctx, r.nverts, r.nfaces, j.faces.data(), &m);
  if (rc) return rc;
  if (!j.fixed.empty()) rc = ccd_mesh_set_fixed(m, j.fixed.data());
  const size_t frame = 3 * (size_t)r.nverts;
  j.vf_off.assign(1, 0);
  j.ee_off.assign(1, 0);
  for (int k = 0; k < r.steps && !rc; k++) {
    const Clock::time_point t0 = Clock::now();
    rc = ccd_mesh_set_positions(m, j.frames + k * frame, j.frames + (k + 1) * frame);
    int64_t nvf = 0, nee = 0;
    // The request's mesh (tree, buffers) stays resident across its steps.
    // (A request's ten steps are too few for a captured step to repay its
    // capture.)
    if (!rc) rc = ccd_mesh_detect(m, r.broadphase_kind, r.outer_eta, r.eta, r.path, &nvf, &nee);
    if (!rc) {
      const size_t ovf = j.vf_t.size(), oee = j.ee_t.size();
      j.vf.resize(4 * (ovf + (size_t)nvf));
      j.ee.resize(4 * (oee + (size_t)nee));
      j.vf_t.resize(ovf + (size_t)nvf);
      j.ee_t.resize(oee + (size_t)nee);
      rc = ccd_mesh_get_collisions(m, j.vf.data() + 4 * ovf, j.vf_t.data() + ovf, j.ee.data() + 4 * oee,
                                   j.ee_t.data() + oee);
      j.vf_hits.push_back(nvf);
      j.ee_hits.push_back(nee);
      j.vf_off.push_back((int64_t)(ovf + nvf));
      j.ee_off.push_back((int64_t)(oee + nee));
    }
    j.step_ms.push_back(ms_between(t0, Clock::now()));
  }
  if (rc) j.error = ccd_last_error(ctx);
  ccd_mesh_destroy(m);
  return rc;
}

void worker_loop(ccd_server *s, int slot) {
  ccd_context *ctx = s->ctxs[(size_t)slot];
  for (;;) {
    std::shared_ptr<Job> job;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      // Queued requests are admitted under the memory budget, also while the
      // server shuts down (it finishes them before its workers exit).
      s->cv.wait(lock, [&] {
        if (s->queue.empty()) return s->stop;
        const int64_t need = s->queue.front()->bytes;
        return s->running == 0 || s->in_use + need <= s->budget;
      });
      if (s->queue.empty()) return;  // woken by the shutdown with nothing left to run
      job = s->queue.front();
      s->queue.pop_front();
      s->in_use += job->bytes;
      s->running++;
      job->started = Clock::now();
    }
    const int rc = run_job(ctx, *job);
    {
      std::lock_guard<std::mutex> lock(s->mu);
      job->status = rc;
      job->finished = Clock::now();
      job->done = true;
      s->in_use -= job->bytes;
      s->running--;
    }
    s->cv.notify_all();
  }
}

int check_request(const ccd_request *r) {
  if (!r || r->nverts <= 0 || r->nfaces < 0 || r->steps < 1 || !r->frames || (r->nfaces > 0 && !r->faces))
    return CCD_ERR_INVALID_ARGUMENT;
  if (r->broadphase_kind != CCD_BROADPHASE_KDOP13 && r->broadphase_kind != CCD_BROADPHASE_AABB &&
      r->broadphase_kind != CCD_BROADPHASE_TRIVIAL)
    return CCD_ERR_INVALID_ARGUMENT;
  if (r->path != CCD_PATH_FP64 && r->path != CCD_PATH_CULL_REFINE && r->path != CCD_PATH_REFINE_ALL)
    return CCD_ERR_INVALID_ARGUMENT;
  return CCD_OK;
}

}  // namespace

extern "C" {

int ccd_server_create(int device, int slots, int64_t memory_budget, ccd_server **out) {
  if (!out || slots < 1 || slots > 64 || memory_budget <= 0) return CCD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  ccd_server *s = new (std::nothrow) ccd_server();
  if (!s) return CCD_ERR_OUT_OF_MEMORY;
  s->device = device;
  s->budget = memory_budget;
  for (int i = 0; i < slots; i++) {
    ccd_context *c = nullptr;
    const int rc = ccd_context_create(device, &c);
    if (rc) {
      for (ccd_context *x : s->ctxs) ccd_context_destroy(x);
      delete s;
      return rc;
    }
    s->ctxs.push_back(c);
  }
  for (int i = 0; i < slots; i++) s->workers.emplace_back(worker_loop, s, i);
  *out = s;
  return CCD_OK;
}

int ccd_server_destroy(ccd_server *s) {
  if (!s) return CCD_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (auto &t : s->workers) t.join();
  for (ccd_context *c : s->ctxs) ccd_context_destroy(c);
  delete s;
  return CCD_OK;
}

int ccd_server_submit(ccd_server *s, const ccd_request *req, uint64_t *ticket) {
  if (!s || !ticket) return CCD_ERR_INVALID_ARGUMENT;
  int rc = check_request(req);
  if (rc) return rc;
  auto job = std::make_shared<Job>();
  job->req = *req;
  job->faces.assign(req->faces, req->faces + 3 * (size_t)req->nfaces);
  for (int64_t i = 0; i < 3 * (int64_t)req->nfaces; i++)
    if (job->faces[(size_t)i] < 0 || job->faces[(size_t)i] >= req->nverts) return CCD_ERR_INVALID_ARGUMENT;
  if (req->fixed) job->fixed.assign(req->fixed, req->fixed + req->nverts);
  job->frames = req->frames;
  job->bytes = footprint(*req);
  job->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    job->ticket = s->next_ticket++;
    s->jobs[job->ticket] = job;
    s->queue.push_back(job);
    *ticket = job->ticket;
  }
  s->cv.notify_all();
  return CCD_OK;
}

int ccd_server_poll(ccd_server *s, uint64_t ticket, int *done) {
  if (!s || !done) return CCD_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return CCD_ERR_INVALID_ARGUMENT;
  *done = it->second->done ? 1 : 0;
  return CCD_OK;
}

int ccd_server_wait(ccd_server *s, uint64_t ticket, ccd_request_result *out) {
  if (!s || !out) return CCD_ERR_INVALID_ARGUMENT;
  std::shared_ptr<Job> job;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return CCD_ERR_INVALID_ARGUMENT;
    job = it->second;
    s->cv.wait(lock, [&] { return job->done; });
  }
  Job &j = *job;
  *out = ccd_request_result{};
  out->status = j.status;
  out->steps = (int32_t)j.step_ms.size();
  out->vf_hits = j.vf_hits.data();
  out->ee_hits = j.ee_hits.data();
  out->vf_offsets = j.vf_off.data();
  out->ee_offsets = j.ee_off.data();
  out->vf = j.vf.data();
  out->ee = j.ee.data();
  out->vf_t = j.vf_t.data();
  out->ee_t = j.ee_t.data();
  out->step_ms = j.step_ms.data();
  out->queue_ms = ms_between(j.submitted, j.started);
  out->total_ms = ms_between(j.submitted, j.finished);
  out->error = j.error.c_str();
  return CCD_OK;
}

int ccd_server_release(ccd_server *s, uint64_t ticket) {
  if (!s) return CCD_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end() || !it->second->done) return CCD_ERR_INVALID_ARGUMENT;
  s->jobs.erase(it);
  return CCD_OK;
}

}  // extern "C"
