// Serving loop (see bl_server.h).
#include "bl_server.h"

#include <cuda_runtime.h>

namespace bl {

namespace {
void cuda_ok(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(3, std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace

Server::Server(int device, int slots, size_t slot_bytes) : device_(device), slot_bytes_(slot_bytes) {
  if (slots < 1 || slot_bytes < (size_t(16) << 20)) throw Error(1, "need >= 1 slot of >= 16 MiB");
  cuda_ok(cudaSetDevice(device), "cudaSetDevice");
  cuda_ok(cudaMalloc(&pool_, size_t(slots) * slot_bytes), "cudaMalloc (serving pool)");
  for (int i = 0; i < slots; ++i) {
    std::unique_ptr<Slot> s(new Slot);
    s->ctx.device = device;
    cuda_ok(cudaStreamCreateWithFlags(&s->ctx.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    cudaEvent_t ev;
    cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    s->event = ev;
    s->base = static_cast<char *>(pool_) + size_t(i) * slot_bytes;
    s->bytes = slot_bytes;
    slots_.push_back(std::move(s));
  }
  worker_ = std::thread([this] { loop(); });
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  if (worker_.joinable()) worker_.join();
  cudaSetDevice(device_);
  for (auto &s : slots_) {
    if (s->ctx.stream) cudaStreamSynchronize(s->ctx.stream);
    s->job.reset();
    if (s->event) cudaEventDestroy(static_cast<cudaEvent_t>(s->event));
  }
  slots_.clear();  // Context destructors release the streams
  if (pool_) cudaFree(pool_);
}

int64_t Server::submit(const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
                       const FidParams &p) {
  auto r = std::make_shared<ServeRequest>(sys, pw, ro, det, p);
  r->t_submit = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(mu_);
    r->id = next_id_++;
    all_[r->id] = r;
    queue_.push_back(r);
  }
  cv_.notify_one();
  return r->id;
}

int Server::poll(int64_t id, double *fid_out, double *sw_out, double *latency_ms, std::string *err) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end()) return -1;
  auto &r = *it->second;
  if (r.state >= 2) {
    if (latency_ms)
      *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    if (err) *err = r.err;
    if (r.state == 2 && sw_out) *sw_out = r.sw;
    if (fid_out) {
      if (r.state == 2) std::copy(r.fid.begin(), r.fid.end(), fid_out);
      int st = r.state;
      all_.erase(it);
      return st;
    }
  }
  return r.state;
}

bool Server::cancel(int64_t id) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end() || it->second->state != 0) return false;  // only queued requests
  it->second->state = 4;
  it->second->t_done = std::chrono::steady_clock::now();
  return true;
}

void Server::stats(int64_t *queued, int64_t *running, int64_t *done) const {
  std::lock_guard<std::mutex> lk(mu_);
  int64_t q = 0, r = 0;
  for (auto &kv : all_) {
    if (kv.second->state == 0) ++q;
    else if (kv.second->state == 1) ++r;
  }
  if (queued) *queued = q;
  if (running) *running = r;
  if (done) *done = n_done_;
}

void Server::loop() {
  cudaSetDevice(device_);
  for (;;) {
    bool progress = false;
    // completions
    for (auto &sp : slots_) {
      Slot &s = *sp;
      if (!s.req) continue;
      cudaError_t q = cudaEventQuery(static_cast<cudaEvent_t>(s.event));
      if (q == cudaErrorNotReady) continue;
      std::vector<double> fid(2 * size_t(s.req->p.npts));
      std::string err;
      try {
        if (q != cudaSuccess) throw Error(3, cudaGetErrorString(q));
        s.job->read(fid.data());
      } catch (const std::exception &e) {
        err = e.what();
      }
      double sw = s.job ? s.job->sw_out() : 0;
      s.job.reset();
      {
        std::lock_guard<std::mutex> lk(mu_);
        s.req->t_done = std::chrono::steady_clock::now();
        s.req->fid.swap(fid);
        s.req->sw = sw;
        s.req->err = err;
        s.req->state = err.empty() ? 2 : 3;
        ++n_done_;
      }
      s.req.reset();
      progress = true;
    }
    bool stopping;
    {
      std::lock_guard<std::mutex> lk(mu_);
      stopping = stop_;
    }
    // admissions, first come first served, while a slot is free
    for (auto &sp : slots_) {
      if (stopping) break;
      Slot &s = *sp;
      if (s.req) continue;
      std::shared_ptr<ServeRequest> r;
      {
        std::lock_guard<std::mutex> lk(mu_);
        while (!queue_.empty() && !r) {
          r = queue_.front();
          queue_.pop_front();
          if (r->state != 0) r.reset();  // cancelled while queued
        }
        if (!r) break;
        r->state = 1;
        r->t_start = std::chrono::steady_clock::now();
      }
      try {
        s.job = job_in_region(s.ctx, s.base, s.bytes, r->sys, r->pw, r->ro, r->det, r->p);
        s.job->run();
        cuda_ok(cudaEventRecord(static_cast<cudaEvent_t>(s.event), s.ctx.stream), "cudaEventRecord");
        s.req = r;
      } catch (const std::exception &e) {
        s.job.reset();
        std::lock_guard<std::mutex> lk(mu_);
        r->err = e.what();
        r->state = 3;
        r->t_done = std::chrono::steady_clock::now();
        ++n_done_;
      }
      progress = true;
    }
    std::unique_lock<std::mutex> lk(mu_);
    if (stop_) {
      bool busy = false;
      for (auto &sp : slots_) busy = busy || bool(sp->req);
      if (!busy) break;
    }
    if (!progress) cv_.wait_for(lk, std::chrono::microseconds(100));
  }
}

}  // namespace bl
