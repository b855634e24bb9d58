// Serving loop (see bl_server.h).
#include "bl_server.h"

#include <cuda_runtime.h>

#include <algorithm>

namespace bl {

namespace {
void cuda_ok(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(3, std::string(what) + ": " + cudaGetErrorString(e));
}
constexpr size_t kAlign = 256;
size_t round_up(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }
}  // namespace

bool RangePool::take(size_t bytes, size_t *off) {
  for (auto it = free_.begin(); it != free_.end(); ++it) {
    if (it->second < bytes) continue;
    *off = it->first;
    size_t rest = it->second - bytes;
    size_t at = it->first + bytes;
    free_.erase(it);
    if (rest) free_[at] = rest;
    return true;
  }
  return false;
}

void RangePool::give(size_t off, size_t bytes) {
  auto it = free_.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != free_.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    free_.erase(nx);
  }
  if (it != free_.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      free_.erase(it);
    }
  }
}

size_t RangePool::free_bytes() const {
  size_t t = 0;
  for (auto &kv : free_) t += kv.second;
  return t;
}

Server::Server(int device, int lanes, size_t pool_bytes)
    : device_(device), pool_bytes_(pool_bytes & ~(kAlign - 1)), ranges_(pool_bytes & ~(kAlign - 1)) {
  if (lanes < 1 || pool_bytes < (size_t(16) << 20)) throw Error(1, "need >= 1 lane and a pool of >= 16 MiB");
  cuda_ok(cudaSetDevice(device), "cudaSetDevice");
  cuda_ok(cudaMalloc(&pool_, pool_bytes_), "cudaMalloc (serving pool)");
  for (int i = 0; i < lanes; ++i) {
    std::unique_ptr<Lane> s(new Lane);
    s->ctx.device = device;
    cuda_ok(cudaStreamCreateWithFlags(&s->ctx.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    cudaEvent_t ev;
    cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    s->event = ev;
    lanes_.push_back(std::move(s));
  }
  worker_ = std::thread([this] { loop(); });
  planner_ = std::thread([this] { plan(); });
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  plan_cv_.notify_all();
  if (planner_.joinable()) planner_.join();
  if (worker_.joinable()) worker_.join();
  cudaSetDevice(device_);
  for (auto &s : lanes_) {
    if (s->ctx.stream) cudaStreamSynchronize(s->ctx.stream);
    s->job.reset();
    if (s->event) cudaEventDestroy(static_cast<cudaEvent_t>(s->event));
  }
  lanes_.clear();  // Context destructors release the streams
  if (pool_) cudaFree(pool_);
}

size_t Server::grant(const ServeRequest &r) const {
  size_t share = pool_bytes_ / lanes_.size();
  return round_up(std::min(r.full_bytes, std::max(r.min_bytes, share)));
}

int64_t Server::submit(std::shared_ptr<const SpinSystem> sys, const Powder &pw, CMatrix ro, CMatrix det,
                       const FidParams &p) {
  auto r = std::make_shared<ServeRequest>(std::move(sys), pw, std::move(ro), std::move(det), p);
  r->t_submit = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> lk(mu_);
    r->id = next_id_++;
    all_[r->id] = r;
    unplanned_.push_back(r);
  }
  plan_cv_.notify_one();
  return r->id;
}

// Planner thread: sizes queued requests in submission order and passes them to admission.
void Server::plan() {
  for (;;) {
    std::shared_ptr<ServeRequest> r;
    {
      std::unique_lock<std::mutex> lk(mu_);
      plan_cv_.wait(lk, [&] { return stop_ || !unplanned_.empty(); });
      if (stop_) return;
      r = unplanned_.front();
      unplanned_.pop_front();
      if (r->state != 0) continue;  // cancelled while waiting
    }
    std::string err;
    try {
      job_bytes(device_, *r->sys, r->pw, r->ro, r->det, r->p, &r->min_bytes, &r->full_bytes);
      if (round_up(r->min_bytes) > pool_bytes_)
        err = "job needs " + std::to_string(r->min_bytes >> 20) + " MiB for one warp of crystallites; the pool has " +
              std::to_string(pool_bytes_ >> 20) + " MiB";
    } catch (const std::exception &e) {
      err = e.what();
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!err.empty()) {
        if (r->state == 0) {
          r->err = err;
          r->state = 3;
          r->t_done = std::chrono::steady_clock::now();
          ++n_done_;
        }
      } else {
        queue_.push_back(r);
      }
    }
    cv_.notify_one();
  }
}

int Server::poll(int64_t id, double *fid_out, double *sw_out, double *latency_ms, std::string *err,
                 double *stmt_out) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end()) return -1;
  auto &r = *it->second;
  if (r.state >= 2) {
    if (latency_ms)
      *latency_ms = std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count();
    if (err) *err = r.err;
    if (r.state == 2 && sw_out) *sw_out = r.sw;
    if (r.state == 2 && stmt_out) *stmt_out = r.stmt;
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

void Server::stats(int64_t *queued, int64_t *running, int64_t *done, double *flops_done) const {
  std::lock_guard<std::mutex> lk(mu_);
  int64_t q = 0, r = 0;
  for (auto &kv : all_) {
    if (kv.second->state == 0) ++q;
    else if (kv.second->state == 1) ++r;
  }
  if (queued) *queued = q;
  if (running) *running = r;
  if (done) *done = n_done_;
  if (flops_done) *flops_done = flops_done_;
}

void Server::loop() {
  cudaSetDevice(device_);
  for (;;) {
    bool progress = false;
    // completions
    for (auto &sp : lanes_) {
      Lane &s = *sp;
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
      double fl = s.job ? s.job->flops() : 0;
      s.job.reset();
      ranges_.give(s.off, s.bytes);
      double stmt = -1;
      if (err.empty() && s.req->p.precision == 1 && s.req->p.error_sample > 0) {
        try {
          stmt = error_statement(s.ctx, *s.req->sys, s.req->pw, s.req->ro, s.req->det, s.req->p,
                                 s.req->p.error_sample);
        } catch (const std::exception &e) {
          err = std::string("error statement: ") + e.what();
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu_);
        s.req->t_done = std::chrono::steady_clock::now();
        s.req->fid.swap(fid);
        s.req->sw = sw;
        s.req->stmt = stmt;
        s.req->err = err;
        s.req->state = err.empty() ? 2 : 3;
        if (err.empty()) flops_done_ += fl;
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
    // admissions while a lane is idle: the head of the queue when its grant fits; otherwise
    // the first of the next kSkipWindow requests whose grant fits, as long as the head has
    // been passed over fewer than kMaxSkips times (then only the head, so it cannot starve)
    for (auto &sp : lanes_) {
      if (stopping) break;
      Lane &s = *sp;
      if (s.req) continue;
      std::shared_ptr<ServeRequest> r;
      size_t bytes = 0, off = 0;
      {
        std::lock_guard<std::mutex> lk(mu_);
        while (!queue_.empty() && queue_.front()->state != 0) queue_.pop_front();  // cancelled
        if (queue_.empty()) break;
        size_t pick = queue_.size();
        bytes = grant(*queue_.front());
        if (ranges_.take(bytes, &off)) {
          pick = 0;
        } else if (queue_.front()->skipped < kMaxSkips) {
          const size_t end = std::min(queue_.size(), size_t(1) + kSkipWindow);
          for (size_t q = 1; q < end; ++q) {
            if (queue_[q]->state != 0) continue;
            bytes = grant(*queue_[q]);
            if (ranges_.take(bytes, &off)) {
              pick = q;
              ++queue_.front()->skipped;
              break;
            }
          }
        }
        if (pick == queue_.size()) break;  // wait for a completion to free memory
        r = queue_[pick];
        queue_.erase(queue_.begin() + std::ptrdiff_t(pick));
        r->state = 1;
        r->t_start = std::chrono::steady_clock::now();
      }
      try {
        s.off = off;
        s.bytes = bytes;
        s.job = job_in_region(s.ctx, static_cast<char *>(pool_) + off, bytes, *r->sys, r->pw, r->ro, r->det, r->p);
        s.job->run();
        cuda_ok(cudaEventRecord(static_cast<cudaEvent_t>(s.event), s.ctx.stream), "cudaEventRecord");
        s.req = r;
      } catch (const std::exception &e) {
        s.job.reset();
        cudaStreamSynchronize(s.ctx.stream);  // nothing of the failed job may still use the range
        ranges_.give(off, bytes);
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
      for (auto &sp : lanes_) busy = busy || bool(sp->req);
      if (!busy) break;
    }
    if (!progress) cv_.wait_for(lk, std::chrono::microseconds(100));
  }
}

}  // namespace bl
