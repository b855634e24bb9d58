// Serving loop: continuous batching of powder-FID jobs on one GPU, admission by free
// device memory.
//
// The reference has no server; its closest analogue is the MPI master/worker farm that
// hands crystallites to free workers as they finish (src/QMspins/driver/oneFID.h:230-286,
// examples/solid-2.0/src/sequencerun.cc:435-526).  Here the unit handed out is a whole
// job (spin system + powder + rho/detect + parameters) and the workers are CUDA streams
// ("lanes") sharing one pool of device memory:
//   * one device allocation at start (the pool) and `lanes` non-blocking streams;
//   * submit() only queues a request; a planner thread sizes requests in submission order
//     (job_bytes: the bytes for one warp of crystallites per batch and for all crystallites
//     at once) and fails those whose one-warp size exceeds the pool, so that submitting
//     never waits on host-side planning;
//   * admission: when a lane is idle, the head of the queue is admitted if the pool holds a
//     free range of its grant, grant = its full size capped at pool/lanes but never below
//     its one-warp size; if it does not, the first of the next kSkipWindow requests whose
//     grant fits is admitted instead (a small job does not wait behind a large one), but the
//     head is passed over at most kMaxSkips times, after which admission waits for it.  The
//     job is built inside that range (no further allocation), batching its crystallites to
//     fit, enqueued on the lane's stream, and its completion recorded with an event;
//   * a worker thread polls completions, copies the FID back and returns the range; a
//     mixed-form request with error_sample > 0 then gets its error statement (two small jobs
//     on the lane's stream, run by the worker before it admits more work);
//   * latency = completion - submission, measured on the host steady clock.
// Jobs never share arithmetic and the crystallite batching does not change the powder sum
// (warp partials are reduced in a fixed order), so a result is bitwise the same alone, in
// the mix, and from a direct call.
#pragma once

#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bl_engine.h"

namespace bl {

struct ServeRequest {
  int64_t id = 0;
  std::shared_ptr<const SpinSystem> sys;  // shared with the caller's handle, never copied
  Powder pw;
  CMatrix ro, det;
  FidParams p;
  size_t min_bytes = 0, full_bytes = 0;
  std::chrono::steady_clock::time_point t_submit, t_start, t_done;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed, 4 cancelled
  int skipped = 0;  // times a later request was admitted ahead of this one at the queue's head
  std::vector<double> fid;
  double sw = 0;
  double stmt = -1;  // stated error (mixed form with error_sample > 0), else -1
  std::string err;
  ServeRequest(std::shared_ptr<const SpinSystem> s, const Powder &w, CMatrix r, CMatrix d, const FidParams &q)
      : sys(std::move(s)), pw(w), ro(std::move(r)), det(std::move(d)), p(q) {}
};

// First-fit ranges of the pool, free neighbours merged on release.
class RangePool {
 public:
  explicit RangePool(size_t bytes) { free_[0] = bytes; }
  bool take(size_t bytes, size_t *off);
  void give(size_t off, size_t bytes);
  size_t free_bytes() const;

 private:
  std::map<size_t, size_t> free_;  // offset -> size
};

class Server {
 public:
  static constexpr size_t kSkipWindow = 16;  // requests behind a blocked head that may go first
  static constexpr int kMaxSkips = 32;       // times the head may be passed over
  Server(int device, int lanes, size_t pool_bytes);
  ~Server();
  // queues the job (the planner fails it later if one warp of it exceeds the pool)
  int64_t submit(std::shared_ptr<const SpinSystem> sys, const Powder &pw, CMatrix ro, CMatrix det, const FidParams &p);
  // state of a ticket; when done and fid_out is given, copies the FID and forgets the ticket
  // (stmt_out: the mixed form's stated error when the request asked for one, else -1)
  int poll(int64_t id, double *fid_out, double *sw_out, double *latency_ms, std::string *err,
           double *stmt_out = nullptr);
  bool cancel(int64_t id);
  // requests queued/running, finished (any outcome), and the algorithmic flop of the
  // completed ones (one complex multiply-add = 8 flop)
  void stats(int64_t *queued, int64_t *running, int64_t *done, double *flops_done) const;
  size_t pool_bytes() const { return pool_bytes_; }

 private:
  struct Lane {
    Context ctx;
    std::unique_ptr<Job> job;
    std::shared_ptr<ServeRequest> req;
    size_t off = 0, bytes = 0;
    void *event = nullptr;  // cudaEvent_t
  };
  void loop();
  void plan();
  size_t grant(const ServeRequest &r) const;
  int device_;
  size_t pool_bytes_;
  void *pool_ = nullptr;
  RangePool ranges_;
  std::vector<std::unique_ptr<Lane>> lanes_;
  mutable std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<ServeRequest>> queue_, unplanned_;
  std::condition_variable plan_cv_;
  std::thread planner_;
  std::unordered_map<int64_t, std::shared_ptr<ServeRequest>> all_;
  int64_t next_id_ = 1, n_done_ = 0;
  double flops_done_ = 0;
  bool stop_ = false;
  std::thread worker_;
};

}  // namespace bl
