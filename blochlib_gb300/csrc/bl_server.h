// Serving loop: continuous batching of powder-FID jobs on one GPU.
//
// The reference has no server; its closest analogue is the MPI master/worker farm that
// hands crystallites to free workers as they finish (src/QMspins/driver/oneFID.h:230-286,
// examples/solid-2.0/src/sequencerun.cc:435-526).  Here the unit handed out is a whole
// job (spin system + powder + rho/detect + parameters) and the workers are slots of device
// memory, each with its own CUDA stream:
//   * one device allocation at start, cut into `slots` regions of `slot_bytes`;
//   * a request is admitted (FIFO) as soon as a slot is free: its job is built inside the
//     slot's region (no further allocation), enqueued on the slot's stream, and its
//     completion recorded with an event, so jobs in different slots overlap on the GPU;
//   * a worker thread polls completions, copies the FID back and frees the slot;
//   * latency = completion - submission, measured on the host steady clock.
// Jobs never share arithmetic, so a result does not depend on what else is in flight.
#pragma once

#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
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
  SpinSystem sys;
  Powder pw;
  CMatrix ro, det;
  FidParams p;
  std::chrono::steady_clock::time_point t_submit, t_start, t_done;
  int state = 0;  // 0 queued, 1 running, 2 done, 3 failed, 4 cancelled
  std::vector<double> fid;
  double sw = 0;
  std::string err;
  ServeRequest(const SpinSystem &s, const Powder &w, const CMatrix &r, const CMatrix &d, const FidParams &q)
      : sys(s), pw(w), ro(r), det(d), p(q) {}
};

class Server {
 public:
  Server(int device, int slots, size_t slot_bytes);
  ~Server();
  int64_t submit(const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det, const FidParams &p);
  // state of a ticket; when done and fid_out is given, copies the FID and forgets the ticket
  int poll(int64_t id, double *fid_out, double *sw_out, double *latency_ms, std::string *err);
  bool cancel(int64_t id);
  void stats(int64_t *queued, int64_t *running, int64_t *done) const;

 private:
  struct Slot {
    Context ctx;
    char *base = nullptr;
    size_t bytes = 0;
    std::unique_ptr<Job> job;
    std::shared_ptr<ServeRequest> req;
    void *event = nullptr;  // cudaEvent_t
  };
  void loop();
  int device_;
  size_t slot_bytes_;
  void *pool_ = nullptr;
  std::vector<std::unique_ptr<Slot>> slots_;
  mutable std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<ServeRequest>> queue_;
  std::unordered_map<int64_t, std::shared_ptr<ServeRequest>> all_;
  int64_t next_id_ = 1, n_done_ = 0;
  bool stop_ = false;
  std::thread worker_;
};

}  // namespace bl
