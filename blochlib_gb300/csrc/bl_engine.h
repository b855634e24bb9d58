// GPU engine for the spinning powder FID (gamma-COMPUTE), internal C++ interface.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "bl_host.h"

namespace bl {

struct FidParams {
  int npts = 0;
  double sw = 0, wr = 0, rotb_deg = 0, start_t = 0;
  int precision = 0;  // 0 = FP64; 1 = mixed (FP64 step, Dyson, Floquet and powder sum;
                      // single-precision eigenframe, Q/R, Fave and FID terms)
  int step_method = 0;  // step exponential: 0 Jacobi eigen-decomposition, 1 Taylor + squaring
  int fave_method = 0;  // Fave correlation: 0 auto (FFT when n <= 2048), 1 direct, 2 FFT
  // mixed form: crystallites (spread evenly over the powder) on which error_statement()
  // recomputes the FID in FP64 and in the mixed form; 0 = no statement
  int error_sample = 0;
  // Point-to-point FID (p2p_base > 0): points every p2p_factor/p2p_base rotor periods,
  // fid[p] = sum_c w_c Tr(rho_c(t_p) det) / Tr(det det^H); each rotor period is cut into
  // p2p_base chunks of ceil(chunk / maxtstep) steps (one step when maxtstep <= 0).  Static
  // (wr == 0 or rotor angle 0): one step of 1/sw per point.
  int p2p_base = 0, p2p_factor = 0;
  double maxtstep = 0;
  // rf that changes within the rotor period (point-to-point only): each field is on during
  // one chunk (0 <= chunk < p2p_base; base and factor are then not reduced by their gcd),
  // on top of the system's continuous rf; the pattern repeats every rotor period
  struct RfChunk {
    int chunk;
    RfField field;
  };
  std::vector<RfChunk> rf_chunks;
};

struct Context {
  int device = 0;
  size_t hbm_budget = 0;  // bytes the engine may hold for one job's work buffers
                          // (0: 60% of the device memory free when the job is created)
  cudaStream_t stream = nullptr;
  ~Context();
};

struct JobImpl;

// A job with all inputs resident on the device; run() recomputes the powder FID.
class Job {
 public:
  Job(Context &ctx, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
      const FidParams &p);
  ~Job();
  void run();                       // enqueue all kernels on the context stream
  void read(double *fid_out);       // device -> host (2*npts doubles), synchronises
  double sw_out() const;
  int npts() const;
  int kernels_per_run() const;      // kernel launches one run() enqueues
  const double *device_fid() const; // device pointer, 2*npts doubles
  std::string describe() const;     // layout summary (JSON)
  // algorithmic FP64 flop count of one run() (one complex MAC = 8 flop)
  double flops() const;
  // BF16 tensor-core flops the last run() issued in its exact-slice products (step, Dyson;
  // 10 slice pairs x 2 b^3 per real b x b product, unpadded); synchronises the stream
  void tensor_flops(double *step, double *dyson) const;

  // Per-stage CUDA-event timing of run() (stages: see stage_name), accumulated while on.
  static constexpr int kStages = 8;
  static const char *stage_name(int s);
  void set_profiling(bool on);
  void stage_times(double *ms, int *launches) const;  // kStages each, accumulated
  void stage_flops(double *flops) const;              // algorithmic flop per run, per stage
  void reset_stage_times();
  // Host<->device bytes moved per bl_powder_fid call (upload at creation, FID read back)
  size_t h2d_bytes() const;
  size_t d2h_bytes() const;
  // Runs run() 'iters' times between two events on the context stream; returns ms total.
  double run_timed(int iters);

 private:
  std::unique_ptr<JobImpl> d_;
};

// Measured FP64 FMA throughput of the device (TFLOP/s), from a short DFMA probe kernel.
// The mixed form's stated error: the relative L2 difference between the mixed-form and the
// FP64 FID of `sample` crystallites of the powder (indices (2k+1) C / (2 sample)), run as two
// jobs on the context's stream (device memory of their own).
double error_statement(Context &ctx, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
                       const FidParams &p, int sample);
double probe_fp64_tflops(Context &ctx);
// Measured FP32 FMA throughput (TFLOP/s): the pipe of the mixed form's double-float stages.
double probe_fp32_tflops(Context &ctx);

// The powder FID with every device buffer taken from one static device array (no device
// allocation or free during the call); see bl_powder_fid_noalloc.
void powder_fid_noalloc(Context &ctx, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
                        const FidParams &p, double *fid_out, double *sw_out);
size_t noalloc_scratch_bytes();

// Device bytes a job needs: *min_bytes with one warp (32) of crystallites per batch,
// *full_bytes with all crystallites in one batch.  Plans the job on the host only.
void job_bytes(int device, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
               const FidParams &p, size_t *min_bytes, size_t *full_bytes);

// A Job whose device buffers are all carved from [base, base + bytes) (no allocation).
std::unique_ptr<Job> job_in_region(Context &ctx, void *base, size_t bytes, const SpinSystem &sys, const Powder &pw,
                                   const CMatrix &ro, const CMatrix &det, const FidParams &p);

}  // namespace bl
