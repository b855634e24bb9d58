// C ABI of the engine (include/blochlib_gb300.h).  Converts exceptions to bl_status.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

#include "../../include/blochlib_gb300.h"
#include "bl_engine.h"
#include "bl_hamgen.h"
#include "bl_host.h"
#include "bl_server.h"

struct bl_ctx {
  bl::Context c;
  // device memory that bl_powder_fid / bl_p2p_fid carve their work buffers from, kept between
  // calls (grown when a job needs more): no cudaMalloc / cudaFree per call once it fits
  std::mutex mu;
  void *region = nullptr;
  size_t region_bytes = 0;
  ~bl_ctx() {
    if (region) cudaFree(region);
  }
};
struct bl_system {
  // shared, so that a serving request keeps the system alive without copying its operators
  std::shared_ptr<const bl::SpinSystem> sp;
  const bl::SpinSystem &s() const { return *sp; }
};
struct bl_powder {
  bl::Powder p;
};
struct bl_job {
  std::unique_ptr<bl::Job> j;
};

namespace {
thread_local std::string g_err;
thread_local double g_stmt = -1.0;  // stated error of this thread's last FID (-1: none)

bl_status fail(int code, const std::string &msg) {
  g_err = msg;
  return static_cast<bl_status>(code);
}

template <class F>
bl_status guarded(F &&f) {
  try {
    g_err.clear();
    f();
    return BL_OK;
  } catch (const bl::Error &e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc &) {
    return fail(BL_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(BL_ERR_INVALID, e.what());
  }
}

bl::CMatrix load_op(const double *m, int N) {
  bl::CMatrix M(N);
  for (size_t i = 0; i < M.a.size(); ++i) M.a[i] = bl::cplx(m[2 * i], m[2 * i + 1]);
  return M;
}

bl::FidParams to_params(const bl_fid_params *p) {
  bl::FidParams f;
  f.npts = p->npts, f.sw = p->sw, f.wr = p->wr, f.rotb_deg = p->rotb_deg, f.start_t = p->start_t;
  f.precision = p->precision;
  f.step_method = p->step_method;
  f.fave_method = p->fave_method;
  f.error_sample = p->error_sample;
  return f;
}

bl::FidParams to_params(const bl_p2p_params *p) {
  bl::FidParams f;
  f.npts = p->npts, f.sw = p->sw, f.wr = p->wr, f.rotb_deg = p->rotb_deg, f.start_t = p->start_t;
  f.precision = p->precision;
  f.step_method = p->step_method;
  if (p->base <= 0 || p->factor <= 0) throw bl::Error(BL_ERR_INVALID, "point-to-point base and factor must be positive");
  f.p2p_base = p->base, f.p2p_factor = p->factor, f.maxtstep = p->maxtstep;
  if (p->nrf < 0 || (p->nrf > 0 && !p->rf)) throw bl::Error(BL_ERR_INVALID, "bad rf schedule");
  for (int k = 0; k < p->nrf; ++k) {
    if (!p->rf[k].iso) throw bl::Error(BL_ERR_INVALID, "rf schedule: null isotope");
    f.rf_chunks.push_back({p->rf[k].chunk, bl::RfField{p->rf[k].iso, p->rf[k].amp_hz, p->rf[k].phase_deg,
                                                      p->rf[k].offset_hz}});
  }
  return f;
}
}  // namespace

extern "C" {

static void release_region(bl_ctx *ctx);
static bool fid_in_region(bl_ctx *ctx, const bl::SpinSystem &s, const bl::Powder &pw, const bl::CMatrix &ro,
                          const bl::CMatrix &det, const bl::FidParams &p, double *fid_out, double *sw_out);

const char *bl_last_error(void) { return g_err.c_str(); }
double bl_last_error_statement(void) { return g_stmt; }
const char *bl_version(void) { return "blochlib_gb300 0.1 (sm_103a, FP64 gamma-COMPUTE)"; }

bl_status bl_ctx_create(int device, size_t hbm_budget, bl_ctx **out) {
  if (!out) return fail(BL_ERR_INVALID, "null output pointer");
  *out = nullptr;
  return guarded([&] {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n)
      throw bl::Error(BL_ERR_CUDA, std::string("no CUDA device ") + std::to_string(device) +
                                       (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : ""));
    if (cudaSetDevice(device) != cudaSuccess) throw bl::Error(BL_ERR_CUDA, "cudaSetDevice failed");
    std::unique_ptr<bl_ctx> c(new bl_ctx);
    c->c.device = device;
    c->c.hbm_budget = hbm_budget;
    if (cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking) != cudaSuccess)
      throw bl::Error(BL_ERR_CUDA, "cudaStreamCreate failed");
    *out = c.release();
  });
}

void bl_ctx_destroy(bl_ctx *ctx) { delete ctx; }
void *bl_ctx_stream(bl_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

bl_status bl_system_create(const char *spin_text, bl_system **out) {
  if (!spin_text || !out) return fail(BL_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] { *out = new bl_system{std::make_shared<const bl::SpinSystem>(bl::SpinSystem::from_text(spin_text))}; });
}

void bl_system_destroy(bl_system *sys) { delete sys; }

bl_status bl_system_set_bfield(bl_system *sys, double bfield) {
  if (!sys) return fail(BL_ERR_INVALID, "null system");
  return guarded([&] {  // a new system object: requests already holding the old one keep it
    auto copy = std::make_shared<bl::SpinSystem>(*sys->sp);
    copy->set_bfield(bfield);
    sys->sp = copy;
  });
}
bl_status bl_hamgen(const bl_system *sys, const char *expr, double theta, double phi, double gamma,
                    const char *const *names, const double *values, int nvars, double *out) {
  if (!sys || !expr || !out || nvars < 0 || (nvars > 0 && (!names || !values))) return fail(BL_ERR_INVALID, "bad arguments");
  return guarded([&] {
    bl::HamiltonianGen gen;
    for (int k = 0; k < nvars; ++k) {
      if (!names[k]) throw bl::Error(BL_ERR_INVALID, "null variable name");
      gen.add_var(names[k], bl::cplx(values[2 * k], values[2 * k + 1]));
    }
    const bl::CMatrix m = gen.evaluate(sys->s(), expr, theta, phi, gamma);
    for (size_t i = 0; i < m.a.size(); ++i) out[2 * i] = m.a[i].real(), out[2 * i + 1] = m.a[i].imag();
  });
}
bl_status bl_system_add_rf(bl_system *sys, const char *iso, double amp_hz, double phase_deg, double offset_hz) {
  if (!sys || !iso) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    auto copy = std::make_shared<bl::SpinSystem>(*sys->sp);
    copy->add_rf(bl::RfField{iso, amp_hz, phase_deg, offset_hz});
    sys->sp = copy;
  });
}
int bl_system_dim(const bl_system *sys) { return sys ? sys->s().dim() : 0; }
int bl_system_spins(const bl_system *sys) { return sys ? sys->s().spins() : 0; }

bl_status bl_system_operator(const bl_system *sys, const char *expr, double *out) {
  if (!sys || !expr || !out) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    bl::CMatrix M = sys->s().op(expr);
    for (size_t i = 0; i < M.a.size(); ++i) out[2 * i] = M.a[i].real(), out[2 * i + 1] = M.a[i].imag();
  });
}

bl_status bl_system_blocks(const bl_system *sys, int *sizes, int cap, int *nblocks) {
  if (!sys || !nblocks) return fail(BL_ERR_INVALID, "null argument");
  const auto &L = sys->s().layout();
  *nblocks = int(L.size.size());
  for (int k = 0; k < *nblocks && k < cap && sizes; ++k) sizes[k] = L.size[k];
  return BL_OK;
}

bl_status bl_powder_zcw(int t, int p, int g, bl_powder **out) {
  if (!out) return fail(BL_ERR_INVALID, "null output pointer");
  *out = nullptr;
  return guarded([&] { *out = new bl_powder{bl::powder_zcw(t, p, g)}; });
}

bl_status bl_powder_read(const char *path, bl_powder **out) {
  if (!path || !out) return fail(BL_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] { *out = new bl_powder{bl::powder_read(path)}; });
}

bl_status bl_powder_from_arrays(const double *theta, const double *phi, const double *gamma, const double *weight,
                                int n, bl_powder **out) {
  if (!out || n < 0 || (n > 0 && (!theta || !phi || !weight))) return fail(BL_ERR_INVALID, "bad powder arrays");
  *out = nullptr;
  return guarded([&] {
    bl::Powder P;
    P.theta.assign(theta, theta + n);
    P.phi.assign(phi, phi + n);
    P.weight.assign(weight, weight + n);
    if (gamma) P.gamma.assign(gamma, gamma + n);
    else P.gamma.assign(n, 0.0);
    *out = new bl_powder{P};
  });
}

int bl_powder_size(const bl_powder *pw) { return pw ? pw->p.size() : 0; }

bl_status bl_powder_get(const bl_powder *pw, double *theta, double *phi, double *gamma, double *weight) {
  if (!pw) return fail(BL_ERR_INVALID, "null powder");
  const auto &P = pw->p;
  if (theta) std::memcpy(theta, P.theta.data(), sizeof(double) * P.size());
  if (phi) std::memcpy(phi, P.phi.data(), sizeof(double) * P.size());
  if (gamma) std::memcpy(gamma, P.gamma.data(), sizeof(double) * P.size());
  if (weight) std::memcpy(weight, P.weight.data(), sizeof(double) * P.size());
  return BL_OK;
}

void bl_powder_destroy(bl_powder *pw) { delete pw; }

bl_status bl_job_create(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro, const double *det,
                        const bl_fid_params *params, bl_job **out) {
  if (!ctx || !sys || !pw || !ro || !det || !params || !out) return fail(BL_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] {
    int N = sys->s().dim();
    release_region(ctx);
    std::unique_ptr<bl_job> j(new bl_job);
    j->j.reset(new bl::Job(ctx->c, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params)));
    *out = j.release();
  });
}

bl_status bl_p2p_job_create(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                            const double *det, const bl_p2p_params *params, bl_job **out) {
  if (!ctx || !sys || !pw || !ro || !det || !params || !out) return fail(BL_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] {
    int N = sys->s().dim();
    release_region(ctx);
    std::unique_ptr<bl_job> j(new bl_job);
    j->j.reset(new bl::Job(ctx->c, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params)));
    *out = j.release();
  });
}

bl_status bl_p2p_fid(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro, const double *det,
                     const bl_p2p_params *params, double *fid_out, double *sw_out) {
  if (!fid_out) return fail(BL_ERR_INVALID, "null output");
  if (!ctx || !sys || !pw || !ro || !det || !params) return fail(BL_ERR_INVALID, "null argument");
  bool done = false;
  const bl_status st0 = guarded([&] {
    const int N = sys->s().dim();
    done = fid_in_region(ctx, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params), fid_out, sw_out);
  });
  if (st0 != BL_OK || done) return st0;
  bl_job *job = nullptr;
  bl_status st = bl_p2p_job_create(ctx, sys, pw, ro, det, params, &job);
  if (st != BL_OK) return st;
  st = bl_job_run(job);
  if (st == BL_OK) st = bl_job_read(job, fid_out);
  if (st == BL_OK && sw_out) *sw_out = job->j->sw_out();
  std::string keep = g_err;
  bl_job_destroy(job);
  g_err = keep;
  return st;
}

bl_status bl_job_run(bl_job *job) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  return guarded([&] { job->j->run(); });
}

bl_status bl_job_read(bl_job *job, double *fid_out) {
  if (!job || !fid_out) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] { job->j->read(fid_out); });
}

bl_status bl_job_sync(bl_job *job) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  return guarded([&] {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) throw bl::Error(BL_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  });
}

int bl_job_launches(const bl_job *job) { return job ? job->j->kernels_per_run() : 0; }
double bl_job_flops(const bl_job *job) { return job ? job->j->flops() : 0.0; }
bl_status bl_job_tensor_flops(const bl_job *job, double *step, double *dyson) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  return guarded([&] { job->j->tensor_flops(step, dyson); });
}
double bl_job_sw(const bl_job *job) { return job ? job->j->sw_out() : 0.0; }

int bl_job_describe(const bl_job *job, char *buf, int cap) {
  if (!job || !buf || cap <= 0) return 0;
  std::string s = job->j->describe();
  int n = int(std::min<size_t>(s.size(), size_t(cap - 1)));
  std::memcpy(buf, s.data(), n);
  buf[n] = 0;
  return n;
}

void bl_job_destroy(bl_job *job) { delete job; }

const char *bl_stage_name(int stage) { return bl::Job::stage_name(stage); }

bl_status bl_job_set_profiling(bl_job *job, int on) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  job->j->set_profiling(on != 0);
  return BL_OK;
}

bl_status bl_job_stage_times(const bl_job *job, double *ms, int *launches) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  job->j->stage_times(ms, launches);
  return BL_OK;
}

bl_status bl_job_stage_flops(const bl_job *job, double *flops) {
  if (!job || !flops) return fail(BL_ERR_INVALID, "null argument");
  job->j->stage_flops(flops);
  return BL_OK;
}

bl_status bl_job_reset_stage_times(bl_job *job) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  job->j->reset_stage_times();
  return BL_OK;
}

bl_status bl_job_run_timed(bl_job *job, int iters, double *ms_total) {
  if (!job || !ms_total || iters < 0) return fail(BL_ERR_INVALID, "bad argument");
  return guarded([&] { *ms_total = job->j->run_timed(iters); });
}

bl_status bl_job_io_bytes(const bl_job *job, size_t *h2d, size_t *d2h) {
  if (!job) return fail(BL_ERR_INVALID, "null job");
  if (h2d) *h2d = job->j->h2d_bytes();
  if (d2h) *d2h = job->j->d2h_bytes();
  return BL_OK;
}

bl_status bl_probe_fp64(bl_ctx *ctx, double *tflops) {
  if (!ctx || !tflops) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] { *tflops = bl::probe_fp64_tflops(ctx->c); });
}

bl_status bl_probe_fp32(bl_ctx *ctx, double *tflops) {
  if (!ctx || !tflops) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] { *tflops = bl::probe_fp32_tflops(ctx->c); });
}

// The context's region back to the device (a resident job sizes its batches from the free
// memory, which the region would otherwise hold).
static void release_region(bl_ctx *ctx) {
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (ctx->region) {
    cudaSetDevice(ctx->c.device);
    cudaFree(ctx->region);
  }
  ctx->region = nullptr, ctx->region_bytes = 0;
}

// One FID with the job in the context's region: the whole powder in one batch when it fits
// the budget, else batches sized to a region of the budget (the batches a job of its own
// would run; results are independent of the batch).  The region stays with the context for
// the next call, so a repeated call allocates and frees nothing (on c2, a job of its own
// spent ~75 ms per call mapping and unmapping its ~170 GB of batch buffers).  Returns false,
// having done nothing, when not even one batch fits: the caller then runs a job of its own,
// which reports the error.
static bool fid_in_region(bl_ctx *ctx, const bl::SpinSystem &s, const bl::Powder &pw, const bl::CMatrix &ro,
                          const bl::CMatrix &det, const bl::FidParams &p, double *fid_out, double *sw_out) {
  std::lock_guard<std::mutex> lock(ctx->mu);
  size_t lo = 0, full = 0;
  bl::job_bytes(ctx->c.device, s, pw, ro, det, p, &lo, &full);
  if (cudaSetDevice(ctx->c.device) != cudaSuccess) return false;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return false;
  const size_t budget = ctx->c.hbm_budget ? ctx->c.hbm_budget : size_t(0.6 * double(fr + ctx->region_bytes));
  const size_t want = std::min(full, budget);
  if (want < lo) {  // not one batch: give the region's memory back to a job of its own
    if (ctx->region) cudaFree(ctx->region);
    ctx->region = nullptr, ctx->region_bytes = 0;
    return false;
  }
  if (want > ctx->region_bytes) {
    if (ctx->region) cudaFree(ctx->region);
    ctx->region = nullptr, ctx->region_bytes = 0;
    if (cudaMalloc(&ctx->region, want) != cudaSuccess) {
      cudaGetLastError();
      ctx->region = nullptr;
      return false;
    }
    ctx->region_bytes = want;
  }
  const size_t saved = ctx->c.hbm_budget;  // job_in_region sets the budget of the region
  struct Restore {
    bl::Context &c;
    size_t v;
    ~Restore() { c.hbm_budget = v; }
  } restore{ctx->c, saved};
  std::unique_ptr<bl::Job> job;
  try {
    job = bl::job_in_region(ctx->c, ctx->region, ctx->region_bytes, s, pw, ro, det, p);
  } catch (const bl::Error &e) {
    if (e.code == BL_ERR_NOMEM) return false;  // more than the planned bytes: a job of its own
    throw;
  }
  job->run();
  job->read(fid_out);
  if (sw_out) *sw_out = job->sw_out();
  return true;
}

bl_status bl_powder_fid(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro, const double *det,
                        const bl_fid_params *params, double *fid_out, double *sw_out) {
  if (!fid_out) return fail(BL_ERR_INVALID, "null output");
  if (!ctx || !sys || !pw || !ro || !det || !params) return fail(BL_ERR_INVALID, "null argument");
  g_stmt = -1.0;
  bool done = false;
  const bl_status st0 = guarded([&] {
    const int N = sys->s().dim();
    done = fid_in_region(ctx, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params), fid_out, sw_out);
  });
  if (st0 != BL_OK) return st0;
  bl_status st = BL_OK;
  if (!done) {
    bl_job *job = nullptr;
    st = bl_job_create(ctx, sys, pw, ro, det, params, &job);
    if (st != BL_OK) return st;
    st = bl_job_run(job);
    if (st == BL_OK) st = bl_job_read(job, fid_out);
    if (st == BL_OK && sw_out) *sw_out = job->j->sw_out();
    std::string keep = g_err;
    bl_job_destroy(job);
    g_err = keep;
  }
  if (st == BL_OK && params->precision == 1 && params->error_sample > 0) {
    double stmt = -1.0;
    st = guarded([&] {
      const int N = sys->s().dim();
      stmt = bl::error_statement(ctx->c, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params),
                                 params->error_sample);
    });
    g_stmt = stmt;
  }
  return st;
}

bl_status bl_powder_fid_noalloc(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                                const double *det, const bl_fid_params *params, double *fid_out, double *sw_out) {
  if (!ctx || !sys || !pw || !ro || !det || !params || !fid_out) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    int N = sys->s().dim();
    bl::powder_fid_noalloc(ctx->c, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params), fid_out,
                           sw_out);
  });
}

struct bl_mat5 {
  bl::Mat5Writer w;
  explicit bl_mat5(const char *path) : w(path) {}
};

bl_status bl_mat5_open(const char *path, bl_mat5 **out) {
  if (!path || !out) return fail(BL_ERR_INVALID, "null argument");
  *out = nullptr;
  return guarded([&] { *out = new bl_mat5(path); });
}

bl_status bl_mat5_put(bl_mat5 *m, const char *name, const double *data, int rows, int cols, int is_complex) {
  if (!m || !name || (!data && rows * cols > 0) || rows < 0 || cols < 0) return fail(BL_ERR_INVALID, "bad arguments");
  return guarded([&] {
    const size_t n = size_t(rows) * size_t(cols);
    std::vector<double> re(n), im(is_complex ? n : 0);
    for (int r = 0; r < rows; ++r)  // row-major in, column-major (MATLAB order) out
      for (int c = 0; c < cols; ++c) {
        const size_t src = size_t(r) * cols + c, dst = size_t(c) * rows + r;
        re[dst] = is_complex ? data[2 * src] : data[src];
        if (is_complex) im[dst] = data[2 * src + 1];
      }
    m->w.put_matrix(name, re.data(), is_complex ? im.data() : nullptr, rows, cols);
  });
}

bl_status bl_mat5_put_string(bl_mat5 *m, const char *name, const char *text) {
  if (!m || !name || !text) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] { m->w.put_string(name, text); });
}

void bl_mat5_close(bl_mat5 *m) { delete m; }

bl_status bl_plotter_fid(const double *fid, int npts, const char *path, double dt) {
  if (!fid || !path || npts <= 0) return fail(BL_ERR_INVALID, "bad arguments");
  return guarded([&] { bl::write_fid_text(path, reinterpret_cast<const bl::cplx *>(fid), npts, dt); });
}

}  // extern "C"

extern "C" {

bl_status bl_rotation3(double alpha, double beta, double gamma, double *R9) {
  if (!R9) return fail(BL_ERR_INVALID, "null output");
  double R[3][3];
  bl::rotation3(alpha, beta, gamma, R);
  for (int i = 0; i < 9; ++i) R9[i] = R[i / 3][i % 3];
  return BL_OK;
}

bl_status bl_rotation2(double phi, double theta, double *R9) {
  if (!R9) return fail(BL_ERR_INVALID, "null output");
  double R[3][3];
  bl::rotation2(phi, theta, R);
  for (int i = 0; i < 9; ++i) R9[i] = R[i / 3][i % 3];
  return BL_OK;
}

}  // extern "C"

struct bl_server {
  std::unique_ptr<bl::Server> s;
};

extern "C" {

bl_status bl_job_bytes(int device, const bl_system *sys, const bl_powder *pw, const double *ro, const double *det,
                       const bl_fid_params *params, size_t *min_bytes, size_t *full_bytes) {
  if (!sys || !pw || !ro || !det || !params) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    int N = sys->s().dim();
    bl::job_bytes(device, sys->s(), pw->p, load_op(ro, N), load_op(det, N), to_params(params), min_bytes, full_bytes);
  });
}

bl_status bl_server_create(int device, int lanes, size_t pool_bytes, bl_server **out) {
  if (!out) return fail(BL_ERR_INVALID, "null output pointer");
  *out = nullptr;
  return guarded([&] {
    std::unique_ptr<bl_server> h(new bl_server);
    h->s.reset(new bl::Server(device, lanes, pool_bytes));
    *out = h.release();
  });
}

void bl_server_destroy(bl_server *srv) { delete srv; }

bl_status bl_server_submit(bl_server *srv, const bl_system *sys, const bl_powder *pw, const double *ro,
                           const double *det, const bl_fid_params *params, long long *ticket) {
  if (!srv || !sys || !pw || !ro || !det || !params || !ticket) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    int N = sys->s().dim();
    if (params->npts <= 0) throw bl::Error(BL_ERR_INVALID, "npts must be positive");
    *ticket = srv->s->submit(sys->sp, pw->p, load_op(ro, N), load_op(det, N), to_params(params));
  });
}

bl_status bl_server_submit_p2p(bl_server *srv, const bl_system *sys, const bl_powder *pw, const double *ro,
                               const double *det, const bl_p2p_params *params, long long *ticket) {
  if (!srv || !sys || !pw || !ro || !det || !params || !ticket) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    int N = sys->s().dim();
    if (params->npts <= 0) throw bl::Error(BL_ERR_INVALID, "npts must be positive");
    *ticket = srv->s->submit(sys->sp, pw->p, load_op(ro, N), load_op(det, N), to_params(params));
  });
}

bl_status bl_server_poll(bl_server *srv, long long ticket, int *state, double *fid_out, double *sw_out,
                         double *latency_ms) {
  if (!srv || !state) return fail(BL_ERR_INVALID, "null argument");
  return guarded([&] {
    std::string err;
    double stmt = -1.0;
    *state = srv->s->poll(ticket, fid_out, sw_out, latency_ms, &err, &stmt);
    if (*state == 3) g_err = err;
    if (*state == 2 && fid_out) g_stmt = stmt;
  });
}

bl_status bl_server_cancel(bl_server *srv, long long ticket) {
  if (!srv) return fail(BL_ERR_INVALID, "null server");
  if (!srv->s->cancel(ticket)) return fail(BL_ERR_INVALID, "ticket is not queued");
  return BL_OK;
}

bl_status bl_server_stats(bl_server *srv, long long *queued, long long *running, long long *done,
                          double *flops_done) {
  if (!srv) return fail(BL_ERR_INVALID, "null server");
  int64_t q = 0, r = 0, d = 0;
  double f = 0;
  srv->s->stats(&q, &r, &d, &f);
  if (queued) *queued = q;
  if (running) *running = r;
  if (done) *done = d;
  if (flops_done) *flops_done = f;
  return BL_OK;
}

}  // extern "C"
