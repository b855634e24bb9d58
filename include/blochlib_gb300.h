/*
 * blochlib_gb300 — C ABI of the GB300 powder-FID engine.
 *
 * Drop-in boundary for BlochLib's spinning powder-FID path (SolidSys + powder +
 * oneFID<SolidSys>::FID + plotterFID).  Plain pointers and sizes only; every call returns
 * a bl_status and never throws or aborts.  A per-thread message for the last failure is
 * available from bl_last_error().  Complex arrays are interleaved (re, im) doubles;
 * operator matrices are N x N, row-major, in the Zeeman product basis with spin 0 the
 * most significant factor (the reference's Kronecker order).
 *
 * Reference interfaces replaced (paths inside the BlochLib tree):
 *   bl_system_create      SolidSys::SolidSys(const Vector<string>&)  src/QMspins/sys.cc:40-42,120-204
 *   bl_system_operator    SpinSys::Fx()/Fy()/Fz()/Fp()/Fmi()/Fe(), Ix(i)...Imi(i)
 *                                                                    src/QMspins/spinsys.h:143-162
 *   bl_powder_zcw         powder::powder(powder::zcw, t, p, g)       src/QMspins/driver/powder.cc:94-113,248-280
 *   bl_powder_read        powder::read(file)                         src/QMspins/driver/powder.cc:333-389
 *   bl_powder_from_arrays powder setters (theta/phi/gamma/weight)    src/QMspins/driver/powder.h:111-141
 *   bl_powder_fid         oneFID<SolidSys>::FID(powder&, ro, det)    src/QMspins/driver/oneFID.h:103-108,200-208
 *                         (spinning branch oneFID.h:339-431, compute.h:86-461)
 *   bl_job_*              the same call split into upload / run / read, for callers that
 *                         keep inputs resident on the GPU between calls (no reference twin;
 *                         oneFID::FID recomputes from host data every call)
 *   bl_p2p_fid            point-to-point FID at dwell = factor/base rotor periods: the dwell
 *                         propagators of PropReduce(base, factor)::generateProps
 *                         (examples/qmsims/MMMQMAS/propreduce.cc:16-60, 455-521; chunk products
 *                         as in mmmqmas.cc:290-341), rho stepped point by point and
 *                         Tr(rho det)/Tr(det det^H) collected per point as the solid-2.0
 *                         point-to-point collector does (examples/solid-2.0/src/
 *                         sequencerun_funcs.cc:624-645; steps of at most maxtstep per chunk,
 *                         propogation.cc:246-296)
 *   bl_hamgen             HamiltonianGen::Hamiltonian(sys, expr, theta, phi, gamma)
 *                                                                    src/QMspins/driver/ham_gen.h:295-299,
 *                                                                    ham_gen.cc:428-1212
 *   bl_plotter_fid        plotterFID(fid, file, dt)                  src/utils/plotter.cc:49-135
 *   bl_mat5_*             Matlab5 / matstream put(name, data)        src/utils/matlab5.h:603-792
 *   bl_rotation3/2        rotationMatrix3D(a,b,g) / (phi,theta)      src/QMspins/space_ten.cc:578-652
 */
#ifndef BLOCHLIB_GB300_H
#define BLOCHLIB_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  BL_OK = 0,
  BL_ERR_INVALID = 1,     /* bad argument (sizes, null pointers, npts<=0, sw/wr<1) */
  BL_ERR_PARSE = 2,       /* malformed spin-system text / unknown isotope */
  BL_ERR_CUDA = 3,        /* CUDA runtime error (message in bl_last_error) */
  BL_ERR_NOMEM = 4,       /* the job does not fit the context's device-memory budget */
  BL_ERR_UNSUPPORTED = 5, /* valid input outside what the GPU engine implements */
  BL_ERR_NUMERIC = 7      /* an eigen-solver exceeded its iteration bound */
} bl_status;

typedef struct bl_ctx bl_ctx;
typedef struct bl_system bl_system;
typedef struct bl_powder bl_powder;
typedef struct bl_job bl_job;

typedef struct {
  int npts;        /* FID points */
  double sw;       /* sweep width, Hz (rounded to n*wr, n = floor(sw/wr+0.5)) */
  double wr;       /* rotor speed, Hz (0 = static powder FID, as is rotor angle 0) */
  double rotb_deg; /* rotor angle, degrees */
  double start_t;  /* start time, s */
  int precision;   /* 0 = FP64; 1 = mixed, <= 1e-6 relative to FP64: for Hamiltonian blocks
                      up to 39 the step exponential and the Dyson products in double-float
                      (hi + lo floats); for blocks 40-74, with step_method 1 and no rf
                      schedule, on the tensor cores as exact BF16 slice products (~2^-32 per
                      product, double-float results); the Floquet decomposition with FP32
                      Jacobi sweeps (FIDs of at most 64 rotor periods) and a double-float or
                      FP64 Cayley transform, eigenvectors and eigenvalues; single-precision
                      eigenframe, Q/R, Fave and FID terms; powder sum in FP64.  Blocks above
                      74 stay FP64. */
  int step_method; /* step exponential exp(-i 2pi tau H): 0 = eigen-decomposition (Jacobi),
                      1 = Taylor series with scaling and squaring; FP64, or in the mixed form
                      as above (blocks up to 8 with step_method 1, blocks 9-74 always) */
  int fave_method; /* correlation over the rotor period: 0 = automatic (FFT for n <= 2048),
                      1 = direct O(n^2) sum, 2 = zero-padded FFT; FP64, single precision in
                      the mixed form */
  int error_sample; /* mixed form: state the result's error.  The FID of this many crystallites
                      (spread evenly over the powder) is computed again in FP64 and in the mixed
                      form; their relative L2 difference is read with bl_last_error_statement.
                      0 = no statement (no extra work).  Honoured by bl_powder_fid and the
                      serving loop; ignored by the job and allocation-free entry points. */
} bl_fid_params;

/* Message of the calling thread's last failed call ("" if none). */
const char *bl_last_error(void);
/* Library version string. */
const char *bl_version(void);

/* Context: one CUDA device and stream; hbm_budget bytes for one job's work buffers (0 = 60%
 * of the device memory free when the job is created).  A job whose crystallites do not fit
 * runs them in equal batches. */
bl_status bl_ctx_create(int device, size_t hbm_budget, bl_ctx **out);
void bl_ctx_destroy(bl_ctx *ctx);

/* Spin system from the reference's text format (numspin/T/C/D/J/Q lines). */
bl_status bl_system_create(const char *spin_text, bl_system **out);
void bl_system_destroy(bl_system *sys);
int bl_system_dim(const bl_system *sys);
int bl_system_spins(const bl_system *sys);
/* SolidSys::setBfield (src/QMspins/sys.cc:206-210): with |B| > 1e-12 each quadrupole adds its
 * second-order term Qp^2/(B nu_rel) (c4 ((r00-r11)^2/4 + r01^2) - c2 (r02^2 + r12^2)), or
 * replaces its first-order term when its Q line's 8th column (order) is 2; order 1 keeps
 * first order only (src/QMspins/qua.cc:219-267).  Default 0.  Jobs created before the call
 * keep the field they were created with. */
bl_status bl_system_set_bfield(bl_system *sys, double bfield);
/* Continuous rf on every spin of isotope 'iso' during the FID, the pulse Hamiltonian of
 * solid-2.0's PulseData::Pulse (examples/solid-2.0/src/pulsedata.cc:110-125):
 * amp (Ix cos phase + Iy sin phase) + offset Iz per spin (Hz, degrees; amp == 0 adds
 * nothing).  Repeatable; fields on one isotope add.  Both FID forms and the static branch
 * see it (H stays periodic with the rotor).  A phase off the x axis needs a Hamiltonian that
 * commutes with the isotope's Fz (a strong J coupling to another isotope does not):
 * BL_ERR_UNSUPPORTED otherwise.  Copy-on-write, as bl_system_set_bfield. */
bl_status bl_system_add_rf(bl_system *sys, const char *iso, double amp_hz, double phase_deg, double offset_hz);
/* Operator expression, e.g. "Fx", "Ip 0", "0.5*Fx + Iz 1"; out = 2*N*N doubles. */
bl_status bl_system_operator(const bl_system *sys, const char *expr, double *out);
/* Block structure of the Hamiltonian: writes up to cap block sizes, returns the count
 * through *nblocks. */
bl_status bl_system_blocks(const bl_system *sys, int *sizes, int cap, int *nblocks);

/* HamiltonianGen expression ("Ix_0 + complexi*Iy_1", "T2m1_0,1*A21", "2*Iz" ...) evaluated
 * for the system at powder angles (theta, phi; gamma is unused, as in the reference) into
 * out (N x N complex).  nvars extra variables: names[k] = values[2k] + i values[2k+1].
 * Grammar, functions and operator set: those of the reference's HamiltonianGen, quirks
 * included (M^2 is M*M*M; "2*-3" is 2*3); a syntax error or a numeric result fails. */
bl_status bl_hamgen(const bl_system *sys, const char *expr, double theta, double phi, double gamma,
                    const char *const *names, const double *values, int nvars, double *out);

/* Powder sets. */
bl_status bl_powder_zcw(int theta_steps, int phi_steps, int gamma_steps, bl_powder **out);
bl_status bl_powder_read(const char *path, bl_powder **out);
bl_status bl_powder_from_arrays(const double *theta, const double *phi, const double *gamma,
                                const double *weight, int n, bl_powder **out);
int bl_powder_size(const bl_powder *pw);
/* Copies the angle columns (any pointer may be NULL). */
bl_status bl_powder_get(const bl_powder *pw, double *theta, double *phi, double *gamma, double *weight);
void bl_powder_destroy(bl_powder *pw);

/* Powder FID: fid_out = 2*npts doubles; *sw_out = the sweep width actually used.  The call
 * builds its job in a device region that the context keeps for the next call (the whole
 * powder in one batch when it fits the context's budget, else batches sized to a region of
 * the budget), so repeated calls allocate nothing; bl_job_create, bl_p2p_job_create and
 * bl_ctx_destroy give the region back. */
bl_status bl_powder_fid(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                        const double *det, const bl_fid_params *params, double *fid_out, double *sw_out);
/* The stated error of the last FID this thread received (bl_powder_fid, or bl_server_poll
 * copying out a finished request) when it was computed in the mixed form with
 * error_sample > 0: the relative L2 difference between the mixed-form and the FP64 FID of the
 * sampled crystallites; -1 when that FID carried no statement.  No counterpart in the
 * reference (its results are FP64 only). */
double bl_last_error_statement(void);

/* Point-to-point powder FID.  A rotor period is cut into 'base' chunks (each of
 * ceil(chunk/maxtstep) steps exp(-i 2pi tau H(t)), one when maxtstep <= 0); point p sits at
 * start_t + p*factor/(base*wr) and
 *   fid[p] = sum_c w_c Tr(U_c(t_p) rho U_c(t_p)^H det) / Tr(det det^H).
 * base and factor are divided by their gcd.  Static (wr == 0 or rotor angle 0): one step of
 * 1/sw per point.  *sw_out = base*wr/factor (sw when static).
 * rf within the rotor period (windowed or phase-cycled trains, solid-2.0's pulse term per
 * chunk, propogation.cc:246-296 with pulsedata.cc:110-125): each bl_rf_chunk is on during
 * one chunk of every period, on top of bl_system_add_rf's continuous fields; base and factor
 * are then taken as given (no gcd reduction). */
typedef struct {
  int chunk;          /* 0 .. base-1 */
  const char *iso;    /* isotope irradiated */
  double amp_hz, phase_deg, offset_hz;
} bl_rf_chunk;

typedef struct {
  int npts;        /* FID points */
  double sw;       /* static only: sweep width, Hz (dwell 1/sw) */
  double wr;       /* rotor speed, Hz */
  double rotb_deg; /* rotor angle, degrees */
  double start_t;  /* time of point 0, s */
  int precision;   /* 0 = FP64, 1 = mixed (as bl_fid_params) */
  int step_method; /* 0 = eigen-decomposition, 1 = Taylor (as bl_fid_params) */
  int base;        /* chunks per rotor period (PropReduce 'base') */
  int factor;      /* chunks per dwell (PropReduce 'factor') */
  double maxtstep; /* longest step inside a chunk, s (<= 0: one step per chunk) */
  const bl_rf_chunk *rf; /* rf schedule (may be NULL) */
  int nrf;               /* its length */
} bl_p2p_params;

bl_status bl_p2p_fid(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                     const double *det, const bl_p2p_params *params, double *fid_out, double *sw_out);
/* The same as a resident job (run with bl_job_run / bl_job_read, free with bl_job_destroy). */
bl_status bl_p2p_job_create(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                            const double *det, const bl_p2p_params *params, bl_job **out);

/* Resident job: inputs uploaded once, each run recomputes the FID on the device. */
bl_status bl_job_create(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                        const double *det, const bl_fid_params *params, bl_job **out);
bl_status bl_job_run(bl_job *job);                    /* enqueue on the context stream */
bl_status bl_job_read(bl_job *job, double *fid_out);  /* synchronises; 2*npts doubles */
bl_status bl_job_sync(bl_job *job);
int bl_job_launches(const bl_job *job);               /* kernel launches per run */
double bl_job_flops(const bl_job *job);               /* algorithmic FP64 flop per run */
/* BF16 tensor-core flops the job's last run issued in the mixed form's exact-slice products
 * (step exponential, Dyson product; 10 slice pairs x 2 b^3 per real b x b product).  Either
 * output may be NULL.  Measurement only; no counterpart in the reference. */
bl_status bl_job_tensor_flops(const bl_job *job, double *step, double *dyson);
double bl_job_sw(const bl_job *job);
/* JSON description of the job's layout; returns the length written (truncated to cap). */
int bl_job_describe(const bl_job *job, char *buf, int cap);
/* The context's CUDA stream (a cudaStream_t), for callers that time runs with events. */
void *bl_ctx_stream(bl_ctx *ctx);
void bl_job_destroy(bl_job *job);

/* Instrumentation (no reference twin: BlochLib has no profiler hooks).  With profiling on,
 * every stage of bl_job_run is bracketed by CUDA events on the context stream. */
#define BL_STAGES 8
const char *bl_stage_name(int stage);
bl_status bl_job_set_profiling(bl_job *job, int on);
bl_status bl_job_stage_times(const bl_job *job, double *ms, int *launches); /* BL_STAGES each */
bl_status bl_job_stage_flops(const bl_job *job, double *flops);             /* BL_STAGES */
bl_status bl_job_reset_stage_times(bl_job *job);
/* Runs the job iters times between two events on the context stream. */
bl_status bl_job_run_timed(bl_job *job, int iters, double *ms_total);
/* Bytes bl_powder_fid moves for this job: host->device at creation, device->host read. */
bl_status bl_job_io_bytes(const bl_job *job, size_t *h2d, size_t *d2h);
/* Measured FP64 FMA throughput of the context's device (TFLOP/s), DFMA probe kernel. */
bl_status bl_probe_fp64(bl_ctx *ctx, double *tflops);
/* Measured FP32 FMA throughput (TFLOP/s), FFMA probe kernel: the pipe of the mixed form's
 * double-float stages.  Measurement only; no counterpart in the reference. */
bl_status bl_probe_fp32(bl_ctx *ctx, double *tflops);

/* Allocation-free powder FID.  No counterpart in the reference: BlochLib has no GPU and
 * no device memory.  Same inputs, outputs and results as bl_powder_fid, for callers that
 * must not allocate device memory during a call: a host program that claims the GPU's
 * memory up front and forbids any other allocator, or a timing-critical loop where
 * cudaMalloc/cudaFree are off limits because they synchronise the whole device.
 * Every device buffer of the call comes from one static device array of
 * BL_NOALLOC_SCRATCH_BYTES that each GPU loading this library keeps until the process
 * exits; nothing is allocated or freed.  Larger powders are processed in crystallite
 * batches that fit it; a job whose smallest batch (32 crystallites plus tables) does not
 * fit returns BL_ERR_NOMEM.  Each call looks up the array's device address
 * (cudaGetSymbolAddress, which allocates nothing).  The first such lookup on a device
 * loads this library's device code and with it the array, so make the first call (or any
 * earlier compute call of this library on that device) before any stream capture and
 * before the host program claims the device's memory.  All calls share
 * the array and it keeps the previous call's contents (each call clears what must start
 * at zero); calls that overlap on the GPU, from any thread or context, race on it. */
#define BL_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
bl_status bl_powder_fid_noalloc(bl_ctx *ctx, const bl_system *sys, const bl_powder *pw, const double *ro,
                                const double *det, const bl_fid_params *params, double *fid_out,
                                double *sw_out);

/* Device bytes one powder FID needs (host-side planning, no device work): *min_bytes with
 * 32 crystallites per batch, *full_bytes with all crystallites in one batch.  Either output
 * may be NULL.  The serving loop sizes every request with this. */
bl_status bl_job_bytes(int device, const bl_system *sys, const bl_powder *pw, const double *ro, const double *det,
                       const bl_fid_params *params, size_t *min_bytes, size_t *full_bytes);

/* Serving loop with continuous batching and admission by free device memory.  No
 * counterpart in the reference beyond its MPI crystallite farm (src/QMspins/driver/
 * oneFID.h:230-286, examples/solid-2.0/src/sequencerun.cc:435-526), which hands work to
 * whichever worker finishes first; here whole jobs go to CUDA streams ("lanes") sharing one
 * pool of device memory allocated at creation.  Submitting only queues a job (the spin system
 * is shared with the caller's handle, the other inputs are copied); a planner thread sizes
 * jobs in submission order (bl_job_bytes) and fails those whose 32 crystallites do not fit
 * the pool (ticket state 3).  A sized job is admitted first come first served when a lane is
 * idle and the pool has a free range of its grant (its full size, capped at pool_bytes/lanes
 * but never below its 32-crystallite size).  The job is built inside that range (no further
 * allocation; crystallites batched to fit) and runs on the lane's stream, overlapping the
 * other lanes.
 * Ticket states: 0 queued, 1 running, 2 done, 3 failed, 4 cancelled; -1 unknown ticket. */
typedef struct bl_server bl_server;
bl_status bl_server_create(int device, int lanes, size_t pool_bytes, bl_server **out);
void bl_server_destroy(bl_server *srv);  /* waits for running jobs */
bl_status bl_server_submit(bl_server *srv, const bl_system *sys, const bl_powder *pw, const double *ro,
                           const double *det, const bl_fid_params *params, long long *ticket);
/* The same for a point-to-point FID (bl_p2p_fid's parameters, rf schedule included). */
bl_status bl_server_submit_p2p(bl_server *srv, const bl_system *sys, const bl_powder *pw, const double *ro,
                               const double *det, const bl_p2p_params *params, long long *ticket);
/* *state as above.  When the job is done (or failed/cancelled) and fid_out is non-NULL, the
 * FID (2*npts doubles) is copied and the ticket is released.  latency_ms: submit to done. */
bl_status bl_server_poll(bl_server *srv, long long ticket, int *state, double *fid_out, double *sw_out,
                         double *latency_ms);
bl_status bl_server_cancel(bl_server *srv, long long ticket);  /* queued jobs only */
/* queued and running requests, finished ones (any outcome), and the algorithmic FP64 flop of
 * the completed ones (as bl_job_flops).  Any output may be NULL. */
bl_status bl_server_stats(bl_server *srv, long long *queued, long long *running, long long *done,
                          double *flops_done);

/* Cartesian rotation matrices of the reference, row-major 3x3 (radians):
 * 3-angle (powder orientation) and 2-angle (rotor phase phi, rotor tilt theta). */
bl_status bl_rotation3(double alpha, double beta, double gamma, double *R9);
bl_status bl_rotation2(double phi, double theta, double *R9);

/* plotterFID-style text file: t, f, Re S, Im S, Re fid, Im fid, |S| (7 columns). */
bl_status bl_plotter_fid(const double *fid, int npts, const char *path, double dt);

/* MAT-file level 5 output, as the reference's Matlab5 / matstream (src/utils/matlab5.h:603-792,
 * e.g. matout.put("vdat", fid) in examples/solid-2.0/src/sequencerun_funcs.cc:786-868): open
 * truncates the file and writes the header; each put appends one variable.  bl_mat5_put takes
 * a rows x cols double matrix in row-major order, interleaved (re, im) when is_complex; a
 * vector is rows x 1 (the reference's put(name, Vector)), a scalar 1 x 1. */
typedef struct bl_mat5 bl_mat5;
bl_status bl_mat5_open(const char *path, bl_mat5 **out);
bl_status bl_mat5_put(bl_mat5 *m, const char *name, const double *data, int rows, int cols, int is_complex);
bl_status bl_mat5_put_string(bl_mat5 *m, const char *name, const char *text);
void bl_mat5_close(bl_mat5 *m);

#ifdef __cplusplus
}
#endif

#endif /* BLOCHLIB_GB300_H */
