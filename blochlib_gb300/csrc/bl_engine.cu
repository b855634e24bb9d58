// GPU engine: spinning powder FID by gamma-COMPUTE, all arithmetic FP64.
//
// Reference algorithm (paths inside the BlochLib tree):
//   per crystallite  oneFID::singleSpinningFID   src/QMspins/driver/oneFID.h:419-431
//   step loop        compute::calcUFID           src/QMspins/driver/compute.h:257-274
//   H(t)             SolidSys::Hamiltonian       src/QMspins/sys.cc:749-770
//   exp(-i2pi tau H) Mexp (Hermitian)            src/container/matrix/matexp.h:240-252
//   reconstruction   compute::calcFID            src/QMspins/driver/compute.h:308-461
//   powder sum       oneFID::spinningFID         src/QMspins/driver/oneFID.h:339-410
//
// GB300 layout.  Every per-crystallite array is stored with the crystallite index
// fastest ([item][c], stride Cpad = C rounded up to 32) and every kernel maps the 32
// lanes of a warp onto 32 consecutive crystallites, so loads/stores are coalesced and
// all control flow (block sizes, steps, element indices) is warp-uniform.  The
// Hamiltonian of every SolidSys commutes with total Fz, so H, U and the Dyson products
// are block diagonal; the host finds the blocks (connected components of the operator
// pattern) and the kernels work per block.  FP64 issue rate is the bound on GB300
// (~1.2 TFLOP/s DFMA), so the kernels avoid FP64 work rather than memory traffic:
//   k_step_prop  (c, block, step)   H_i block, Jacobi eigh, U_i = V e^{-i2pi tau L} V^T
//   k_dyson      (c, block, column) A_{i+1} = U_i A_i, one column per thread
//   k_floquet    (c, block)         unitary eig of A_n (Cayley transform + Jacobi)
//   k_eigframe   (c, block, step)   W_i = A_{i+1} V_F  (in place)
//   k_qr         (c, step, pair)    Q_i = W^H D W (and R_i = W^H rho W when needed)
//   k_fave       (c, element, p)    G_p = sum_i q_{(i+p)%n} r_i (with the period twist)
//   k_p2p_elems  (c, element)       point-to-point FID terms from Q/R and the Floquet phases
//   k_fid        (c, j, p)          fid[jn+p] = sum_e z_e^j G_p(e); weighted warp sum
//   k_reduce     (k)                compensated sum of warp partials (fixed order)
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <type_traits>

#include "bl_engine.h"

namespace bl {

namespace {

constexpr int kMaxBlock = 8;      // largest Hamiltonian block handled by this engine
constexpr int kMaxSweeps = 40;    // bound on Jacobi sweeps; exceeding it sets a status bit
constexpr int kMaxP2PSteps = 16384;  // steps per rotor period of a point-to-point FID
constexpr int kThreads = 128;
constexpr double kPi = 3.14159265358979323846;
constexpr double kPi2 = 2.0 * kPi;

enum StatusBits { kNoConvergeStep = 1, kNoConvergeFloquet = 2, kSingularCayley = 4 };

#define CUDA_OK(x)                                                                          \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) throw Error(3, std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------------ complex helpers
__device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return cmk(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cconj(double2 a) { return cmk(a.x, -a.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return cmk(a.x * s, a.y * s); }
// acc + a*b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  return cmk(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
// acc + conj(a)*b
__device__ __forceinline__ double2 cfmaconj(double2 a, double2 b, double2 acc) {
  return cmk(fma(a.x, b.x, fma(a.y, b.y, acc.x)), fma(a.x, b.y, fma(-a.y, b.x, acc.y)));
}
__device__ __forceinline__ double2 cexp(double2 z) {
  double s, c, e = exp(z.x);
  sincos(z.y, &s, &c);
  return cmk(e * c, e * s);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  double d = b.x * b.x + b.y * b.y;
  return cmk((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double chop1(double v, double eps) { return fabs(v) < eps ? 0.0 : v; }

// Single-precision twins for the mixed-precision form (same names, float2 arguments).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 acc) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y)));
}
__device__ __forceinline__ float2 cdiv(float2 a, float2 b) {
  float d = b.x * b.x + b.y * b.y;
  return make_float2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ float2 cfmaconj(float2 a, float2 b, float2 acc) {
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, acc.y)));
}
template <class C>
__device__ __forceinline__ C mkc(double r, double i);
template <>
__device__ __forceinline__ double2 mkc<double2>(double r, double i) { return make_double2(r, i); }
template <>
__device__ __forceinline__ float2 mkc<float2>(double r, double i) { return make_float2(float(r), float(i)); }
template <class C>
__device__ __forceinline__ C cvt(double2 v) { return mkc<C>(v.x, v.y); }
template <class C>
__device__ __forceinline__ double2 todbl(C v) { return make_double2(double(v.x), double(v.y)); }

// Double-float values (hi + lo, ~2^-48 relative) for the mixed form's Dyson products, where
// GB300's FP32 pipe (about 64 times the FP64 rate) does the work.  A complex element is one
// float4 (re.hi, im.hi, re.lo, im.lo) in the 16-byte slot a double2 would take.  Sums use the
// compensated dot product of Ogita, Rump and Oishi (2005) with the error-free two-sum of Knuth
// and the FMA two-product; the _rn intrinsics keep the compiler from contracting them.
__device__ __forceinline__ float4 df_store(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, ih, __double2float_rn(v.x - double(rh)), __double2float_rn(v.y - double(ih)));
}
__device__ __forceinline__ double2 df_load(float4 v) {
  return make_double2(double(v.x) + double(v.z), double(v.y) + double(v.w));
}
// running compensated sum of products: s + c
struct DfAcc {
  float s, c;
};
__device__ __forceinline__ void df_dot(DfAcc &a, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh), pe = __fmaf_rn(xh, yh, -p);       // two-product
  const float s = __fadd_rn(a.s, p), bb = __fsub_rn(s, a.s);           // two-sum
  const float se = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  a.s = s;
  a.c = __fadd_rn(a.c, __fadd_rn(__fadd_rn(pe, se), __fmaf_rn(xh, yl, __fmul_rn(xl, yh))));
}
__device__ __forceinline__ float2 df_fin(const DfAcc &a) {  // (hi, lo) of s + c
  const float h = __fadd_rn(a.s, a.c);
  return make_float2(h, __fsub_rn(a.c, __fsub_rn(h, a.s)));
}
// double-float scalars (x = hi, y = lo) for the mixed form's step exponential
__device__ __forceinline__ float2 dfv_of(double d) {
  const float h = __double2float_rn(d);
  return make_float2(h, __double2float_rn(d - double(h)));
}
__host__ __device__ __forceinline__ constexpr float2 dfv_const(double d) {
  return float2{float(d), float(d - double(float(d)))};
}
__device__ __forceinline__ float2 dfv_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x), bb = __fsub_rn(s, a.x);
  const float e = __fadd_rn(__fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb)), __fadd_rn(a.y, b.y));
  const float h = __fadd_rn(s, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ float2 dfv_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  const float e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, __fmaf_rn(a.x, b.x, -p)));
  const float h = __fadd_rn(p, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, p)));
}

// ------------------------------------------------------------------ job description
struct DevSys {
  int C, Cpad, n, npts, N, nb, S2, nint, nq, nr, ne, J, rosym, step_method;
  int M, logM, fave_method;  // FFT length for the Fave correlation; 0 direct, 1 FFT
  int fave_twist;            // 1: M == n, circular correlation of the twisted sequences
  int is_static;             // static powder FID (oneFID.h:292-336): dt = 1/sw, n = p-period
  int gper;                  // period of the FID split fid[j*gper + p] (n, or the p2p base)
  int p2p, pb, pf, psub;     // point-to-point FID: base, factor, steps per chunk
  // mixed form: 1 when the Floquet sweeps over K may run in FP32, i.e. the FID raises the
  // Floquet eigenvalues to at most kFloq32MaxPeriods periods (phase errors grow with the power)
  int floq32;
  double dt;
  const int *srp, *seo;      // per D pair (a,b): the rho pair (b,a) and first element, or -1
  const double2 *tw;         // exp(-2 pi i k / M), k < M/2
  double tau, wr, sin_rotb, cos_rotb, scale;
  // per block
  const int *bs, *boff, *bpoff;
  // per interaction: crystal tensor (xx xy xz yy yz zz), scale, packed operator
  const double *pas, *iscale, *Tk, *Hc;
  const double *fk;  // per (step, term, crystallite): the term coefficients of k_coef, or null
  // point-to-point rf schedule: hc_chunks > 0 gives one Hc per chunk of the period (step i in
  // chunk i / psub); frames (chunk x N, permuted index) rotate each step's U into the lab frame
  int hc_chunks;
  const double2 *frames;
  // double-float copies for the mixed form's step (hi, lo): term operators, constant parts,
  // and fk_df = 1 when k_coef stores the coefficients as float2 in fk's slots
  const float2 *Tk_df, *Hc_df;
  // the same operators by element for the tensor-core step: element e (packed block index)
  // holds entries [tk_ptr[e], tk_ptr[e+1]) of (term, double-float value), terms ascending
  const int *tk_ptr, *tk_term, *tk_order;
  const float2 *tk_val;
  int fk_df;
  float2 tpdf;  // 2 pi tau as double-float
  const int *ikind;  // per term: 0 first order, 1 / 2 second-order quadrupolar (c4 / c2)
  int has2;
  // Q pairs (D blocks) and R pairs (rho blocks)
  int npq, npr;
  const int *qa, *qb, *qoff, *doff;
  const int *ra, *rb, *roff, *rhooff;
  const double2 *Dblk, *Rhoblk;
  // elements of the Fave/FID sums
  const int *eq, *erev, *er, *erg, *esg;
  // per crystallite (this batch): Rp (9 x Cpad), t0, weight
  const double *Rp, *t0, *w;
  // work buffers
  double2 *U, *A, *VF, *L, *Q, *R, *G, *Z, *partial;
  // mixed-precision form: eigenframe, Q/R, Fave and FID arrays in single precision
  int mixed;
  float2 *Wf, *Qf, *Rf, *Gf, *Zf;
  const float2 *twf;
  int warp_base;  // global warp index of this batch's first crystallite
  int ft_jt, ft_pt, ft_r;  // k_fid_tiled: thread rows (4 j each), columns (4 p each), element ranges
  int *status;
  unsigned long long *tc_flops;  // [2]: BF16 tensor flops issued by the step and Dyson kernels
  // 1: in the mixed form, A and W of the large blocks (kMaxBlock < b <= kMaxBigBlock) are
  // stored crystallite-major inside each (step, block) region (big_at), so that the
  // one-CTA-per-crystallite kernels move contiguous rows; the other blocks keep [item][c]
  int clay;
};

// Precision-dependent arrays: W (eigenframe; in place over A in FP64), Q, R, G, Z, twiddles.
template <class C> struct Bufs;
template <> struct Bufs<double2> {
  static __device__ double2 *W(const DevSys &s) { return s.A; }
  static __device__ double2 *Q(const DevSys &s) { return s.Q; }
  static __device__ double2 *R(const DevSys &s) { return s.R; }
  static __device__ double2 *G(const DevSys &s) { return s.G; }
  static __device__ double2 *Z(const DevSys &s) { return s.Z; }
  static __device__ const double2 *tw(const DevSys &s) { return s.tw; }
};
template <> struct Bufs<float2> {
  static __device__ float2 *W(const DevSys &s) { return s.Wf; }
  static __device__ float2 *Q(const DevSys &s) { return s.Qf; }
  static __device__ float2 *R(const DevSys &s) { return s.Rf; }
  static __device__ float2 *G(const DevSys &s) { return s.Gf; }
  static __device__ float2 *Z(const DevSys &s) { return s.Zf; }
  static __device__ const float2 *tw(const DevSys &s) { return s.twf; }
};

// ------------------------------------------------------------------ eigen-solvers
// Cyclic Jacobi, real symmetric, B x B in registers.  a becomes diagonal, v the
// eigenvectors (columns).  Returns false if kMaxSweeps was not enough.
template <int B>
__device__ bool jacobi_sym(double (&a)[B][B], double (&v)[B][B]) {
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = 0; q < B; ++q) v[p][q] = (p == q) ? 1.0 : 0.0;
  if (B == 1) return true;
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    double off = 0, dg = 0;
#pragma unroll
    for (int p = 0; p < B; ++p) {
      dg = fma(a[p][p], a[p][p], dg);
#pragma unroll
      for (int q = p + 1; q < B; ++q) off = fma(a[p][q], a[p][q], off);
    }
    if (off <= 1e-34 * dg || off == 0.0) return true;
#pragma unroll
    for (int p = 0; p < B - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < B; ++q) {
        double apq = a[p][q];
        if (apq != 0.0) {
          double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
          double t;
          if (fabs(theta) > 1e100) t = 0.5 / theta;
          else t = copysign(1.0, theta) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
          double c = rsqrt(fma(t, t, 1.0));
          double s = t * c, tz = s / (1.0 + c);
          a[p][p] = fma(-t, apq, a[p][p]);
          a[q][q] = fma(t, apq, a[q][q]);
          a[p][q] = 0.0;
          a[q][p] = 0.0;
#pragma unroll
          for (int r = 0; r < B; ++r) {
            if (r != p && r != q) {
              double arp = a[r][p], arq = a[r][q];
              double nrp = arp - s * fma(tz, arp, arq);
              double nrq = arq + s * fma(-tz, arq, arp);
              a[r][p] = nrp, a[p][r] = nrp;
              a[r][q] = nrq, a[q][r] = nrq;
            }
          }
#pragma unroll
          for (int r = 0; r < B; ++r) {
            double vrp = v[r][p], vrq = v[r][q];
            v[r][p] = vrp - s * fma(tz, vrp, vrq);
            v[r][q] = vrq + s * fma(-tz, vrq, vrp);
          }
        }
      }
  }
  return false;
}

// Cyclic Jacobi, complex Hermitian (B x B).  Same rotation as the oracle's.
template <int B>
__device__ bool jacobi_herm(double2 (&h)[B][B], double2 (&v)[B][B]) {
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = 0; q < B; ++q) v[p][q] = cmk(p == q ? 1.0 : 0.0, 0.0);
  if (B == 1) return true;
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    double off = 0, dg = 0;
#pragma unroll
    for (int p = 0; p < B; ++p) {
      dg = fma(h[p][p].x, h[p][p].x, dg);
#pragma unroll
      for (int q = p + 1; q < B; ++q) off += h[p][q].x * h[p][q].x + h[p][q].y * h[p][q].y;
    }
    if (off <= 1e-34 * dg || off == 0.0) return true;
#pragma unroll
    for (int p = 0; p < B - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < B; ++q) {
        double2 hpq = h[p][q];
        double ab = hypot(hpq.x, hpq.y);
        if (ab != 0.0) {
          double2 ph = cmk(hpq.x / ab, hpq.y / ab);
          double theta = 0.5 * (h[q][q].x - h[p][p].x) / ab;
          double t;
          if (fabs(theta) > 1e100) t = 0.5 / theta;
          else t = copysign(1.0, theta) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
          double c = rsqrt(fma(t, t, 1.0)), s = t * c;
          double2 sp = cscale(ph, s), spc = cconj(sp);
#pragma unroll
          for (int k = 0; k < B; ++k) {  // columns p, q
            double2 hkp = h[k][p], hkq = h[k][q];
            h[k][p] = csub(cscale(hkp, c), cmul(spc, hkq));
            h[k][q] = cadd(cmul(sp, hkp), cscale(hkq, c));
          }
#pragma unroll
          for (int k = 0; k < B; ++k) {  // rows p, q
            double2 hpk = h[p][k], hqk = h[q][k];
            h[p][k] = csub(cscale(hpk, c), cmul(sp, hqk));
            h[q][k] = cadd(cmul(spc, hpk), cscale(hqk, c));
          }
          h[p][q] = cmk(0, 0);
          h[q][p] = cmk(0, 0);
          h[p][p].y = 0.0;
          h[q][q].y = 0.0;
#pragma unroll
          for (int k = 0; k < B; ++k) {
            double2 vkp = v[k][p], vkq = v[k][q];
            v[k][p] = csub(cscale(vkp, c), cmul(spc, vkq));
            v[k][q] = cadd(cmul(sp, vkp), cscale(vkq, c));
          }
        }
      }
  }
  return false;
}

// Eigen-decomposition of a unitary U = V diag(lam) V^H via the Cayley transform of
// W = e^{ia} U: K = i (I+W)^{-1} (I-W) is Hermitian with U's eigenvectors.  A first
// pass (a = 0.5) locates the spectrum; the second puts -1 in its widest gap.
template <int B>
__device__ int unitary_eig(const double2 (&U)[B][B], double2 (&lam)[B], double2 (&V)[B][B]) {
  int st = 0;
  if (B == 1) {
    lam[0] = U[0][0];
    V[0][0] = cmk(1, 0);
    return 0;
  }
  double a = 0.5;
  for (int pass = 0; pass < 2; ++pass) {
    double sa, ca;
    sincos(a, &sa, &ca);
    double2 ea = cmk(ca, sa);
    double2 M[B][B], X[B][B];
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
      for (int c = 0; c < B; ++c) {
        double2 w = cmul(ea, U[r][c]);
        double id = (r == c) ? 1.0 : 0.0;
        M[r][c] = cmk(id + w.x, w.y);
        X[r][c] = cmk(id - w.x, -w.y);
      }
    // Gaussian elimination with partial pivoting: M X' = X
#pragma unroll
    for (int k = 0; k < B; ++k) {
      int piv = k;
      double best = M[k][k].x * M[k][k].x + M[k][k].y * M[k][k].y;
#pragma unroll
      for (int i = k + 1; i < B; ++i) {
        double m2 = M[i][k].x * M[i][k].x + M[i][k].y * M[i][k].y;
        if (m2 > best) best = m2, piv = i;
      }
      if (best == 0.0) {
        st |= kSingularCayley;
        best = 1e-300;
      }
#pragma unroll
      for (int i = k + 1; i < B; ++i) {
        if (i == piv) {
#pragma unroll
          for (int j = 0; j < B; ++j) {
            double2 t = M[k][j];
            M[k][j] = M[i][j];
            M[i][j] = t;
            t = X[k][j];
            X[k][j] = X[i][j];
            X[i][j] = t;
          }
        }
      }
      double2 inv = cdiv(cmk(1, 0), M[k][k]);
#pragma unroll
      for (int i = k + 1; i < B; ++i) {
        double2 f = cmul(M[i][k], inv);
#pragma unroll
        for (int j = k; j < B; ++j) M[i][j] = csub(M[i][j], cmul(f, M[k][j]));
#pragma unroll
        for (int j = 0; j < B; ++j) X[i][j] = csub(X[i][j], cmul(f, X[k][j]));
      }
    }
#pragma unroll
    for (int k = B - 1; k >= 0; --k) {
      double2 inv = cdiv(cmk(1, 0), M[k][k]);
#pragma unroll
      for (int j = 0; j < B; ++j) {
        double2 s = X[k][j];
#pragma unroll
        for (int i = k + 1; i < B; ++i) s = csub(s, cmul(M[k][i], X[i][j]));
        X[k][j] = cmul(s, inv);
      }
    }
    // K = i X, Hermitian part
    double2 K[B][B];
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
      for (int c = 0; c < B; ++c) {
        double2 krc = cmk(-X[r][c].y, X[r][c].x);
        double2 kcr = cmk(-X[c][r].y, X[c][r].x);
        K[r][c] = cscale(cadd(krc, cconj(kcr)), 0.5);
      }
    if (!jacobi_herm<B>(K, V)) st |= kNoConvergeFloquet;
    // Rayleigh quotients
#pragma unroll
    for (int r = 0; r < B; ++r) {
      double2 s = cmk(0, 0);
#pragma unroll
      for (int k = 0; k < B; ++k) {
        double2 uv = cmk(0, 0);
#pragma unroll
        for (int l = 0; l < B; ++l) uv = cfma(U[k][l], V[l][r], uv);
        s = cfmaconj(V[k][r], uv, s);
      }
      lam[r] = s;
    }
    if (pass == 0) {
      // well conditioned already (every |1 + e^{ia} lambda| >= 1/4): keep this pass
      double mind = 4.0;
#pragma unroll
      for (int r = 0; r < B; ++r) {
        double2 w = cmul(ea, lam[r]);
        mind = fmin(mind, (1.0 + w.x) * (1.0 + w.x) + w.y * w.y);
      }
      if (mind >= 0.0625) break;
      double th[B];
#pragma unroll
      for (int r = 0; r < B; ++r) th[r] = atan2(lam[r].y, lam[r].x);
      // insertion sort
#pragma unroll
      for (int i = 1; i < B; ++i) {
#pragma unroll
        for (int j = i; j > 0; --j) {
          if (th[j] < th[j - 1]) {
            double t = th[j];
            th[j] = th[j - 1];
            th[j - 1] = t;
          }
        }
      }
      double best = -1, mid = 0;
#pragma unroll
      for (int r = 0; r < B; ++r) {
        double lo = th[r], hi = (r + 1 < B) ? th[r + 1] : th[0] + kPi2;
        if (hi - lo > best) best = hi - lo, mid = 0.5 * (lo + hi);
      }
      a = kPi - mid;
    }
  }
  return st;
}

// ------------------------------------------------------------------ kernels
__device__ __forceinline__ size_t at(int item, int c, int Cpad) { return size_t(item) * Cpad + c; }

// Rows of M = R_rotor(phi, beta) R_powder for crystallite c, phi the rotor phase (sin sp,
// cos cp): row 2 always, rows 0 and 1 only when second-order quadrupolar terms need them.
__device__ __forceinline__ void orient_rows(const DevSys &s, int c, double sp, double cp, double (&m)[3][3]) {
  const double rr[3][3] = {{cp, sp, 0.0}, {-s.cos_rotb * sp, cp * s.cos_rotb, s.sin_rotb},
                           {sp * s.sin_rotb, -cp * s.sin_rotb, s.cos_rotb}};
#pragma unroll
  for (int i = 2; i >= 0; --i) {
    if (i < 2 && !s.has2) break;
#pragma unroll
    for (int j = 0; j < 3; ++j)
      m[i][j] = rr[i][0] * s.Rp[at(0 * 3 + j, c, s.Cpad)] + rr[i][1] * s.Rp[at(1 * 3 + j, c, s.Cpad)] +
                rr[i][2] * s.Rp[at(2 * 3 + j, c, s.Cpad)];
  }
}

// u PAS' v for the packed symmetric crystal tensor of term kk
__device__ __forceinline__ double pas_form(const double *P, const double *u, const double *v) {
  return u[0] * (P[0] * v[0] + P[1] * v[1] + P[2] * v[2]) + u[1] * (P[1] * v[0] + P[3] * v[1] + P[4] * v[2]) +
         u[2] * (P[2] * v[0] + P[4] * v[1] + P[5] * v[2]);
}

// Coefficient of term kk: scale (M PAS' M^T)_22 (kind 0); second-order quadrupolar
// scale ((r00-r11)^2/4 + r01^2) (kind 1) and scale (r02^2 + r12^2) (kind 2), r = M PAS' M^T.
__device__ __forceinline__ double term_coef(const DevSys &s, int kk, const double (&m)[3][3]) {
  const double *P = s.pas + 6 * kk;
  const int kind = s.has2 ? s.ikind[kk] : 0;
  double a;
  if (kind == 0) {
    a = pas_form(P, m[2], m[2]);
  } else if (kind == 1) {
    const double r00 = pas_form(P, m[0], m[0]), r11 = pas_form(P, m[1], m[1]), r01 = pas_form(P, m[0], m[1]);
    a = (r00 - r11) * (r00 - r11) / 4.0 + r01 * r01;
  } else {
    const double r02 = pas_form(P, m[0], m[2]), r12 = pas_form(P, m[1], m[2]);
    a = r02 * r02 + r12 * r12;
  }
  return s.iscale[kk] * a;
}

// Constant part of H and rf frame of step i: one per chunk under a point-to-point rf
// schedule (chunk i / psub), else the single Hc and no frame.
__device__ __forceinline__ const double *hc_of(const DevSys &s, int i) {
  return s.hc_chunks ? s.Hc + size_t(i / s.psub) * s.S2 : s.Hc;
}
__device__ __forceinline__ const double2 *frame_of(const DevSys &s, int i) {
  return s.frames ? s.frames + size_t(i / s.psub) * s.N : nullptr;
}

// Stores u = U'(p,q) = U'(q,p) of a step's real-symmetric-H block; with a frame r the lab-frame
// U = R U' R^H takes r_p u conj(r_q) at (p,q) and r_q u conj(r_p) at (q,p).
__device__ __forceinline__ void store_u_pair(double2 *Ub, int c, int Cpad, int bp, int bo, int B, int p, int q,
                                             double2 u, const double2 *fr, bool dfl) {
  double2 upq = u, uqp = u;
  if (fr) {
    const double2 rp = fr[bo + p], rq = fr[bo + q];
    upq = cmul(cmul(rp, u), cconj(rq));
    uqp = cmul(cmul(rq, u), cconj(rp));
  }
  if (dfl) {  // mixed form: double-float for k_dyson_df
    float4 *U4 = reinterpret_cast<float4 *>(Ub);
    U4[at(bp + p * B + q, c, Cpad)] = df_store(upq);
    if (q != p) U4[at(bp + q * B + p, c, Cpad)] = df_store(uqp);
    return;
  }
  Ub[at(bp + p * B + q, c, Cpad)] = upq;
  if (q != p) Ub[at(bp + q * B + p, c, Cpad)] = uqp;
}

// H_i block at the midpoint of step i (sys.cc:749-770): rotor phase 2 pi wr t_mid,
// a = (M PAS M^T)_22 with M = R_rotor R_powder, H = Hc + sum_k scale_k a_k T_k.
template <int B>
__device__ __forceinline__ void build_h_at(const DevSys &s, int c, double sp, double cp, const double *Hcb,
                                           int bp, double (&h)[B][B]) {
  double m[3][3];
  orient_rows(s, c, sp, cp, m);
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = 0; q < B; ++q) h[p][q] = Hcb[p * B + q];
  for (int kk = 0; kk < s.nint; ++kk) {
    const double f = term_coef(s, kk, m);
    const double *T = s.Tk + size_t(kk) * s.S2 + bp;
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) {
        const double t = T[p * B + q];  // same for every lane: the skip is warp-uniform
        if (t != 0.0) h[p][q] = fma(f, t, h[p][q]);
      }
  }
}

// Term coefficients of step i for every crystallite, once per (crystallite, step): the
// small-block step kernels of all blocks read them instead of each recomputing them.
__global__ void __launch_bounds__(kThreads) k_coef(DevSys s, double *fk) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int c = int(tid % s.Cpad), i = int(tid / s.Cpad);
  if (i >= s.n || c >= s.C) return;
  double t1 = s.t0[c] + double(i) * s.tau, t2 = t1 + s.tau;
  double tmid = (t2 - t1) / 2.0 + t1;
  double sp, cp;
  sincos(tmid * s.wr * kPi2, &sp, &cp);
  double m[3][3];
  orient_rows(s, c, sp, cp, m);
  float2 *fk2 = reinterpret_cast<float2 *>(fk);
  for (int kk = 0; kk < s.nint; ++kk) {
    const double f = term_coef(s, kk, m);
    if (s.fk_df) fk2[at(i * s.nint + kk, c, s.Cpad)] = dfv_of(f);
    else fk[at(i * s.nint + kk, c, s.Cpad)] = f;
  }
}

template <int B>
__device__ __forceinline__ void build_h(const DevSys &s, int c, int i, int bp, double (&h)[B][B]) {
  const double *Hcb = hc_of(s, i) + bp;
  if (s.fk) {  // coefficients from k_coef
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) h[p][q] = Hcb[p * B + q];
    for (int kk = 0; kk < s.nint; ++kk) {
      const double f = s.fk[at(i * s.nint + kk, c, s.Cpad)];
      const double *T = s.Tk + size_t(kk) * s.S2 + bp;
#pragma unroll
      for (int p = 0; p < B; ++p)
#pragma unroll
        for (int q = 0; q < B; ++q) {
          const double t = T[p * B + q];
          if (t != 0.0) h[p][q] = fma(f, t, h[p][q]);
        }
    }
    return;
  }
  double t1 = s.t0[c] + double(i) * s.tau, t2 = t1 + s.tau;
  double tmid = (t2 - t1) / 2.0 + t1;
  double sp, cp;
  sincos(tmid * s.wr * kPi2, &sp, &cp);
  build_h_at<B>(s, c, sp, cp, Hcb, bp, h);
}

// Static powder FID, step 1 (oneFID.h:301-311): one thread per (crystallite, block): H at
// rotor phase 0 (Hamiltonian(0, dt), wr = 0), Jacobi eigen-decomposition; V (real) goes to
// VF, the eigenvalues to L.x.
template <int B>
__global__ void __launch_bounds__(kThreads) k_static_eig(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= nblist) return;
  int k = blist[rest];
  if (c >= s.C) return;
  const int bp = s.bpoff[k], bo = s.boff[k];
  double h[B][B], v[B][B];
  build_h_at<B>(s, c, 0.0, 1.0, s.Hc + bp, bp, h);
  if (!jacobi_sym<B>(h, v)) atomicOr(s.status, kNoConvergeStep);
#pragma unroll
  for (int r = 0; r < B; ++r) {
#pragma unroll
    for (int q = 0; q < B; ++q) s.VF[at(bp + r * B + q, c, s.Cpad)] = cmk(v[r][q], 0.0);
    s.L[at(bo + r, c, s.Cpad)] = cmk(h[r][r], 0.0);
  }
}

// Static powder FID, step 2 (oneFID.h:312-334): one thread per (crystallite, block pair
// (a,b) of D with rho_ba != 0).  Do = V_a^T D_ab V_b, sig0 = V_b^T rho_ba V_a,
// A_ij = Do(i,j) sig0(j,i) (dropped when |A|^2 <= 1e-10, as the reference does),
// B_ij = conj(e_i) e_j with e = exp(-2 pi i dt lambda).  fid[k] = sum A B^k is written for
// the reconstruction kernel as G_p = A B^p (p < ns) and Z_j = (B^ns)^j.
__global__ void __launch_bounds__(kThreads) k_static_elems(DevSys s) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= s.npq) return;
  const int pq = int(rest);
  if (c >= s.C || s.srp[pq] < 0) return;
  const int a = s.qa[pq], b = s.qb[pq], rp = s.srp[pq], e0 = s.seo[pq];
  const int ba = s.bs[a], bb = s.bs[b], pa = s.bpoff[a], pb = s.bpoff[b];
  const double2 *D = s.Dblk + s.doff[pq], *Rh = s.Rhoblk + s.rhooff[rp];  // D_ab (ba x bb), rho_ba (bb x ba)
  double2 X[kMaxBlock * kMaxBlock], Do[kMaxBlock * kMaxBlock];
  // Do = V_a^T (D_ab V_b)
  for (int l = 0; l < ba; ++l)
    for (int q = 0; q < bb; ++q) {
      double2 acc = cmk(0, 0);
      for (int m = 0; m < bb; ++m) {
        double2 d = D[l * bb + m];
        if (d.x == 0.0 && d.y == 0.0) continue;
        acc = cfma(d, cmk(s.VF[at(pb + m * bb + q, c, s.Cpad)].x, 0.0), acc);
      }
      X[l * bb + q] = acc;
    }
  for (int r = 0; r < ba; ++r)
    for (int q = 0; q < bb; ++q) {
      double2 acc = cmk(0, 0);
      for (int l = 0; l < ba; ++l) acc = cfma(cmk(s.VF[at(pa + l * ba + r, c, s.Cpad)].x, 0.0), X[l * bb + q], acc);
      Do[r * bb + q] = acc;
    }
  // sig0_ba = V_b^T (rho_ba V_a)   (bb x ba)
  for (int m = 0; m < bb; ++m)
    for (int r = 0; r < ba; ++r) {
      double2 acc = cmk(0, 0);
      for (int l = 0; l < ba; ++l) {
        double2 d = Rh[m * ba + l];
        if (d.x == 0.0 && d.y == 0.0) continue;
        acc = cfma(d, cmk(s.VF[at(pa + l * ba + r, c, s.Cpad)].x, 0.0), acc);
      }
      X[m * ba + r] = acc;
    }
  const double z = s.dt * kPi2;
  for (int i = 0; i < ba; ++i)
    for (int j = 0; j < bb; ++j) {
      double2 sg = cmk(0, 0);
      for (int m = 0; m < bb; ++m) sg = cfma(cmk(s.VF[at(pb + m * bb + j, c, s.Cpad)].x, 0.0), X[m * ba + i], sg);
      double2 A = cmul(Do[i * bb + j], sg);
      if (A.x * A.x + A.y * A.y <= 1.0e-10) A = cmk(0, 0);
      double si, ci, sj, cj;
      sincos(z * s.L[at(s.boff[a] + i, c, s.Cpad)].x, &si, &ci);
      sincos(z * s.L[at(s.boff[b] + j, c, s.Cpad)].x, &sj, &cj);
      const double2 B = cmul(cmk(ci, si), cmk(cj, -sj));  // conj(e_i) e_j
      const int e = e0 + i * bb + j;
      double2 g = A;
      for (int p = 0; p < s.n; ++p) {
        s.G[at(p * s.ne + e, c, s.Cpad)] = g;
        g = cmul(g, B);
      }
      // g = A B^ns now; Z_j = (B^ns)^j
      double2 bn = cmk(1, 0);
      for (int p = 0; p < s.n; ++p) bn = cmul(bn, B);
      double2 zj = cmk(1, 0);
      for (int j2 = 0; j2 < s.J; ++j2) {
        s.Z[at(j2 * s.ne + e, c, s.Cpad)] = zj;
        zj = cmul(zj, bn);
      }
    }
}

// One thread per (crystallite, block k, step i): U_i = V diag(chop(e^{-i 2pi tau L})) V^T
// from a cyclic Jacobi eigen-decomposition of the real symmetric H_i block (the
// reference's method, matexp.h:240-252).
template <int B>
__global__ void __launch_bounds__(kThreads) k_step_prop(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= long(nblist) * s.n) return;
  int i = int(rest % s.n);
  int k = blist[rest / s.n];
  if (c >= s.C) return;
  const int bp = s.bpoff[k];
  double h[B][B];
  build_h<B>(s, c, i, bp, h);
  double v[B][B];
  if (!jacobi_sym<B>(h, v)) atomicOr(s.status, kNoConvergeStep);
  double2 e[B];
  const double tp = s.tau * kPi2;
#pragma unroll
  for (int j = 0; j < B; ++j) {
    double sn, cs;
    sincos(tp * h[j][j], &sn, &cs);
    e[j] = cmk(chop1(cs, 1e-12), chop1(-sn, 1e-12));
  }
  double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
  const double2 *fr = frame_of(s, i);
  const int bo = s.boff[k];
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) {
      double2 u = cmk(0, 0);
#pragma unroll
      for (int j = 0; j < B; ++j) {
        double vv = v[p][j] * v[q][j];
        u.x = fma(vv, e[j].x, u.x);
        u.y = fma(vv, e[j].y, u.y);
      }
      store_u_pair(Ub, c, s.Cpad, bp, bo, B, p, q, u, fr, s.mixed != 0);
    }
}

// Largest power of the period propagator (periods the FID spans: npts/n for the gamma-COMPUTE
// FID, npts*factor/base for the point-to-point one) for which the mixed form sweeps over the
// Floquet K in FP32: the residual ~1e-7 off-diagonal of V's basis grows into the eigenphases
// with the power; the benchmark FIDs (2048-4096 points, 100-200 steps a period) span at most 21.
constexpr long kFloq32MaxPeriods = 64;
constexpr int kTaylorTerms = 15;  // ||x|| <= 1/2: remainder 0.5^16/16! < 1e-18

// Taylor degree for exp(-iX) with ||X||_inf = x <= 1/2: the smallest K whose first omitted
// term bound x^(K+1)/(K+1)! is at most 2^-56, i.e. x <= ((K+1)! 2^-56)^(1/(K+1)) (table for
// K = 1..14; K = 15 covers x <= 0.601).  The mixed form, whose target is 1e-6 relative and
// whose eigenframe onwards is single precision, takes 2^-40 instead (<= 1e-12 per step,
// <= 1e-10 over a period of 128 steps): two to four fewer terms.
__device__ __forceinline__ int taylor_degree(double x, bool loose) {
  constexpr double thr[14] = {5.268356063861754e-09, 4.3667382909901915e-06, 0.00013509300777591815,
                              0.0011073892359697527, 0.004640970307744106,   0.013203184215395692,
                              0.029408989058618194,  0.05554895835340547,    0.09337020827678472,
                              0.14404487618659187,   0.2082354986608797,     0.2861946964536857,
                              0.3778659482136564,    0.4829712994609099};
  constexpr double thr40[14] = {1.3486991523486091e-06, 0.00017605585575041613, 0.0021614881244146904,
                                0.010176449549599028,   0.029468324594664686,   0.06437944735017741,
                                0.11763595623447277,    0.19047604120885106,    0.2830455430072978,
                                0.39478407585236897,    0.524720576196396,      0.671676320302853,
                                0.8343956619942197,     1.0116260068329037};
  int K = kTaylorTerms;
#pragma unroll
  for (int j = 13; j >= 0; --j)
    if (x <= (loose ? thr40[j] : thr[j])) K = j + 1;
  return K;
}

// Upper-triangle index of a symmetric B x B matrix stored packed.
template <int B>
__device__ __forceinline__ constexpr int sx(int p, int q) {
  return p <= q ? p * B - p * (p - 1) / 2 + (q - p) : q * B - q * (q - 1) / 2 + (p - q);
}

// C = X Y for commuting real symmetric X, Y (the product is symmetric): upper triangle.
template <int B>
__device__ __forceinline__ void sym_mul(const double *X, const double *Y, double *C, double scale) {
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) {
      double acc = 0;
#pragma unroll
      for (int l = 0; l < B; ++l) acc = fma(X[sx<B>(p, l)], Y[sx<B>(l, q)], acc);
      C[sx<B>(p, q)] = acc * scale;
    }
}

// cos X = sum_j c_j Y^j, sin X = X sum_j s_j Y^j (Y = X^2): c_j = (-1)^j/(2j)!, s_j = (-1)^j/(2j+1)!
__device__ __forceinline__ constexpr double cos_coef(int j) {
  return j == 0 ? 1.0 : j == 1 ? -1.0 / 2 : j == 2 ? 1.0 / 24 : j == 3 ? -1.0 / 720 : j == 4 ? 1.0 / 40320
       : j == 5 ? -1.0 / 3628800 : j == 6 ? 1.0 / 479001600 : -1.0 / 87178291200.0;
}
__device__ __forceinline__ constexpr double sin_coef(int j) {
  return j == 0 ? 1.0 : j == 1 ? -1.0 / 6 : j == 2 ? 1.0 / 120 : j == 3 ? -1.0 / 5040 : j == 4 ? 1.0 / 362880
       : j == 5 ? -1.0 / 39916800 : j == 6 ? 1.0 / 6227020800.0 : -1.0 / 1307674368000.0;
}

// acc = sum_{j <= d} coef_j Y^j (d <= 7) for this thread's d: pairs L_m = coef_2m I +
// coef_2m+1 Y (zero beyond d); acc = L_top, then acc = acc Y2 + L_m for m = top-1 .. 0
// (Paterson-Stockmeyer with Y2 = Y^2: d/2 symmetric products).
template <int B, bool SIN>
__device__ __forceinline__ void ps_poly(int d, const double *Y, const double *Y2, double *acc, double *tmp) {
  constexpr int NP = B * (B + 1) / 2;
  const int top = d / 2;
#pragma unroll
  for (int m = 3; m >= 0; --m) {
    if (m > top) continue;
    const double a0 = SIN ? sin_coef(2 * m) : cos_coef(2 * m);
    const double a1 = (2 * m + 1 <= d) ? (SIN ? sin_coef(2 * m + 1) : cos_coef(2 * m + 1)) : 0.0;
    if (m < top) sym_mul<B>(acc, Y2, tmp, 1.0);
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = p; q < B; ++q) {
        const int j = sx<B>(p, q);
        const double l = fma(a1, Y[j], p == q ? a0 : 0.0);
        acc[j] = (m < top) ? tmp[j] + l : l;
      }
  }
  (void)NP;
}

// The same in double-float (float2 = hi, lo): compensated dot products over l.
template <int B>
__device__ __forceinline__ void sym_mul_df(const float2 *X, const float2 *Y, float2 *C, float scale) {
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) {
      DfAcc acc = {0.f, 0.f};
#pragma unroll
      for (int l = 0; l < B; ++l) {
        const float2 x = X[sx<B>(p, l)], y = Y[sx<B>(l, q)];
        df_dot(acc, x.x, x.y, y.x, y.y);
      }
      const float2 v = df_fin(acc);
      C[sx<B>(p, q)] = make_float2(v.x * scale, v.y * scale);  // scale is +-1 or 2: exact
    }
}
template <int B, bool SIN>
__device__ __forceinline__ void ps_poly_df(int d, const float2 *Y, const float2 *Y2, float2 *acc, float2 *tmp) {
  const int top = d / 2;
#pragma unroll
  for (int m = 3; m >= 0; --m) {
    if (m > top) continue;
    const float2 a0 = dfv_const(SIN ? sin_coef(2 * m) : cos_coef(2 * m));
    const float2 a1 = (2 * m + 1 <= d) ? dfv_const(SIN ? sin_coef(2 * m + 1) : cos_coef(2 * m + 1)) : float2{0.f, 0.f};
    if (m < top) sym_mul_df<B>(acc, Y2, tmp, 1.f);
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = p; q < B; ++q) {
        const int j = sx<B>(p, q);
        float2 l = dfv_mul(a1, Y[j]);
        if (p == q) l = dfv_add(l, a0);
        acc[j] = (m < top) ? dfv_add(tmp[j], l) : l;
      }
  }
}

// H of step i in double-float from the double-float copies of Hc, the operators and k_coef's
// coefficients.
template <int B>
__device__ __forceinline__ void build_h_df(const DevSys &s, int c, int i, int bp, float2 (&h)[B][B]) {
  const float2 *Hcb = s.Hc_df + (s.hc_chunks ? size_t(i / s.psub) * s.S2 : 0) + bp;
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = 0; q < B; ++q) h[p][q] = Hcb[p * B + q];
  const float2 *fk2 = reinterpret_cast<const float2 *>(s.fk);
  for (int kk = 0; kk < s.nint; ++kk) {
    const float2 f = fk2[at(i * s.nint + kk, c, s.Cpad)];
    const float2 *T = s.Tk_df + size_t(kk) * s.S2 + bp;
#pragma unroll
    for (int p = 0; p < B; ++p)
#pragma unroll
      for (int q = 0; q < B; ++q) {
        const float2 t = T[p * B + q];  // same for every lane: the skip is warp-uniform
        if (t.x != 0.f) h[p][q] = dfv_add(h[p][q], dfv_mul(f, t));
      }
  }
}

// The mixed form's step exponential in double-float on the FP32 pipe (~2^-48, against the
// form's 2^-40 truncation): H from build_h_df, its norm from the high parts (it only picks the
// scaling and the degree), the polynomial and the squarings; U stored as double-float for
// k_dyson_df.
template <int B>
__global__ void __launch_bounds__(kThreads) k_step_taylor_df(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= long(nblist) * s.n) return;
  int i = int(rest % s.n);
  int k = blist[rest / s.n];
  if (c >= s.C) return;
  const int bp = s.bpoff[k];
  constexpr int NP = B * (B + 1) / 2;
  float2 h[B][B];
  build_h_df<B>(s, c, i, bp, h);
  const float tpf = float(s.tau * kPi2);
  float nrm = 0.f;
#pragma unroll
  for (int p = 0; p < B; ++p) {
    float rs = 0.f;
#pragma unroll
    for (int q = 0; q < B; ++q) rs += fabsf(h[p][q].x);
    nrm = fmaxf(nrm, rs);
  }
  nrm *= tpf * (1.f + 1e-6f);  // margin over the rounding of the high parts
  int sq = 0;
  if (nrm > 0.5f) {
    frexpf(nrm / 0.5f, &sq);
    sq = min(sq, 60);
  }
  float2 sc = make_float2(ldexpf(s.tpdf.x, -sq), ldexpf(s.tpdf.y, -sq));  // 2 pi tau 2^-sq, exact scaling
  const int K = taylor_degree(double(ldexpf(nrm, -sq)), true);
  __shared__ float2 Xs[NP * kThreads];
  float2 Y[NP], Y2[NP], R[NP], S[NP], T[NP];
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) T[sx<B>(p, q)] = dfv_mul(sc, h[p][q]);
#pragma unroll
  for (int j = 0; j < NP; ++j) Xs[j * blockDim.x + threadIdx.x] = T[j];
  sym_mul_df<B>(T, T, Y, 1.f);
  sym_mul_df<B>(Y, Y, Y2, 1.f);
  ps_poly_df<B, false>(K / 2, Y, Y2, R, T);
  ps_poly_df<B, true>((K - 1) / 2, Y, Y2, S, T);
#pragma unroll
  for (int j = 0; j < NP; ++j) T[j] = Xs[j * blockDim.x + threadIdx.x];
  float2 *I = Y2;
  sym_mul_df<B>(T, S, I, -1.f);
  for (int t = 0; t < sq; ++t) {
    sym_mul_df<B>(R, R, Y, 1.f);
    sym_mul_df<B>(I, I, S, 1.f);
    sym_mul_df<B>(R, I, T, 2.f);
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      R[j] = dfv_add(Y[j], make_float2(-S[j].x, -S[j].y));
      I[j] = T[j];
    }
  }
  double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
  float4 *U4 = reinterpret_cast<float4 *>(Ub);
  const double2 *fr = frame_of(s, i);
  const int bo = s.boff[k];
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) {
      const float2 re = R[sx<B>(p, q)], im = I[sx<B>(p, q)];
      if (fr) {  // rf schedule frames: through FP64
        const double2 u = cmk(double(re.x) + double(re.y), double(im.x) + double(im.y));
        store_u_pair(Ub, c, s.Cpad, bp, bo, B, p, q, u, fr, true);
      } else {
        const float4 v = make_float4(re.x, im.x, re.y, im.y);
        U4[at(bp + p * B + q, c, s.Cpad)] = v;
        if (q != p) U4[at(bp + q * B + p, c, s.Cpad)] = v;
      }
    }
}

// One thread per (crystallite, block k, step i): U_i = exp(-i 2pi tau H_i) by a Taylor
// series of the scaled real symmetric block plus repeated squaring.  Real and imaginary
// parts of U are polynomials in H, hence symmetric and commuting, so every product is a
// real symmetric one (B^2(B+1)/2 FMA) and no division or square root is needed.
template <int B>
__global__ void __launch_bounds__(kThreads) k_step_taylor(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= long(nblist) * s.n) return;
  int i = int(rest % s.n);
  int k = blist[rest / s.n];
  if (c >= s.C) return;
  const int bp = s.bpoff[k];
  constexpr int NP = B * (B + 1) / 2;
  double h[B][B];
  build_h<B>(s, c, i, bp, h);
  const double tp = s.tau * kPi2;
  double nrm = 0;
#pragma unroll
  for (int p = 0; p < B; ++p) {
    double rs = 0;
#pragma unroll
    for (int q = 0; q < B; ++q) rs += fabs(h[p][q]);
    nrm = fmax(nrm, rs);
  }
  nrm *= tp;
  int sq = 0;
  if (nrm > 0.5) {
    frexp(nrm / 0.5, &sq);  // nrm / 0.5 < 2^sq
    sq = min(sq, 60);
  }
  const double sc = ldexp(tp, -sq);
  const int K = taylor_degree(ldexp(nrm, -sq), s.mixed != 0);
  // The degree-K Taylor polynomial of exp(-iX) as cos X - i sin X with cos X = C(Y) of degree
  // K/2 and sin X = X S(Y) of degree (K-1)/2 in Y = X^2, each by Paterson-Stockmeyer in Y^2
  // (K = 11: 7 symmetric products instead of 10).  X waits in this thread's slice of shared
  // memory, so that five packed arrays are live in registers.
  __shared__ double Xs[NP * kThreads];
  double Y[NP], Y2[NP], R[NP], S[NP], T[NP];
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) T[sx<B>(p, q)] = sc * h[p][q];
#pragma unroll
  for (int j = 0; j < NP; ++j) Xs[j * blockDim.x + threadIdx.x] = T[j];
  sym_mul<B>(T, T, Y, 1.0);
  sym_mul<B>(Y, Y, Y2, 1.0);
  ps_poly<B, false>(K / 2, Y, Y2, R, T);        // R = cos X
  ps_poly<B, true>((K - 1) / 2, Y, Y2, S, T);   // S(Y)
#pragma unroll
  for (int j = 0; j < NP; ++j) T[j] = Xs[j * blockDim.x + threadIdx.x];
  double *I = Y2;
  sym_mul<B>(T, S, I, -1.0);  // I = -sin X = -X S(Y)
  // (R + iI)^2 = (R R - I I) + i 2 R I
  for (int t = 0; t < sq; ++t) {
    sym_mul<B>(R, R, Y, 1.0);
    sym_mul<B>(I, I, S, 1.0);
    sym_mul<B>(R, I, T, 2.0);
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      R[j] = Y[j] - S[j];
      I[j] = T[j];
    }
  }
  double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
  const double2 *fr = frame_of(s, i);
  const int bo = s.boff[k];
#pragma unroll
  for (int p = 0; p < B; ++p)
#pragma unroll
    for (int q = p; q < B; ++q) {
      double2 u = cmk(R[sx<B>(p, q)], I[sx<B>(p, q)]);
      store_u_pair(Ub, c, s.Cpad, bp, bo, B, p, q, u, fr, s.mixed != 0);
    }
}

// One thread per (crystallite, block, column j): column j of A_{i+1} = U_i A_i.
template <int B>
__global__ void __launch_bounds__(kThreads) k_dyson(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= long(nblist) * B) return;
  int j = int(rest % B);
  int k = blist[rest / B];
  if (c >= s.C) return;
  const int bp = s.bpoff[k];
  double2 x[B];
#pragma unroll
  for (int r = 0; r < B; ++r) x[r] = cmk(r == j ? 1.0 : 0.0, 0.0);
  for (int i = 0; i < s.n; ++i) {
    const double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
    double2 y[B];
#pragma unroll
    for (int r = 0; r < B; ++r) {
      double2 acc = cmk(0, 0);
#pragma unroll
      for (int l = 0; l < B; ++l) acc = cfma(Ub[at(bp + r * B + l, c, s.Cpad)], x[l], acc);
      y[r] = acc;
    }
    double2 *Ab = s.A + size_t(i) * s.S2 * s.Cpad;
#pragma unroll
    for (int r = 0; r < B; ++r) {
      x[r] = y[r];
      Ab[at(bp + r * B + j, c, s.Cpad)] = y[r];
    }
  }
}

// The mixed form's Dyson product in double-float: one lane per (crystallite, block, column,
// row), U_i and A_{i+1} as float4 double-float elements; each element of U_i x is four
// compensated dot products (re and im, each of a U-hi/lo x-hi/lo expansion).
template <int B>
__global__ void __launch_bounds__(kThreads) k_dyson_df(DevSys s, const int *__restrict__ blist, int nblist) {
  // G lanes per (crystallite, column j): lane r < B owns row r of the column; a warp holds
  // 32/G consecutive crystallites of one (block, column), so the U rows it loads are whole
  // 16-byte runs of consecutive crystallites.  y_r = sum_l U_rl x_l, l ascending, each x_l
  // broadcast from lane l of the group: the same sums in the same order as one thread per
  // column, with B times the threads on the chain of n dependent steps.  The next step's U
  // row is loaded while this step is summed.
  constexpr int G = B <= 1 ? 1 : B <= 2 ? 2 : B <= 4 ? 4 : 8;
  static_assert(B <= 8, "k_dyson_df takes blocks of at most 8");
  const long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int r = int(tid % G);
  const long rest = tid / G;
  const int c = int(rest % s.Cpad);
  const long rest2 = rest / s.Cpad;
  if (rest2 >= long(nblist) * B) return;  // warp-uniform (G Cpad is a multiple of 32)
  const int j = int(rest2 % B), k = blist[rest2 / B];
  const int bp = s.bpoff[k];
  const bool own = r < B;
  const int lane0 = int(threadIdx.x & 31) & ~(G - 1);
  float4 u[B], un[B];
  auto load_row = [&](int i, float4(&d)[B]) {
    const float4 *Ub = reinterpret_cast<const float4 *>(s.U + size_t(i) * s.S2 * s.Cpad);
#pragma unroll
    for (int l = 0; l < B; ++l) d[l] = own ? Ub[at(bp + r * B + l, c, s.Cpad)] : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  load_row(0, u);
  float4 x = make_float4(r == j ? 1.f : 0.f, 0.f, 0.f, 0.f);
  for (int i = 0; i < s.n; ++i) {
    if (i + 1 < s.n) load_row(i + 1, un);
    DfAcc re = {0.f, 0.f}, im = {0.f, 0.f};
#pragma unroll
    for (int l = 0; l < B; ++l) {
      float4 xl;
      xl.x = __shfl_sync(0xffffffffu, x.x, lane0 + l);
      xl.y = __shfl_sync(0xffffffffu, x.y, lane0 + l);
      xl.z = __shfl_sync(0xffffffffu, x.z, lane0 + l);
      xl.w = __shfl_sync(0xffffffffu, x.w, lane0 + l);
      const float4 uu = u[l];
      df_dot(re, uu.x, uu.z, xl.x, xl.z);    // ur xr
      df_dot(re, -uu.y, -uu.w, xl.y, xl.w);  // - ui xi
      df_dot(im, uu.x, uu.z, xl.y, xl.w);    // ur xi
      df_dot(im, uu.y, uu.w, xl.x, xl.z);    // ui xr
    }
    const float2 a = df_fin(re), b = df_fin(im);
    x = make_float4(a.x, b.x, a.y, b.y);
    if (own && c < s.C) {
      float4 *Ab = reinterpret_cast<float4 *>(s.A + size_t(i) * s.S2 * s.Cpad);
      Ab[at(bp + r * B + j, c, s.Cpad)] = x;
    }
#pragma unroll
    for (int l = 0; l < B; ++l) u[l] = un[l];
  }
}

// One thread per (crystallite, block): Floquet eigen-decomposition of A_n.
template <int B>
__global__ void __launch_bounds__(kThreads) k_floquet(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= nblist) return;
  int k = blist[rest];
  if (c >= s.C) return;
  const int bp = s.bpoff[k], bo = s.boff[k];
  const double2 *An = s.A + size_t(s.n - 1) * s.S2 * s.Cpad;
  const float4 *An4 = reinterpret_cast<const float4 *>(An);  // mixed form: double-float A
  double2 U[B][B], lam[B], V[B][B];
#pragma unroll
  for (int r = 0; r < B; ++r)
#pragma unroll
    for (int q = 0; q < B; ++q)
      U[r][q] = s.mixed ? df_load(An4[at(bp + r * B + q, c, s.Cpad)]) : An[at(bp + r * B + q, c, s.Cpad)];
  int st = unitary_eig<B>(U, lam, V);
  if (st) atomicOr(s.status, st);
#pragma unroll
  for (int r = 0; r < B; ++r) {
#pragma unroll
    for (int q = 0; q < B; ++q) s.VF[at(bp + r * B + q, c, s.Cpad)] = V[r][q];
    // principal-branch log: (ln|lam|, atan2)   (complex.h:1058-1061)
    s.L[at(bo + r, c, s.Cpad)] = cmk(log(hypot(lam[r].x, lam[r].y)), atan2(lam[r].y, lam[r].x));
  }
}


// ------------------------------------------------------------------ Floquet, lanes per matrix
// The FP64 pipe costs a warp instruction whatever its active lanes, so one thread per
// (crystallite, block) leaves most SM sub-partitions idle when there are few blocks.  Here B
// lanes work on one matrix (lane r owns row r), 32/B matrices per warp: the same Cayley
// transform with partial pivoting and back substitution as unitary_eig, then a parallel
// (round-robin) complex Jacobi on K as in floquet_cta, and the Rayleigh quotients.  Every
// index into a lane's row is a compile-time constant (the rounds and pairs are unrolled);
// rows move between lanes by shuffles within the group.
template <int B>
struct LaneGroup {
  unsigned mask;
  int base;
  __device__ __forceinline__ double shfl(double v, int src) const { return __shfl_sync(mask, v, base + src); }
  __device__ __forceinline__ double2 shfl(double2 v, int src) const { return cmk(shfl(v.x, src), shfl(v.y, src)); }
  __device__ __forceinline__ int shfl(int v, int src) const { return __shfl_sync(mask, v, base + src); }
  __device__ __forceinline__ float shfl(float v, int src) const { return __shfl_sync(mask, v, base + src); }
  __device__ __forceinline__ float2 shfl(float2 v, int src) const {
    return make_float2(shfl(v.x, src), shfl(v.y, src));
  }
};
template <class T> struct LaneCx;
template <> struct LaneCx<double> { using type = double2; };
template <> struct LaneCx<float> { using type = float2; };
__device__ __forceinline__ double2 cxm(double r, double i) { return make_double2(r, i); }
__device__ __forceinline__ float2 cxm(float r, float i) { return make_float2(r, i); }

//
// T = double: the FP64 form.  T = float (mixed form): the Cayley transform and the sweeps
// over K in single precision; the sweeps stop one sweep after off(K)^2 <= 1e-10 diag(K)^2
// (quadratic convergence takes that to the float floor).  V accumulates the rotations in FP64,
// each scaled to exact unitarity first: the FID's reconstruction takes V^-1 = V^H, which a
// single-precision V (unitary to ~1e-7 per rotation) breaks by more than 1e-6.  The
// eigenvalues stay FP64 Rayleigh quotients of the double-float A_n: their error is quadratic
// in V's, so the phases that the FID carries over npts points keep FP64 accuracy.
template <int B, class T>
__global__ void __launch_bounds__(kThreads) k_floquet_lanes(DevSys s, const int *__restrict__ blist, int nblist) {
  using CT = typename LaneCx<T>::type;
  constexpr bool F32 = sizeof(T) == sizeof(float);
  constexpr int GPW = 32 / B;             // matrices per warp
  constexpr int BQ = B + (B & 1), NP = BQ / 2;  // round-robin players (one dummy when B is odd)
  const int lane = threadIdx.x & 31;
  const long warp = (long(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int gi = lane / B, r = lane % B;
  if (gi >= GPW) return;
  const long item = warp * GPW + gi;
  if (item >= long(nblist) * s.Cpad) return;
  const int c = int(item % s.Cpad), k = blist[item / s.Cpad];
  if (c >= s.C) return;  // the whole group leaves together
  const LaneGroup<B> g{((1u << B) - 1u) << (gi * B), gi * B};
  const int bp = s.bpoff[k], bo = s.boff[k];
  const double2 *An = s.A + size_t(s.n - 1) * s.S2 * s.Cpad;
  const float4 *An4 = reinterpret_cast<const float4 *>(An);  // mixed form: double-float A
  double2 U[B], lam[B], V[B];  // V accumulates in FP64 in both forms
  CT K[B];
#pragma unroll
  for (int q = 0; q < B; ++q)
    U[q] = s.mixed ? df_load(An4[at(bp + r * B + q, c, s.Cpad)]) : An[at(bp + r * B + q, c, s.Cpad)];
  int st = 0;
  double a = 0.5;
  for (int pass = 0; pass < 2; ++pass) {
    double sa, ca;
    sincos(a, &sa, &ca);
    const double2 ea = cmk(ca, sa);
    CT M[B], X[B];
#pragma unroll
    for (int q = 0; q < B; ++q) {
      const double2 w = cmul(ea, U[q]);
      const double id = (q == r) ? 1.0 : 0.0;
      M[q] = cxm(T(id + w.x), T(w.y));
      X[q] = cxm(T(id - w.x), T(-w.y));
    }
    // Gaussian elimination with partial pivoting (first largest |M[i][k]|, i >= k): M X' = X
#pragma unroll
    for (int kc = 0; kc < B; ++kc) {
      const T m2 = (r >= kc) ? M[kc].x * M[kc].x + M[kc].y * M[kc].y : T(-1);
      int piv = kc;
      T best = g.shfl(m2, kc);
#pragma unroll
      for (int i = kc + 1; i < B; ++i) {
        const T v = g.shfl(m2, i);
        if (v > best) best = v, piv = i;
      }
      if (best == T(0)) st |= kSingularCayley;
      const int src = (r == kc) ? piv : (r == piv ? kc : r);
#pragma unroll
      for (int q = 0; q < B; ++q) M[q] = g.shfl(M[q], src), X[q] = g.shfl(X[q], src);
      CT Mk[B], Xk[B];
#pragma unroll
      for (int q = 0; q < B; ++q) Mk[q] = g.shfl(M[q], kc), Xk[q] = g.shfl(X[q], kc);
      if (r > kc) {
        const CT f = cmul(M[kc], cdiv(cxm(T(1), T(0)), Mk[kc]));
#pragma unroll
        for (int q = kc; q < B; ++q) M[q] = csub(M[q], cmul(f, Mk[q]));
#pragma unroll
        for (int q = 0; q < B; ++q) X[q] = csub(X[q], cmul(f, Xk[q]));
      }
    }
    // back substitution, row kc on lane kc from the final rows below it
#pragma unroll
    for (int kc = B - 1; kc >= 0; --kc) {
      CT acc[B];
#pragma unroll
      for (int q = 0; q < B; ++q) acc[q] = X[q];
#pragma unroll
      for (int i = kc + 1; i < B; ++i) {
        const CT mki = M[i];  // M[kc][i] on lane kc
#pragma unroll
        for (int q = 0; q < B; ++q) {
          const CT xiq = g.shfl(X[q], i);
          acc[q] = csub(acc[q], cmul(mki, xiq));
        }
      }
      if (r == kc) {
        const CT inv = cdiv(cxm(T(1), T(0)), M[kc]);
#pragma unroll
        for (int q = 0; q < B; ++q) X[q] = cmul(acc[q], inv);
      }
    }
    // K = Hermitian part of i X (row r needs column r of X: X[q][r] from lane q), V = I
#pragma unroll
    for (int q = 0; q < B; ++q) {
      CT xqr = cxm(T(0), T(0));
#pragma unroll
      for (int t = 0; t < B; ++t) {
        const CT v = g.shfl(X[t], q);
        if (t == r) xqr = v;
      }
      const CT krq = cxm(-X[q].y, X[q].x), kqr = cxm(-xqr.y, xqr.x);
      K[q] = cscale(cadd(krq, cconj(kqr)), T(0.5));
      V[q] = cmk(q == r ? 1.0 : 0.0, 0.0);
    }
#pragma unroll
    for (int q = 0; q < B; ++q)
      if (q == r) K[q].y = T(0);
    bool conv = false, polish = false;
    for (int sweep = 0; sweep < kMaxSweeps && !conv; ++sweep) {
      T off = 0, dg = 0;
#pragma unroll
      for (int q = 0; q < B; ++q) {
        if (q > r) off += K[q].x * K[q].x + K[q].y * K[q].y;
        if (q == r) dg += K[q].x * K[q].x;
      }
      T offs = 0, dgs = 0;
#pragma unroll
      for (int t = 0; t < B; ++t) offs += g.shfl(off, t), dgs += g.shfl(dg, t);
      if (F32) {
        const bool small = offs <= T(1e-10) * dgs || offs == T(0);
        if (small && (polish || offs == T(0))) {
          conv = true;
          break;
        }
        polish = polish || small;
      } else if (offs <= 1e-34 * dgs || offs == 0.0) {
        conv = true;
        break;
      }
#pragma unroll
      for (int round = 0; round < BQ - 1; ++round) {
        // this lane's pair (mp, mq) of the round, or none
        int mp = r, mq = r;
        bool paired = false;
#pragma unroll
        for (int t = 0; t < NP; ++t) {
          const int j1 = t, j2 = BQ - 1 - t;
          int p = j1 == 0 ? 0 : 1 + (j1 - 1 + round) % (BQ - 1);
          int q = j2 == 0 ? 0 : 1 + (j2 - 1 + round) % (BQ - 1);
          if (p > q) { const int x = p; p = q; q = x; }
          if (q < B && (r == p || r == q)) mp = p, mq = q, paired = true;
        }
        // the pair's rotation, computed identically by both of its lanes from K[p][q]
        // (lane p's entry q), K[p][p] and K[q][q]
        CT own_q = cxm(T(0), T(0)), own_d = cxm(T(0), T(0));
#pragma unroll
        for (int q2 = 0; q2 < B; ++q2) {
          if (q2 == mq) own_q = K[q2];
          if (q2 == r) own_d = K[q2];
        }
        const CT hpq = g.shfl(own_q, mp);
        const T kpp = g.shfl(own_d.x, mp), kqq = g.shfl(own_d.x, mq);
        T cs = T(1);
        CT sp = cxm(T(0), T(0));
        if (paired) {
          const T ab = hypot(hpq.x, hpq.y);
          if (ab != T(0)) {
            const CT ph = cxm(hpq.x / ab, hpq.y / ab);
            const T theta = T(0.5) * (kqq - kpp) / ab;
            T tt;
            if (fabs(theta) > T(F32 ? 1e18 : 1e100)) tt = T(0.5) / theta;  // theta^2 stays finite
            else tt = copysign(T(1), theta) / (fabs(theta) + sqrt(fma(theta, theta, T(1))));
            cs = rsqrt(fma(tt, tt, T(1)));
            sp = cscale(ph, tt * cs);
          }
        }
        // columns p, q of K and V for every pair: K <- K G, V <- V G, G = [[c, sp], [-conj(sp), c]]
#pragma unroll
        for (int t = 0; t < NP; ++t) {
          const int j1 = t, j2 = BQ - 1 - t;
          int p = j1 == 0 ? 0 : 1 + (j1 - 1 + round) % (BQ - 1);
          int q = j2 == 0 ? 0 : 1 + (j2 - 1 + round) % (BQ - 1);
          if (p > q) { const int x = p; p = q; q = x; }
          if (q >= B) continue;
          const T cst = g.shfl(cs, p);
          const CT spt = g.shfl(sp, p), spc = cconj(spt);
          const CT kp = K[p], kq = K[q];
          K[p] = csub(cscale(kp, cst), cmul(spc, kq));
          K[q] = cadd(cmul(spt, kp), cscale(kq, cst));
          // V in FP64; a single-precision rotation is first scaled to c^2 + |s|^2 = 1 in FP64,
          // so that V stays unitary to FP64 rounding
          double cd = cst;
          double2 sd = todbl(spt);
          if (F32) {
            const double nn = 1.0 / sqrt(fma(cd, cd, fma(sd.x, sd.x, sd.y * sd.y)));
            cd *= nn, sd = cscale(sd, nn);
          }
          const double2 vp = V[p], vq = V[q];
          V[p] = csub(cscale(vp, cd), cmul(cconj(sd), vq));
          V[q] = cadd(cmul(sd, vp), cscale(vq, cd));
        }
        // rows p, q of K: K <- G^H K, as row = alpha row_p + beta row_q in every lane
        // (lane p: cs, -sp; lane q: conj(sp), cs; a lane without a pair keeps its row)
        const bool isp = paired && r == mp;
        const CT al = !paired ? cxm(T(1), T(0)) : (isp ? cxm(cs, T(0)) : cconj(sp));
        const CT be = !paired ? cxm(T(0), T(0)) : (isp ? cxm(-sp.x, -sp.y) : cxm(cs, T(0)));
#pragma unroll
        for (int q2 = 0; q2 < B; ++q2) {
          const CT kpk = g.shfl(K[q2], mp), kqk = g.shfl(K[q2], mq);
          if (paired) K[q2] = cadd(cmul(al, kpk), cmul(be, kqk));
        }
        if (paired && !(sp.x == T(0) && sp.y == T(0))) {
          const int other = isp ? mq : mp;
#pragma unroll
          for (int q2 = 0; q2 < B; ++q2) {
            if (q2 == other) K[q2] = cxm(T(0), T(0));
            if (q2 == r) K[q2].y = T(0);
          }
        }
      }
    }
    if (!conv) st |= kNoConvergeFloquet;
    // Rayleigh quotients lam_r = v_r^H U v_r (columns of V), in every lane
    double2 uv[B];
#pragma unroll
    for (int q = 0; q < B; ++q) uv[q] = cmk(0, 0);
#pragma unroll
    for (int l = 0; l < B; ++l)
#pragma unroll
      for (int q = 0; q < B; ++q) uv[q] = cfma(U[l], todbl(g.shfl(V[q], l)), uv[q]);  // (U V)[r][q], l ascending
#pragma unroll
    for (int q = 0; q < B; ++q) lam[q] = cmk(0, 0);
#pragma unroll
    for (int kk = 0; kk < B; ++kk)
#pragma unroll
      for (int q = 0; q < B; ++q) lam[q] = cfmaconj(todbl(g.shfl(V[q], kk)), g.shfl(uv[q], kk), lam[q]);
    if (pass == 1) break;
    double mind = 4.0;
#pragma unroll
    for (int q = 0; q < B; ++q) {
      const double2 w = cmul(ea, lam[q]);
      mind = fmin(mind, (1.0 + w.x) * (1.0 + w.x) + w.y * w.y);
    }
    if (mind >= 0.0625) break;
    // widest gap of the eigenphases (every lane, same values): -1 into its middle
    double th[B];
#pragma unroll
    for (int q = 0; q < B; ++q) th[q] = atan2(lam[q].y, lam[q].x);
#pragma unroll
    for (int i = 1; i < B; ++i)
#pragma unroll
      for (int j = i; j > 0; --j)
        if (th[j - 1] > th[j]) { const double x = th[j]; th[j] = th[j - 1]; th[j - 1] = x; }
    double best = -1, mid = 0;
#pragma unroll
    for (int q = 0; q < B; ++q) {
      const double lo = th[q], hi = (q + 1 < B) ? th[q + 1] : th[0] + kPi2;
      if (hi - lo > best) best = hi - lo, mid = 0.5 * (lo + hi);
    }
    a = kPi - mid;
  }
  if (st && r == 0) atomicOr(s.status, st);
#pragma unroll
  for (int q = 0; q < B; ++q) s.VF[at(bp + r * B + q, c, s.Cpad)] = todbl(V[q]);
  double2 lr = cmk(0, 0);
#pragma unroll
  for (int q = 0; q < B; ++q)
    if (q == r) lr = lam[q];
  // principal-branch log: (ln|lam|, atan2)   (complex.h:1058-1061)
  s.L[at(bo + r, c, s.Cpad)] = cmk(log(hypot(lr.x, lr.y)), atan2(lr.y, lr.x));
}

// One thread per (crystallite, block, step): W_i = A_{i+1} V_F (in place over A in FP64;
// into the single-precision W array in the mixed form).
template <int B, class C>
__global__ void __launch_bounds__(kThreads) k_eigframe(DevSys s, const int *__restrict__ blist, int nblist) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= long(nblist) * s.n) return;
  int i = int(rest % s.n);
  int k = blist[rest / s.n];
  if (c >= s.C) return;
  const int bp = s.bpoff[k];
  C V[B][B];
#pragma unroll
  for (int r = 0; r < B; ++r)
#pragma unroll
    for (int q = 0; q < B; ++q) V[r][q] = cvt<C>(s.VF[at(bp + r * B + q, c, s.Cpad)]);
  const double2 *Ab = s.A + size_t(i) * s.S2 * s.Cpad;
  const float4 *Ab4 = reinterpret_cast<const float4 *>(Ab);  // mixed form: double-float A
  C *Wb = Bufs<C>::W(s) + size_t(i) * s.S2 * s.Cpad;
#pragma unroll
  for (int r = 0; r < B; ++r) {
    C a[B];
#pragma unroll
    for (int l = 0; l < B; ++l) {
      if (s.mixed) {  // single precision from here on: the high parts
        const float4 v = Ab4[at(bp + r * B + l, c, s.Cpad)];
        a[l] = mkc<C>(v.x, v.y);
      } else {
        a[l] = cvt<C>(Ab[at(bp + r * B + l, c, s.Cpad)]);
      }
    }
#pragma unroll
    for (int q = 0; q < B; ++q) {
      C acc = mkc<C>(0, 0);
#pragma unroll
      for (int l = 0; l < B; ++l) acc = cfma(a[l], V[l][q], acc);
      Wb[at(bp + r * B + q, c, s.Cpad)] = acc;
    }
  }
}

// One thread per (crystallite, step, pair): Q^{ab} = W_a^H D_ab W_b  (and R pairs).
// compute.h:378-383: Qs[i] = adjprop(evect, adjprop(As[i+1], det)).
template <class C>
__global__ void __launch_bounds__(kThreads) k_qr(DevSys s) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  int npair = s.npq + s.npr;
  if (rest >= long(npair) * s.n) return;
  int i = int(rest % s.n);
  int pr = int(rest / s.n);
  if (c >= s.C) return;
  bool isq = pr < s.npq;
  int a, b, off, moff;
  const double2 *M;
  C *out;
  int nitems;
  if (isq) {
    a = s.qa[pr], b = s.qb[pr], off = s.qoff[pr], moff = s.doff[pr], M = s.Dblk, out = Bufs<C>::Q(s), nitems = s.nq;
  } else {
    int p2 = pr - s.npq;
    a = s.ra[p2], b = s.rb[p2], off = s.roff[p2], moff = s.rhooff[p2], M = s.Rhoblk, out = Bufs<C>::R(s);
    nitems = s.nr;
  }
  const int ba = s.bs[a], bb = s.bs[b], pa = s.bpoff[a], pb = s.bpoff[b];
  if (ba > kMaxBlock || bb > kMaxBlock) return;  // k_big_qr handles pairs with a large block
  const C *W = Bufs<C>::W(s) + size_t(i) * s.S2 * s.Cpad;
  C X[kMaxBlock * kMaxBlock];
  // X = M_ab W_b  (ba x bb)
  for (int l = 0; l < ba; ++l)
    for (int q = 0; q < bb; ++q) X[l * bb + q] = mkc<C>(0, 0);
  for (int l = 0; l < ba; ++l)
    for (int m = 0; m < bb; ++m) {
      double2 d2 = M[moff + l * bb + m];
      if (d2.x == 0.0 && d2.y == 0.0) continue;
      const C d = cvt<C>(d2);
      for (int q = 0; q < bb; ++q) X[l * bb + q] = cfma(d, W[at(pb + m * bb + q, c, s.Cpad)], X[l * bb + q]);
    }
  C *ob = out + size_t(i) * nitems * s.Cpad;
  for (int r = 0; r < ba; ++r)
    for (int q = 0; q < bb; ++q) {
      C acc = mkc<C>(0, 0);
      for (int l = 0; l < ba; ++l) acc = cfmaconj(W[at(pa + l * ba + r, c, s.Cpad)], X[l * bb + q], acc);
      ob[at(off + r * bb + q, c, s.Cpad)] = acc;
    }
}

constexpr int kFavePT = 8;

// One thread per (crystallite, element, tile of kFavePT values of p).
// G_p = sum_{i<n-p} q_{i+p} r_i + z sum_{i>=n-p} q_{i+p-n} r_i with z = e^{i n tau w}.
// Equals compute.h:406-427's Fave_p(r,s) times e^{i p tau w_rs}, so that
// fid[jn+p] = sum_e z_e^j G_p(e) reproduces compute.h:440-459.
__global__ void __launch_bounds__(kThreads) k_fave(DevSys s) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  int ntile = (s.n + kFavePT - 1) / kFavePT;
  if (rest >= long(s.ne) * ntile) return;
  int tile = int(rest % ntile);
  int e = int(rest / ntile);
  if (c >= s.C) return;
  const int eq = s.eq[e], erev = s.erev[e], er = s.er[e];
  // w_rs = chop((l_r - l_s)/(i n tau), 1e-10)   (compute.h:327-335)
  double2 lr = s.L[at(s.erg[e], c, s.Cpad)], ls = s.L[at(s.esg[e], c, s.Cpad)];
  double2 d = csub(lr, ls);
  double nt = double(s.n) * s.tau;
  double2 w = cmk(chop1(d.y / nt, 1e-10), chop1(-d.x / nt, 1e-10));
  // z = exp(i n tau w)
  double2 z = cexp(cmk(-nt * w.y, nt * w.x));
  if (tile == 0) {
    for (int j = 0; j < s.J; ++j) {
      double2 zj = cexp(cmk(-double(j) * nt * w.y, double(j) * nt * w.x));
      s.Z[at(j * s.ne + e, c, s.Cpad)] = zj;
    }
  }
  // Three phases over i for the tile p0..p0+PT-1: all j = i+p < n (no wrap), the mixed
  // band of at most PT-1 steps, and all wrapped.  Only the band tests j < n per p, so
  // the bulk issues exactly one complex FMA per (i, p).  q_{(i+p) mod n} for the tile
  // sits in a register window that shifts by one element per step.
  const int n = s.n, p0 = tile * kFavePT;
  const size_t qstride = size_t(s.nq) * s.Cpad, rstride = size_t(s.nr) * s.Cpad;
  const double2 *qb = s.Q + at(eq, c, s.Cpad);
  const double2 *qr = s.Q + at(erev >= 0 ? erev : 0, c, s.Cpad);
  const double2 *rb = s.R + at(er >= 0 ? er : 0, c, s.Cpad);
  const bool rosym = s.rosym != 0, has_rev = erev >= 0;
  double2 s1[kFavePT], s2[kFavePT], win[kFavePT];
#pragma unroll
  for (int t = 0; t < kFavePT; ++t) {
    s1[t] = s2[t] = cmk(0, 0);
    win[t] = qb[size_t((p0 + t) % n) * qstride];
  }
  int jl = (p0 + kFavePT) % n;  // next window element to load
  auto rho_at = [&](int i) -> double2 {
    if (rosym) {
      double2 r = cconj(qb[size_t(i) * qstride]);
      if (has_rev) r = cadd(r, qr[size_t(i) * qstride]);
      return r;
    }
    return rb[size_t(i) * rstride];
  };
  auto shift = [&]() {
#pragma unroll
    for (int t = 0; t < kFavePT - 1; ++t) win[t] = win[t + 1];
    win[kFavePT - 1] = qb[size_t(jl) * qstride];
    jl = (jl + 1 == n) ? 0 : jl + 1;
  };
  int iA = n - p0 - (kFavePT - 1);
  if (iA < 0) iA = 0;
  const int iC = n - p0;
  int i = 0;
  for (; i < iA; ++i) {
    double2 rho = rho_at(i);
#pragma unroll
    for (int t = 0; t < kFavePT; ++t) s1[t] = cfma(win[t], rho, s1[t]);
    shift();
  }
  for (; i < iC; ++i) {
    double2 rho = rho_at(i);
#pragma unroll
    for (int t = 0; t < kFavePT; ++t) {
      if (i + p0 + t < n) s1[t] = cfma(win[t], rho, s1[t]);
      else s2[t] = cfma(win[t], rho, s2[t]);
    }
    shift();
  }
  for (; i < n; ++i) {
    double2 rho = rho_at(i);
#pragma unroll
    for (int t = 0; t < kFavePT; ++t) s2[t] = cfma(win[t], rho, s2[t]);
    shift();
  }
#pragma unroll
  for (int t = 0; t < kFavePT; ++t) {
    int p = p0 + t;
    if (p < n) s.G[at(p * s.ne + e, c, s.Cpad)] = cfma(z, s2[t], s1[t]);
  }
}

// Radix-2 decimation-in-time FFT (negative exponent) of CG interleaved sequences of length
// M = 2^logM held in shared memory as X[i * CG + cc], input in bit-reversed order, output in
// natural order.  tw[k] = exp(-2 pi i k / (M twm)), k < M twm / 2 (twm = 2: a half-length
// transform on the table of the full length).  Stage st pairs the points i and i + 2^st of
// each block of 2^(st+1) with twiddle tw[(i mod 2^st) (M >> (st+1)) twm]; stages 0 and 1
// multiply by 1 and -i only.  The stages run in passes of up to three: a thread holds the
// 2^LR points of one group in registers and applies LR stages to them, so a pass costs one
// shared-memory round trip and one barrier, and every point sees the same butterflies in
// the same order as stage by stage (the result does not depend on the grouping).

// Stages st .. st+LR-1 on x[k] = point (group base) + pos + k 2^st, pos < 2^st.
template <class C, int LR>
__device__ __forceinline__ void fft_regs(C (&x)[1 << LR], int st, int pos, int M, const C *__restrict__ tw,
                                         int twm) {
#pragma unroll
  for (int l = 0; l < LR; ++l) {
    const int sl = st + l, tstride = M >> (sl + 1);
#pragma unroll
    for (int k = 0; k < (1 << LR); ++k) {
      if ((k >> l) & 1) continue;
      const int k1 = k + (1 << l);
      const int p = pos + ((k & ((1 << l) - 1)) << st);  // position within the half block
      const C a = x[k], d = x[k1];
      C t = d;
      if (sl == 1) {
        if (p) t.x = d.y, t.y = -d.x;
      } else if (sl > 1) {
        t = cmul(tw[p * tstride * twm], d);
      }
      x[k] = cadd(a, t), x[k1] = csub(a, t);
    }
  }
}

// One pass of LR stages from st over X (and Y), in place; ends with a barrier.
template <int CG, class C, int LR>
__device__ void fft_pass(C *X, C *Y, int M, int st, const C *__restrict__ tw, int twm) {
  constexpr int R = 1 << LR;
  const int h = 1 << st, items = (M >> LR) * CG;
  for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
    const int cc = idx % CG, b = idx / CG;
    const int pos = b & (h - 1), grp = b >> st;
    const int base = ((grp << (st + LR)) + pos) * CG + cc;
    for (int w = 0; w < (Y ? 2 : 1); ++w) {
      C *V = w ? Y : X;
      C x[R];
#pragma unroll
      for (int k = 0; k < R; ++k) x[k] = V[base + k * h * CG];
      fft_regs<C, LR>(x, st, pos, M, tw, twm);
#pragma unroll
      for (int k = 0; k < R; ++k) V[base + k * h * CG] = x[k];
    }
  }
  __syncthreads();
}

// Stages st0 .. logM-1 in passes of three (the last pass two or one).
template <int CG, class C>
__device__ void fft_dit(C *X, C *Y, int M, int logM, const C *__restrict__ tw, int twm = 1, int st0 = 0) {
  int st = st0;
  for (; st + 3 <= logM; st += 3) fft_pass<CG, C, 3>(X, Y, M, st, tw, twm);
  if (logM - st == 2) fft_pass<CG, C, 2>(X, Y, M, st, tw, twm);
  else if (logM - st == 1) fft_pass<CG, C, 1>(X, Y, M, st, tw, twm);
}

// The first pass (stages 0..2, logM >= 3) fused with the load: point (bit-reversed position)
// j of column cc is load(natural index brev(j), cc, x, y); the transformed groups go to X
// (and Y when it is given).  Ends with a barrier; fft_dit(..., st0 = 3) continues.
template <int CG, class C, class F>
__device__ void fft_first_pass(C *X, C *Y, int M, int logM, const C *__restrict__ tw, int twm, F &&load) {
  const int items = (M >> 3) * CG;
  for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
    const int cc = idx % CG, grp = idx / CG;
    C x[8], y[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int i = int(__brev(unsigned(grp * 8 + k)) >> (32 - logM));
      load(i, cc, x[k], y[k]);
    }
    fft_regs<C, 3>(x, 0, 0, M, tw, twm);
#pragma unroll
    for (int k = 0; k < 8; ++k) X[(grp * 8 + k) * CG + cc] = x[k];
    if (Y) {
      fft_regs<C, 3>(y, 0, 0, M, tw, twm);
#pragma unroll
      for (int k = 0; k < 8; ++k) Y[(grp * 8 + k) * CG + cc] = y[k];
    }
  }
  __syncthreads();
}

// z^j in float for z = e^{a + i b}, from e = (a, b_hi, b_lo): b = b_hi + b_lo with |b| < 2 pi
// (a difference of two principal-branch arguments).  The phase j b is j b_hi (with its exact
// rounding error, by fma) plus j b_lo, reduced modulo 2 pi against a three-term float 2 pi
// (Cody-Waite: 6.28125 has 8 significant bits, so k 6.28125 is exact); then float sincos
// with the small remainder added to the argument and a float exp of j a.  All float
// arithmetic; error a few float ulp.
__device__ __forceinline__ float2 z_pow_f(float4 e, int j) {
  constexpr float kInv2Pi = 0.15915494f, kP1 = 6.28125f, kP2 = 0.0019353071693331003f, kP3 = 1.0253131677018246e-11f;
  const float jf = float(j);
  const float p = jf * e.y, pe = __fmaf_rn(jf, e.y, -p), corr = __fmaf_rn(jf, e.z, pe);
  const float k = rintf(p * kInv2Pi);
  float r = __fmaf_rn(-k, kP1, p);
  r = __fmaf_rn(-k, kP2, r);
  r = __fmaf_rn(-k, kP3, r) + corr;
  float sn, cs;
  sincosf(r, &sn, &cs);
  const float m = expf(jf * e.x);
  return make_float2(m * cs, m * sn);
}

// Fave by FFT.  One CTA per (element e, group of CG crystallites).  With q zero outside
// [0, n), Lin_d = sum_i q_{i+d} r_i for |d| < n is the linear cross-correlation, obtained
// from zero-padded transforms of length M >= 2n:  Lin = IFFT(FFT(q) . conj(FFT(conj r))).
// Then G_p = Lin_p + z Lin_{p-n} (the same G as k_fave).  When r = conj(q) (rho = (D+D^H)/2
// and D has no block pair (b,a) for this element) the product is |FFT(q)|^2 and the second
// forward transform is skipped.
// Twisted form (fave_twist, n a power of two, M = n): with zeta^n = z, u_i = zeta^-i q_i and
// v_i = zeta^i r_i, the circular correlation C_p = sum_i v_i u_{(i+p) mod n} equals
// zeta^-p G_p (the wrapped terms carry zeta^n = z), so G_p = zeta^p C_p from transforms of
// length n instead of 2n.  zeta = e^{i tau w}; in the autocorrelation case r = conj(q) needs
// |zeta| = 1, and zeta = e^{i tau Re w} is used there: exact when the chop has zeroed Im w,
// otherwise G_p carries z e^{-n tau Im w} in place of z on its wrapped part (relative error
// at most n tau |Im w|).
template <int CG, class C>
__global__ void __launch_bounds__(128) k_fave_fft(DevSys s) {
  extern __shared__ __align__(16) unsigned char fsm_raw[];
  const int M = s.M, logM = s.logM, n = s.n;
  C *X = reinterpret_cast<C *>(fsm_raw), *Y = X + size_t(M) * CG;
  // twist tables per column: zeta^b (b < 8), zeta^8a (a < M/8), and those of zeta^-1
  double2 *tp1 = reinterpret_cast<double2 *>(Y + size_t(M) * CG), *tp8 = tp1 + 8 * CG;
  double2 *tm1 = tp8 + (M / 8) * CG, *tm8 = tm1 + 8 * CG;
  __shared__ C zc[CG];
  const int groups = s.Cpad / CG;
  const int e = blockIdx.x / groups;
  const int c0 = (blockIdx.x % groups) * CG;
  const int eq = s.eq[e], erev = s.erev[e], er = s.er[e];
  const bool autoc = s.rosym && erev < 0;
  const size_t qstride = size_t(s.nq) * s.Cpad, rstride = size_t(s.nr) * s.Cpad;
  const C *Qb = Bufs<C>::Q(s), *Rb = Bufs<C>::R(s);
  const double nt = double(n) * s.tau;
  // per crystallite of the group: w_rs = chop((l_r - l_s)/(i n tau), 1e-10), z = e^{i n tau w},
  // and the powers z^j of the FID reconstruction.  FP64 form: four powers per thread, one
  // cexp and three products (error a few ulp).  Single-precision form (the powers are stored
  // as float): the exponent of z^j in FP64, then z_pow_f per power (after the first pass).
  constexpr bool kF = std::is_same<C, float2>::value;
  __shared__ float4 zexp[CG];
  if constexpr (kF) {  // z = e^{n tau (i w)} = e^{d} with d = l_r - l_s, chopped as w is
    for (int cc = threadIdx.x; cc < CG; cc += blockDim.x) {
      const int c = c0 + cc;
      float4 ze = make_float4(0.f, 0.f, 0.f, 0.f);
      if (c < s.C) {
        const double2 d = csub(s.L[at(s.erg[e], c, s.Cpad)], s.L[at(s.esg[e], c, s.Cpad)]);
        const double thr = 1e-10 * nt;
        const double dx = fabs(d.x) < thr ? 0.0 : d.x, dy = fabs(d.y) < thr ? 0.0 : d.y;
        const float yh = float(dy);
        ze = make_float4(float(dx), yh, float(dy - double(yh)), 0.f);
      }
      zexp[cc] = ze;
    }
  } else {
    constexpr int kZrun = 4;
    const int nzr = (s.J + 1 + kZrun - 1) / kZrun;
    for (int idx = threadIdx.x; idx < CG * nzr; idx += blockDim.x) {
      const int cc = idx % CG, j0 = (idx / CG) * kZrun, c = c0 + cc;
      if (c >= s.C) continue;
      double2 d = csub(s.L[at(s.erg[e], c, s.Cpad)], s.L[at(s.esg[e], c, s.Cpad)]);
      double2 w = cmk(chop1(d.y / nt, 1e-10), chop1(-d.x / nt, 1e-10));
      const double2 z1 = cexp(cmk(-nt * w.y, nt * w.x));
      double2 zj = cexp(cmk(-double(j0) * nt * w.y, double(j0) * nt * w.x));
      for (int j = j0; j < min(j0 + kZrun, s.J + 1); ++j) {
        if (j == s.J) zc[cc] = cvt<C>(z1);
        else Bufs<C>::Z(s)[at(j * s.ne + e, c, s.Cpad)] = cvt<C>(zj);
        zj = cmul(zj, z1);
      }
    }
  }
  const bool twist = s.fave_twist;
  if (twist) {
    // one thread per column: zeta^b by products, zeta^8a by products restarted from cexp
    // every 16 entries; zeta^-k the same from -log zeta (the conjugate when |zeta| = 1)
    for (int cc = threadIdx.x; cc < CG; cc += blockDim.x) {
      const int c = c0 + cc;
      double2 zl = cmk(0, 0);
      if (c < s.C) {
        double2 d = csub(s.L[at(s.erg[e], c, s.Cpad)], s.L[at(s.esg[e], c, s.Cpad)]);
        double2 w = cmk(chop1(d.y / nt, 1e-10), chop1(-d.x / nt, 1e-10));
        zl = autoc ? cmk(0.0, s.tau * w.x) : cmk(-s.tau * w.y, s.tau * w.x);
      }
      // |zeta| = 1 in the autocorrelation case: zeta^-k is conj(zeta^k) (bit for bit, as the
      // products of conjugates are the conjugated products)
      for (int sgn = 0; sgn < 2; ++sgn) {
        const double2 l = sgn ? cmk(-zl.x, -zl.y) : zl;
        double2 *t1 = sgn ? tm1 : tp1, *t8 = sgn ? tm8 : tp8;
        if (sgn && autoc) {
          for (int b = 0; b < 8; ++b) t1[b * CG + cc] = cconj(tp1[b * CG + cc]);
          for (int a = 0; a < M / 8; ++a) t8[a * CG + cc] = cconj(tp8[a * CG + cc]);
          continue;
        }
        const double2 z1 = cexp(l);
        t1[cc] = cmk(1, 0);
        for (int b = 1; b < 8; ++b) t1[b * CG + cc] = cmul(t1[(b - 1) * CG + cc], z1);
        const double2 z8 = cmul(t1[7 * CG + cc], z1);
        t8[cc] = cmk(1, 0);
        for (int a = 1; a < M / 8; ++a)
          t8[a * CG + cc] = (a % 16 == 0) ? cexp(cmk(8.0 * a * l.x, 8.0 * a * l.y)) : cmul(t8[(a - 1) * CG + cc], z8);
      }
    }
    __syncthreads();
  }
  // q (and conj r) at natural index i, zero-padded
  auto load = [&](int i, int cc, C &qo, C &yo) {
    const int c = c0 + cc;
    C q = mkc<C>(0, 0), y = mkc<C>(0, 0);
    if (i < n && c < s.C) {
      q = Qb[i * qstride + at(eq, c, s.Cpad)];
      C r;
      if (!autoc) {
        if (s.rosym) r = cadd(cconj(q), Qb[i * qstride + at(erev, c, s.Cpad)]);
        else r = Rb[i * rstride + at(er, c, s.Cpad)];
        y = cconj(r);
      }
      if (twist) {  // u_i = zeta^-i q_i, conj(v_i) = conj(zeta^i r_i)
        const int a = i >> 3, b = i & 7;
        q = cvt<C>(cmul(cmul(tm8[a * CG + cc], tm1[b * CG + cc]), todbl(q)));
        if (!autoc) y = cconj(cvt<C>(cmul(cmul(tp8[a * CG + cc], tp1[b * CG + cc]), todbl(r))));
      }
    }
    qo = q, yo = y;
  };
  const C *tw = Bufs<C>::tw(s);
  C *Yf = autoc ? nullptr : Y;
  if (logM >= 3) {
    fft_first_pass<CG, C>(X, Yf, M, logM, tw, 1, load);
  } else {
    for (int idx = threadIdx.x; idx < M * CG; idx += blockDim.x) {
      const int cc = idx % CG, i = idx / CG;
      const int ri = int(__brev(unsigned(i)) >> (32 - logM));
      C q, y;
      load(i, cc, q, y);
      X[ri * CG + cc] = q;
      if (!autoc) Y[ri * CG + cc] = y;
    }
    __syncthreads();
  }
  if constexpr (kF) {  // z^j, j < J, and z itself (the exponents were written before the first pass's barrier)
    for (int idx = threadIdx.x; idx < CG * (s.J + 1); idx += blockDim.x) {
      const int cc = idx % CG, j = idx / CG, c = c0 + cc;
      if (c >= s.C) continue;
      if (j == s.J) zc[cc] = z_pow_f(zexp[cc], 1);
      else Bufs<C>::Z(s)[at(j * s.ne + e, c, s.Cpad)] = z_pow_f(zexp[cc], j);
    }
  }
  fft_dit<CG, C>(X, Yf, M, logM, tw, 1, logM >= 3 ? 3 : 0);
  // Inverse transform by a forward one: conj(FFT(x))/M.  Autocorrelation: the spectrum
  // S = |FFT q|^2 is real, so its transform takes one of half length on z_k = S_2k + i S_2k+1
  // (each column on its own, so a crystallite's result does not depend on its neighbours):
  // with Z = FFT_{M/2}(z), E_p = (Z_p + conj Z_-p)/2, O_p = (Z_p - conj Z_-p)/(2i),
  // FFT(S)_p = E_p + w^p O_p and FFT(S)_{p+M/2} = E_p - w^p O_p, w = exp(-2 pi i / M).
  const int Mh = M / 2;
  const bool half = autoc && M >= 4;
  const C *twb = tw;
  if (half) {
    auto spow = [&](int k, int cc, C &zo, C &) {
      const C xe = X[(2 * k) * CG + cc], xo = X[(2 * k + 1) * CG + cc];
      zo = mkc<C>(xe.x * xe.x + xe.y * xe.y, xo.x * xo.x + xo.y * xo.y);
    };
    if (logM - 1 >= 3) {
      fft_first_pass<CG, C>(Y, nullptr, Mh, logM - 1, twb, 2, spow);
    } else {
      for (int idx = threadIdx.x; idx < Mh * CG; idx += blockDim.x) {
        const int cc = idx % CG, k = idx / CG;
        C z, u;
        spow(k, cc, z, u);
        Y[int(__brev(unsigned(k)) >> (33 - logM)) * CG + cc] = z;
      }
      __syncthreads();
    }
    fft_dit<CG, C>(Y, nullptr, Mh, logM - 1, twb, 2, logM - 1 >= 3 ? 3 : 0);
  } else {
    // conj of the cross spectrum, in place in X (same index read and written)
    for (int idx = threadIdx.x; idx < M * CG; idx += blockDim.x) {
      C x = X[idx];
      if (autoc) X[idx] = mkc<C>(x.x * x.x + x.y * x.y, 0.0);
      else X[idx] = cconj(cmul(x, cconj(Y[idx])));
    }
    __syncthreads();
    auto fromX = [&](int f, int cc, C &xo, C &) { xo = X[f * CG + cc]; };
    if (logM >= 3) {
      fft_first_pass<CG, C>(Y, nullptr, M, logM, tw, 1, fromX);
    } else {
      for (int idx = threadIdx.x; idx < M * CG; idx += blockDim.x) {
        const int cc = idx % CG, f = idx / CG;
        Y[int(__brev(unsigned(f)) >> (32 - logM)) * CG + cc] = X[idx];
      }
      __syncthreads();
    }
    fft_dit<CG, C>(Y, nullptr, M, logM, tw, 1, logM >= 3 ? 3 : 0);
  }
  // transform of column cc at frequency p
  auto spec = [&](int p, int cc) -> C {
    if (!half) return Y[p * CG + cc];
    const int q = p & (Mh - 1);
    const C zp = Y[q * CG + cc], zm = cconj(Y[((Mh - q) & (Mh - 1)) * CG + cc]);
    const C ev = cscale(cadd(zp, zm), 0.5), d = csub(zp, zm);
    const C wo = cmul(twb[q], mkc<C>(0.5 * d.y, -0.5 * d.x));
    return p < Mh ? cadd(ev, wo) : csub(ev, wo);
  };
  const double invM = 1.0 / double(M);
  C *Gb = Bufs<C>::G(s);
  if (half && twist) {  // n == M: frequencies q and q + M/2 share E_q and w^q O_q
    for (int idx = threadIdx.x; idx < Mh * CG; idx += blockDim.x) {
      const int cc = idx % CG, q = idx / CG, c = c0 + cc;
      if (c >= s.C) continue;
      const C zp = Y[q * CG + cc], zm = cconj(Y[((Mh - q) & (Mh - 1)) * CG + cc]);
      const C ev = cscale(cadd(zp, zm), 0.5), d = csub(zp, zm);
      const C wo = cmul(twb[q], mkc<C>(0.5 * d.y, -0.5 * d.x));
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int p = q + hh * Mh;
        const C lp = cscale(cconj(hh ? csub(ev, wo) : cadd(ev, wo)), invM);
        const C g = cvt<C>(cmul(cmul(tp8[(p >> 3) * CG + cc], tp1[(p & 7) * CG + cc]), todbl(lp)));
        Gb[at(p * s.ne + e, c, s.Cpad)] = g;
      }
    }
    return;
  }
  for (int idx = threadIdx.x; idx < n * CG; idx += blockDim.x) {
    const int cc = idx % CG, p = idx / CG, c = c0 + cc;
    if (c >= s.C) continue;
    C lp = cscale(cconj(spec(p, cc)), invM);
    C g = lp;
    if (twist) {  // G_p = zeta^p C_p
      g = cvt<C>(cmul(cmul(tp8[(p >> 3) * CG + cc], tp1[(p & 7) * CG + cc]), todbl(lp)));
    } else if (p > 0) {
      C lm = cscale(cconj(spec(M + p - n, cc)), invM);
      g = cfma(zc[cc], lm, lp);
    }
    Gb[at(p * s.ne + e, c, s.Cpad)] = g;
  }
}

// Shared memory of k_fave_fft's twist tables (four per column, 8 or M/8 entries).
static size_t fave_twist_bytes(const DevSys &s, int cg) {
  return s.fave_twist ? sizeof(double2) * size_t(cg) * 2 * (8 + s.M / 8) : 0;
}

#include "bl_big.cuh"
#include "bl_huge.cuh"
#include "bl_tc.cuh"

constexpr int kFidJT = 4, kFidPT = 4;

// One thread per (crystallite, tile of kFidJT j's, tile of kFidPT p's); lanes are
// 32 consecutive crystallites, reduced with the powder weights by warp shuffles.
template <class C, int JT = kFidJT, int PT = kFidPT>
__global__ void __launch_bounds__(kThreads) k_fid(DevSys s) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  int npt = (s.gper + PT - 1) / PT, njt = (s.J + JT - 1) / JT;
  if (rest >= long(npt) * njt) return;  // warp-uniform: whole warp leaves together
  int pt = int(rest % npt), jt = int(rest / npt);
  int p0 = pt * PT, j0 = jt * JT;
  C acc[JT][PT];
#pragma unroll
  for (int a = 0; a < JT; ++a)
#pragma unroll
    for (int b = 0; b < PT; ++b) acc[a][b] = mkc<C>(0, 0);
  const C *Zb = Bufs<C>::Z(s), *Gb = Bufs<C>::G(s);
  // Partial sums over chunks of kFidChunk elements in C, folded into FP64 accumulators:
  // in single precision this keeps the summation error at ~sqrt(chunk) eps instead of
  // ~sqrt(ne) eps (ne reaches 10^4 for 8 spins); in FP64 it changes nothing.
  constexpr int kFidChunk = 32;
  double2 acc64[JT][PT];
#pragma unroll
  for (int a = 0; a < JT; ++a)
#pragma unroll
    for (int b = 0; b < PT; ++b) acc64[a][b] = cmk(0, 0);
  if (c < s.C) {
    for (int e0 = 0; e0 < s.ne; e0 += kFidChunk) {
      const int e1 = min(s.ne, e0 + kFidChunk);
      for (int e = e0; e < e1; ++e) {
        C zj[JT], gp[PT];
#pragma unroll
        for (int a = 0; a < JT; ++a)
          zj[a] = (j0 + a < s.J) ? Zb[at((j0 + a) * s.ne + e, c, s.Cpad)] : mkc<C>(0, 0);
#pragma unroll
        for (int b = 0; b < PT; ++b)
          gp[b] = (p0 + b < s.gper) ? Gb[at((p0 + b) * s.ne + e, c, s.Cpad)] : mkc<C>(0, 0);
#pragma unroll
        for (int a = 0; a < JT; ++a)
#pragma unroll
          for (int b = 0; b < PT; ++b) acc[a][b] = cfma(zj[a], gp[b], acc[a][b]);
      }
#pragma unroll
      for (int a = 0; a < JT; ++a)
#pragma unroll
        for (int b = 0; b < PT; ++b) {
          acc64[a][b] = cadd(acc64[a][b], todbl(acc[a][b]));
          acc[a][b] = mkc<C>(0, 0);
        }
    }
  }
  double wc = (c < s.C) ? s.w[c] * s.scale : 0.0;
  int lane = threadIdx.x & 31;
  int wglob = s.warp_base + c / 32;
#pragma unroll
  for (int a = 0; a < JT; ++a)
#pragma unroll
    for (int b = 0; b < PT; ++b) {
      double2 v = cscale(acc64[a][b], wc);  // powder weight and the warp sum in FP64
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
      }
      int k = (j0 + a) * s.gper + p0 + b;
      if (lane == 0 && p0 + b < s.gper && k < s.npts) s.partial[size_t(wglob) * s.npts + k] = v;
    }
}

// Point-to-point FID terms, one thread per (crystallite, element (r,s)).
// With W_i = A_{i+1} V (A_n = Omega = V diag(lam) V^H), Q_i = W_i^H D W_i and R_{n-1} =
// W_{n-1}^H rho W_{n-1} = diag(lam)^H (V^H rho V) diag(lam), the density matrix after
// m_tot chunks, G = A_{j'} Omega^{q'} with m_tot = q' b + j' (1 <= j' <= b), gives
//   Tr(D G rho G^H) = sum_rs Q_i(r,s) R_{n-1}(s,r) e^{i m (th_s - th_r)},
//   i = j' sub - 1, m = q' + 1   (m_tot = 0: i = n - 1, m = 0).
// Point p = j b + k has m_tot = p f: its i depends on k only and m grows by f per j, so
// G[k] = Q_{i_k}(r,s) R(s,r) e^{i m_k d} and Z[j] = e^{i j f d} (d = th_s - th_r) feed
// k_fid's fid[j b + k] = sum_e Z[j] G[k].  The chunk products are never formed: the
// reference's PropReduce (examples/qmsims/MMMQMAS/propreduce.cc:455-521) builds every
// dwell propagator from shared sub-products; here the Floquet powers replace them.
template <class C>
__global__ void __launch_bounds__(kThreads) k_p2p_elems(DevSys s) {
  long tid = long(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = int(tid % s.Cpad);
  long rest = tid / s.Cpad;
  if (rest >= s.ne) return;
  const int e = int(rest);
  if (c >= s.C) return;
  const C *Q = Bufs<C>::Q(s), *R = Bufs<C>::R(s);
  const int qlast = (s.n - 1) * s.nq;
  double2 rsr;  // R_{n-1}(s,r)
  if (s.rosym) {  // rho = (D + D^H)/2: R = (Q(s,r) + conj(Q(r,s)))/2
    double2 v = cconj(todbl(Q[at(qlast + s.eq[e], c, s.Cpad)]));
    if (s.erev[e] >= 0) v = cadd(v, todbl(Q[at(qlast + s.erev[e], c, s.Cpad)]));
    rsr = cscale(v, 0.5);
  } else {
    rsr = todbl(R[at((s.n - 1) * s.nr + s.er[e], c, s.Cpad)]);
  }
  const double d = s.L[at(s.esg[e], c, s.Cpad)].y - s.L[at(s.erg[e], c, s.Cpad)].y;
  for (int k = 0; k < s.pb; ++k) {
    const long mt = long(k) * s.pf;
    int i = s.n - 1;
    long m = 0;
    if (mt > 0) {
      const long jp = (mt - 1) % s.pb + 1, qp = (mt - jp) / s.pb;
      i = int(jp) * s.psub - 1;
      m = qp + 1;
    }
    double sn, cs;
    sincos(double(m) * d, &sn, &cs);
    const double2 g = cmul(cmul(todbl(Q[at(i * s.nq + s.eq[e], c, s.Cpad)]), rsr), cmk(cs, sn));
    Bufs<C>::G(s)[at(k * s.ne + e, c, s.Cpad)] = cvt<C>(g);
  }
  // Z[j] = e^{i j f d}: a running product, re-anchored by an exact sincos every 64 powers
  // (its rounding then stays near 64 eps; arguments reach ~10^4 rad)
  double2 z1;
  sincos(double(s.pf) * d, &z1.y, &z1.x);
  double2 zj = cmk(1, 0);
  for (int j = 0; j < s.J; ++j) {
    if ((j & 63) == 0 && j) sincos(double(j) * double(s.pf) * d, &zj.y, &zj.x);
    Bufs<C>::Z(s)[at(j * s.ne + e, c, s.Cpad)] = cvt<C>(zj);
    zj = cmul(zj, z1);
  }
}

// Compensated (Kahan) sum of the warp partials in fixed order: deterministic.
// Mixed form: the FID terms as a tiled product.  fid[j gper + p] = sum_c w_c sum_e
// z_e^j(c) G_p(e, c) is a product with K = (crystallite, element); one CTA takes a group of
// 32 crystallites (one warp of the batch layout), a range of the elements (ft_r ranges, a
// function of the element count only) and a (j, p) tile of ft_jt x ft_pt threads, each
// thread a 4 x 4 register tile (the tile shape follows J and gper, so little is padded).
// Per element it stages z_e^j and G_p(e) of its 32 crystallites in shared memory by
// asynchronous copies (coalesced: crystallites are fastest in HBM; double-buffered, so the
// next element's copies are in flight while this one is summed), and each thread updates its
// tile with w_c scale z, accumulating one element in FP32 and folding it into double-float
// (hi + lo) sums.  The CTA writes its tile to partial row (warp * ft_r + range); k_reduce
// sums the rows of the populated warps in a fixed order.  Each output's summation order
// (crystallites 0..31 per element, elements in order within a range) depends on neither
// the tile shape nor the batch, so a crystallite's contribution does not depend on its
// neighbours.
constexpr int kFtThreads = 64, kFtR = 16, kFtJmax = 32;
// 8-byte asynchronous copy global -> shared (cp.async); src_bytes 0 writes zeros
__device__ __forceinline__ void cp_async8(void *dst, const void *src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(uint32_t(__cvta_generic_to_shared(dst))), "l"(src),
               "r"(src_bytes)
               : "memory");
}
// Dynamic shared memory of k_fid_tiled: two buffers of 32 crystallites x (4 jt + 4 pt).
static size_t fid_tiled_smem(int jt, int pt) { return sizeof(float2) * 2 * 32 * 4 * size_t(jt + pt); }
__global__ void __launch_bounds__(kFtThreads) k_fid_tiled(DevSys s) {
  extern __shared__ __align__(16) float2 ftsm[];
  const int JT = 4 * s.ft_jt, PT = 4 * s.ft_pt;
  float2 *zs = ftsm, *gs = ftsm + 2 * 32 * JT;  // [buffer][c][j], [buffer][c][p]
  __shared__ float ws[32];
  const int tid = threadIdx.x;
  const int g = blockIdx.x;  // group of 32 crystallites in this batch
  const int npr = (s.gper + PT - 1) / PT;
  const int pr = blockIdx.y % npr, jr = blockIdx.y / npr, er = blockIdx.z;
  const int p0 = pr * PT, j0 = jr * JT;
  const int e_lo = int((long(s.ne) * er) / s.ft_r), e_hi = int((long(s.ne) * (er + 1)) / s.ft_r);
  const int c0 = g * 32;
  if (tid < 32) {
    const int c = c0 + tid;
    ws[tid] = c < s.C ? float(s.w[c] * s.scale) : 0.f;
  }
  const bool active = tid < s.ft_jt * s.ft_pt;
  const int jt = active ? tid / s.ft_pt : 0, pt = active ? tid % s.ft_pt : 0;  // j0 + 4 jt + a, p0 + 4 pt + b
  float2 acc[4][4];
  float2 hi[4][4], lo[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) hi[a][b] = lo[a][b] = make_float2(0.f, 0.f);
  const float2 *Zb = s.Zf, *Gb = s.Gf;
  // z (JT x 32) and G (PT x 32) of element e into buffer buf, zeros outside J, gper and C
  auto stage = [&](int e, int buf) {
    for (int t = tid; t < JT * 32; t += kFtThreads) {
      const int jj = t / 32, c = t % 32, j = j0 + jj;
      const bool ok = j < s.J && c0 + c < s.C;
      cp_async8(&zs[(buf * 32 + c) * JT + jj], ok ? &Zb[at(j * s.ne + e, c0 + c, s.Cpad)] : Zb, ok ? 8 : 0);
    }
    for (int t = tid; t < PT * 32; t += kFtThreads) {
      const int pp = t / 32, c = t % 32, p = p0 + pp;
      const bool ok = p < s.gper && c0 + c < s.C;
      cp_async8(&gs[(buf * 32 + c) * PT + pp], ok ? &Gb[at(p * s.ne + e, c0 + c, s.Cpad)] : Gb, ok ? 8 : 0);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  if (e_lo < e_hi) stage(e_lo, 0);
  int buf = 0;
  for (int e = e_lo; e < e_hi; ++e) {
    if (e + 1 < e_hi) {
      stage(e + 1, buf ^ 1);  // in flight while this element is summed
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.f, 0.f);
      const float2 *zrow = zs + buf * 32 * JT + 4 * jt, *grow = gs + buf * 32 * PT + 4 * pt;
#pragma unroll 2
      for (int c = 0; c < 32; ++c) {
        const float w = ws[c];
        const float4 z01 = *reinterpret_cast<const float4 *>(zrow + c * JT);
        const float4 z23 = *reinterpret_cast<const float4 *>(zrow + c * JT + 2);
        const float4 g01 = *reinterpret_cast<const float4 *>(grow + c * PT);
        const float4 g23 = *reinterpret_cast<const float4 *>(grow + c * PT + 2);
        const float2 zz[4] = {make_float2(w * z01.x, w * z01.y), make_float2(w * z01.z, w * z01.w),
                              make_float2(w * z23.x, w * z23.y), make_float2(w * z23.z, w * z23.w)};
        const float2 gg[4] = {make_float2(g01.x, g01.y), make_float2(g01.z, g01.w), make_float2(g23.x, g23.y),
                              make_float2(g23.z, g23.w)};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = cfma(zz[a], gg[b], acc[a][b]);
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const float2 x = dfv_add(make_float2(hi[a][b].x, lo[a][b].x), make_float2(acc[a][b].x, 0.f));
          const float2 y = dfv_add(make_float2(hi[a][b].y, lo[a][b].y), make_float2(acc[a][b].y, 0.f));
          hi[a][b] = make_float2(x.x, y.x), lo[a][b] = make_float2(x.y, y.y);
        }
    }
    __syncthreads();  // the next stage() overwrites this buffer
    buf ^= 1;
  }
  if (!active) return;
  const long row = long(s.warp_base + g) * s.ft_r + er;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + 4 * jt + a, p = p0 + 4 * pt + b;
      const long k = long(j) * s.gper + p;
      if (j < s.J && p < s.gper && k < s.npts)
        s.partial[row * s.npts + k] = make_double2(double(hi[a][b].x) + double(lo[a][b].x),
                                                   double(hi[a][b].y) + double(lo[a][b].y));
    }
}

__global__ void k_reduce(const double2 *__restrict__ partial, int nw, int npts, double2 *__restrict__ fid) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npts) return;
  double sx = 0, sy = 0, cx = 0, cy = 0;
  for (int w = 0; w < nw; ++w) {
    double2 v = partial[size_t(w) * npts + k];
    double yx = v.x - cx, tx = sx + yx;
    cx = (tx - sx) - yx, sx = tx;
    double yy = v.y - cy, ty = sy + yy;
    cy = (ty - sy) - yy, sy = ty;
  }
  fid[k] = make_double2(sx, sy);
}

inline unsigned grid_for(long threads) { return unsigned((threads + kThreads - 1) / kThreads); }

}  // namespace

// ------------------------------------------------------------------ host side
Context::~Context() {
  if (stream) cudaStreamDestroy(stream);
}

static thread_local size_t *g_upload_counter = nullptr;  // set while a Job uploads its inputs

// Bump allocator over a caller-provided device region.  The allocation-free entry point
// (powder_fid_noalloc) and job_in_region install one while they build a Job.
struct ScratchArena {
  char *base = nullptr;
  size_t cap = 0, used = 0;
  const char *label = "static device scratch of the allocation-free entry point";
  bool aux_streams = false;  // the Job may create its own streams (not on the allocation-free path)
};
static thread_local ScratchArena *g_arena = nullptr;
// Set by job_bytes: the Job constructor records its memory plan here and returns before
// touching the device.
struct JobSizing {
  size_t per_c = 0;
  long cpad = 0;
  size_t extra = 0;   // bytes independent of the batch size (huge-block workspace)
  size_t tables = 0;  // the system's operator tables on the device (and their double-float copies)
};
static thread_local JobSizing *g_sizing = nullptr;

template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  bool owned = true;  // false: carved from a ScratchArena, never freed here
  void alloc(size_t count) {
    n = count;
    if (!count) return;
    if (g_arena) {
      size_t off = (g_arena->used + 255) & ~size_t(255);
      size_t bytes = count * sizeof(T);
      if (off + bytes > g_arena->cap)
        throw Error(4, "job needs more than the " + std::to_string(g_arena->cap >> 20) + " MiB " + g_arena->label);
      p = reinterpret_cast<T *>(g_arena->base + off);
      g_arena->used = off + bytes;
      owned = false;
      return;
    }
    CUDA_OK(cudaMalloc(&p, count * sizeof(T)));
  }
  DevBuf() {}
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n), owned(o.owned) { o.p = nullptr, o.n = 0; }
  void upload(const std::vector<T> &v, cudaStream_t st) {
    alloc(v.size());
    if (!v.empty()) CUDA_OK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    if (g_upload_counter) *g_upload_counter += v.size() * sizeof(T);
  }
  ~DevBuf() {
    if (p && owned) cudaFree(p);
  }
};

struct JobImpl {
  Context *ctx;
  FidParams P;
  int C = 0, n = 0, gammaloop = 1, J = 0, rosym = 0, is_static = 0;
  double tau = 0, sw_out = 0, dt = 0;
  BlockLayout L;
  int nint = 0, nq = 0, nr = 0, ne = 0, npq = 0, npr = 0;
  int Cb = 0, nbatch = 0, nwarps_total = 0;
  int ft_jt = 1, ft_pt = 1, ft_r = 1;  // k_fid_tiled tile shape and element ranges
  std::vector<std::vector<int>> blocks_by_size;  // size -> list of block indices (size <= kMaxBlock)
  std::vector<int> big_blocks;                   // blocks kMaxBlock < b <= kMaxBigBlock
  std::vector<BigPair> big_pairs;                // Q/R pairs whose largest block is one of those
  std::vector<int> huge_blocks;                  // blocks larger than kMaxBigBlock
  std::vector<int> huge_sq;                      // per huge block: squarings that bound every step's
  std::vector<BigPair> huge_pairs;               // Q/R pairs with a huge block
  size_t huge_ws_bytes = 0;                      // workspace of the huge-block products
  int huge_items = 0;                            // largest chunk of exponential items
  DevBuf<double2> huge_ws;
  DevBuf<double> hfk, hsc;
  DevBuf<int> hsq, hsqmax;
  std::vector<size_t> big_rp_off, huge_rp_off;   // each pair's row pointers in big_rp
  DevBuf<int> big_rp, big_ci;                    // non-zeros of M_ab by row, all big pairs
  DevBuf<double2> big_cv;
  DevBuf<int> bs, boff, bpoff, qa, qb, qoff, doff, ra, rb, roff, rhooff, eq, erev, er, erg, esg, status, srp, seo;
  std::vector<DevBuf<int>> blist;
  DevBuf<double> pas, iscale, Tk, Hc, Rp_all, t0_all, w_all;
  DevBuf<int> ikind;
  int has2 = 0;  // second-order quadrupolar terms present
  int p2p = 0, pb = 1, pf = 1, psub = 1;  // point-to-point FID: base, factor, steps per chunk
  DevBuf<double> fkc;                      // k_coef's term coefficients (small blocks)
  DevBuf<double2> frames;                  // rf schedule: per chunk frame (permuted index)
  DevBuf<float2> Tk_df, Hc_df;             // mixed form: double-float operators and constant parts
  DevBuf<int> tk_ptr, tk_term, tk_order;  // tensor-core step: the operators' non-zeros by element
  DevBuf<float2> tk_val;
  DevBuf<double2> Dblk, Rhoblk;
  DevBuf<double2> U, A, VF, Lb, Q, R, G, Z, partial, fid, tw;
  DevBuf<float2> Wf, Qf, Rf, Gf, Zf, twf;  // mixed-precision form
  // mixed form on the tensor cores (large blocks): the step writes each (crystallite, step)'s
  // U slices to a slab the Dyson product reads; one region per large block
  bool tc = false;
  DevBuf<unsigned char> usl;
  DevBuf<unsigned long long> tcf;  // the two tensor-flop counters
  std::vector<size_t> usl_off;  // per block index: byte offset of its region (large blocks)
  int mixed = 0;
  DevBuf<double> Rp_b, t0_b, w_b;
  std::vector<double> h_Rp, h_t0, h_w;  // all virtual crystallites (C * gammaloop)
  int Ceff = 0;
  double flops = 0;
  int launches = 0;
  size_t h2d = 0;
  bool profiling = false;
  double stage_ms[Job::kStages] = {0};
  int stage_launch[Job::kStages] = {0};
  double stage_fl[Job::kStages] = {0};
  std::vector<cudaEvent_t> evpool;  // stage-boundary events (created when profiling)
  struct Mark {
    int stage, b, e, nlaunch;
  };
  std::vector<Mark> marks;
  int evnext = 0;
  // streams on which the large blocks of one stage run side by side (fork/join on the
  // context stream), so that their one-CTA-per-crystallite launches fill the SMs together
  std::vector<cudaStream_t> aux;
  cudaEvent_t fork_ev = nullptr;
  std::vector<cudaEvent_t> join_ev;
  ~JobImpl() {
    for (auto &e : evpool) cudaEventDestroy(e);
    for (auto &e : join_ev) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (auto &a : aux) cudaStreamDestroy(a);
  }
  double cos_rotb = 1, sin_rotb = 0;
  DevSys base{};
};

static bool any_nonzero(const CMatrix &M, const BlockLayout &L, int a, int b) {
  for (int r = 0; r < L.size[a]; ++r)
    for (int s = 0; s < L.size[b]; ++s)
      if (M(L.perm[L.off[a] + r], L.perm[L.off[b] + s]) != cplx(0, 0)) return true;
  return false;
}

Job::Job(Context &ctx, const SpinSystem &sys, const Powder &pw, const CMatrix &ro_in, const CMatrix &det_in,
         const FidParams &p)
    : d_(new JobImpl) {
  JobImpl &J = *d_;
  J.ctx = &ctx;
  J.P = p;
  if (!g_sizing) CUDA_OK(cudaSetDevice(ctx.device));
  if (p.precision != 0 && p.precision != 1) throw Error(1, "precision must be 0 (FP64) or 1 (mixed)");
  if (p.step_method != 0 && p.step_method != 1) throw Error(1, "step_method must be 0 (eigh) or 1 (Taylor)");
  if (p.fave_method < 0 || p.fave_method > 2) throw Error(1, "fave_method must be 0 (auto), 1 (direct) or 2 (FFT)");
  if (p.npts <= 0) throw Error(1, "npts must be positive");
  if (pw.size() <= 0) throw Error(1, "empty powder");
  const int N = sys.dim();
  if (ro_in.n != N || det_in.n != N) throw Error(1, "rho/detect dimension does not match the spin system");
  // oneFID::FID dispatch (oneFID.h:206): no spinning or rotor angle 0 -> static powder FID
  J.is_static = (p.wr == 0.0 || p.rotb_deg == 0.0) ? 1 : 0;
  double tmin = p.start_t;
  J.p2p = p.p2p_base > 0 ? 1 : 0;
  if (J.p2p) {
    if (p.p2p_factor <= 0) throw Error(1, "the point-to-point factor must be positive");
    // PropReduce::setParams (examples/qmsims/MMMQMAS/propreduce.cc:16-33): base and factor
    // divided by their greatest common divisor
    int u = p.p2p_base, v = p.p2p_factor;
    while (v) {
      const int t = u % v;
      u = v, v = t;
    }
    J.pb = p.p2p_base / u, J.pf = p.p2p_factor / u;
    if (!p.rf_chunks.empty()) {  // the schedule is given on the caller's chunks
      if (J.is_static) throw Error(1, "an rf schedule within the rotor period needs spinning (wr > 0, rotor angle != 0)");
      J.pb = p.p2p_base, J.pf = p.p2p_factor;
      for (const auto &rc : p.rf_chunks)
        if (rc.chunk < 0 || rc.chunk >= J.pb) throw Error(1, "rf schedule: chunk outside 0 .. base-1");
    }
    J.gammaloop = 1;
    if (J.is_static) {  // time-independent H: one step of 1/sw per point
      if (!(p.sw > 0)) throw Error(1, "sw must be positive");
      J.pb = J.pf = J.psub = J.n = 1;
      J.tau = 1.0 / p.sw;
      J.sw_out = p.sw;
    } else {
      // chunk of 1/(wr base); steps of at most maxtstep in it, as Propogation::propogator
      // splits a pulse (examples/solid-2.0/src/propogation.cc:246-253)
      const double chunk = 1.0 / (p.wr * J.pb);
      double sub = p.maxtstep > 0 ? std::ceil(chunk / p.maxtstep) : 1.0;
      if (!(sub >= 1.0)) sub = 1.0;
      if (double(J.pb) * sub > double(kMaxP2PSteps))
        throw Error(5, "point-to-point FID needs more than " + std::to_string(kMaxP2PSteps) +
                           " steps per rotor period (base x ceil(chunk/maxtstep))");
      J.psub = int(sub);
      J.n = J.pb * J.psub;
      J.tau = chunk / J.psub;
      J.sw_out = p.wr * J.pb / J.pf;
    }
    J.is_static = 0;  // spinning machinery: steps, Dyson, Floquet, Q/R, then the p2p terms
  } else if (!p.rf_chunks.empty()) {
    throw Error(1, "an rf schedule within the rotor period needs the point-to-point form");
  } else if (J.is_static) {
    // oneFID::singleStaticFID (oneFID.h:292-336): dt = 1/sw as given; the FID index k is
    // split as k = j*ns + p for the reconstruction kernel
    if (!(p.sw > 0)) throw Error(1, "sw must be positive");
    J.n = std::min(64, p.npts);
    J.gammaloop = 1;
    J.sw_out = p.sw;
    J.tau = 0.0;
    J.dt = 1.0 / p.sw;
  } else {
    // compute::CalcComputeStep and the constructor (compute.h:86-97, 213-235)
    J.n = int(std::floor(p.sw / p.wr + 0.5));
    if (J.n < 1) throw Error(1, "sw/wr gives fewer than one step per rotor period");
    int gamma_step = 10;
    J.gammaloop = gamma_step >= J.n ? gamma_step / J.n : 1;
    if (J.gammaloop < 1) J.gammaloop = 1;
    J.sw_out = double(J.n * p.wr);
    double tmax = p.start_t + 1.0 / p.wr;
    J.tau = (tmax - tmin) / J.n;
    if (!(J.tau > 0)) throw Error(1, "the propagator time step is not positive");
  }
  // rf schedule: one system per chunk (the system's own rf plus the chunk's fields) for its
  // constant H and rf frame; the block layout of a system with every scheduled isotope
  // irradiated holds all of them
  const bool sched = !p.rf_chunks.empty();
  std::vector<SpinSystem> chunk_sys;
  if (sched) {
    SpinSystem su = sys;
    std::vector<std::string> isos;
    for (const auto &rc : p.rf_chunks)
      if (rc.field.amp != 0.0 && std::find(isos.begin(), isos.end(), rc.field.iso) == isos.end())
        isos.push_back(rc.field.iso);
    for (const auto &iso : isos) su.add_rf(RfField{iso, 1.2345, 0.0, 0.0});
    J.L = su.layout();
    for (int kc = 0; kc < J.pb; ++kc) {
      chunk_sys.push_back(sys);
      for (const auto &rc : p.rf_chunks)
        if (rc.chunk == kc) chunk_sys.back().add_rf(rc.field);
    }
  } else {
    J.L = sys.layout();
  }
  const BlockLayout &L = J.L;
  if (L.max_block > kMaxHugeBlock)
    throw Error(5, "Hamiltonian block of size " + std::to_string(L.max_block) + " exceeds this engine's limit of " +
                       std::to_string(kMaxHugeBlock));
  if (J.is_static && L.max_block > kMaxBlock)
    throw Error(5, "static powder FIDs support Hamiltonian blocks up to " + std::to_string(kMaxBlock));
  const int nb = int(L.size.size());
  // rosym: exact test ro == 0.5*(det + det^H) on the caller's matrices   (compute.h:75-83)
  J.rosym = 1;
  for (int r = 0; r < N && J.rosym; ++r)
    for (int s = 0; s < N; ++s)
      if (ro_in(r, s) != 0.5 * (det_in(r, s) + std::conj(det_in(s, r)))) {
        J.rosym = 0;
        break;
      }
  // rf phases: the engine propagates the real H' = R^H H R, so rho and det enter as R^H X R
  // (under an rf schedule each step's U is turned back into the lab frame instead)
  const CMatrix ro = sched ? ro_in : sys.to_frame(ro_in), det = sched ? det_in : sys.to_frame(det_in);
  if (J.is_static) J.rosym = 0;  // the static FID always transforms rho itself
  // Hamiltonian terms, packed per block
  const int nhc = sched ? J.pb : 1;
  std::vector<double> pas, isc, Tk, Hc(size_t(L.S2) * nhc, 0.0);
  auto pack = [&](const std::vector<double> &M, double *dst) {
    for (int k = 0; k < nb; ++k)
      for (int r = 0; r < L.size[k]; ++r)
        for (int q = 0; q < L.size[k]; ++q)
          dst[L.poff[k] + r * L.size[k] + q] = M[size_t(L.perm[L.off[k] + r]) * N + L.perm[L.off[k] + q]];
  };
  if (!g_sizing) {  // planning needs only the counts
    if (sched)
      for (int kc = 0; kc < J.pb; ++kc) pack(chunk_sys[kc].h_const(), Hc.data() + size_t(kc) * L.S2);
    else
      pack(sys.h_const(), Hc.data());
  }
  // orientation-dependent terms: kind 0 = scale (M PAS' M^T)_22 T; a quadrupole in a field
  // adds kind 1 = s2 ((r00-r11)^2/4 + r01^2) c4 and kind 2 = -s2 (r02^2 + r12^2) c2 with
  // s2 = Qp^2/(B nu_rel), r = M PAS' M^T (qua.cc:219-267: order 1 or |B| <= 1e-12 first order
  // only, order 2 second order only, otherwise both)
  const auto &ints = sys.interactions();
  const double Bf = sys.bfield();
  std::vector<int> ikind;
  auto add_term = [&](const Interaction &I, int kind, double scale, const std::vector<double> &op) {
    pas.insert(pas.end(), {I.pas[0][0], I.pas[0][1], I.pas[0][2], I.pas[1][1], I.pas[1][2], I.pas[2][2]});
    isc.push_back(scale);
    ikind.push_back(kind);
    if (!g_sizing) {
      size_t o = Tk.size();
      Tk.resize(o + L.S2);
      pack(op, Tk.data() + o);
    }
    ++J.nint;
  };
  for (size_t kk = 0; kk < ints.size(); ++kk) {
    const auto &I = ints[kk];
    if (I.kind == 'J') continue;
    const bool quad = I.kind == 'Q';
    const bool first_only = !quad || I.order == 1 || std::fabs(Bf) <= 1e-12;
    const bool second_only = !first_only && I.order == 2;
    if (!second_only) add_term(I, 0, I.op_scale, sys.h_ops()[kk]);
    if (!first_only) {
      const double s2 = I.op_scale * I.op_scale / (Bf * isotope_rel_freq(sys.isotopes()[I.s1]));
      add_term(I, 1, s2, sys.h_ops_q4()[kk]);
      add_term(I, 2, -s2, sys.h_ops_q2()[kk]);
    }
  }
  J.has2 = std::any_of(ikind.begin(), ikind.end(), [](int k) { return k != 0; }) ? 1 : 0;
  // Q pairs (blocks of D) and R pairs (blocks of rho when rho != (D + D^H)/2)
  std::vector<int> qa, qb, qoff, doff, ra, rb, roff, rhooff;
  std::vector<double2> Dblk, Rhoblk;
  std::vector<std::vector<int>> qpair(nb, std::vector<int>(nb, -1)), rpair(nb, std::vector<int>(nb, -1));
  for (int a = 0; a < nb; ++a)
    for (int b = 0; b < nb; ++b) {
      if (any_nonzero(det, L, a, b)) {
        qpair[a][b] = int(qa.size());
        qa.push_back(a), qb.push_back(b), qoff.push_back(J.nq), doff.push_back(int(Dblk.size()));
        for (int r = 0; r < L.size[a]; ++r)
          for (int s = 0; s < L.size[b]; ++s) {
            cplx v = det(L.perm[L.off[a] + r], L.perm[L.off[b] + s]);
            Dblk.push_back(make_double2(v.real(), v.imag()));
          }
        J.nq += L.size[a] * L.size[b];
      }
      if (!J.rosym && any_nonzero(ro, L, a, b)) {
        rpair[a][b] = int(ra.size());
        ra.push_back(a), rb.push_back(b), roff.push_back(J.nr), rhooff.push_back(int(Rhoblk.size()));
        for (int r = 0; r < L.size[a]; ++r)
          for (int s = 0; s < L.size[b]; ++s) {
            cplx v = ro(L.perm[L.off[a] + r], L.perm[L.off[b] + s]);
            Rhoblk.push_back(make_double2(v.real(), v.imag()));
          }
        J.nr += L.size[a] * L.size[b];
      }
    }
  J.npq = int(qa.size());
  J.npr = int(ra.size());
  // elements (r,s): Q(r,s) structurally non-zero and R(s,r) structurally non-zero
  std::vector<int> eq, erev, er, erg, esg, srp(J.npq, -1), seo(J.npq, -1);
  for (int pq = 0; pq < J.npq; ++pq) {
    int a = qa[pq], b = qb[pq];
    if (!J.rosym && rpair[b][a] >= 0) srp[pq] = rpair[b][a], seo[pq] = int(eq.size());
    for (int r = 0; r < L.size[a]; ++r)
      for (int s = 0; s < L.size[b]; ++s) {
        int rv = -1, ri = -1;
        if (J.rosym) {
          if (qpair[b][a] >= 0) rv = qoff[qpair[b][a]] + s * L.size[a] + r;
        } else {
          if (rpair[b][a] < 0) continue;
          ri = roff[rpair[b][a]] + s * L.size[a] + r;
        }
        eq.push_back(qoff[pq] + r * L.size[b] + s);
        erev.push_back(rv);
        er.push_back(ri);
        erg.push_back(L.off[a] + r);
        esg.push_back(L.off[b] + s);
      }
  }
  J.ne = int(eq.size());
  J.J = (p.npts + (J.p2p ? J.pb : J.n) - 1) / (J.p2p ? J.pb : J.n);
  {  // k_fid_tiled: up to kFtJmax j's per tile, then as few p tiles as fit 64 threads, each
     // as narrow as it can be; element ranges of at least 64 elements (a function of ne only)
    const int gp = J.p2p ? J.pb : J.n;
    J.ft_jt = std::max(1, std::min(kFtJmax / 4, (J.J + 3) / 4));
    const int pt_max = std::max(1, kFtThreads / J.ft_jt);
    const int ntile = (gp + 4 * pt_max - 1) / (4 * pt_max);
    J.ft_pt = std::max(1, (gp + 4 * ntile - 1) / (4 * ntile));
    J.ft_r = std::max(1, std::min(kFtR, J.ne / 64));
  }
  // crystallites, expanded by the gamma loop (compute.h:294-306: fid summed over q)
  J.C = pw.size();
  J.Ceff = J.C * J.gammaloop;
  const double d2r = kPi / 180.0;
  for (int c = 0; c < J.C; ++c) {
    double R[3][3];
    rotation3(pw.phi[c], pw.theta[c], pw.gamma[c], R);  // setPowderAngles(phi, theta, gamma)
    for (int q = 0; q < J.gammaloop; ++q) {
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) J.h_Rp.push_back(R[a][b]);
      J.h_t0.push_back(q == 0 ? tmin : tmin + kPi2 * double(q) / double(J.gammaloop * J.n) / p.wr);
      J.h_w.push_back(pw.weight[c]);
    }
  }
  J.cos_rotb = std::cos(p.rotb_deg * d2r);
  J.sin_rotb = std::sin(p.rotb_deg * d2r);
  // batch size from the memory budget
  const size_t nsteps = J.is_static ? 0 : size_t(J.n);  // U, A, Q, R exist only when spinning
  // mixed form (spinning only): eigenframe W, Q/R, Fave G and z powers Z in single precision
  J.mixed = (p.precision == 1 && !J.is_static) ? 1 : 0;
  const size_t wide = nsteps * (J.nq + J.nr) + size_t(J.n) * J.ne + size_t(J.J) * J.ne;
  size_t per_c = J.mixed ? sizeof(double2) * (nsteps * L.S2 * 2 + L.S2 + N) + sizeof(float2) * (nsteps * L.S2 + wide)
                         : sizeof(double2) * (nsteps * L.S2 * 2 + L.S2 + N + wide);
  per_c += sizeof(double) * 11;
  // term coefficients per (step, term), computed once for all small blocks (k_coef)
  const bool use_fk = !J.is_static && J.nint > 0;
  if (use_fk) per_c += sizeof(double) * size_t(J.n) * size_t(J.nint);
  // tensor-core step and Dyson of the mixed form's large blocks (double-float coefficients
  // from k_coef, no rf schedule): the U slab of every (step, large block)
  J.tc = J.mixed && use_fk && p.step_method == 1 && !sched;
  size_t usl_per_c = 0;
  if (J.tc) {
    J.usl_off.assign(nb, 0);
    for (int k = 0; k < nb; ++k)
      if (L.size[k] >= tc::kMinB && L.size[k] <= tc::kMaxB) usl_per_c += nsteps * tc::slab_bytes(L.size[k]);
    per_c += usl_per_c;
  }
  long cpad_all = ((long(J.Ceff) + 31) / 32) * 32;
  // huge blocks: one workspace for their batched products, at least one item of each use
  // (exponential: 7 real b x b; Floquet: 2 complex b x b, 3 in the mixed form; eigenframe, Q/R: one complex
  // matrix), else 1 GiB
  size_t huge_fixed = 0;
  {
    size_t need = 0;
    int bmin = 0;
    for (int k = 0; k < nb; ++k) {
      const size_t b = size_t(L.size[k]);
      if (L.size[k] <= kMaxBigBlock) continue;
      need = std::max(need, std::max(sizeof(double) * kHugeSlots * b * b,
                                     (p.precision == 1 ? 3 : 2) * sizeof(double2) * b * b));
      bmin = bmin ? std::min(bmin, L.size[k]) : L.size[k];
    }
    for (int pr = 0; pr < J.npq + J.npr; ++pr) {
      const bool isq = pr < J.npq;
      const int ba = L.size[isq ? qa[pr] : ra[pr - J.npq]], bb = L.size[isq ? qb[pr] : rb[pr - J.npq]];
      if (std::max(ba, bb) > kMaxBigBlock) need = std::max(need, sizeof(double2) * size_t(ba) * bb);
    }
    if (need && !J.is_static) {
      J.huge_ws_bytes = (std::max(need, size_t(1) << 30) + 255) / 256 * 256;
      J.huge_items = int(std::min<size_t>(kHugeMaxItems, J.huge_ws_bytes / (sizeof(double) * kHugeSlots *
                                                                            size_t(bmin) * size_t(bmin))));
      huge_fixed = J.huge_ws_bytes + size_t(J.huge_items) * (sizeof(double) * (J.nint + 1) + sizeof(int)) + 4096;
    }
  }
  if (g_sizing) {
    g_sizing->per_c = per_c;
    g_sizing->cpad = cpad_all;
    g_sizing->extra = huge_fixed;
    // Tk and Hc (per chunk), their double-float copies in the mixed form, the D and rho
    // blocks, the rf frames, and 256-byte alignment per buffer
    const size_t tk = size_t(J.nint) * L.S2, hc = size_t(L.S2) * (sched ? J.pb : 1);
    g_sizing->tables = (tk + hc) * sizeof(double) * ((p.precision == 1 && !J.is_static) ? 2 : 1) +
                       (Dblk.size() + Rhoblk.size()) * sizeof(double2) + size_t(N) * J.pb * sizeof(double2) +
                       64 * 256;
    return;
  }
  size_t budget = ctx.hbm_budget;
  if (!budget) {  // default: 60% of the device memory free when the job is created
    size_t fr = 0, tot = 0;
    CUDA_OK(cudaMemGetInfo(&fr, &tot));
    budget = size_t(0.6 * double(fr));
  }
  budget = budget > huge_fixed ? budget - huge_fixed : 0;
  long cb = long(budget / std::max<size_t>(per_c, 1));
  cb = (cb / 32) * 32;
  if (cb < 32) throw Error(4, "job does not fit the device memory budget (one warp of crystallites)");
  // as few batches as the budget allows, of equal size (no small remainder batch)
  const long nb_min = (cpad_all + cb - 1) / cb;
  J.Cb = int(((long(J.Ceff) + nb_min - 1) / nb_min + 31) / 32 * 32);
  J.nbatch = int((cpad_all + J.Cb - 1) / J.Cb);
  J.nwarps_total = J.nbatch * (J.Cb / 32);
  // block lists by size
  J.blocks_by_size.assign(kMaxBlock + 1, {});
  for (int k = 0; k < nb; ++k) {
    if (L.size[k] <= kMaxBlock) J.blocks_by_size[L.size[k]].push_back(k);
    else if (L.size[k] <= kMaxBigBlock) J.big_blocks.push_back(k);
    else J.huge_blocks.push_back(k);
  }
  // per huge block: squarings enough for every step, from a rotation-free bound on
  // ||2 pi tau H||_inf (|a_k| <= ||PAS'_k||_F); the kernels skip items that need fewer
  for (int k : J.huge_blocks) {
    const int b = L.size[k], bp = L.poff[k];
    double nrm = 0;
    for (int r = 0; r < b; ++r) {
      double rs = 0;
      for (int q = 0; q < b; ++q) {
        double v = 0;  // the largest constant part over the chunks of an rf schedule
        for (int kc = 0; kc < nhc; ++kc) v = std::max(v, std::fabs(Hc[size_t(kc) * L.S2 + bp + r * b + q]));
        for (int kk = 0; kk < J.nint; ++kk) {
          const double *Pa = pas.data() + 6 * kk;
          const double fro = std::sqrt(Pa[0] * Pa[0] + Pa[3] * Pa[3] + Pa[5] * Pa[5] +
                                       2 * (Pa[1] * Pa[1] + Pa[2] * Pa[2] + Pa[4] * Pa[4]));
          // |r_ij| <= ||PAS'||_F: first order |a| <= fro, second order |a| <= 2 fro^2
          const double amax = ikind[kk] == 0 ? fro : 2.0 * fro * fro;
          v += std::fabs(isc[kk]) * amax * std::fabs(Tk[size_t(kk) * L.S2 + bp + r * b + q]);
        }
        rs += v;
      }
      nrm = std::max(nrm, rs);
    }
    nrm *= J.tau * kPi2 * (1.0 + 1e-12);  // margin over the device's rounding of the same sum
    int q = 0;
    if (nrm > 0.5) {
      std::frexp(nrm / 0.5, &q);
      q = std::min(q, 60);
    }
    J.huge_sq.push_back(q);
  }
  std::vector<int> big_rp_h, big_ci_h;
  std::vector<double2> big_cv_h;
  if (!J.big_blocks.empty() || !J.huge_blocks.empty()) {
    if (!J.big_blocks.empty() && J.nint > kMaxInt)
      throw Error(5, "more than " + std::to_string(kMaxInt) + " anisotropic interactions");
    const size_t csz = J.mixed ? sizeof(float2) : sizeof(double2);
    size_t smem_step = 0, smem_mat = 0, smem_qr[2] = {0, 0};
    for (int k : J.big_blocks) {
      smem_step = std::max(smem_step, big_step_smem(L.size[k]));
      smem_mat = std::max(smem_mat, sizeof(double2) * 2 * size_t(L.size[k]) * L.size[k]);
    }
    // Q/R pairs with a big block: M_ab's non-zeros by row, and the W_b column chunk that
    // keeps W_a, W_b and X within half the shared memory (two CTAs per SM) where it can
    for (int pr = 0; pr < J.npq + J.npr; ++pr) {
      const bool isq = pr < J.npq;
      const int a = isq ? qa[pr] : ra[pr - J.npq], b = isq ? qb[pr] : rb[pr - J.npq];
      const int ba = L.size[a], bb = L.size[b];
      if (ba <= kMaxBlock && bb <= kMaxBlock) continue;
      const double2 *M = isq ? Dblk.data() + doff[pr] : Rhoblk.data() + rhooff[pr - J.npq];
      const size_t rp_off = big_rp_h.size();
      for (int l = 0; l < ba; ++l) {
        big_rp_h.push_back(int(big_ci_h.size()));
        for (int m = 0; m < bb; ++m) {
          const double2 v = M[l * bb + m];
          if (v.x != 0.0 || v.y != 0.0) big_ci_h.push_back(m), big_cv_h.push_back(v);
        }
      }
      big_rp_h.push_back(int(big_ci_h.size()));
      int nch = 1, w = bb;
      for (;;) {
        w = (bb + nch - 1) / nch;
        if (csz * (size_t(ba) * ba + size_t(bb + ba) * w) <= (size_t(113) << 10) || w <= 8) break;
        ++nch;
      }
      BigPair P{a, b, isq ? qoff[pr] : roff[pr - J.npq], isq ? J.nq : J.nr, isq ? 1 : 0, w, nullptr, nullptr, nullptr};
      if (std::max(ba, bb) > kMaxBigBlock) {  // k_huge_mx + k_huge_zgemm
        J.huge_pairs.push_back(P);
        J.huge_rp_off.push_back(rp_off);
        continue;
      }
      J.big_pairs.push_back(P);
      J.big_rp_off.push_back(rp_off);
      const size_t sm = J.mixed ? big_qr_smem<float2>(ba, bb, w) : big_qr_smem<double2>(ba, bb, w);
      smem_qr[big_nt(ba, w) - 1] = std::max(smem_qr[big_nt(ba, w) - 1], sm);
    }
    if (!g_sizing) {
      auto attr = [](const void *f, size_t bytes) {
        if (bytes) CUDA_OK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
      };
      attr((const void *)k_big_step, smem_step);
      attr((const void *)k_big_dyson<1>, smem_mat);
      attr((const void *)k_big_dyson<2>, smem_mat);
      attr((const void *)k_big_step_df, smem_step);  // 5 b^2 float2 <= the FP64 step's 5 or 7 b^2 doubles
      attr((const void *)k_big_dyson_df<1>, smem_mat);
      attr((const void *)k_big_dyson_df<2>, smem_mat);
      if (J.tc) {
        size_t sm_step = 0, sm_dy = 0;
        for (int k : J.big_blocks)
          if (L.size[k] >= tc::kMinB)
            sm_step = std::max(sm_step, tc_step_smem(L.size[k])), sm_dy = std::max(sm_dy, tc_dyson_smem(L.size[k]));
        attr((const void *)k_tc_step, sm_step);
        attr((const void *)k_tc_dyson, sm_dy);
        attr((const void *)k_tc_dyson_stk, tc_dyson_stk_smem(64));
        attr((const void *)k_tc_step_stk, tc_step_stk_smem(64));
      }
      attr((const void *)k_big_eigframe<1, double2>, smem_mat);
      attr((const void *)k_big_eigframe<2, double2>, smem_mat);
      attr((const void *)k_big_eigframe<1, float2>, smem_mat);
      attr((const void *)k_big_eigframe<2, float2>, smem_mat);
      attr((const void *)k_big_eigframe4, smem_mat);
      attr((const void *)k_big_floquet, smem_mat + (J.mixed ? smem_mat / 4 : 0));  // + b^2 float2 (K)
      size_t smem_hf = 0;
      for (int k : J.huge_blocks) smem_hf = std::max(smem_hf, huge_floquet_smem(L.size[k]));
      if (smem_hf > (size_t(48) << 10)) attr((const void *)k_huge_floquet, smem_hf);
      if (J.mixed) {
        attr((const void *)k_big_qr<1, float2>, smem_qr[0]);
        attr((const void *)k_big_qr<2, float2>, smem_qr[1]);
      } else {
        attr((const void *)k_big_qr<1, double2>, smem_qr[0]);
        attr((const void *)k_big_qr<2, double2>, smem_qr[1]);
      }
    }
  }
  if (!g_sizing && !J.big_blocks.empty() && (!g_arena || g_arena->aux_streams)) {
    const int naux = int(std::min<size_t>(4, std::max(J.big_blocks.size(), J.big_pairs.size())));
    CUDA_OK(cudaEventCreateWithFlags(&J.fork_ev, cudaEventDisableTiming));
    for (int a = 0; a < naux; ++a) {
      cudaStream_t x;
      cudaEvent_t e;
      CUDA_OK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
      J.aux.push_back(x);
      CUDA_OK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      J.join_ev.push_back(e);
    }
  }
  J.blist.resize(kMaxBlock + 1);
  cudaStream_t st = ctx.stream;
  g_upload_counter = &J.h2d;
  struct CounterReset {
    ~CounterReset() { g_upload_counter = nullptr; }
  } counter_reset;
  for (int b = 1; b <= kMaxBlock; ++b) J.blist[b].upload(J.blocks_by_size[b], st);
  J.bs.upload(L.size, st), J.boff.upload(L.off, st), J.bpoff.upload(L.poff, st);
  J.qa.upload(qa, st), J.qb.upload(qb, st), J.qoff.upload(qoff, st), J.doff.upload(doff, st);
  J.ra.upload(ra, st), J.rb.upload(rb, st), J.roff.upload(roff, st), J.rhooff.upload(rhooff, st);
  J.eq.upload(eq, st), J.erev.upload(erev, st), J.er.upload(er, st), J.erg.upload(erg, st), J.esg.upload(esg, st);
  J.srp.upload(srp, st), J.seo.upload(seo, st);
  J.big_rp.upload(big_rp_h, st), J.big_ci.upload(big_ci_h, st), J.big_cv.upload(big_cv_h, st);
  for (size_t t = 0; t < J.big_pairs.size(); ++t)
    J.big_pairs[t].rp = J.big_rp.p + J.big_rp_off[t], J.big_pairs[t].ci = J.big_ci.p, J.big_pairs[t].cv = J.big_cv.p;
  for (size_t t = 0; t < J.huge_pairs.size(); ++t)
    J.huge_pairs[t].rp = J.big_rp.p + J.huge_rp_off[t], J.huge_pairs[t].ci = J.big_ci.p,
    J.huge_pairs[t].cv = J.big_cv.p;
  J.pas.upload(pas, st), J.iscale.upload(isc, st), J.Tk.upload(Tk, st), J.Hc.upload(Hc, st);
  if (p.precision == 1 && !J.is_static) {  // hi, lo splits for the mixed form's double-float step
    auto split = [](const std::vector<double> &v) {
      std::vector<float2> o(v.size());
      for (size_t x = 0; x < v.size(); ++x) {
        const float h = float(v[x]);
        o[x] = make_float2(h, float(v[x] - double(h)));
      }
      return o;
    };
    J.Tk_df.upload(split(Tk), st);
    J.Hc_df.upload(split(Hc), st);
    if (J.tc) {
      std::vector<int> ptr(size_t(L.S2) + 1, 0), term;
      std::vector<float2> val;
      for (size_t e = 0; e < size_t(L.S2); ++e) {
        ptr[e] = int(term.size());
        for (int kk = 0; kk < J.nint; ++kk) {
          const double v = Tk[size_t(kk) * L.S2 + e];
          if (v != 0.0) {
            const float h = float(v);
            term.push_back(kk), val.push_back(make_float2(h, float(v - double(h))));
          }
        }
      }
      ptr[L.S2] = int(term.size());
      // per block, its elements by descending term count (ties in element order): the
      // step's H build visits them in this order, so a warp's lanes walk similar lengths
      std::vector<int> order(size_t(L.S2), 0);
      for (size_t kb = 0; kb < L.size.size(); ++kb) {
        const int b = L.size[kb], bp = L.poff[kb];
        int *o = order.data() + bp;
        for (int e = 0; e < b * b; ++e) o[e] = e;
        std::stable_sort(o, o + b * b, [&](int x, int y) {
          return ptr[bp + x + 1] - ptr[bp + x] > ptr[bp + y + 1] - ptr[bp + y];
        });
      }
      J.tk_ptr.upload(ptr, st), J.tk_term.upload(term, st), J.tk_val.upload(val, st);
      J.tk_order.upload(order, st);
    }
  }
  if (sched) {  // per chunk: the rf frame of each permuted index (1 where a chunk has none)
    bool any = false;
    for (const auto &cs : chunk_sys) any = any || !cs.frame().empty();
    if (any) {
      std::vector<double2> fr(size_t(J.pb) * N, make_double2(1.0, 0.0));
      for (int kc = 0; kc < J.pb; ++kc) {
        const auto &f = chunk_sys[kc].frame();
        if (f.empty()) continue;
        for (int x = 0; x < N; ++x) fr[size_t(kc) * N + x] = make_double2(f[L.perm[x]].real(), f[L.perm[x]].imag());
      }
      J.frames.upload(fr, st);
    }
  }
  J.ikind.upload(ikind, st);
  J.Dblk.upload(Dblk, st), J.Rhoblk.upload(Rhoblk, st);
  J.status.upload(std::vector<int>(1, 0), st);
  // per-crystallite inputs, all batches, transposed to [item][c] per batch at run time
  // (stored here already in batch-major, crystallite-fastest order)
  {
    std::vector<double> Rp(size_t(J.nbatch) * 9 * J.Cb, 0.0), t0(size_t(J.nbatch) * J.Cb, 0.0),
        w(size_t(J.nbatch) * J.Cb, 0.0);
    for (int cg = 0; cg < J.Ceff; ++cg) {
      int bi = cg / J.Cb, c = cg % J.Cb;
      for (int x = 0; x < 9; ++x) Rp[(size_t(bi) * 9 + x) * J.Cb + c] = J.h_Rp[size_t(cg) * 9 + x];
      t0[size_t(bi) * J.Cb + c] = J.h_t0[cg];
      w[size_t(bi) * J.Cb + c] = J.h_w[cg];
    }
    J.Rp_all.upload(Rp, st), J.t0_all.upload(t0, st), J.w_all.upload(w, st);
  }
  size_t Cb = J.Cb;
  J.U.alloc(std::max<size_t>(1, nsteps * L.S2 * Cb));
  J.A.alloc(std::max<size_t>(1, nsteps * L.S2 * Cb));
  J.VF.alloc(size_t(L.S2) * Cb);
  J.Lb.alloc(size_t(N) * Cb);
  const size_t nQ = std::max<size_t>(1, nsteps * J.nq * Cb), nR = std::max<size_t>(1, nsteps * J.nr * Cb);
  const size_t nG = std::max<size_t>(1, size_t(J.n) * J.ne * Cb), nZ = std::max<size_t>(1, size_t(J.J) * J.ne * Cb);
  if (J.mixed) {
    J.Wf.alloc(std::max<size_t>(1, nsteps * L.S2 * Cb));
    J.Qf.alloc(nQ), J.Rf.alloc(nR), J.Gf.alloc(nG), J.Zf.alloc(nZ);
    J.Q.alloc(1), J.R.alloc(1), J.G.alloc(1), J.Z.alloc(1);
  } else {
    J.Q.alloc(nQ), J.R.alloc(nR), J.G.alloc(nG), J.Z.alloc(nZ);
  }
  J.partial.alloc(size_t(J.nwarps_total) * (J.mixed ? J.ft_r : 1) * p.npts);
  if (J.huge_ws_bytes) {
    J.huge_ws.alloc(J.huge_ws_bytes / sizeof(double2));
    J.hfk.alloc(size_t(J.huge_items) * std::max(J.nint, 1));
    J.hsc.alloc(size_t(J.huge_items));
    J.hsq.alloc(size_t(J.huge_items));
    J.hsqmax.alloc(1);
  }
  J.fid.alloc(p.npts);
  if (use_fk) J.fkc.alloc(size_t(J.n) * J.nint * Cb);
  J.tcf.alloc(2);
  if (J.tc && usl_per_c) {
    J.usl.alloc(usl_per_c * Cb);
    size_t off = 0;
    for (int k = 0; k < nb; ++k)
      if (L.size[k] >= tc::kMinB && L.size[k] <= tc::kMaxB) {
        J.usl_off[k] = off;
        off += nsteps * tc::slab_bytes(L.size[k]) * Cb;
      }
  }
  CUDA_OK(cudaMemsetAsync(J.partial.p, 0, J.partial.n * sizeof(double2), st));
  CUDA_OK(cudaStreamSynchronize(st));
  // algorithmic flop count (one complex MAC = 8 flop; eigh counted as 32 b^3, the
  // Floquet eig as 100 b^3)
  double S3 = 0;
  for (int k = 0; k < nb; ++k) S3 += double(L.size[k]) * L.size[k] * L.size[k];
  double pairs = 0;
  for (int pq = 0; pq < J.npq + J.npr; ++pq) {
    int a = pq < J.npq ? qa[pq] : ra[pq - J.npq], b = pq < J.npq ? qb[pq] : rb[pq - J.npq];
    pairs += double(L.size[a]) * L.size[b] * (L.size[a] + L.size[b]);
  }
  double S2H = 0;  // H build: one FMA per operator entry per interaction
  for (int k = 0; k < nb; ++k) S2H += double(L.size[k]) * L.size[k];
  double Ce = J.Ceff;
  J.stage_fl[0] = Ce * (J.is_static ? 1 : J.n) * (11.0 * S3 + 2.0 * J.nint * S2H);  // eigh + U + H build
  const double spin_steps = J.is_static ? 0.0 : double(J.n);
  J.stage_fl[1] = Ce * spin_steps * 8.0 * S3;                   // Dyson
  J.stage_fl[2] = J.is_static ? 0.0 : Ce * 100.0 * S3;          // Floquet eig
  J.stage_fl[3] = Ce * spin_steps * 8.0 * S3;                   // W = A V_F
  J.stage_fl[4] = Ce * spin_steps * 8.0 * pairs;               // Q, R transforms
  {
    // Fave correlation: direct 8 n^2 per element; FFT: 5 M log2 M per length-M transform
    // (two when r = conj(q), three otherwise), 8 M for the spectrum product, 8 n for G
    // (length n with 6 flop per twisted point when n is a power of two, else length >= 2n)
    const bool twist = !J.mixed && J.n >= 8 && (J.n & (J.n - 1)) == 0;
    int lm = 1;
    while ((1 << lm) < (twist ? J.n : 2 * J.n)) ++lm;
    double M = double(1 << lm), fftf = 5.0 * M * lm;
    bool fft = p.fave_method != 1 && M <= 4096;
    double per = 0;
    for (int e = 0; e < J.ne; ++e) {
      bool autoc = J.rosym && erev[e] < 0;
      per += fft ? (autoc ? 2 : 3) * fftf + 8.0 * M + 8.0 * J.n + (twist ? (autoc ? 12.0 : 18.0) * J.n : 0.0)
                 : 8.0 * J.n * J.n;
    }
    J.stage_fl[5] = J.is_static ? Ce * (16.0 * pairs + 8.0 * J.n * J.ne) : Ce * per;
    if (J.p2p) J.stage_fl[5] = Ce * 16.0 * J.pb * J.ne;  // two complex products per (k, element)
  }
  J.stage_fl[6] = Ce * 8.0 * p.npts * J.ne;                     // FID reconstruction
  J.stage_fl[7] = 4.0 * p.npts * J.nwarps_total * (J.mixed ? J.ft_r : 1);  // compensated powder sum
  J.flops = 0;
  for (double f : J.stage_fl) J.flops += f;
  // static part of the device description
  DevSys &s = J.base;
  s.n = J.n, s.npts = p.npts, s.N = N, s.nb = nb, s.S2 = L.S2, s.nint = J.nint, s.nq = J.nq, s.nr = J.nr;
  s.ne = J.ne, s.J = J.J, s.rosym = J.rosym, s.step_method = p.step_method;
  // FFT length: n itself when it is a power of two (twisted circular correlation; FP64 form
  // only, its twist factors are FP64 work), else the power of two >= 2n (zero-padded linear
  // correlation, the single-precision transforms of the mixed form)
  if (!J.p2p) {
    s.fave_twist = (!J.mixed && J.n >= 8 && (J.n & (J.n - 1)) == 0) ? 1 : 0;
    s.logM = 1;
    while ((1 << s.logM) < (s.fave_twist ? J.n : 2 * J.n)) ++s.logM;
    s.M = 1 << s.logM;
    // FFT correlation up to M = 4096 (its shared-memory tile is M * max(1, 2048/M) * 32 B)
    if (p.fave_method == 2 && s.M > 4096) throw Error(5, "FFT Fave supports at most 2048 steps per period");
    s.fave_method = (p.fave_method != 1 && s.M <= 4096) ? 1 : 0;
    if (J.mixed && !s.fave_method) throw Error(5, "the mixed form needs the FFT correlation (at most 2048 steps)");
    {
      std::vector<double2> tw(s.M / 2);
      for (int k = 0; k < s.M / 2; ++k) {
        double a = kPi2 * double(k) / double(s.M);
        tw[k] = make_double2(std::cos(a), -std::sin(a));
      }
      std::vector<float2> twf(tw.size());
      for (size_t k = 0; k < tw.size(); ++k) twf[k] = make_float2(float(tw[k].x), float(tw[k].y));
      g_upload_counter = &J.h2d;
      J.tw.upload(tw, st);
      J.twf.upload(twf, st);
      g_upload_counter = nullptr;
      s.tw = J.tw.p;
      s.twf = J.twf.p;
      // one cap for every job (jobs on other threads launch these kernels concurrently): the
      // largest M (4096, for 2048 steps) with its twist tables
      const size_t shm_max = sizeof(double2) * 4096 * 2 + sizeof(double2) * 2 * (8 + 4096 / 8);
      for (auto f : {k_fave_fft<8, double2>, k_fave_fft<4, double2>, k_fave_fft<2, double2>, k_fave_fft<1, double2>,
                     k_fave_fft<8, float2>, k_fave_fft<4, float2>, k_fave_fft<2, float2>, k_fave_fft<1, float2>})
        CUDA_OK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, int(shm_max)));
    }
    CUDA_OK(cudaFuncSetAttribute(k_fid_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(fid_tiled_smem(kFtJmax / 4, kFtThreads))));
  } else {  // no Fave: the point-to-point terms come from Q/R and the Floquet phases
    s.fave_twist = 0, s.logM = 0, s.M = 0, s.fave_method = 0;
    s.tw = nullptr, s.twf = nullptr;
  }
  s.tau = J.tau, s.wr = p.wr, s.sin_rotb = J.sin_rotb, s.cos_rotb = J.cos_rotb;
  s.is_static = J.is_static, s.dt = J.dt, s.srp = J.srp.p, s.seo = J.seo.p;
  s.scale = J.is_static ? 1.0 : double(1. / double(J.n / (J.rosym ? 2 : 1)));
  s.gper = J.n, s.p2p = J.p2p, s.pb = J.pb, s.pf = J.pf, s.psub = J.psub;
  s.ft_jt = J.ft_jt, s.ft_pt = J.ft_pt, s.ft_r = J.ft_r;
  if (J.p2p) {  // fid = sum_c w_c Tr(rho_c det) / Tr(det det^H)  (sequencerun_funcs.cc:624-645)
    double dd = 0;
    for (const auto &v : det.a) dd += std::norm(v);
    if (!(dd > 0)) throw Error(1, "the detection operator is zero");
    s.scale = 1.0 / dd;
    s.gper = J.pb;
  }
  s.bs = J.bs.p, s.boff = J.boff.p, s.bpoff = J.bpoff.p;
  s.pas = J.pas.p, s.iscale = J.iscale.p, s.Tk = J.Tk.p, s.Hc = J.Hc.p;
  s.fk = use_fk ? J.fkc.p : nullptr;
  s.hc_chunks = sched ? J.pb : 0;
  s.frames = J.frames.n ? J.frames.p : nullptr;
  s.Tk_df = J.Tk_df.p, s.Hc_df = J.Hc_df.p;
  s.tk_ptr = J.tk_ptr.p, s.tk_term = J.tk_term.p, s.tk_val = J.tk_val.p, s.tk_order = J.tk_order.p;
  s.fk_df = (J.mixed && p.step_method == 1 && use_fk) ? 1 : 0;
  {
    const double tp = J.tau * kPi2;
    const float h = float(tp);
    s.tpdf = make_float2(h, float(tp - double(h)));
  }
  s.ikind = J.ikind.p, s.has2 = J.has2;
  s.npq = J.npq, s.npr = J.npr;
  s.qa = J.qa.p, s.qb = J.qb.p, s.qoff = J.qoff.p, s.doff = J.doff.p;
  s.ra = J.ra.p, s.rb = J.rb.p, s.roff = J.roff.p, s.rhooff = J.rhooff.p;
  s.Dblk = J.Dblk.p, s.Rhoblk = J.Rhoblk.p;
  s.mixed = J.mixed;
  s.floq32 = 0;
  if (J.mixed && J.n > 0 && J.pb > 0) {  // the mixed form spins (never static)
    const long periods = J.p2p ? (long(p.npts) - 1) * J.pf / J.pb + 1 : (long(p.npts) - 1) / J.n + 1;
    s.floq32 = periods <= kFloq32MaxPeriods ? 1 : 0;
  }
  s.Wf = J.Wf.p, s.Qf = J.Qf.p, s.Rf = J.Rf.p, s.Gf = J.Gf.p, s.Zf = J.Zf.p;
  s.eq = J.eq.p, s.erev = J.erev.p, s.er = J.er.p, s.erg = J.erg.p, s.esg = J.esg.p;
  s.U = J.U.p, s.A = J.A.p, s.VF = J.VF.p, s.L = J.Lb.p, s.Q = J.Q.p, s.R = J.R.p, s.G = J.G.p, s.Z = J.Z.p;
  s.partial = J.partial.p;
  s.status = J.status.p;
  s.tc_flops = J.tcf.p;
  s.clay = (J.mixed && J.huge_blocks.empty()) ? 1 : 0;
  s.Cpad = J.Cb;
}

Job::~Job() {}

template <int B>
static void launch_block_kernels(JobImpl &J, DevSys &s, int stage) {
  const auto &lst = J.blocks_by_size[B];
  if (lst.empty()) return;
  int nl = int(lst.size());
  const int *bl = J.blist[B].p;
  cudaStream_t st = J.ctx->stream;
  long Cp = s.Cpad;
  if (s.is_static) {
    if (stage == 0) k_static_eig<B><<<grid_for(Cp * nl), kThreads, 0, st>>>(s, bl, nl);
    else return;
    ++J.launches;
    return;
  }
  switch (stage) {
    case 0:
      if (s.step_method == 1 && s.mixed) k_step_taylor_df<B><<<grid_for(Cp * nl * s.n), kThreads, 0, st>>>(s, bl, nl);
      else if (s.step_method == 1) k_step_taylor<B><<<grid_for(Cp * nl * s.n), kThreads, 0, st>>>(s, bl, nl);
      else k_step_prop<B><<<grid_for(Cp * nl * s.n), kThreads, 0, st>>>(s, bl, nl);
      break;
    case 1:
      if (s.mixed) {
        constexpr int G = B <= 1 ? 1 : B <= 2 ? 2 : B <= 4 ? 4 : 8;
        k_dyson_df<B><<<grid_for(Cp * nl * B * G), kThreads, 0, st>>>(s, bl, nl);
      }
      else k_dyson<B><<<grid_for(Cp * nl * B), kThreads, 0, st>>>(s, bl, nl);
      break;
    case 2:
      if (B == 1) {
        k_floquet<B><<<grid_for(Cp * nl), kThreads, 0, st>>>(s, bl, nl);
      } else {  // B lanes per matrix, 32/B matrices per warp
        const long warps = (Cp * nl + (32 / B) - 1) / (32 / B);
        if (s.floq32) k_floquet_lanes<B, float><<<grid_for(warps * 32), kThreads, 0, st>>>(s, bl, nl);
        else k_floquet_lanes<B, double><<<grid_for(warps * 32), kThreads, 0, st>>>(s, bl, nl);
      }
      break;
    case 3:
      if (s.mixed) k_eigframe<B, float2><<<grid_for(Cp * nl * s.n), kThreads, 0, st>>>(s, bl, nl);
      else k_eigframe<B, double2><<<grid_for(Cp * nl * s.n), kThreads, 0, st>>>(s, bl, nl);
      break;
  }
  ++J.launches;
}

// Work enqueued on the auxiliary streams after fork() waits for everything before it on
// the context stream; join() makes the context stream wait for all of it.
static void fork(JobImpl &J) {
  if (J.aux.empty()) return;
  CUDA_OK(cudaEventRecord(J.fork_ev, J.ctx->stream));
  for (auto a : J.aux) CUDA_OK(cudaStreamWaitEvent(a, J.fork_ev, 0));
}
static void join(JobImpl &J) {
  for (size_t a = 0; a < J.aux.size(); ++a) {
    CUDA_OK(cudaEventRecord(J.join_ev[a], J.aux[a]));
    CUDA_OK(cudaStreamWaitEvent(J.ctx->stream, J.join_ev[a], 0));
  }
}
static cudaStream_t aux_stream(JobImpl &J, size_t idx) {
  return J.aux.empty() ? J.ctx->stream : J.aux[idx % J.aux.size()];
}


// ------------------------------------------------------------------ huge blocks (bl_huge.cuh)
// All on the context stream; every launch covers at most kHugeMaxItems items and the
// workspace holds one launch's items.
template <class T>
static HMat<T> item_mat(T *p, long off, long sstr, int ld, int Cpad) {
  return HMat<T>{p, off, sstr, long(ld), long(Cpad), 1};
}
template <class T>
static HMat<T> ws_mat(T *p, long j0, long mat, int C, int ld) {
  return HMat<T>{p, -j0 * mat, long(C) * mat, long(ld), 1, mat};
}
static unsigned tiles(int m, int n) { return unsigned(((m + kHT - 1) / kHT) * ((n + kHT - 1) / kHT)); }

// U_i of huge block k for every (crystallite, step): symmetric Paterson-Stockmeyer.
static void huge_step(JobImpl &J, DevSys &s, size_t kh) {
  const int k = J.huge_blocks[kh], b = J.L.size[k], bp = J.L.poff[k];
  const long bb = long(b) * b, total = long(s.C) * J.n;
  const long per = std::min<long>(J.huge_items, long(J.huge_ws_bytes / (sizeof(double) * kHugeSlots * bb)));
  cudaStream_t st = J.ctx->stream;
  double *ws = reinterpret_cast<double *>(J.huge_ws.p);
  const unsigned ge = unsigned((bb + 255) / 256), tm = unsigned((b + kHT - 1) / kHT), gs = tm * (tm + 1) / 2;
  for (long j0 = 0; j0 < total; j0 += per) {
    const int items = int(std::min(per, total - j0));
    auto sym = [&](int a, int bsl, int o, int akind, double alpha, int round, bool low, double c0, double c1,
                   double c2, double c3) {
      SymArgs g{ws, J.hsc.p, J.hsq.p, bb, b, a, bsl, o, akind, alpha, round, low ? 1 : 0, c0, c1, c2, c3};
      if (s.mixed) k_huge_sym_df<<<dim3(gs, unsigned(items)), kHThreads, 0, st>>>(g);
      else k_huge_sym<<<dim3(gs, unsigned(items)), kHThreads, 0, st>>>(g);
      ++J.launches;
    };
    k_huge_fk<<<unsigned((items + 127) / 128), 128, 0, st>>>(s, j0, items, J.hfk.p);
    k_huge_hbuild<<<dim3(ge, unsigned(items)), 256, 0, st>>>(s, bp, b, J.hfk.p, ws, j0);
    CUDA_OK(cudaMemsetAsync(J.hsqmax.p, 0, sizeof(int), st));
    k_huge_norm<<<unsigned(items), 256, 0, st>>>(ws, b, s.tau * kPi2, J.hsc.p, J.hsq.p, J.hsqmax.p);
    J.launches += 3;
    sym(0, 0, 1, 1, 1.0, -1, false, 0, 0, 0, 0);  // Y = sc^2 H H
    sym(1, 1, 2, 0, 1.0, -1, false, 0, 0, 0, 0);  // Y^2
    sym(2, 1, 3, 0, 1.0, -1, false, 0, 0, 0, 0);  // Y^3
    sym(2, 2, 4, 0, 1.0, -1, false, 0, 0, 0, 0);  // Y^4
    // cos X = C(Y), coefficients (-1)^j/(2j)!;  sin X = X S(Y), (-1)^j/(2j+1)!
    k_huge_low<<<dim3(ge, unsigned(items)), 256, 0, st>>>(ws, b, 1.0 / 40320, -1.0 / 3628800, 1.0 / 479001600,
                                                          -1.0 / 87178291200.0);
    sym(4, 5, 6, 0, 1.0, -1, true, 1.0, -1.0 / 2, 1.0 / 24, -1.0 / 720);  // R = cos X
    k_huge_low<<<dim3(ge, unsigned(items)), 256, 0, st>>>(ws, b, 1.0 / 362880, -1.0 / 39916800,
                                                          1.0 / 6227020800.0, -1.0 / 1307674368000.0);
    sym(4, 5, 3, 0, 1.0, -1, true, 1.0, -1.0 / 6, 1.0 / 120, -1.0 / 5040);  // S(Y) over Y^3
    sym(0, 3, 1, 2, 1.0, -1, false, 0, 0, 0, 0);                            // I = -sc H S
    J.launches += 2;
    // squarings: the host bound for the block; each item skips the rounds it does not need
    for (int t = 0; t < J.huge_sq[kh]; ++t) {
      sym(6, 6, 2, 0, 1.0, t, false, 0, 0, 0, 0);
      sym(1, 1, 4, 0, 1.0, t, false, 0, 0, 0, 0);
      sym(6, 1, 5, 0, 2.0, t, false, 0, 0, 0, 0);
      k_huge_sqcomb<<<dim3(ge, unsigned(items)), 256, 0, st>>>(ws, b, J.hsq.p, t);
      ++J.launches;
    }
    k_huge_store_u<<<dim3(ge, unsigned(items)), 256, 0, st>>>(s, ws, bp, J.L.off[k], b, j0);
    ++J.launches;
  }
}

// A_{i+1} = U_i A_i for huge block k, one product launch per step.
static void huge_dyson(JobImpl &J, DevSys &s, size_t kh) {
  const int k = J.huge_blocks[kh], b = J.L.size[k], bp = J.L.poff[k];
  const long bb = long(b) * b;
  cudaStream_t st = J.ctx->stream;
  k_huge_copy_u0<<<dim3(unsigned((bb + 255) / 256), unsigned(s.C)), 256, 0, st>>>(s, bp, b);
  ++J.launches;
  const auto U = item_mat<const double2>(s.U, bp, s.S2, b, s.Cpad);
  const auto Ain = item_mat<const double2>(s.A, long(bp) - s.S2, s.S2, b, s.Cpad);
  const auto Aout = item_mat<double2>(s.A, bp, s.S2, b, s.Cpad);
  for (int i = 1; i < J.n; ++i) {
    if (s.mixed)  // double-float products, FP64 storage
      k_huge_zgemm_df<<<dim3(tiles(b, b), unsigned(s.C)), kHThreads, 0, st>>>(U, Ain, Aout, b, b, b, s.C,
                                                                              long(i) * s.C, 1.0);
    else
      k_huge_zgemm<double2, false, double2, double2, double2>
          <<<dim3(tiles(b, b), unsigned(s.C)), kHThreads, 0, st>>>(U, Ain, Aout, b, b, b, s.C, long(i) * s.C, 1.0);
    ++J.launches;
  }
}

// Floquet of all huge blocks: one launch per group of kMaxHugeLaunch blocks and chunk of
// crystallites, each (crystallite, block) with its own part of the workspace.
static void huge_floquet_all(JobImpl &J, DevSys &s) {
  const size_t nh = J.huge_blocks.size();
  for (size_t g0 = 0; g0 < nh; g0 += kMaxHugeLaunch) {
    HugeFloq hf{};
    hf.n = int(std::min<size_t>(kMaxHugeLaunch, nh - g0));
    hf.mats = s.floq32 ? 3 : 2;  // the mixed form's FP32 K takes half a third matrix
    size_t per_c = 0, smem = 0;
    for (int t = 0; t < hf.n; ++t) {
      const size_t b = size_t(J.L.size[J.huge_blocks[g0 + t]]);
      per_c += size_t(hf.mats) * b * b;
      smem = std::max(smem, huge_floquet_smem(int(b)));
    }
    const int per = int(std::min<size_t>(size_t(s.C), J.huge_ws_bytes / (sizeof(double2) * per_c)));
    if (per < 1) throw Error(3, "the huge-block workspace holds no crystallite's Floquet matrices");
    long off = 0;
    for (int t = 0; t < hf.n; ++t) {
      const long b = J.L.size[J.huge_blocks[g0 + t]];
      hf.k[t] = J.huge_blocks[g0 + t];
      hf.ws[t] = off;
      off += long(per) * hf.mats * b * b;
    }
    for (int c0 = 0; c0 < s.C; c0 += per) {
      k_huge_floquet<<<dim3(unsigned(std::min(per, s.C - c0)), unsigned(hf.n)), kHugeFloqThreads, smem,
                       J.ctx->stream>>>(s, hf, J.huge_ws.p, c0);
      ++J.launches;
    }
  }
}

// W_i = A_{i+1} V_F for huge block k: straight into W in the mixed form; through the
// workspace and back over A in FP64 (a product may not overwrite its own operand).
static void huge_eigframe(JobImpl &J, DevSys &s, size_t kh) {
  const int k = J.huge_blocks[kh], b = J.L.size[k], bp = J.L.poff[k];
  const long bb = long(b) * b, total = long(s.C) * J.n;
  cudaStream_t st = J.ctx->stream;
  const auto A = item_mat<const double2>(s.A, bp, s.S2, b, s.Cpad);
  const auto V = item_mat<const double2>(s.VF, bp, 0, b, s.Cpad);
  if (s.mixed) {
    const auto W = item_mat<float2>(s.Wf, bp, s.S2, b, s.Cpad);
    for (long j0 = 0; j0 < total; j0 += kHugeMaxItems) {
      const int items = int(std::min<long>(kHugeMaxItems, total - j0));
      k_huge_zgemm<float2, false, double2, double2, float2>
          <<<dim3(tiles(b, b), unsigned(items)), kHThreads, 0, st>>>(A, V, W, b, b, b, s.C, j0, 1.0);
      ++J.launches;
    }
    return;
  }
  const long per = std::min<long>(kHugeMaxItems, long(J.huge_ws_bytes / (sizeof(double2) * bb)));
  for (long j0 = 0; j0 < total; j0 += per) {
    const int items = int(std::min(per, total - j0));
    const auto O = ws_mat<double2>(J.huge_ws.p, j0, bb, s.C, b);
    k_huge_zgemm<double2, false, double2, double2, double2>
        <<<dim3(tiles(b, b), unsigned(items)), kHThreads, 0, st>>>(A, V, O, b, b, b, s.C, j0, 1.0);
    k_huge_copy_back<<<dim3(unsigned((bb + 255) / 256), unsigned(items)), 256, 0, st>>>(s, J.huge_ws.p, bp, b, j0);
    J.launches += 2;
  }
}

// Q^{ab} (or R) = W_a^H (M_ab W_b) for a pair with a huge block, every (crystallite, step).
template <class C>
static void huge_qr(JobImpl &J, DevSys &s, const BigPair &P, C *Wbuf, C *out) {
  const int ba = J.L.size[P.a], bb = J.L.size[P.b], pa = J.L.poff[P.a];
  const long ne = long(ba) * bb, total = long(s.C) * J.n;
  const long per = std::min<long>(kHugeMaxItems, long(J.huge_ws_bytes / (sizeof(C) * ne)));
  cudaStream_t st = J.ctx->stream;
  C *ws = reinterpret_cast<C *>(J.huge_ws.p);
  const auto Wa = item_mat<const C>(Wbuf, pa, s.S2, ba, s.Cpad);
  const auto O = item_mat<C>(out, P.off, P.nitems, bb, s.Cpad);
  for (long j0 = 0; j0 < total; j0 += per) {
    const int items = int(std::min(per, total - j0));
    k_huge_mx<C><<<dim3(unsigned((ne + 255) / 256), unsigned(items)), 256, 0, st>>>(s, P, j0, ws);
    const auto X = ws_mat<const C>(ws, j0, ne, s.C, bb);
    k_huge_zgemm<C, true, C, C, C><<<dim3(tiles(ba, bb), unsigned(items)), kHThreads, 0, st>>>(Wa, X, O, ba, bb, ba,
                                                                                             s.C, j0, 1.0);
    J.launches += 2;
  }
}

static void launch_stage(JobImpl &J, DevSys &s, int stage) {
  if (stage == 0 && s.fk) {  // the small blocks' term coefficients, before the streams fork
    k_coef<<<grid_for(long(s.Cpad) * s.n), kThreads, 0, J.ctx->stream>>>(s, J.fkc.p);
    ++J.launches;
  }
  if (!J.big_blocks.empty()) fork(J);
  launch_block_kernels<1>(J, s, stage);
  launch_block_kernels<2>(J, s, stage);
  launch_block_kernels<3>(J, s, stage);
  launch_block_kernels<4>(J, s, stage);
  launch_block_kernels<5>(J, s, stage);
  launch_block_kernels<6>(J, s, stage);
  launch_block_kernels<7>(J, s, stage);
  launch_block_kernels<8>(J, s, stage);
  // blocks larger than kMaxBlock: one CTA per crystallite (per step for the exponential),
  // each block on its own auxiliary stream
  for (size_t kb = 0; kb < J.big_blocks.size(); ++kb) {
    const int k = J.big_blocks[kb];
    const int b = J.L.size[k];
    cudaStream_t st = aux_stream(J, kb);
    const size_t smat = sizeof(double2) * 2 * size_t(b) * b;
    const size_t sw = (s.mixed ? sizeof(float2) : sizeof(double2)) * 2 * size_t(b) * b;
    const unsigned th = big_threads(b, b), th_step = unsigned((big_sym_tiles(b) + 31) / 32 * 32);
    const bool nt1 = big_nt(b, b) == 1;
    switch (stage) {
      case 0:
        if (J.tc && b >= tc::kMinB && tc::up16(b) <= 64)  // the two Horner chains stacked in one M = 128 tile
          k_tc_step_stk<<<unsigned(s.C) * unsigned(s.n), tc::kTcThreads, tc_step_stk_smem(b), st>>>(
              s, k, J.usl.p + J.usl_off[k]);
        else if (J.tc && b >= tc::kMinB)
          k_tc_step<<<unsigned(s.C) * unsigned(s.n), tc::kTcThreads, tc_step_smem(b), st>>>(s, k, J.usl.p + J.usl_off[k]);
        else if (s.mixed) k_big_step_df<<<unsigned(s.C) * unsigned(s.n), th_step, big_step_df_smem(b), st>>>(s, k);
        else k_big_step<<<unsigned(s.C) * unsigned(s.n), th_step, big_step_smem(b), st>>>(s, k);
        break;
      case 1:
        if (J.tc && b >= tc::kMinB) {  // exact-slice BF16 products on the tensor cores
          if (tc::up16(b) <= 64)  // re and im stacked in one M = 128 tile
            k_tc_dyson_stk<<<unsigned(s.C), tc::kTcThreads, tc_dyson_stk_smem(b), st>>>(s, k, J.usl.p + J.usl_off[k]);
          else
            k_tc_dyson<<<unsigned(s.C), tc::kTcThreads, tc_dyson_smem(b), st>>>(s, k, J.usl.p + J.usl_off[k]);
        } else if (s.mixed) {
          if (nt1) k_big_dyson_df<1><<<unsigned(s.C), th, smat, st>>>(s, k);
          else k_big_dyson_df<2><<<unsigned(s.C), th, smat, st>>>(s, k);
        } else {
          if (nt1) k_big_dyson<1><<<unsigned(s.C), th, smat, st>>>(s, k);
          else k_big_dyson<2><<<unsigned(s.C), th, smat, st>>>(s, k);
        }
        break;
      case 2:  // the mixed form's single-precision K follows the two b x b double2 arrays
        k_big_floquet<<<unsigned(s.C), kBigThreads, smat + (s.floq32 ? sizeof(float2) * size_t(b) * b : 0), st>>>(s, k);
        break;
      case 3:
        if (s.mixed) {
          k_big_eigframe4<<<unsigned(s.C), unsigned(big4_threads(b, b)), sw, st>>>(s, k);
        } else {
          if (nt1) k_big_eigframe<1, double2><<<unsigned(s.C), th, sw, st>>>(s, k);
          else k_big_eigframe<2, double2><<<unsigned(s.C), th, sw, st>>>(s, k);
        }
        break;
    }
    ++J.launches;
  }
  // blocks larger than kMaxBigBlock: batched products on the context stream, alongside the
  // large blocks on the auxiliary streams
  for (size_t kh = 0; kh < J.huge_blocks.size(); ++kh) {
    switch (stage) {
      case 0: huge_step(J, s, kh); break;
      case 1: huge_dyson(J, s, kh); break;
      case 2:
        if (kh == 0) huge_floquet_all(J, s);
        break;
      case 3: huge_eigframe(J, s, kh); break;
    }
  }
  if (!J.big_blocks.empty()) join(J);
}

static void mark_begin(JobImpl &J, int stage);
static void mark_end(JobImpl &J, int stage, int nlaunch);

// k_fid with a (j, p) register tile of about 16 accumulators whose p-width wastes the least of
// the period gper (a point-to-point period of 9 takes 3-wide tiles instead of 4-wide)
template <int JT, int PT, class C>
static void launch_fid_tile(const DevSys &s, long Cp, int Jn, cudaStream_t st) {
  const int npt = (s.gper + PT - 1) / PT, njt = (Jn + JT - 1) / JT;
  k_fid<C, JT, PT><<<grid_for(Cp * npt * njt), kThreads, 0, st>>>(s);
}
template <class C>
static void launch_fid(const DevSys &s, long Cp, int Jn, cudaStream_t st) {
  int pt = kFidPT;
  if (s.gper % kFidPT != 0 && s.gper < 64) {
    int waste = 1 << 30;
    for (int w = kFidPT; w >= 1; --w) {
      const int ws = (s.gper + w - 1) / w * w - s.gper;
      if (ws < waste) waste = ws, pt = w;
    }
  }
  switch (pt) {
    case 1: launch_fid_tile<16, 1, C>(s, Cp, Jn, st); break;
    case 2: launch_fid_tile<8, 2, C>(s, Cp, Jn, st); break;
    case 3: launch_fid_tile<5, 3, C>(s, Cp, Jn, st); break;
    default: launch_fid_tile<kFidJT, kFidPT, C>(s, Cp, Jn, st); break;
  }
}

void Job::run() {
  JobImpl &J = *d_;
  CUDA_OK(cudaSetDevice(J.ctx->device));
  cudaStream_t st = J.ctx->stream;
  J.launches = 0;
  J.marks.clear();
  J.evnext = 0;
  if (J.profiling && J.evpool.empty()) {
    J.evpool.resize(size_t(2) * Job::kStages * (J.nbatch + 1));
    for (auto &e : J.evpool) CUDA_OK(cudaEventCreate(&e));
  }
  CUDA_OK(cudaMemsetAsync(J.status.p, 0, sizeof(int), st));
  CUDA_OK(cudaMemsetAsync(J.tcf.p, 0, 2 * sizeof(unsigned long long), st));
  for (int bi = 0; bi < J.nbatch; ++bi) {
    DevSys s = J.base;
    int c0 = bi * J.Cb;
    s.C = std::min(J.Cb, J.Ceff - c0);
    s.Cpad = J.Cb;
    s.Rp = J.Rp_all.p + size_t(bi) * 9 * J.Cb;
    s.t0 = J.t0_all.p + size_t(bi) * J.Cb;
    s.w = J.w_all.p + size_t(bi) * J.Cb;
    s.warp_base = c0 / 32;
    for (int stage = 0; stage < 4; ++stage) {
      mark_begin(J, stage);
      int before = J.launches;
      launch_stage(J, s, stage);
      mark_end(J, stage, J.launches - before);
    }
    long Cp = s.Cpad;
    mark_begin(J, 4);
    const int qr_before = J.launches;
    if (!J.is_static && J.npq + J.npr > 0) {
      if (!J.big_pairs.empty()) fork(J);
      if (s.mixed) k_qr<float2><<<grid_for(Cp * (J.npq + J.npr) * J.n), kThreads, 0, st>>>(s);
      else k_qr<double2><<<grid_for(Cp * (J.npq + J.npr) * J.n), kThreads, 0, st>>>(s);
      ++J.launches;
      for (size_t t = 0; t < J.big_pairs.size(); ++t) {
        const BigPair &P = J.big_pairs[t];
        cudaStream_t st = aux_stream(J, t);
        const int ba = J.L.size[P.a], bb = J.L.size[P.b];
        const unsigned grid = unsigned(s.C) * unsigned(J.n), th = big_threads(ba, P.wchunk);
        const bool nt1 = big_nt(ba, P.wchunk) == 1;
        if (s.mixed) {
          const size_t sm = big_qr_smem<float2>(ba, bb, P.wchunk);
          if (nt1) k_big_qr<1, float2><<<grid, th, sm, st>>>(s, P);
          else k_big_qr<2, float2><<<grid, th, sm, st>>>(s, P);
        } else {
          const size_t sm = big_qr_smem<double2>(ba, bb, P.wchunk);
          if (nt1) k_big_qr<1, double2><<<grid, th, sm, st>>>(s, P);
          else k_big_qr<2, double2><<<grid, th, sm, st>>>(s, P);
        }
        ++J.launches;
      }
      for (const BigPair &P : J.huge_pairs) {
        if (s.mixed) huge_qr<float2>(J, s, P, s.Wf, P.isq ? s.Qf : s.Rf);
        else huge_qr<double2>(J, s, P, s.A, P.isq ? s.Q : s.R);
      }
      if (!J.big_pairs.empty()) join(J);
    }
    mark_end(J, 4, J.launches - qr_before);
    mark_begin(J, 5);
    if (J.is_static && J.ne > 0) {
      k_static_elems<<<grid_for(Cp * J.npq), kThreads, 0, st>>>(s);
      ++J.launches;
    } else if (J.p2p && J.ne > 0) {
      if (s.mixed) k_p2p_elems<float2><<<grid_for(Cp * J.ne), kThreads, 0, st>>>(s);
      else k_p2p_elems<double2><<<grid_for(Cp * J.ne), kThreads, 0, st>>>(s);
      ++J.launches;
    } else if (J.ne > 0) {
      if (s.fave_method == 1) {
        int cg = std::max(1, std::min(8, 2048 / s.M));
        const size_t shm = sizeof(double2) * size_t(s.M) * cg * 2 + fave_twist_bytes(s, cg);
        const size_t shmf = sizeof(float2) * size_t(s.M) * cg * 2 + fave_twist_bytes(s, cg);
        unsigned grid = unsigned(J.ne) * unsigned(Cp / cg);
        switch (cg) {
          case 8:
            if (s.mixed) k_fave_fft<8, float2><<<grid, 128, shmf, st>>>(s);
            else k_fave_fft<8, double2><<<grid, 128, shm, st>>>(s);
            break;
          case 4:
            if (s.mixed) k_fave_fft<4, float2><<<grid, 128, shmf, st>>>(s);
            else k_fave_fft<4, double2><<<grid, 128, shm, st>>>(s);
            break;
          case 2:
            if (s.mixed) k_fave_fft<2, float2><<<grid, 128, shmf, st>>>(s);
            else k_fave_fft<2, double2><<<grid, 128, shm, st>>>(s);
            break;
          default:
            if (s.mixed) k_fave_fft<1, float2><<<grid, 128, shmf, st>>>(s);
            else k_fave_fft<1, double2><<<grid, 128, shm, st>>>(s);
            break;
        }
      } else {
        int ntile = (J.n + kFavePT - 1) / kFavePT;
        k_fave<<<grid_for(Cp * J.ne * ntile), kThreads, 0, st>>>(s);
      }
      ++J.launches;
    }
    mark_end(J, 5, J.ne > 0 ? 1 : 0);
    // k_fid writes every (warp, k) of this batch, so partials need no clearing; it exits
    // per warp, and rows it does not cover (p >= n or k >= npts) do not exist
    mark_begin(J, 6);
    if (s.mixed) {
      const unsigned npr = unsigned((s.gper + 4 * s.ft_pt - 1) / (4 * s.ft_pt));
      const unsigned njr = unsigned((J.J + 4 * s.ft_jt - 1) / (4 * s.ft_jt));
      k_fid_tiled<<<dim3(unsigned(Cp / 32), npr * njr, unsigned(s.ft_r)), kFtThreads,
                    fid_tiled_smem(s.ft_jt, s.ft_pt), st>>>(s);
    } else {
      launch_fid<double2>(s, Cp, J.J, st);
    }
    ++J.launches;
    mark_end(J, 6, 1);
  }
  mark_begin(J, 7);
  // only warps that hold crystallites: the sum is then independent of the batch size
  k_reduce<<<(J.P.npts + 255) / 256, 256, 0, st>>>(J.partial.p, (J.Ceff + 31) / 32 * (J.mixed ? J.ft_r : 1),
                                                    J.P.npts, J.fid.p);
  ++J.launches;
  mark_end(J, 7, 1);
  CUDA_OK(cudaGetLastError());
  if (J.profiling && !J.marks.empty()) {
    CUDA_OK(cudaEventSynchronize(J.evpool[J.marks.back().e]));
    for (const auto &m : J.marks) {
      float ms = 0;
      CUDA_OK(cudaEventElapsedTime(&ms, J.evpool[m.b], J.evpool[m.e]));
      J.stage_ms[m.stage] += ms;
      J.stage_launch[m.stage] += m.nlaunch;
    }
  }
}

// Stage markers: with profiling on, an event pair on the launching stream brackets each
// stage; run() folds the elapsed times into the per-stage totals once its last event
// has completed (one synchronisation per run, none between stages).
static void mark_begin(JobImpl &J, int stage) {
  if (!J.profiling) return;
  CUDA_OK(cudaEventRecord(J.evpool[J.evnext], J.ctx->stream));
  J.marks.push_back({stage, J.evnext, -1, 0});
  ++J.evnext;
}

static void mark_end(JobImpl &J, int stage, int nlaunch) {
  if (!J.profiling) return;
  CUDA_OK(cudaEventRecord(J.evpool[J.evnext], J.ctx->stream));
  J.marks.back().e = J.evnext;
  J.marks.back().nlaunch = nlaunch;
  (void)stage;
  ++J.evnext;
}

void Job::read(double *fid_out) {
  JobImpl &J = *d_;
  CUDA_OK(cudaMemcpyAsync(fid_out, J.fid.p, sizeof(double2) * J.P.npts, cudaMemcpyDeviceToHost, J.ctx->stream));
  int status = 0;
  CUDA_OK(cudaMemcpyAsync(&status, J.status.p, sizeof(int), cudaMemcpyDeviceToHost, J.ctx->stream));
  CUDA_OK(cudaStreamSynchronize(J.ctx->stream));
  if (status & (kNoConvergeStep | kNoConvergeFloquet))
    throw Error(7, "an eigen-decomposition did not converge within its sweep limit");
  if (status & kSingularCayley) throw Error(7, "singular Cayley transform in the Floquet eigen-decomposition");
  if (status & kTcTimeout) throw Error(7, "a tensor-core product did not complete within its wait limit");
}

const char *Job::stage_name(int s) {
  static const char *names[kStages] = {"k_step_prop", "k_dyson",  "k_floquet", "k_eigframe",
                                       "k_qr",        "k_fave",   "k_fid",     "k_reduce"};
  return (s >= 0 && s < kStages) ? names[s] : "";
}
void Job::set_profiling(bool on) { d_->profiling = on; }
void Job::stage_times(double *ms, int *launches) const {
  for (int i = 0; i < kStages; ++i) {
    if (ms) ms[i] = d_->stage_ms[i];
    if (launches) launches[i] = d_->stage_launch[i];
  }
}
void Job::stage_flops(double *f) const {
  for (int i = 0; i < kStages; ++i) f[i] = d_->stage_fl[i];
}
void Job::reset_stage_times() {
  for (int i = 0; i < kStages; ++i) d_->stage_ms[i] = 0, d_->stage_launch[i] = 0;
}
size_t Job::h2d_bytes() const { return d_->h2d; }
size_t Job::d2h_bytes() const { return sizeof(double2) * d_->P.npts; }
double Job::run_timed(int iters) {
  JobImpl &J = *d_;
  cudaEvent_t a, b;
  CUDA_OK(cudaEventCreate(&a));
  CUDA_OK(cudaEventCreate(&b));
  CUDA_OK(cudaEventRecord(a, J.ctx->stream));
  for (int i = 0; i < iters; ++i) run();
  CUDA_OK(cudaEventRecord(b, J.ctx->stream));
  CUDA_OK(cudaEventSynchronize(b));
  float ms = 0;
  CUDA_OK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

namespace {
// 8 independent DFMA chains per thread; 2*8*iters flop per thread.
__global__ void k_dfma_probe(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = threadIdx.x + c;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
// The same with FP32 FMA chains: the FP32 pipe that the mixed form's double-float stages use.
__global__ void k_ffma_probe(float *out, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = threadIdx.x + c;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fmaf(x[c], a, b);
  float s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

double error_statement(Context &ctx, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
                       const FidParams &p, int sample) {
  const int C = pw.size();
  const int m = std::min(std::max(sample, 1), C);
  Powder sub;
  for (int k = 0; k < m; ++k) {
    const int c = int((2L * k + 1) * C / (2L * m));
    sub.theta.push_back(pw.theta[c]), sub.phi.push_back(pw.phi[c]), sub.gamma.push_back(pw.gamma[c]);
    sub.weight.push_back(pw.weight[c]);
  }
  FidParams p1 = p, p0 = p;
  p1.precision = 1, p0.precision = 0;
  p1.error_sample = p0.error_sample = 0;
  std::vector<double> f1(2 * size_t(p.npts)), f0(2 * size_t(p.npts));
  {
    Job j(ctx, sys, sub, ro, det, p1);
    j.run();
    j.read(f1.data());
  }
  {
    Job j(ctx, sys, sub, ro, det, p0);
    j.run();
    j.read(f0.data());
  }
  double num = 0, den = 0;
  for (size_t x = 0; x < f0.size(); ++x) num += (f1[x] - f0[x]) * (f1[x] - f0[x]), den += f0[x] * f0[x];
  return den > 0 ? std::sqrt(num / den) : 0.0;
}

double probe_fp32_tflops(Context &ctx) {
  CUDA_OK(cudaSetDevice(ctx.device));
  int sms = 0;
  CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  int blocks = sms * 8, threads = 256, iters = 40000;
  DevBuf<float> out;
  out.alloc(size_t(blocks) * threads);
  cudaEvent_t a, b;
  CUDA_OK(cudaEventCreate(&a));
  CUDA_OK(cudaEventCreate(&b));
  k_ffma_probe<<<blocks, threads, 0, ctx.stream>>>(out.p, 10, 0.999f, 0.001f);
  double best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    CUDA_OK(cudaEventRecord(a, ctx.stream));
    k_ffma_probe<<<blocks, threads, 0, ctx.stream>>>(out.p, iters, 0.999f, 0.001f);
    CUDA_OK(cudaEventRecord(b, ctx.stream));
    CUDA_OK(cudaEventSynchronize(b));
    float ms = 0;
    CUDA_OK(cudaEventElapsedTime(&ms, a, b));
    best = std::max(best, 2.0 * 8 * double(iters) * blocks * threads / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

double probe_fp64_tflops(Context &ctx) {
  CUDA_OK(cudaSetDevice(ctx.device));
  int sms = 0;
  CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx.device));
  int blocks = sms * 4, threads = 256, iters = 4000;
  DevBuf<double> out;
  out.alloc(size_t(blocks) * threads);
  cudaEvent_t a, b;
  CUDA_OK(cudaEventCreate(&a));
  CUDA_OK(cudaEventCreate(&b));
  k_dfma_probe<<<blocks, threads, 0, ctx.stream>>>(out.p, 10, 0.999, 0.001);
  double best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    CUDA_OK(cudaEventRecord(a, ctx.stream));
    k_dfma_probe<<<blocks, threads, 0, ctx.stream>>>(out.p, iters, 0.999, 0.001);
    CUDA_OK(cudaEventRecord(b, ctx.stream));
    CUDA_OK(cudaEventSynchronize(b));
    float ms = 0;
    CUDA_OK(cudaEventElapsedTime(&ms, a, b));
    best = std::max(best, 2.0 * 8 * double(iters) * blocks * threads / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

double Job::sw_out() const { return d_->sw_out; }
int Job::npts() const { return d_->P.npts; }
int Job::kernels_per_run() const { return d_->launches; }
const double *Job::device_fid() const { return reinterpret_cast<const double *>(d_->fid.p); }
double Job::flops() const { return d_->flops; }
void Job::tensor_flops(double *step, double *dyson) const {
  unsigned long long v[2] = {0, 0};
  CUDA_OK(cudaMemcpyAsync(v, d_->tcf.p, sizeof(v), cudaMemcpyDeviceToHost, d_->ctx->stream));
  CUDA_OK(cudaStreamSynchronize(d_->ctx->stream));
  if (step) *step = double(v[0]);
  if (dyson) *dyson = double(v[1]);
}

std::string Job::describe() const {
  const JobImpl &J = *d_;
  std::ostringstream o;
  o << "{\"N\": " << J.L.N << ", \"blocks\": [";
  for (size_t k = 0; k < J.L.size.size(); ++k) o << (k ? ", " : "") << J.L.size[k];
  o << "], \"S2\": " << J.L.S2 << ", \"n\": " << J.n << ", \"gammaloop\": " << J.gammaloop
    << ", \"crystallites\": " << J.C << ", \"rosym\": " << J.rosym << ", \"q_pairs\": " << J.npq
    << ", \"r_pairs\": " << J.npr << ", \"elements\": " << J.ne << ", \"batch\": " << J.Cb
    << ", \"batches\": " << J.nbatch << ", \"flops\": " << J.flops << "}";
  return o.str();
}

// ------------------------------------------------------------------ allocation-free entry
// Some callers may not allocate device memory at all: a host program that reserves the
// GPU's memory for itself up front and forbids other allocators, or a timing-critical loop
// in which cudaMalloc/cudaFree (which synchronise the device) are not allowed.  For them
// powder_fid_noalloc runs the same pipeline with every device buffer (inputs, tables, work
// buffers, warp partials, FID, status word) carved from one static device array of
// kNoAllocScratch bytes; larger jobs are processed in crystallite batches that fit it, and
// a job whose smallest batch does not fit is rejected with BL_ERR_NOMEM.  Every GPU that
// loads this library holds the array until the process exits.  All calls share it and it
// keeps the previous call's contents: each call zeroes what must start at zero (the status
// word and the warp partials), and calls that overlap on the GPU race on it.
namespace {
constexpr size_t kNoAllocScratch = size_t(64) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratch];
}  // namespace

size_t noalloc_scratch_bytes() { return kNoAllocScratch; }

// Device address of the static array in the current device's context.  Host code may not
// use the symbol itself as a device pointer, so every call asks the runtime (a host-side
// lookup that allocates nothing); an address kept from an earlier call would dangle once the
// host program resets the device or its primary context is rebuilt.  The first lookup on a
// device loads this library's device code, and with it the array, so the first call should
// come before any stream capture and before the host program claims the device's memory.
static char *noalloc_base() {
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr) throw Error(3, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  return static_cast<char *>(ptr);
}

// Device bytes outside the batch-sized work buffers: tables, per-crystallite inputs (11
// doubles each, padded by up to one batch), warp partials and the FID.
static size_t fixed_bytes(const Powder &pw, const FidParams &p) {
  long n = p.wr != 0.0 ? long(std::floor(p.sw / p.wr + 0.5)) : 1;
  long g = (n >= 1 && n <= 10) ? std::max(1L, 10 / n) : 1;
  size_t ceff = size_t(pw.size()) * size_t(g) + 32;
  // warp partials: up to kFtR rows per warp in the mixed form (k_fid_tiled's element ranges)
  return (size_t(8) << 20) + 2 * ceff * 11 * sizeof(double) +
         (ceff / 32 + 1) * size_t(p.precision == 1 ? kFtR : 1) * size_t(std::max(p.npts, 0)) * sizeof(double2);
}

void job_bytes(int device, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
               const FidParams &p, size_t *min_bytes, size_t *full_bytes) {
  Context ctx;
  ctx.device = device;
  JobSizing plan;
  struct Scope {
    JobSizing *prev;
    explicit Scope(JobSizing *z) : prev(g_sizing) { g_sizing = z; }
    ~Scope() { g_sizing = prev; }
  } scope(&plan);
  Job job(ctx, sys, pw, ro, det, p);
  // work buffers are carved with 256-byte alignment: allow for it on each of ~40 buffers
  size_t fixed = fixed_bytes(pw, p) + 40 * 256 + plan.extra + plan.tables;
  if (min_bytes) *min_bytes = fixed + plan.per_c * 32;
  if (full_bytes) *full_bytes = fixed + plan.per_c * size_t(plan.cpad);
}

void powder_fid_noalloc(Context &ctx, const SpinSystem &sys, const Powder &pw, const CMatrix &ro, const CMatrix &det,
                        const FidParams &p, double *fid_out, double *sw_out) {
  CUDA_OK(cudaSetDevice(ctx.device));
  // the host-side plan (no device memory is touched): the batch-independent bytes as the
  // arena will carve them, and the bytes each crystallite of a batch adds
  JobSizing plan;
  {
    struct Scope {
      JobSizing *prev;
      explicit Scope(JobSizing *z) : prev(g_sizing) { g_sizing = z; }
      ~Scope() { g_sizing = prev; }
    } scope(&plan);
    Context probe;
    probe.device = ctx.device;
    Job sizing(probe, sys, pw, ro, det, p);
  }
  // work buffers are carved with 256-byte alignment: allow for it on each of ~40 buffers
  const size_t fixed = fixed_bytes(pw, p) + 40 * 256 + plan.extra + plan.tables;
  const size_t smallest = fixed + plan.per_c * 32;  // with one 32-crystallite batch
  if (smallest > kNoAllocScratch)
    throw Error(4, "job needs " + std::to_string((smallest + (size_t(1) << 20) - 1) >> 20) +
                       " MiB for its smallest batch, more than the " + std::to_string(kNoAllocScratch >> 20) +
                       " MiB static device scratch of the allocation-free entry point");
  ScratchArena arena;
  arena.base = noalloc_base();
  arena.cap = kNoAllocScratch;
  Context view;  // same device and stream; budget = what the scratch leaves for work buffers
  view.device = ctx.device;
  view.stream = ctx.stream;
  view.hbm_budget = kNoAllocScratch - (fixed - plan.extra);  // the Job sets the workspace (extra) aside itself
  struct Release {
    Context &c;
    ~Release() { c.stream = nullptr; }  // the stream belongs to the caller's context
  } release{view};
  struct Scope {
    ScratchArena *prev;
    explicit Scope(ScratchArena *a) : prev(g_arena) { g_arena = a; }
    ~Scope() { g_arena = prev; }
  } scope(&arena);
  try {
    Job job(view, sys, pw, ro, det, p);
    job.run();
    job.read(fid_out);
    if (sw_out) *sw_out = job.sw_out();
  } catch (const Error &e) {
    if (e.code == 4 && std::string(e.what()).find("static device scratch") == std::string::npos)
      throw Error(4, std::string("job does not fit the ") + std::to_string(kNoAllocScratch >> 20) +
                         " MiB static device scratch of the allocation-free entry point: " + e.what());
    throw;
  }
}

// A resident Job whose every device buffer lives in [base, base + bytes): the serving loop
// gives each slot such a region, so admitting a request allocates nothing.  The caller's
// Context (device, stream) must outlive the Job; its hbm_budget is set here.
std::unique_ptr<Job> job_in_region(Context &ctx, void *base, size_t bytes, const SpinSystem &sys, const Powder &pw,
                                   const CMatrix &ro, const CMatrix &det, const FidParams &p) {
  CUDA_OK(cudaSetDevice(ctx.device));
  ScratchArena arena;
  arena.base = static_cast<char *>(base);
  arena.cap = bytes;
  arena.label = "device region given to the job";
  arena.aux_streams = true;
  size_t fixed = fixed_bytes(pw, p);
  if (fixed >= bytes) throw Error(4, "job does not fit a device region of " + std::to_string(bytes >> 20) + " MiB");
  ctx.hbm_budget = bytes - fixed;
  struct Scope {
    ScratchArena *prev;
    explicit Scope(ScratchArena *a) : prev(g_arena) { g_arena = a; }
    ~Scope() { g_arena = prev; }
  } scope(&arena);
  return std::unique_ptr<Job>(new Job(ctx, sys, pw, ro, det, p));
}

}  // namespace bl
