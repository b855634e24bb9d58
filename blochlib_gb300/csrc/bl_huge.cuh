// Huge-block kernels (Hamiltonian blocks kMaxBigBlock < b <= kMaxHugeBlock, 9-12 like
// spins 1/2), included by bl_engine.cu after bl_big.cuh.  A block no longer fits shared
// memory, so each stage is a sequence of batched products of per-crystallite matrices:
// 64 x 64 output tiles per CTA, 16-wide k panels staged in shared memory, 4 x 4 outputs
// per thread.  Operands are addressed in place in the engine's [item][c] buffers (HMat
// with element stride Cpad) or in a workspace of contiguous per-item matrices (element
// stride 1).  With FP64 issue as the bound (one 64x64x16 complex panel is 262k FMA against
// 32 KB of loads), the strided panel loads cost well under 1 B/clock per SM.
//   step       k_huge_fk, k_huge_hbuild, k_huge_norm, k_huge_sym x 7, k_huge_low, squarings,
//              k_huge_store_u: the same symmetric Paterson-Stockmeyer exponential as
//              k_big_step, over a chunk of (crystallite, step) items at a time
//   Dyson      k_huge_zgemm per step (A_{i+1} = U_i A_i), A_1 = U_0 by k_huge_copy_u0
//   Floquet    k_huge_floquet: floquet_cta with its two b x b matrices in global memory
//   eigenframe k_huge_zgemm (A_{i+1} V_F) into the workspace, copied back in FP64
//   Q/R        k_huge_mx (X = M_ab W_b from M's non-zeros) and k_huge_zgemm (W_a^H X)
// Items are numbered g = sl*C + c (crystallite c, step sl); a launch covers
// g = j0 + blockIdx.y, and the workspace holds the launch's items by blockIdx.y.

constexpr int kMaxHugeBlock = 1024;
constexpr int kHT = 64;          // output tile
constexpr int kHK = 16;          // k panel
constexpr int kHThreads = 256;   // 16 x 16 threads, 4 x 4 outputs each
constexpr int kHugeSlots = 7;    // X, Y, Y2, Y3, Y4, T, R per item of the exponential
constexpr int kHugeMaxItems = 65535;  // items per launch (grid y)

// Operand of a batched product.  Element (r, q) of item (c, sl) is at
// p[(off + sl*sstr + r*ld + q)*es + c*cs]: es = Cpad, cs = 1 for the [item][c] buffers;
// es = 1, cs = mat, sstr = C*mat, off = -j0*mat for a workspace of contiguous matrices
// indexed by blockIdx.y.
template <class T>
struct HMat {
  T *p;
  long off, sstr, ld, es, cs;
  __device__ __forceinline__ T &operator()(int c, int sl, int r, int q) const {
    return p[(off + long(sl) * sstr + long(r) * ld + q) * es + long(c) * cs];
  }
};

template <class C>
__device__ __forceinline__ C to(double2 v) { return mkc<C>(v.x, v.y); }
template <class C>
__device__ __forceinline__ C to(float2 v) { return mkc<C>(v.x, v.y); }

// O = alpha * op(A) (m x k) * B (k x n) for items g = j0 + blockIdx.y; op(A) = A, or A^H
// when CONJ_A (A stored k x m).  Compute type C (double2, or float2 in the mixed form);
// operands are converted on load.
template <class C, bool CONJ_A, class TA, class TB, class TO>
__global__ void __launch_bounds__(kHThreads) k_huge_zgemm(HMat<const TA> A, HMat<const TB> B, HMat<TO> O, int m,
                                                         int n, int k, int Cb, long j0, double alpha) {
  __shared__ C As[kHK][kHT + 1], Bs[kHK][kHT + 1];
  const long g = j0 + blockIdx.y;
  const int c = int(g % Cb), sl = int(g / Cb);
  const int tn = (n + kHT - 1) / kHT;
  const int r0 = (blockIdx.x / tn) * kHT, q0 = (blockIdx.x % tn) * kHT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  C acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = mkc<C>(0, 0);
  for (int k0 = 0; k0 < k; k0 += kHK) {
    for (int idx = threadIdx.x; idx < kHT * kHK; idx += kHThreads) {
      const int rr = idx / kHK, kk = idx % kHK, r = r0 + rr, l = k0 + kk;
      C v = mkc<C>(0, 0);
      if (r < m && l < k) v = CONJ_A ? cconj(to<C>(A(c, sl, l, r))) : to<C>(A(c, sl, r, l));
      As[kk][rr] = v;
      const int kb = idx / kHT, qq = idx % kHT, lb = k0 + kb, q = q0 + qq;
      C w = mkc<C>(0, 0);
      if (lb < k && q < n) w = to<C>(B(c, sl, lb, q));
      Bs[kb][qq] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kHK; ++kk) {
      C a[4], b[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) a[t] = As[kk][ty + 16 * t], b[t] = Bs[kk][tx + 16 * t];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = cfma(a[x], b[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int r = r0 + ty + 16 * x, q = q0 + tx + 16 * y;
      if (r < m && q < n) O(c, sl, r, q) = to<TO>(mkc<C>(double(acc[x][y].x) * alpha, double(acc[x][y].y) * alpha));
    }
}

// The mixed form's Dyson product for huge blocks: O = alpha A B (FP64 storage, as
// k_huge_zgemm<double2>) with double-float arithmetic on the FP32 pipe: operands split into
// hi + lo floats as they are staged, each output a compensated complex dot product (cdf_mac),
// rounded to FP64 once at the end (~2^-44 relative against FP64's 2^-53).
__global__ void __launch_bounds__(kHThreads) k_huge_zgemm_df(HMat<const double2> A, HMat<const double2> B,
                                                            HMat<double2> O, int m, int n, int k, int Cb, long j0,
                                                            double alpha) {
  __shared__ float4 As[kHK][kHT + 1], Bs[kHK][kHT + 1];
  const long g = j0 + blockIdx.y;
  const int c = int(g % Cb), sl = int(g / Cb);
  const int tn = (n + kHT - 1) / kHT;
  const int r0 = (blockIdx.x / tn) * kHT, q0 = (blockIdx.x % tn) * kHT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  CdfAcc acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = CdfAcc{{0.f, 0.f}, {0.f, 0.f}};
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k0 = 0; k0 < k; k0 += kHK) {
    for (int idx = threadIdx.x; idx < kHT * kHK; idx += kHThreads) {
      const int rr = idx / kHK, kk = idx % kHK, r = r0 + rr, l = k0 + kk;
      As[kk][rr] = (r < m && l < k) ? df_store(A(c, sl, r, l)) : z4;
      const int kb = idx / kHT, qq = idx % kHT, lb = k0 + kb, q = q0 + qq;
      Bs[kb][qq] = (lb < k && q < n) ? df_store(B(c, sl, lb, q)) : z4;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kHK; ++kk) {
      float4 a[4], b[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) a[t] = As[kk][ty + 16 * t], b[t] = Bs[kk][tx + 16 * t];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) cdf_mac(acc[x][y], a[x], b[y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int r = r0 + ty + 16 * x, q = q0 + tx + 16 * y;
      if (r < m && q < n) O(c, sl, r, q) = cscale(df_load(cdf_fin(acc[x][y])), alpha);
    }
}

// Arguments of k_huge_sym: workspace of kHugeSlots real b x b matrices per item (slot t of
// item j at ws + (j*kHugeSlots + t)*bb) and per-item scale sc_j = 2 pi tau 2^-sq_j.
struct SymArgs {
  double *ws;
  const double *sc;
  const int *sq;
  long bb;
  int b, a, bsl, o;  // operand and output slots
  int akind;         // alpha: 0 -> alpha, 1 -> sc_j^2, 2 -> -sc_j
  double alpha;
  int round;         // >= 0: squaring round, items with sq_j <= round are skipped
  int low;           // epilogue adds c0 I + c1 Y + c2 Y2 + c3 Y3 (slots 1, 2, 3)
  double c0, c1, c2, c3;
};

// O = alpha_j A B (+ low terms) for commuting real symmetric A, B of item j (blockIdx.y):
// upper-triangle tiles only, each value stored at (r, q) and (q, r).  The low terms are read
// at the upper element only, so S may overwrite Y3 in place.
__global__ void __launch_bounds__(kHThreads) k_huge_sym(SymArgs g) {
  __shared__ double As[kHK][kHT + 1], Bs[kHK][kHT + 1];
  const int j = blockIdx.y;
  if (g.round >= 0 && g.sq[j] <= g.round) return;
  const int b = g.b, tm = (b + kHT - 1) / kHT;
  int ti, tj;
  sym_tile(blockIdx.x, tm, ti, tj);
  const int r0 = ti * kHT, q0 = tj * kHT;
  double *base = g.ws + long(j) * kHugeSlots * g.bb;
  const double *A = base + g.a * g.bb, *B = base + g.bsl * g.bb;
  double *O = base + g.o * g.bb;
  const double *Y = base + g.bb, *Y2 = base + 2 * g.bb, *Y3 = base + 3 * g.bb;
  const double scj = g.sc[j];
  const double alpha = g.akind == 0 ? g.alpha : (g.akind == 1 ? scj * scj : -scj);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = 0.0;
  for (int k0 = 0; k0 < b; k0 += kHK) {
    for (int idx = threadIdx.x; idx < kHT * kHK; idx += kHThreads) {
      const int rr = idx / kHK, kk = idx % kHK, r = r0 + rr, l = k0 + kk;
      As[kk][rr] = (r < b && l < b) ? A[long(r) * b + l] : 0.0;
      const int kb = idx / kHT, qq = idx % kHT, lb = k0 + kb, q = q0 + qq;
      Bs[kb][qq] = (lb < b && q < b) ? B[long(lb) * b + q] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kHK; ++kk) {
      double a[4], bv[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) a[t] = As[kk][ty + 16 * t], bv[t] = Bs[kk][tx + 16 * t];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], bv[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int r = r0 + ty + 16 * x, q = q0 + tx + 16 * y;
      if (r >= b || q >= b || r > q) continue;  // upper triangle (r > q only on diagonal tiles)
      const long e = long(r) * b + q;
      double v = alpha * acc[x][y];
      if (g.low) v += fma(g.c3, Y3[e], fma(g.c2, Y2[e], fma(g.c1, Y[e], r == q ? g.c0 : 0.0)));
      O[e] = v;
      if (r != q) O[long(q) * b + r] = v;
    }
}

// k_huge_sym with double-float arithmetic (the mixed form): FP64 workspace, operands split
// into hi + lo floats as they are staged, compensated dot products, the FP64 epilogue of
// k_huge_sym (scale, low terms, mirrored store).
__global__ void __launch_bounds__(kHThreads) k_huge_sym_df(SymArgs g) {
  __shared__ float2 As[kHK][kHT + 1], Bs[kHK][kHT + 1];
  const int j = blockIdx.y;
  if (g.round >= 0 && g.sq[j] <= g.round) return;
  const int b = g.b, tm = (b + kHT - 1) / kHT;
  int ti, tj;
  sym_tile(blockIdx.x, tm, ti, tj);
  const int r0 = ti * kHT, q0 = tj * kHT;
  double *base = g.ws + long(j) * kHugeSlots * g.bb;
  const double *A = base + g.a * g.bb, *B = base + g.bsl * g.bb;
  double *O = base + g.o * g.bb;
  const double *Y = base + g.bb, *Y2 = base + 2 * g.bb, *Y3 = base + 3 * g.bb;
  const double scj = g.sc[j];
  const double alpha = g.akind == 0 ? g.alpha : (g.akind == 1 ? scj * scj : -scj);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  DfAcc acc[4][4];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = DfAcc{0.f, 0.f};
  const float2 z2 = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < b; k0 += kHK) {
    for (int idx = threadIdx.x; idx < kHT * kHK; idx += kHThreads) {
      const int rr = idx / kHK, kk = idx % kHK, r = r0 + rr, l = k0 + kk;
      As[kk][rr] = (r < b && l < b) ? dfv_of(A[long(r) * b + l]) : z2;
      const int kb = idx / kHT, qq = idx % kHT, lb = k0 + kb, q = q0 + qq;
      Bs[kb][qq] = (lb < b && q < b) ? dfv_of(B[long(lb) * b + q]) : z2;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kHK; ++kk) {
      float2 a[4], bv[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) a[t] = As[kk][ty + 16 * t], bv[t] = Bs[kk][tx + 16 * t];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) df_dot(acc[x][y], a[x].x, a[x].y, bv[y].x, bv[y].y);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int r = r0 + ty + 16 * x, q = q0 + tx + 16 * y;
      if (r >= b || q >= b || r > q) continue;  // upper triangle (r > q only on diagonal tiles)
      const long e = long(r) * b + q;
      const float2 d = df_fin(acc[x][y]);
      double v = alpha * (double(d.x) + double(d.y));
      if (g.low) v += fma(g.c3, Y3[e], fma(g.c2, Y2[e], fma(g.c1, Y[e], r == q ? g.c0 : 0.0)));
      O[e] = v;
      if (r != q) O[long(q) * b + r] = v;
    }
}

// Interaction coefficients f_k = scale_k (M PAS'_k M^T)_22 of items g = j0 + j, as in
// build_h.
__global__ void k_huge_fk(DevSys s, long j0, int items, double *fk) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= items) return;
  const long g = j0 + j;
  const int c = int(g % s.C), i = int(g / s.C);
  double t1 = s.t0[c] + double(i) * s.tau, t2 = t1 + s.tau;
  double tmid = (t2 - t1) / 2.0 + t1;
  double sp, cp;
  sincos(tmid * s.wr * kPi2, &sp, &cp);
  double m[3][3];
  orient_rows(s, c, sp, cp, m);
  for (int kk = 0; kk < s.nint; ++kk) fk[long(j) * s.nint + kk] = term_coef(s, kk, m);
}

// X = H of block (bp, b): slot 0 of item blockIdx.y.
__global__ void k_huge_hbuild(DevSys s, int bp, int b, const double *fk, double *ws, long j0) {
  const long bb = long(b) * b, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (e >= bb) return;
  double h = hc_of(s, int((j0 + j) / s.C))[bp + e];
  const double *f = fk + long(j) * s.nint;
  for (int kk = 0; kk < s.nint; ++kk) {
    const double t = s.Tk[size_t(kk) * s.S2 + bp + e];
    if (t != 0.0) h = fma(f[kk], t, h);
  }
  ws[long(j) * kHugeSlots * bb + e] = h;
}

// Per item: ||2 pi tau H||_inf -> squarings sq_j (so that the scaled norm is <= 1/2) and
// sc_j = 2 pi tau 2^-sq_j; the largest sq of the launch into *sq_max.
__global__ void __launch_bounds__(256) k_huge_norm(const double *ws, int b, double tp, double *sc, int *sq,
                                                   int *sq_max) {
  __shared__ double red[256];
  const long bb = long(b) * b;
  const int j = blockIdx.x;
  const double *X = ws + long(j) * kHugeSlots * bb;
  double m = 0;
  for (int r = threadIdx.x; r < b; r += blockDim.x) {
    double rs = 0;
    for (int q = 0; q < b; ++q) rs += fabs(X[long(r) * b + q]);
    m = fmax(m, rs);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double nrm = 0;
    for (int t = 0; t < blockDim.x; ++t) nrm = fmax(nrm, red[t]);
    nrm *= tp;
    int q = 0;
    if (nrm > 0.5) {
      frexp(nrm / 0.5, &q);
      q = min(q, 60);
    }
    sc[j] = ldexp(tp, -q);
    sq[j] = q;
    atomicMax(sq_max, q);
  }
}

// T (slot 5) = c0 I + c1 Y + c2 Y2 + c3 Y3, every item.
__global__ void k_huge_low(double *ws, int b, double c0, double c1, double c2, double c3) {
  const long bb = long(b) * b, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= bb) return;
  double *base = ws + long(blockIdx.y) * kHugeSlots * bb;
  const int r = int(e / b), q = int(e % b);
  base[5 * bb + e] = fma(c3, base[3 * bb + e], fma(c2, base[2 * bb + e], fma(c1, base[bb + e], r == q ? c0 : 0.0)));
}

// One squaring round: R = P - Q, I = Z (slots: R 6, I 1, P 2, Q 4, Z 5) for items with sq > round.
__global__ void k_huge_sqcomb(double *ws, int b, const int *sq, int round) {
  const long bb = long(b) * b, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (e >= bb || sq[j] <= round) return;
  double *base = ws + long(j) * kHugeSlots * bb;
  base[6 * bb + e] = base[2 * bb + e] - base[4 * bb + e];
  base[bb + e] = base[5 * bb + e];
}

// U block (bp, b) of item g = j0 + blockIdx.y = R + i I (slots 6 and 1).
__global__ void k_huge_store_u(DevSys s, const double *ws, int bp, int bo, int b, long j0) {
  const long bb = long(b) * b, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (e >= bb) return;
  const long g = j0 + j;
  const int c = int(g % s.C), i = int(g / s.C);
  const double *base = ws + long(j) * kHugeSlots * bb;
  double2 u = cmk(base[6 * bb + e], base[bb + e]);
  const double2 *fr = frame_of(s, i);
  if (fr) u = cmul(cmul(fr[bo + e / b], u), cconj(fr[bo + e % b]));  // lab frame: U = R U' R^H
  s.U[(size_t(i) * s.S2 + bp + e) * s.Cpad + c] = u;
}

// A_1 = U_0 for block (bp, b), crystallite blockIdx.y.
__global__ void k_huge_copy_u0(DevSys s, int bp, int b) {
  const long bb = long(b) * b, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (e >= bb) return;
  const size_t a0 = (size_t(bp) + e) * s.Cpad + c;
  s.A[a0] = s.U[a0];
}

// W of item g = j0 + blockIdx.y = workspace (contiguous b x b per item), back over A in the
// FP64 form.
__global__ void k_huge_copy_back(DevSys s, const double2 *ws, int bp, int b, long j0) {
  const long bb = long(b) * b, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (e >= bb) return;
  const long g = j0 + j;
  const int c = int(g % s.C), i = int(g / s.C);
  s.A[(size_t(i) * s.S2 + bp + e) * s.Cpad + c] = ws[long(j) * bb + e];
}

// X of item g = j0 + blockIdx.y (ba x bb, contiguous) = M_ab W_b(step g / C) from M's
// non-zeros by row.
template <class C>
__global__ void k_huge_mx(DevSys s, BigPair P, long j0, C *ws) {
  const int ba = s.bs[P.a], bb = s.bs[P.b], pb = s.bpoff[P.b];
  const long ne = long(ba) * bb, e = long(blockIdx.x) * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (e >= ne) return;
  const long g = j0 + j;
  const int c = int(g % s.C), i = int(g / s.C);
  const int l = int(e / bb), q = int(e % bb);
  const C *W = Bufs<C>::W(s) + size_t(i) * s.S2 * s.Cpad;
  C x = mkc<C>(0, 0);
  for (int t = P.rp[l]; t < P.rp[l + 1]; ++t) x = cfma(cvt<C>(P.cv[t]), W[at(pb + P.ci[t] * bb + q, c, s.Cpad)], x);
  ws[long(j) * ne + e] = x;
}

constexpr int kHugeFloqThreads = 1024;
constexpr int kHugeFloqSweeps0 = 4;  // first pass: locate the spectrum only
constexpr int kMaxHugeLaunch = 16;   // huge blocks per Floquet launch

__host__ __device__ constexpr size_t huge_floquet_smem(int b) {
  return sizeof(double2) * (2 * size_t(b / 2 + 1) + 2 * size_t(b)) +
         sizeof(double) * size_t(b > kHugeFloqThreads ? b : kHugeFloqThreads) + sizeof(int) * 2 * size_t(b / 2 + 1);
}

// Huge blocks of one Floquet launch and each one's workspace (2 b^2 per crystallite).
struct HugeFloq {
  int n;
  int mats;  // b x b double2 matrices per (crystallite, block): 2, or 3 with the FP32 K
  int k[kMaxHugeLaunch];
  long ws[kMaxHugeLaunch];
};

// One CTA per (crystallite c0 + blockIdx.x, huge block blockIdx.y): Floquet eigen-
// decomposition with its two b x b matrices in the workspace, the small arrays in shared
// memory; all huge blocks of the system in one launch.
__global__ void __launch_bounds__(kHugeFloqThreads) k_huge_floquet(DevSys s, HugeFloq hf, double2 *ws, int c0) {
  extern __shared__ __align__(16) unsigned char fsm[];
  const int k = hf.k[blockIdx.y], b = s.bs[k], c = c0 + blockIdx.x;
  const int np1 = b / 2 + 1;
  double2 *rot = reinterpret_cast<double2 *>(fsm), *fv = rot + 2 * np1, *lam = fv + b;
  double *red = reinterpret_cast<double *>(lam + b);
  int *rpair = reinterpret_cast<int *>(red + (b > kHugeFloqThreads ? b : kHugeFloqThreads));
  double2 *Mm = ws + hf.ws[blockIdx.y] + size_t(blockIdx.x) * hf.mats * b * b;
  if (s.floq32)  // mixed form: FP32 sweeps, double-float Cayley solve, V and Rayleigh quotients
    floquet_cta_df(s, k, c,
                   FloqWork{Mm, Mm + size_t(b) * b, rot, fv, lam, rpair, red,
                            reinterpret_cast<float2 *>(Mm + 2 * size_t(b) * b)},
                   true);
  else
    floquet_cta<false, false>(s, k, c, FloqWork{Mm, Mm + size_t(b) * b, rot, fv, lam, rpair, red, nullptr},
                              kHugeFloqSweeps0);
}
