// Large-block kernels (Hamiltonian blocks of kMaxBlock < b <= kMaxBigBlock), included by
// bl_engine.cu after DevSys and the complex helpers.  One CTA works on one crystallite's
// block with the matrices in shared memory; products are CTA-wide FP64 GEMMs with 2x2
// output tiles, one tile per thread (NT = 1) or two (NT = 2, blocks above 64), and CTAs of
// about one thread per tile so that registers stay low and several CTAs share an SM.
// Same arithmetic as the small-block kernels:
//   k_big_step      (c, step)   H_i, U_i = exp(-i 2pi tau H_i) by Taylor + squaring
//   k_big_dyson     (c)         A_{i+1} = U_i A_i for i < n (A stays in shared memory)
//   k_big_floquet   (c)         A_n = V diag(lam) V^H: Cayley transform, parallel Jacobi
//   k_big_eigframe  (c)         W_i = A_{i+1} V_F for i < n
//   k_big_qr        (c, step) per pair  Q = W_a^H M_ab W_b for block pairs with a big block
// and, for the mixed form, the same step and Dyson in double-float on the FP32 pipe:
//   k_big_step_df   (c, step)   U_i in double-float (the Taylor series term by term)
//   k_big_dyson_df  (c)         A_{i+1} = U_i A_i in double-float

constexpr int kMaxBigBlock = 74;   // 5 real b x b matrices fit 227 KB of shared memory
constexpr int kBigThreads = 256;   // k_big_floquet
constexpr int kBigPSMax = 63;      // 7 real b x b matrices (Paterson-Stockmeyer step) fit
constexpr int kMaxInt = 128;       // interactions per system on the large-block path

// Element e of block (size b, packed offset bp) of crystallite c inside one step's A or W
// array: [item][c] as at(), or, for the large blocks of a crystallite-major job (s.clay), the
// block's region [bp Cpad, (bp + b^2) Cpad) taken as [c][e].
__device__ __forceinline__ size_t big_at(const DevSys &s, int b, int bp, int e, int c) {
  return (s.clay && b > kMaxBlock && b <= kMaxBigBlock) ? size_t(bp) * s.Cpad + size_t(c) * b * b + e
                                                        : size_t(bp + e) * s.Cpad + c;
}

__host__ __device__ constexpr int big_tiles(int m, int n) { return ((m + 1) / 2) * ((n + 1) / 2); }
// tiles per thread of an m x n product, and the CTA size that gives each thread NT tiles
__host__ __device__ constexpr int big_nt(int m, int n) { return big_tiles(m, n) <= 1024 ? 1 : 2; }
__host__ __device__ constexpr int big_threads(int m, int n) {
  return ((big_tiles(m, n) + big_nt(m, n) - 1) / big_nt(m, n) + 31) / 32 * 32;
}

// C (m x n) = alpha * A (m x k) * B (k x n) (+ epilogue), real, shared memory, row-major.
// ep(e, v) returns the value stored at C[e] for the product value v.
template <class EP>
__device__ void cta_mm_real(const double *A, int lda, const double *B, int ldb, double *C, int ldc, int m, int n,
                            int k, double alpha, EP ep) {
  const int tm = (m + 1) / 2, tn = (n + 1) / 2;
  for (int t = threadIdx.x; t < tm * tn; t += blockDim.x) {
    const int i0 = (t / tn) * 2, j0 = (t % tn) * 2;
    const int i1 = min(i0 + 1, m - 1), j1 = min(j0 + 1, n - 1);
    double c00 = 0, c01 = 0, c10 = 0, c11 = 0;
    for (int l = 0; l < k; ++l) {
      const double a0 = A[i0 * lda + l], a1 = A[i1 * lda + l];
      const double b0 = B[l * ldb + j0], b1 = B[l * ldb + j1];
      c00 = fma(a0, b0, c00), c01 = fma(a0, b1, c01), c10 = fma(a1, b0, c10), c11 = fma(a1, b1, c11);
    }
    C[i0 * ldc + j0] = ep(i0 * ldc + j0, alpha * c00);
    if (j0 + 1 < n) C[i0 * ldc + j0 + 1] = ep(i0 * ldc + j0 + 1, alpha * c01);
    if (i0 + 1 < m) {
      C[(i0 + 1) * ldc + j0] = ep((i0 + 1) * ldc + j0, alpha * c10);
      if (j0 + 1 < n) C[(i0 + 1) * ldc + j0 + 1] = ep((i0 + 1) * ldc + j0 + 1, alpha * c11);
    }
  }
}
__device__ __forceinline__ void cta_mm_real(const double *A, int lda, const double *B, int ldb, double *C, int ldc,
                                            int m, int n, int k, double alpha) {
  cta_mm_real(A, lda, B, ldb, C, ldc, m, n, k, alpha, [](int, double v) { return v; });
}

// Upper-triangle 2x2 tiles of an m x m matrix: tile t -> (ti, tj), ti <= tj, t < big_sym_tiles.
// Rows pr and tm-1-pr together hold tm+1 tiles; an odd tm's middle row comes last.
__host__ __device__ constexpr int big_sym_tiles(int m) { return ((m + 1) / 2) * ((m + 1) / 2 + 1) / 2; }
__device__ __forceinline__ void sym_tile(int t, int tm, int &ti, int &tj) {
  const int h = tm / 2, pr = t / (tm + 1), q = t % (tm + 1);
  if (pr < h) {
    if (q < tm - pr) ti = pr, tj = pr + q;
    else ti = tm - 1 - pr, tj = ti + (q - (tm - pr));
  } else {
    ti = h, tj = h + (t - h * (tm + 1));
  }
}

// C = alpha * A * B (+ epilogue) for m x m real A, B that are symmetric and commute, so
// that C is symmetric: only upper-triangle tiles are computed, each value stored at (i, j)
// and (j, i).  ep(e, v) gives the stored value for the upper element e = i*m + j (called
// once per upper element, by the thread that stores it and its mirror).
template <class EP>
__device__ void cta_mm_sym(const double *A, const double *B, double *C, int m, double alpha, EP ep) {
  const int tm = (m + 1) / 2;
  for (int t = threadIdx.x; t < big_sym_tiles(m); t += blockDim.x) {
    int ti, tj;
    sym_tile(t, tm, ti, tj);
    const int i0 = 2 * ti, j0 = 2 * tj;
    const int i1 = min(i0 + 1, m - 1), j1 = min(j0 + 1, m - 1);
    double c00 = 0, c01 = 0, c10 = 0, c11 = 0;
    for (int l = 0; l < m; ++l) {
      const double a0 = A[i0 * m + l], a1 = A[i1 * m + l];
      const double b0 = B[l * m + j0], b1 = B[l * m + j1];
      c00 = fma(a0, b0, c00), c01 = fma(a0, b1, c01), c10 = fma(a1, b0, c10), c11 = fma(a1, b1, c11);
    }
    auto put = [&](int i, int j, double v) {
      const double x = ep(i * m + j, alpha * v);
      C[i * m + j] = x;
      if (i != j) C[j * m + i] = x;
    };
    put(i0, j0, c00);
    if (j0 + 1 < m) put(i0, j0 + 1, c01);
    if (i0 + 1 < m) {
      if (ti != tj) put(i0 + 1, j0, c10);  // on a diagonal tile (i0+1, i0) mirrors c01
      if (j0 + 1 < m) put(i0 + 1, j0 + 1, c11);
    }
  }
}
__device__ __forceinline__ void cta_mm_sym(const double *A, const double *B, double *C, int m, double alpha) {
  cta_mm_sym(A, B, C, m, alpha, [](int, double v) { return v; });
}

// Complex 2x2-tiled product into per-thread registers: acc[q] for the tiles
// t = threadIdx.x + q*blockDim.x.  CONJ_A: use A^H (A stored k x m).
template <int NT, bool CONJ_A, class C>
__device__ void cta_mm_cplx_regs(const C *A, int lda, const C *B, int ldb, int m, int n, int k, C (&acc)[NT][4]) {
  const int tm = (m + 1) / 2, tn = (n + 1) / 2;
#pragma unroll
  for (int q = 0; q < NT; ++q) {
    const int t = threadIdx.x + q * blockDim.x;
    acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = mkc<C>(0, 0);
    if (t >= tm * tn) continue;
    const int i0 = (t / tn) * 2, j0 = (t % tn) * 2;
    const int i1 = min(i0 + 1, m - 1), j1 = min(j0 + 1, n - 1);
    C c00 = mkc<C>(0, 0), c01 = c00, c10 = c00, c11 = c00;
    for (int l = 0; l < k; ++l) {
      C a0, a1;
      if (CONJ_A) {
        a0 = cconj(A[l * lda + i0]), a1 = cconj(A[l * lda + i1]);
      } else {
        a0 = A[i0 * lda + l], a1 = A[i1 * lda + l];
      }
      const C b0 = B[l * ldb + j0], b1 = B[l * ldb + j1];
      c00 = cfma(a0, b0, c00), c01 = cfma(a0, b1, c01), c10 = cfma(a1, b0, c10), c11 = cfma(a1, b1, c11);
    }
    acc[q][0] = c00, acc[q][1] = c01, acc[q][2] = c10, acc[q][3] = c11;
  }
}

// Visits this thread's tile outputs: f(row, col, value).
template <int NT, class C, class F>
__device__ void cta_tiles_store(int m, int n, const C (&acc)[NT][4], F f) {
  const int tm = (m + 1) / 2, tn = (n + 1) / 2;
#pragma unroll
  for (int q = 0; q < NT; ++q) {
    const int t = threadIdx.x + q * blockDim.x;
    if (t >= tm * tn) continue;
    const int i0 = (t / tn) * 2, j0 = (t % tn) * 2;
    f(i0, j0, acc[q][0]);
    if (j0 + 1 < n) f(i0, j0 + 1, acc[q][1]);
    if (i0 + 1 < m) {
      f(i0 + 1, j0, acc[q][2]);
      if (j0 + 1 < n) f(i0 + 1, j0 + 1, acc[q][3]);
    }
  }
}

// Shared memory of k_big_step for a block of size b.
__host__ __device__ constexpr size_t big_step_smem(int b) {
  return sizeof(double) * size_t(b <= kBigPSMax ? 7 : 5) * size_t(b) * size_t(b);
}

// One CTA per (crystallite, step): U_i of a large block, exp(-iX) with X = 2pi tau H_i / 2^sq
// (||X||_inf <= 1/2) by its Taylor polynomial, then sq squarings.  Blocks above kBigPSMax
// sum the series term by term up to the degree taylor_degree gives for the step's norm.
// Blocks up to kBigPSMax evaluate the polynomial as cos X = C(Y), sin X = X S(Y), Y = X^2,
// C and S of degree 7 in Y by Paterson-Stockmeyer with Y^4 (Y, Y^2, Y^3, Y^4, C, S, X S:
// 7 real products); larger blocks accumulate the terms one product at a time (14).  All
// factors are polynomials in X, hence symmetric and commuting: products are symmetric
// and only their upper triangles are computed (cta_mm_sym).
__global__ void __launch_bounds__(1024) k_big_step(DevSys s, int k) {
  extern __shared__ double bsm[];
  __shared__ double fk[kMaxInt];
  __shared__ double red[kMaxBigBlock];
  __shared__ double scl[3];
  const int c = blockIdx.x % s.C, i = blockIdx.x / s.C;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  if (s.fk && !s.fk_df) {  // k_coef's coefficients (same arithmetic), read in parallel
    for (int kk = threadIdx.x; kk < s.nint; kk += blockDim.x) fk[kk] = s.fk[at(i * s.nint + kk, c, s.Cpad)];
  } else if (threadIdx.x == 0) {
    double t1 = s.t0[c] + double(i) * s.tau, t2 = t1 + s.tau;
    double tmid = (t2 - t1) / 2.0 + t1;
    double sp, cp;
    sincos(tmid * s.wr * kPi2, &sp, &cp);
    double m[3][3];
    orient_rows(s, c, sp, cp, m);
    for (int kk = 0; kk < s.nint; ++kk) fk[kk] = term_coef(s, kk, m);
  }
  __syncthreads();
  double *X = bsm;
  const double *Hcb = hc_of(s, i) + bp;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) {
    double h = Hcb[e];
    for (int kk = 0; kk < s.nint; ++kk) {
      const double t = s.Tk[size_t(kk) * s.S2 + bp + e];
      if (t != 0.0) h = fma(fk[kk], t, h);
    }
    X[e] = h;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < b; p += blockDim.x) {
    double rs = 0;
    for (int q = 0; q < b; ++q) rs += fabs(X[p * b + q]);
    red[p] = rs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double nrm = 0;
    for (int p = 0; p < b; ++p) nrm = fmax(nrm, red[p]);
    const double tp = s.tau * kPi2;
    nrm *= tp;
    int sq = 0;
    if (nrm > 0.5) {
      frexp(nrm / 0.5, &sq);
      sq = min(sq, 60);
    }
    scl[0] = ldexp(tp, -sq);
    scl[1] = double(sq);
    scl[2] = double(taylor_degree(ldexp(nrm, -sq), s.mixed != 0));  // terms the series needs
  }
  __syncthreads();
  const double sc = scl[0];
  const int sq = int(scl[1]), nterms = int(scl[2]);
  double *R, *I, *F0, *F1, *F2;  // result R + iI and three free b x b buffers for squaring
  if (b <= kBigPSMax) {
    double *Y = X + bb, *Y2 = Y + bb, *Y3 = Y2 + bb, *Y4 = Y3 + bb, *T = Y4 + bb;
    R = T + bb;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) X[e] *= sc;
    __syncthreads();
    cta_mm_sym(X, X, Y, b, 1.0);
    __syncthreads();
    cta_mm_sym(Y, Y, Y2, b, 1.0);
    __syncthreads();
    cta_mm_sym(Y2, Y, Y3, b, 1.0);
    cta_mm_sym(Y2, Y2, Y4, b, 1.0);
    // c0 I + c1 Y + c2 Y^2 + c3 Y^3 at element e; cos: (-1)^j / (2j)!, sin: (-1)^j / (2j+1)!
    auto low = [&](double c0, double c1, double c2, double c3, int e) {
      const double d = (e / b == e % b) ? c0 : 0.0;
      return fma(c3, Y3[e], fma(c2, Y2[e], fma(c1, Y[e], d)));
    };
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x)
      T[e] = low(1.0 / 40320, -1.0 / 3628800, 1.0 / 479001600, -1.0 / 87178291200.0, e);
    __syncthreads();
    cta_mm_sym(Y4, T, R, b, 1.0,
                [&](int e, double v) { return v + low(1.0, -1.0 / 2, 1.0 / 24, -1.0 / 720, e); });
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x)
      T[e] = low(1.0 / 362880, -1.0 / 39916800, 1.0 / 6227020800.0, -1.0 / 1307674368000.0, e);
    __syncthreads();
    // S(Y) over Y3 in place: element e's epilogue reads Y3[e] before the same thread writes it
    cta_mm_sym(Y4, T, Y3, b, 1.0,
                [&](int e, double v) { return v + low(1.0, -1.0 / 6, 1.0 / 120, -1.0 / 5040, e); });
    __syncthreads();
    I = Y;  // -sin X = -X S(Y)
    cta_mm_sym(X, Y3, I, b, -1.0);
    F0 = Y2, F1 = Y4, F2 = T;
  } else {
    double *P = X + bb, *Q = P + bb;
    R = Q + bb, I = R + bb;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const double x = sc * X[e];
      X[e] = x, P[e] = x;
      R[e] = (e / b == e % b) ? 1.0 : 0.0;
      I[e] = -x;
    }
    __syncthreads();
    for (int kt = 2; kt <= nterms; ++kt) {  // the degree the step's norm needs (<= 15)
      cta_mm_sym(P, X, Q, b, 1.0 / kt);
      __syncthreads();
      const int m4 = kt & 3;
      for (int e = threadIdx.x; e < bb; e += blockDim.x) {
        const double v = Q[e];
        if (m4 == 2) R[e] -= v;
        else if (m4 == 3) I[e] += v;
        else if (m4 == 0) R[e] += v;
        else I[e] -= v;
      }
      double *t = P;
      P = Q, Q = t;
      __syncthreads();
    }
    F0 = P, F1 = Q, F2 = X;
  }
  __syncthreads();
  for (int t = 0; t < sq; ++t) {  // (R + iI)^2 = (RR - II) + i 2RI
    cta_mm_sym(R, R, F0, b, 1.0);
    cta_mm_sym(I, I, F1, b, 1.0);
    cta_mm_sym(R, I, F2, b, 2.0);
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x) R[e] = F0[e] - F1[e], I[e] = F2[e];
    __syncthreads();
  }
  double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
  const double2 *fr = frame_of(s, i);
  if (fr) {  // lab frame of a chunk rf phase: U = R U' R^H
    const int bo = s.boff[k];
    for (int e = threadIdx.x; e < bb; e += blockDim.x)
      Ub[at(bp + e, c, s.Cpad)] = cmul(cmul(fr[bo + e / b], cmk(R[e], I[e])), cconj(fr[bo + e % b]));
  } else {
    for (int e = threadIdx.x; e < bb; e += blockDim.x) Ub[at(bp + e, c, s.Cpad)] = cmk(R[e], I[e]);
  }
}

// One CTA per crystallite: A_{i+1} = U_i A_i for all steps; A lives in shared memory.
template <int NT>
__global__ void __launch_bounds__(NT == 1 ? 1024 : 768) k_big_dyson(DevSys s, int k) {
  extern __shared__ double2 bsc[];
  const int c = blockIdx.x;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  double2 *Us = bsc, *As = Us + bb;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) As[e] = cmk(e / b == e % b ? 1.0 : 0.0, 0.0);
  double2 acc[NT][4];
  for (int i = 0; i < s.n; ++i) {
    const double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) Us[e] = Ub[at(bp + e, c, s.Cpad)];
    __syncthreads();
    cta_mm_cplx_regs<NT, false, double2>(Us, b, As, b, b, b, b, acc);
    __syncthreads();
    double2 *Ab = s.A + size_t(i) * s.S2 * s.Cpad;
    cta_tiles_store<NT>(b, b, acc, [&](int r, int q, double2 v) {
      As[r * b + q] = v;
      Ab[at(bp + r * b + q, c, s.Cpad)] = v;
    });
    __syncthreads();
  }
}

// One CTA per crystallite: W_i = A_{i+1} V_F (in place over A in FP64; into the
// single-precision W array in the mixed form).
template <int NT, class C>
__global__ void __launch_bounds__(NT == 1 ? 1024 : 768) k_big_eigframe(DevSys s, int k) {
  extern __shared__ __align__(16) unsigned char bsr[];
  const int c = blockIdx.x;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  C *Vs = reinterpret_cast<C *>(bsr), *As = Vs + bb;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) Vs[e] = cvt<C>(s.VF[at(bp + e, c, s.Cpad)]);
  C acc[NT][4];
  for (int i = 0; i < s.n; ++i) {
    const double2 *Ab = s.A + size_t(i) * s.S2 * s.Cpad;
    C *Wb = Bufs<C>::W(s) + size_t(i) * s.S2 * s.Cpad;
    const float4 *Ab4 = reinterpret_cast<const float4 *>(Ab);  // mixed form: double-float A, high parts
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      if (s.mixed) {
        const float4 v = Ab4[big_at(s, b, bp, e, c)];
        As[e] = mkc<C>(v.x, v.y);
      } else {
        As[e] = cvt<C>(Ab[at(bp + e, c, s.Cpad)]);
      }
    }
    __syncthreads();
    cta_mm_cplx_regs<NT, false, C>(As, b, Vs, b, b, b, b, acc);
    cta_tiles_store<NT>(b, b, acc, [&](int r, int q, C v) { Wb[big_at(s, b, bp, r * b + q, c)] = v; });
    __syncthreads();
  }
}

// One big Q/R block pair as the kernel sees it: blocks a, b, the output offset, and the
// non-zeros of M_ab (D or rho) by row: row l holds entries [rp[l], rp[l+1]) of (ci, cv).
struct BigPair {
  int a, b, off, nitems, isq, wchunk;
  const int *rp, *ci;
  const double2 *cv;
};

// Shared memory of k_big_qr: W_a, a column chunk of W_b and of X = M_ab W_b.
template <class C>
__host__ __device__ constexpr size_t big_qr_smem(int ba, int bb, int w) {
  return sizeof(C) * (size_t(ba) * ba + size_t(bb) * w + size_t(ba) * w);
}

// One CTA per (crystallite, step) of one block pair: Q^{ab} = W_a^H (M_ab W_b), M = D (or
// rho), over column chunks of width wchunk; M's non-zeros come from the host.
template <int NT, class C>
__global__ void __launch_bounds__(NT == 1 ? 1024 : 768) k_big_qr(DevSys s, BigPair bp2) {
  extern __shared__ __align__(16) unsigned char bsr[];
  const int c = blockIdx.x % s.C, i = blockIdx.x / s.C;
  const int ba = s.bs[bp2.a], bb = s.bs[bp2.b], pa = s.bpoff[bp2.a], pb = s.bpoff[bp2.b];
  const int w = bp2.wchunk;
  C *out = bp2.isq ? Bufs<C>::Q(s) : Bufs<C>::R(s);
  const C *W = Bufs<C>::W(s) + size_t(i) * s.S2 * s.Cpad;
  C *Wa = reinterpret_cast<C *>(bsr), *Wb = Wa + ba * ba, *X = Wb + bb * w;
  for (int e = threadIdx.x; e < ba * ba; e += blockDim.x) Wa[e] = W[big_at(s, ba, pa, e, c)];
  C *ob = out + size_t(i) * bp2.nitems * s.Cpad;
  C acc[NT][4];
  for (int q0 = 0; q0 < bb; q0 += w) {
    const int wc = min(w, bb - q0);
    for (int e = threadIdx.x; e < bb * wc; e += blockDim.x) {
      const int m = e / wc, q = e % wc;
      Wb[e] = W[big_at(s, bb, pb, m * bb + q0 + q, c)];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ba * wc; e += blockDim.x) {
      const int l = e / wc, q = e % wc;
      C x = mkc<C>(0, 0);
      for (int j = __ldg(bp2.rp + l); j < __ldg(bp2.rp + l + 1); ++j)
        x = cfma(cvt<C>(__ldg(bp2.cv + j)), Wb[__ldg(bp2.ci + j) * wc + q], x);
      X[e] = x;
    }
    __syncthreads();
    cta_mm_cplx_regs<NT, true, C>(Wa, ba, X, wc, ba, wc, ba, acc);
    cta_tiles_store<NT>(ba, wc, acc, [&](int r, int q, C v) { ob[at(bp2.off + r * bb + q0 + q, c, s.Cpad)] = v; });
    __syncthreads();
  }
}

// One CTA per crystallite: unitary eigen-decomposition of a block of A_n by the Cayley
// transform K = i (I+W)^{-1}(I-W), W = e^{ia} A_n, and a parallel (round-robin) complex
// Jacobi on K; a second pass moves -1 into the widest spectral gap when the first is ill
// conditioned.  Work arrays of floquet_cta: Mm, Xk (b x b each), rot and rpair ((b/2+1) x 2),
// fv and lam (b each), red (max(b, blockDim.x)); in shared memory for blocks up to
// kMaxBigBlock, Mm and Xk in global memory above.
struct FloqWork {
  double2 *Mm, *Xk, *rot, *fv, *lam;
  int *rpair;
  double *red;
  float2 *Kf;  // MIX: b x b single-precision K
};

// The parallel Jacobi sweeps of floquet_cta over K (Xk, element type KC) with V (Mm, FP64)
// accumulating the rotations; returns convergence.  KC = double2: the FP64 form.  KC =
// float2 (mixed form): K in single precision, the sweeps stop one sweep after
// off(K)^2 <= 1e-10 diag(K)^2, and each rotation is scaled to c^2 + |s|^2 = 1 in FP64
// before V takes it, so that V stays unitary to FP64 rounding.
template <class KC>
__device__ bool floquet_sweeps(KC *Xk, double2 *Mm, int b, int max_sweeps, const FloqWork &wk) {
  using R = decltype(KC::x);
  constexpr bool F32 = sizeof(R) == sizeof(float);
  auto rot = [&](int t, int q) -> double2 & { return wk.rot[2 * t + q]; };
  auto rpair = [&](int t, int q) -> int & { return wk.rpair[2 * t + q]; };
  double *red = wk.red;
  const int bb = b * b;
  const int bq = b + (b & 1);  // players in the round-robin (one dummy when b is odd)
  const int np = bq / 2;
  bool conv = false, polish = false;
  const int nw = (blockDim.x + 31) / 32, wid = threadIdx.x >> 5, lid = threadIdx.x & 31;
  for (int sweep = 0; sweep < max_sweeps && !conv; ++sweep) {
    // off(K)^2 and diag(K)^2: FP64 sums per thread, a fixed shuffle tree per warp, the warps'
    // sums added by one thread
    double off = 0, dg = 0;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const int r = e / b, q = e % b;
      const double2 v = todbl(Xk[e]);
      if (r < q) off += v.x * v.x + v.y * v.y;
      else if (r == q) dg += v.x * v.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dg += __shfl_xor_sync(0xffffffffu, dg, o);
    }
    if (lid == 0) red[2 * wid] = off, red[2 * wid + 1] = dg;
    __syncthreads();
    if (threadIdx.x == 0) {
      double so = 0, sd = 0;
      for (int t = 0; t < nw; ++t) so += red[2 * t], sd += red[2 * t + 1];
      red[2 * nw] = so, red[2 * nw + 1] = sd;
    }
    __syncthreads();
    const double offs = red[2 * nw], dgs = red[2 * nw + 1];
    __syncthreads();
    if (F32) {  // offs, dgs are the same in every thread: polish too
      const bool small = offs <= 1e-10 * dgs || offs == 0.0;
      if (small && (polish || offs == 0.0)) {
        conv = true;
        break;
      }
      polish = polish || small;
    } else if (offs <= 1e-34 * dgs || offs == 0.0) {
      conv = true;
      break;
    }
    for (int round = 0; round < bq - 1; ++round) {
      for (int t = threadIdx.x; t < np; t += blockDim.x) {
        auto player = [&](int j) { return j == 0 ? 0 : 1 + (j - 1 + round) % (bq - 1); };
        int p = player(t), q = player(bq - 1 - t);
        if (p > q) {
          int tmp = p;
          p = q, q = tmp;
        }
        rpair(t, 0) = p, rpair(t, 1) = q;
        rot(t, 0) = cmk(1, 0), rot(t, 1) = cmk(0, 0);
        if (q < b) {
          const KC hpq = Xk[p * b + q];
          const R ab = hypot(hpq.x, hpq.y);
          if (ab != R(0)) {
            const R phx = hpq.x / ab, phy = hpq.y / ab;
            const R theta = R(0.5) * (Xk[q * b + q].x - Xk[p * b + p].x) / ab;
            R tt;
            if (fabs(theta) > R(F32 ? 1e18 : 1e100)) tt = R(0.5) / theta;  // theta^2 stays finite
            else tt = copysign(R(1), theta) / (fabs(theta) + sqrt(fma(theta, theta, R(1))));
            const R cc = rsqrt(fma(tt, tt, R(1)));
            double cd = cc;
            double2 sd = cmk(double(phx * (tt * cc)), double(phy * (tt * cc)));
            if (F32) {
              const double nn = 1.0 / sqrt(fma(cd, cd, fma(sd.x, sd.x, sd.y * sd.y)));
              cd *= nn, sd = cscale(sd, nn);
            }
            rot(t, 0) = cmk(cd, 0.0);
            rot(t, 1) = sd;
          }
        }
      }
      __syncthreads();
      // columns p, q of K and V:  K <- K G, V <- V G  with G = [[c, sp], [-conj(sp), c]];
      // the pair index runs fastest, so a warp's accesses stay within one row of K (or V)
      for (int e = threadIdx.x; e < np * b * 2; e += blockDim.x) {
        const int t = e % np, rest = e / np, kk = rest % b;
        const int p = rpair(t, 0), q = rpair(t, 1);
        if (q >= b) continue;
        const double cc = rot(t, 0).x;
        const double2 sp = rot(t, 1), spc = cconj(sp);
        if (rest < b) {
          const R ccr = R(cc);
          const KC spr = cxm(R(sp.x), R(sp.y)), spcr = cxm(R(spc.x), R(spc.y));
          const KC xkp = Xk[kk * b + p], xkq = Xk[kk * b + q];
          Xk[kk * b + p] = csub(cscale(xkp, ccr), cmul(spcr, xkq));
          Xk[kk * b + q] = cadd(cmul(spr, xkp), cscale(xkq, ccr));
        } else {
          const double2 xkp = Mm[kk * b + p], xkq = Mm[kk * b + q];
          Mm[kk * b + p] = csub(cscale(xkp, cc), cmul(spc, xkq));
          Mm[kk * b + q] = cadd(cmul(sp, xkp), cscale(xkq, cc));
        }
      }
      __syncthreads();
      // rows p, q of K:  K <- G^H K; a non-trivial rotation then zeroes K_pq, K_qp and the
      // imaginary parts of K_pp, K_qq (written by the items of columns p and q)
      for (int e = threadIdx.x; e < np * b; e += blockDim.x) {
        const int t = e / b, kk = e % b;
        const int p = rpair(t, 0), q = rpair(t, 1);
        if (q >= b) continue;
        const R cc = R(rot(t, 0).x);
        const KC sp = cxm(R(rot(t, 1).x), R(rot(t, 1).y)), spc = cconj(sp);
        const KC xpk = Xk[p * b + kk], xqk = Xk[q * b + kk];
        KC np_ = csub(cscale(xpk, cc), cmul(sp, xqk)), nq_ = cadd(cmul(spc, xpk), cscale(xqk, cc));
        if ((kk == p || kk == q) && !(rot(t, 1).x == 0.0 && rot(t, 1).y == 0.0)) {
          if (kk == p) np_.y = R(0), nq_ = cxm(R(0), R(0));
          else np_ = cxm(R(0), R(0)), nq_.y = R(0);
        }
        Xk[p * b + kk] = np_;
        Xk[q * b + kk] = nq_;
      }
      __syncthreads();
    }
  }
  return conv;
}

// sweeps0 < kMaxSweeps: the first pass only locates the spectrum (that many sweeps); the
// second pass, with -1 in the widest gap of those eigenphases, always follows.  DFA: A_n is
// double-float (mixed form).  K32: the sweeps run over a single-precision K (wk.Kf); the
// eigenvalues stay FP64 Rayleigh quotients, whose error is quadratic in V's.
template <bool DFA, bool K32>
__device__ void floquet_cta(const DevSys &s, int k, int c, FloqWork wk, int sweeps0 = kMaxSweeps) {
  constexpr bool dfA = DFA;
  __shared__ int piv_s;
  __shared__ double a_s;
  __shared__ int done_s;
  const int b = s.bs[k], bp = s.bpoff[k], bo = s.boff[k], bb = b * b;
  double2 *Mm = wk.Mm, *Xk = wk.Xk, *fv = wk.fv, *lam = wk.lam;
  double *red = wk.red;
  const double2 *U = s.A + size_t(s.n - 1) * s.S2 * s.Cpad;  // U(r,q) = U[at(bp + r*b + q, c)]
  const float4 *U4 = reinterpret_cast<const float4 *>(U);      // dfA: double-float A (mixed form)
  auto Ug = [&](int r, int q) {
    return dfA ? df_load(U4[big_at(s, b, bp, r * b + q, c)]) : U[big_at(s, b, bp, r * b + q, c)];
  };
  if (threadIdx.x == 0) a_s = 0.5, done_s = 0;
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    double sa, ca;
    sincos(a_s, &sa, &ca);
    const double2 ea = cmk(ca, sa);
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const double2 w = cmul(ea, Ug(e / b, e % b));
      const double id = (e / b == e % b) ? 1.0 : 0.0;
      Mm[e] = cmk(id + w.x, w.y);
      Xk[e] = cmk(id - w.x, -w.y);
    }
    __syncthreads();
    // Gaussian elimination with partial pivoting: Mm Xk' = Xk
    for (int kc = 0; kc < b; ++kc) {
      if (threadIdx.x == 0) {
        int pv = kc;
        double best = -1;
        for (int r = kc; r < b; ++r) {
          const double2 v = Mm[r * b + kc];
          const double m2 = v.x * v.x + v.y * v.y;
          if (m2 > best) best = m2, pv = r;
        }
        piv_s = pv;
        if (best == 0.0) atomicOr(s.status, kSingularCayley);
      }
      __syncthreads();
      const int pv = piv_s;
      if (pv != kc)
        for (int j = threadIdx.x; j < 2 * b; j += blockDim.x) {
          double2 *Mx = j < b ? Mm : Xk;
          const int jj = j < b ? j : j - b;
          const double2 t = Mx[kc * b + jj];
          Mx[kc * b + jj] = Mx[pv * b + jj];
          Mx[pv * b + jj] = t;
        }
      __syncthreads();
      const double2 inv = cdiv(cmk(1, 0), Mm[kc * b + kc]);
      for (int r = kc + 1 + threadIdx.x; r < b; r += blockDim.x) fv[r] = cmul(Mm[r * b + kc], inv);
      __syncthreads();
      const int rows = b - kc - 1;
      for (int e = threadIdx.x; e < rows * (2 * b); e += blockDim.x) {
        const int r = kc + 1 + e / (2 * b), j = e % (2 * b);
        if (j < b) {
          if (j > kc) Mm[r * b + j] = csub(Mm[r * b + j], cmul(fv[r], Mm[kc * b + j]));
        } else {
          Xk[r * b + (j - b)] = csub(Xk[r * b + (j - b)], cmul(fv[r], Xk[kc * b + (j - b)]));
        }
      }
      __syncthreads();
    }
    for (int kr = b - 1; kr >= 0; --kr) {  // back substitution, columns in parallel
      const double2 inv = cdiv(cmk(1, 0), Mm[kr * b + kr]);
      for (int j = threadIdx.x; j < b; j += blockDim.x) {
        double2 acc = Xk[kr * b + j];
        for (int r = kr + 1; r < b; ++r) acc = csub(acc, cmul(Mm[kr * b + r], Xk[r * b + j]));
        Xk[kr * b + j] = cmul(acc, inv);
      }
      __syncthreads();
    }
    // K = Hermitian part of i X, in Xk; V = I in Mm
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const int r = e / b, q = e % b;
      if (r <= q) {
        const double2 xrq = Xk[r * b + q], xqr = Xk[q * b + r];
        const double2 krq = cmk(-xrq.y, xrq.x), kqr = cmk(-xqr.y, xqr.x);
        const double2 h = cscale(cadd(krq, cconj(kqr)), 0.5);
        Xk[r * b + q] = h;
        Xk[q * b + r] = cconj(h);
      }
    }
    for (int e = threadIdx.x; e < bb; e += blockDim.x) Mm[e] = cmk(e / b == e % b ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int e = threadIdx.x; e < b; e += blockDim.x) Xk[e * b + e].y = 0.0;
    __syncthreads();
    const int max_sweeps = pass == 0 ? sweeps0 : kMaxSweeps;
    bool conv;
    if (K32) {
      for (int e = threadIdx.x; e < bb; e += blockDim.x) wk.Kf[e] = make_float2(float(Xk[e].x), float(Xk[e].y));
      __syncthreads();
      conv = floquet_sweeps<float2>(wk.Kf, Mm, b, max_sweeps, wk);
    } else {
      conv = floquet_sweeps<double2>(Xk, Mm, b, max_sweeps, wk);
    }
    if (!conv && max_sweeps == kMaxSweeps) atomicOr(s.status, kNoConvergeFloquet);
    // Rayleigh quotients lam_r = v_r^H U v_r
    for (int r = threadIdx.x; r < b; r += blockDim.x) {
      double2 acc = cmk(0, 0);
      for (int kk = 0; kk < b; ++kk) {
        double2 uv = cmk(0, 0);
        for (int l = 0; l < b; ++l) uv = cfma(Ug(kk, l), Mm[l * b + r], uv);
        acc = cfmaconj(Mm[kk * b + r], uv, acc);
      }
      lam[r] = acc;
    }
    __syncthreads();
    if (pass == 1) break;
    if (threadIdx.x == 0) {
      double mind = 4.0;
      for (int r = 0; r < b; ++r) {
        const double2 w = cmul(ea, lam[r]);
        mind = fmin(mind, (1.0 + w.x) * (1.0 + w.x) + w.y * w.y);
      }
      done_s = conv && mind >= 0.0625;
      if (!done_s) {
        // widest gap of the eigenphases: sort them (insertion sort into red[])
        for (int r = 0; r < b; ++r) {
          const double th = atan2(lam[r].y, lam[r].x);
          int j = r;
          while (j > 0 && red[j - 1] > th) red[j] = red[j - 1], --j;
          red[j] = th;
        }
        double best = -1, mid = 0;
        for (int r = 0; r < b; ++r) {
          const double lo = red[r], hi = (r + 1 < b) ? red[r + 1] : red[0] + kPi2;
          if (hi - lo > best) best = hi - lo, mid = 0.5 * (lo + hi);
        }
        a_s = kPi - mid;
      }
    }
    __syncthreads();
    if (done_s) break;
  }
  for (int e = threadIdx.x; e < bb; e += blockDim.x) s.VF[at(bp + e, c, s.Cpad)] = Mm[e];
  for (int r = threadIdx.x; r < b; r += blockDim.x)
    s.L[at(bo + r, c, s.Cpad)] = cmk(log(hypot(lam[r].x, lam[r].y)), atan2(lam[r].y, lam[r].x));
}

__device__ void floquet_cta_df(const DevSys &s, int k, int c, FloqWork wk, bool a64 = false);

// One CTA per crystallite: unitary eigen-decomposition of a large block of A_n.
__global__ void __launch_bounds__(kBigThreads) k_big_floquet(DevSys s, int k) {
  extern __shared__ double2 bsc[];
  __shared__ double2 rot[(kMaxBigBlock / 2 + 1) * 2];  // (c, 0), (s e^{i ph}) per pair
  __shared__ int rpair[(kMaxBigBlock / 2 + 1) * 2];
  __shared__ double2 fv[kMaxBigBlock];
  __shared__ double2 lam[kMaxBigBlock];
  __shared__ double red[kBigThreads];
  const int b = s.bs[k];
  if (s.floq32) {  // K in single precision after the two b x b arrays; the rest double-float
    floquet_cta_df(s, k, blockIdx.x, FloqWork{bsc, bsc + b * b, rot, fv, lam, rpair, red,
                                              reinterpret_cast<float2 *>(bsc + 2 * b * b)});
  } else if (s.mixed) {
    floquet_cta<true, false>(s, k, blockIdx.x, FloqWork{bsc, bsc + b * b, rot, fv, lam, rpair, red, nullptr});
  } else {
    floquet_cta<false, false>(s, k, blockIdx.x, FloqWork{bsc, bsc + b * b, rot, fv, lam, rpair, red, nullptr});
  }
}

// ------------------------------------------------------------------ mixed form, double-float
// The large-block step and Dyson of the mixed form in double-float on the FP32 pipe (float2 =
// hi, lo; complex elements float4 = re.hi, im.hi, re.lo, im.lo), with the same tiling as the
// FP64 kernels and sums as compensated dot products.

// C = alpha A B for symmetric commuting A, B (upper tiles, mirrored), double-float.
__device__ void cta_mm_sym_df(const float2 *A, const float2 *B, float2 *C, int m, float2 alpha) {
  const int tm = (m + 1) / 2;
  for (int t = threadIdx.x; t < big_sym_tiles(m); t += blockDim.x) {
    int ti, tj;
    sym_tile(t, tm, ti, tj);
    const int i0 = 2 * ti, j0 = 2 * tj;
    const int i1 = min(i0 + 1, m - 1), j1 = min(j0 + 1, m - 1);
    DfAcc c00 = {0.f, 0.f}, c01 = c00, c10 = c00, c11 = c00;
    for (int l = 0; l < m; ++l) {
      const float2 a0 = A[i0 * m + l], a1 = A[i1 * m + l], b0 = B[l * m + j0], b1 = B[l * m + j1];
      df_dot(c00, a0.x, a0.y, b0.x, b0.y);
      df_dot(c01, a0.x, a0.y, b1.x, b1.y);
      df_dot(c10, a1.x, a1.y, b0.x, b0.y);
      df_dot(c11, a1.x, a1.y, b1.x, b1.y);
    }
    auto put = [&](int i, int j, const DfAcc &v) {
      const float2 x = dfv_mul(alpha, df_fin(v));
      C[i * m + j] = x;
      if (i != j) C[j * m + i] = x;
    };
    put(i0, j0, c00);
    if (j0 + 1 < m) put(i0, j0 + 1, c01);
    if (i0 + 1 < m) {
      if (ti != tj) put(i0 + 1, j0, c10);
      if (j0 + 1 < m) put(i0 + 1, j0 + 1, c11);
    }
  }
}

// 1/k for the Taylor terms, double-float
static_assert(kTaylorTerms == 15, "inv_df covers the terms 2..15");
__device__ __forceinline__ float2 inv_df(int kt) {
  switch (kt) {
    case 2: return dfv_const(1.0 / 2); case 3: return dfv_const(1.0 / 3); case 4: return dfv_const(1.0 / 4);
    case 5: return dfv_const(1.0 / 5); case 6: return dfv_const(1.0 / 6); case 7: return dfv_const(1.0 / 7);
    case 8: return dfv_const(1.0 / 8); case 9: return dfv_const(1.0 / 9); case 10: return dfv_const(1.0 / 10);
    case 11: return dfv_const(1.0 / 11); case 12: return dfv_const(1.0 / 12); case 13: return dfv_const(1.0 / 13);
    case 14: return dfv_const(1.0 / 14); default: return dfv_const(1.0 / 15);
  }
}

__host__ __device__ constexpr size_t big_step_df_smem(int b) { return sizeof(float2) * 5 * size_t(b) * size_t(b); }

// One CTA per (crystallite, step): the large block's U_i in double-float: H from the hi/lo
// tables, the series term by term to the degree taylor_degree gives at 2^-40, squarings.
__global__ void __launch_bounds__(1024) k_big_step_df(DevSys s, int k) {
  extern __shared__ __align__(16) unsigned char bsd[];
  __shared__ float2 fk[kMaxInt];
  __shared__ float red[kMaxBigBlock];
  __shared__ float2 scl;
  __shared__ int nsq, nterms;
  const int c = blockIdx.x % s.C, i = blockIdx.x / s.C;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  if (s.fk) {  // k_coef's coefficients: hi/lo pairs after the Taylor step, doubles after eigh
    const float2 *fk2 = reinterpret_cast<const float2 *>(s.fk);
    for (int kk = threadIdx.x; kk < s.nint; kk += blockDim.x) {
      const size_t a = at(i * s.nint + kk, c, s.Cpad);
      fk[kk] = s.fk_df ? fk2[a] : dfv_of(s.fk[a]);
    }
  } else if (threadIdx.x == 0) {
    double t1 = s.t0[c] + double(i) * s.tau, t2 = t1 + s.tau;
    double tmid = (t2 - t1) / 2.0 + t1;
    double sp, cp;
    sincos(tmid * s.wr * kPi2, &sp, &cp);
    double m[3][3];
    orient_rows(s, c, sp, cp, m);
    for (int kk = 0; kk < s.nint; ++kk) fk[kk] = dfv_of(term_coef(s, kk, m));
  }
  __syncthreads();
  float2 *X = reinterpret_cast<float2 *>(bsd), *P = X + bb, *Q = P + bb, *R = Q + bb, *I = R + bb;
  const float2 *Hcb = s.Hc_df + (s.hc_chunks ? size_t(i / s.psub) * s.S2 : 0) + bp;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) {
    float2 h = Hcb[e];
    for (int kk = 0; kk < s.nint; ++kk) {
      const float2 t = s.Tk_df[size_t(kk) * s.S2 + bp + e];
      if (t.x != 0.f) h = dfv_add(h, dfv_mul(fk[kk], t));
    }
    X[e] = h;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < b; p += blockDim.x) {
    float rs = 0.f;
    for (int q = 0; q < b; ++q) rs += fabsf(X[p * b + q].x);
    red[p] = rs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float nrm = 0.f;
    for (int p = 0; p < b; ++p) nrm = fmaxf(nrm, red[p]);
    nrm *= float(s.tau * kPi2) * (1.f + 1e-6f);
    int sq = 0;
    if (nrm > 0.5f) {
      frexpf(nrm / 0.5f, &sq);
      sq = min(sq, 60);
    }
    scl = make_float2(ldexpf(s.tpdf.x, -sq), ldexpf(s.tpdf.y, -sq));
    nsq = sq;
    nterms = taylor_degree(double(ldexpf(nrm, -sq)), true);
  }
  __syncthreads();
  const float2 sc = scl;
  const int sq = nsq, K = nterms;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) {
    const float2 x = dfv_mul(sc, X[e]);
    X[e] = x, P[e] = x;
    R[e] = make_float2((e / b == e % b) ? 1.f : 0.f, 0.f);
    I[e] = make_float2(-x.x, -x.y);
  }
  __syncthreads();
  for (int kt = 2; kt <= K; ++kt) {
    cta_mm_sym_df(P, X, Q, b, inv_df(kt));
    __syncthreads();
    const int m4 = kt & 3;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const float2 v = Q[e], nv = make_float2(-v.x, -v.y);
      if (m4 == 2) R[e] = dfv_add(R[e], nv);
      else if (m4 == 3) I[e] = dfv_add(I[e], v);
      else if (m4 == 0) R[e] = dfv_add(R[e], v);
      else I[e] = dfv_add(I[e], nv);
    }
    float2 *t = P;
    P = Q, Q = t;
    __syncthreads();
  }
  // squarings: (R + iI)^2 = (RR - II) + i 2RI, in P, Q, X
  for (int t = 0; t < sq; ++t) {
    cta_mm_sym_df(R, R, P, b, make_float2(1.f, 0.f));
    cta_mm_sym_df(I, I, Q, b, make_float2(1.f, 0.f));
    cta_mm_sym_df(R, I, X, b, make_float2(2.f, 0.f));
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const float2 q = Q[e];
      R[e] = dfv_add(P[e], make_float2(-q.x, -q.y)), I[e] = X[e];
    }
    __syncthreads();
  }
  double2 *Ub = s.U + size_t(i) * s.S2 * s.Cpad;
  float4 *U4 = reinterpret_cast<float4 *>(Ub);
  const double2 *fr = frame_of(s, i);
  const int bo = s.boff[k];
  for (int e = threadIdx.x; e < bb; e += blockDim.x) {
    const float2 re = R[e], im = I[e];
    if (fr) {  // rf schedule frames: through FP64
      const double2 u = cmk(double(re.x) + double(re.y), double(im.x) + double(im.y));
      U4[at(bp + e, c, s.Cpad)] = df_store(cmul(cmul(fr[bo + e / b], u), cconj(fr[bo + e % b])));
    } else {
      U4[at(bp + e, c, s.Cpad)] = make_float4(re.x, im.x, re.y, im.y);
    }
  }
}

// Complex double-float 2x2-tiled product into registers (compensated sums per re / im).
struct CdfAcc {
  DfAcc re, im;
};
__device__ __forceinline__ void cdf_mac(CdfAcc &a, float4 x, float4 y) {  // a += x y
  df_dot(a.re, x.x, x.z, y.x, y.z);
  df_dot(a.re, -x.y, -x.w, y.y, y.w);
  df_dot(a.im, x.x, x.z, y.y, y.w);
  df_dot(a.im, x.y, x.w, y.x, y.z);
}
__device__ __forceinline__ float4 cdf_fin(const CdfAcc &a) {
  const float2 r = df_fin(a.re), m = df_fin(a.im);
  return make_float4(r.x, m.x, r.y, m.y);
}

template <int NT>
__global__ void __launch_bounds__(NT == 1 ? 1024 : 768) k_big_dyson_df(DevSys s, int k) {
  extern __shared__ __align__(16) unsigned char bsy[];
  const int c = blockIdx.x;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  float4 *Us = reinterpret_cast<float4 *>(bsy), *As = Us + bb;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) As[e] = make_float4(e / b == e % b ? 1.f : 0.f, 0.f, 0.f, 0.f);
  const int tm = (b + 1) / 2;
  for (int i = 0; i < s.n; ++i) {
    const float4 *Ub = reinterpret_cast<const float4 *>(s.U + size_t(i) * s.S2 * s.Cpad);
    for (int e = threadIdx.x; e < bb; e += blockDim.x) Us[e] = Ub[at(bp + e, c, s.Cpad)];
    __syncthreads();
    float4 out[NT][4];
#pragma unroll
    for (int q = 0; q < NT; ++q) {
      const int t = threadIdx.x + q * blockDim.x;
      if (t >= tm * tm) continue;
      const int i0 = (t / tm) * 2, j0 = (t % tm) * 2;
      const int i1 = min(i0 + 1, b - 1), j1 = min(j0 + 1, b - 1);
      CdfAcc c00 = {{0.f, 0.f}, {0.f, 0.f}}, c01 = c00, c10 = c00, c11 = c00;
      for (int l = 0; l < b; ++l) {
        const float4 a0 = Us[i0 * b + l], a1 = Us[i1 * b + l], b0 = As[l * b + j0], b1 = As[l * b + j1];
        cdf_mac(c00, a0, b0), cdf_mac(c01, a0, b1), cdf_mac(c10, a1, b0), cdf_mac(c11, a1, b1);
      }
      out[q][0] = cdf_fin(c00), out[q][1] = cdf_fin(c01), out[q][2] = cdf_fin(c10), out[q][3] = cdf_fin(c11);
    }
    __syncthreads();
    float4 *Ab = reinterpret_cast<float4 *>(s.A + size_t(i) * s.S2 * s.Cpad);
#pragma unroll
    for (int q = 0; q < NT; ++q) {
      const int t = threadIdx.x + q * blockDim.x;
      if (t >= tm * tm) continue;
      const int i0 = (t / tm) * 2, j0 = (t % tm) * 2;
      for (int d = 0; d < 4; ++d) {
        const int r = i0 + (d >> 1), col = j0 + (d & 1);
        if (r < b && col < b) {
          As[r * b + col] = out[q][d];
          Ab[big_at(s, b, bp, r * b + col, c)] = out[q][d];
        }
      }
    }
    __syncthreads();
  }
}


// ------------------------------------------------------------------ mixed form, Floquet step
// floquet_cta's algorithm for the mixed form's large blocks when the FID spans at most
// kFloq32MaxPeriods periods, with every FP64 part moved to double-float on the FP32 pipe
// (GB300 issues about 2 FP64 FMAs per clock per SM against 128 FP32 FMAs): the Cayley
// transform, by Gauss-Jordan elimination with partial pivoting (the pivot search is a warp
// reduction; every update is parallel, no serial back substitution); V's accumulation of the
// Jacobi rotations, each rotation renormalised in double-float to c^2 + |s|^2 = 1; and the
// Rayleigh quotients lam_r = v_r^H A_n v_r through the CTA-wide product A_n V.  The sweeps over
// K run in FP32 with floquet_sweeps' rules.  Complex double-float elements are float4
// (re.hi, im.hi, re.lo, im.lo) in the 16-byte slots of the FP64 work arrays; the results
// (V, ln lambda) are stored in FP64 as by floquet_cta.

// x - f y, complex double-float
__device__ __forceinline__ float4 cdf_fms(float4 x, float4 f, float4 y) {
  CdfAcc a = {{x.x, x.z}, {x.y, x.w}};
  cdf_mac(a, make_float4(-f.x, -f.y, -f.z, -f.w), y);
  return cdf_fin(a);
}
__device__ __forceinline__ float4 cdf_mul(float4 x, float4 y) {
  CdfAcc a = {{0.f, 0.f}, {0.f, 0.f}};
  cdf_mac(a, x, y);
  return cdf_fin(a);
}

// q = e / d and r = e - q d without an integer division: (e + 1/2) / d in FP32 is at least
// 1/(2 d) away from an integer and its rounding error is far smaller (e < 2^20, d <= 2^8)
__device__ __forceinline__ int fdiv(int e, float invd, int d, int &r) {
  const int q = __float2int_rz((float(e) + 0.5f) * invd);
  r = e - q * d;
  return q;
}

// The sweeps over the FP32 K (Kf) with V (double-float, Vd) accumulating the rotations.
__device__ bool floquet_sweeps_df(float2 *Xk, float4 *Vd, int b, int max_sweeps, const FloqWork &wk) {
  float4 *rot = reinterpret_cast<float4 *>(wk.rot);  // per pair: (c.hi, 0, c.lo, 0), (s as complex df)
  auto rpair = [&](int t, int q) -> int & { return wk.rpair[2 * t + q]; };
  double *red = wk.red;
  const int bb = b * b;
  const float invb = 1.f / float(b);
  const int bq = b + (b & 1);
  const int np = bq / 2;
  bool conv = false, polish = false;
  const int nw = (blockDim.x + 31) / 32, wid = threadIdx.x >> 5, lid = threadIdx.x & 31;
  for (int sweep = 0; sweep < max_sweeps && !conv; ++sweep) {
    // off(K)^2 and diag(K)^2 for the stopping test: FP32 sums per thread (K is FP32), a fixed
    // shuffle tree per warp, the warps' sums added in FP64 by one thread
    float off = 0.f, dg = 0.f;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      int q;
      const int r = fdiv(e, invb, b, q);
      const float2 v = Xk[e];
      if (r < q) off = fmaf(v.x, v.x, fmaf(v.y, v.y, off));
      else if (r == q) dg = fmaf(v.x, v.x, dg);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dg += __shfl_xor_sync(0xffffffffu, dg, o);
    }
    if (lid == 0) red[2 * wid] = off, red[2 * wid + 1] = dg;
    __syncthreads();
    if (threadIdx.x == 0) {
      double so = 0, sd = 0;
      for (int t = 0; t < nw; ++t) so += red[2 * t], sd += red[2 * t + 1];
      red[2 * nw] = so, red[2 * nw + 1] = sd;
    }
    __syncthreads();
    const double offs = red[2 * nw], dgs = red[2 * nw + 1];
    __syncthreads();
    const bool small = offs <= 1e-10 * dgs || offs == 0.0;
    if (small && (polish || offs == 0.0)) {
      conv = true;
      break;
    }
    polish = polish || small;
    for (int round = 0; round < bq - 1; ++round) {
      for (int t = threadIdx.x; t < np; t += blockDim.x) {
        auto player = [&](int j) { return j == 0 ? 0 : 1 + (j - 1 + round) % (bq - 1); };
        int p = player(t), q = player(bq - 1 - t);
        if (p > q) {
          const int tmp = p;
          p = q, q = tmp;
        }
        rpair(t, 0) = p, rpair(t, 1) = q;
        float4 cr = make_float4(1.f, 0.f, 0.f, 0.f), sr = make_float4(0.f, 0.f, 0.f, 0.f);
        if (q < b) {
          const float2 hpq = Xk[p * b + q];
          const float ab = hypotf(hpq.x, hpq.y);
          if (ab != 0.f) {
            const float phx = hpq.x / ab, phy = hpq.y / ab;
            const float theta = 0.5f * (Xk[q * b + q].x - Xk[p * b + p].x) / ab;
            float tt;
            if (fabsf(theta) > 1e18f) tt = 0.5f / theta;
            else tt = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
            const float cc = rsqrtf(fmaf(tt, tt, 1.f));
            const float sx = phx * (tt * cc), sy = phy * (tt * cc);
            // renormalise: n2 = c^2 + |s|^2 in double-float (exact products), nn = n2^-1/2
            // = 1 - d/2 + 3d^2/8 with d = n2 - 1 (|d| ~ 1e-7)
            DfAcc n2 = {0.f, 0.f};
            df_dot(n2, cc, 0.f, cc, 0.f);
            df_dot(n2, sx, 0.f, sx, 0.f);
            df_dot(n2, sy, 0.f, sy, 0.f);
            const float2 nv = df_fin(n2);
            const float d = __fadd_rn(__fsub_rn(nv.x, 1.f), nv.y);
            const float2 nn = dfv_add(make_float2(1.f, 0.f), make_float2(fmaf(0.375f * d, d, -0.5f * d), 0.f));
            const float2 c2 = dfv_mul(nn, make_float2(cc, 0.f)), s2x = dfv_mul(nn, make_float2(sx, 0.f)),
                         s2y = dfv_mul(nn, make_float2(sy, 0.f));
            cr = make_float4(c2.x, 0.f, c2.y, 0.f);
            sr = make_float4(s2x.x, s2y.x, s2x.y, s2y.y);
          }
        }
        rot[2 * t] = cr, rot[2 * t + 1] = sr;
      }
      __syncthreads();
      // columns p, q of K (FP32) and of V (double-float): X <- X G, G = [[c, sp], [-conj(sp), c]];
      // one (pair, row) per iteration updates both; the pair index runs fastest, so a warp's
      // accesses stay within one row of K and of V
      for (int e = threadIdx.x; e < np * b; e += blockDim.x) {
        const int t = e % np, kk = e / np;
        const int p = rpair(t, 0), q = rpair(t, 1);
        if (q >= b) continue;
        const float4 cr = rot[2 * t], sp = rot[2 * t + 1];
        {
          const float ccr = cr.x + cr.z;
          const float2 spr = make_float2(sp.x + sp.z, sp.y + sp.w), spcr = cconj(spr);
          const float2 xkp = Xk[kk * b + p], xkq = Xk[kk * b + q];
          Xk[kk * b + p] = csub(cscale(xkp, ccr), cmul(spcr, xkq));
          Xk[kk * b + q] = cadd(cmul(spr, xkp), cscale(xkq, ccr));
        }
        {
          const float4 vp = Vd[kk * b + p], vq = Vd[kk * b + q];
          // vp' = c vp - conj(sp) vq,  vq' = sp vp + c vq
          CdfAcc ap = {{0.f, 0.f}, {0.f, 0.f}}, aq = ap;
          cdf_mac(ap, cr, vp);
          cdf_mac(ap, make_float4(-sp.x, sp.y, -sp.z, sp.w), vq);
          cdf_mac(aq, sp, vp);
          cdf_mac(aq, cr, vq);
          Vd[kk * b + p] = cdf_fin(ap);
          Vd[kk * b + q] = cdf_fin(aq);
        }
      }
      __syncthreads();
      // rows p, q of K:  K <- G^H K
      for (int e = threadIdx.x; e < np * b; e += blockDim.x) {
        int kk;
        const int t = fdiv(e, invb, b, kk);
        const int p = rpair(t, 0), q = rpair(t, 1);
        if (q >= b) continue;
        const float4 cr = rot[2 * t], s4 = rot[2 * t + 1];
        const float cc = cr.x + cr.z;
        const float2 sp = make_float2(s4.x + s4.z, s4.y + s4.w), spc = cconj(sp);
        const float2 xpk = Xk[p * b + kk], xqk = Xk[q * b + kk];
        float2 np_ = csub(cscale(xpk, cc), cmul(sp, xqk)), nq_ = cadd(cmul(spc, xpk), cscale(xqk, cc));
        // a non-trivial rotation zeroes K_pq, K_qp and the imaginary parts of K_pp, K_qq
        if ((kk == p || kk == q) && !(s4.x == 0.f && s4.y == 0.f)) {
          if (kk == p) np_.y = 0.f, nq_ = make_float2(0.f, 0.f);
          else np_ = make_float2(0.f, 0.f), nq_.y = 0.f;
        }
        Xk[p * b + kk] = np_;
        Xk[q * b + kk] = nq_;
      }
      __syncthreads();
    }
  }
  return conv;
}

// a64: A_n is FP64 (double2, the huge-block path's storage) instead of double-float
__device__ void floquet_cta_df(const DevSys &s, int k, int c, FloqWork wk, bool a64) {
  __shared__ int piv_s;
  __shared__ double a_s;
  __shared__ int done_s;
  __shared__ float4 inv_s;
  const int b = s.bs[k], bp = s.bpoff[k], bo = s.boff[k], bb = b * b;
  float4 *M4 = reinterpret_cast<float4 *>(wk.Mm), *X4 = reinterpret_cast<float4 *>(wk.Xk);
  float4 *fv = reinterpret_cast<float4 *>(wk.fv);
  double2 *lam = wk.lam;
  double *red = wk.red;
  float2 *Kf = wk.Kf;
  const double2 *An = s.A + size_t(s.n - 1) * s.S2 * s.Cpad;
  const float4 *U4 = reinterpret_cast<const float4 *>(An);
  auto Ug = [&](int r, int q) {
    return a64 ? df_store(An[at(bp + r * b + q, c, s.Cpad)]) : U4[big_at(s, b, bp, r * b + q, c)];
  };
  if (threadIdx.x == 0) a_s = 0.5, done_s = 0;
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    double sa, ca;
    sincos(a_s, &sa, &ca);
    const float4 ea = df_store(cmk(ca, sa));
    // M = I + e^{ia} A_n, X = I - e^{ia} A_n
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const float4 w = cdf_mul(ea, Ug(e / b, e % b));
      const float id = (e / b == e % b) ? 1.f : 0.f;
      const float2 re = dfv_add(make_float2(id, 0.f), make_float2(w.x, w.z));
      const float2 mre = dfv_add(make_float2(id, 0.f), make_float2(-w.x, -w.z));
      M4[e] = make_float4(re.x, w.y, re.y, w.w);
      X4[e] = make_float4(mre.x, -w.y, mre.y, -w.w);
    }
    __syncthreads();
    // Gauss-Jordan with partial pivoting: M X' = X, then X' = diag(M)^-1 X
    for (int kc = 0; kc < b; ++kc) {
      if (threadIdx.x < 32) {
        float best = -1.f;
        int pv = kc;
        for (int r = kc + threadIdx.x; r < b; r += 32) {
          const float4 v = M4[r * b + kc];
          const float m2 = v.x * v.x + v.y * v.y;
          if (m2 > best) best = m2, pv = r;
        }
        for (int o = 16; o; o >>= 1) {
          const float ob = __shfl_xor_sync(0xffffffffu, best, o);
          const int op = __shfl_xor_sync(0xffffffffu, pv, o);
          if (ob > best || (ob == best && op < pv)) best = ob, pv = op;
        }
        if (threadIdx.x == 0) {
          piv_s = pv;
          if (!(best > 0.f)) atomicOr(s.status, kSingularCayley);
        }
      }
      __syncthreads();
      const int pv = piv_s;
      if (pv != kc)
        for (int j = threadIdx.x; j < 2 * b; j += blockDim.x) {
          float4 *Mx = j < b ? M4 : X4;
          const int jj = j < b ? j : j - b;
          const float4 t = Mx[kc * b + jj];
          Mx[kc * b + jj] = Mx[pv * b + jj];
          Mx[pv * b + jj] = t;
        }
      __syncthreads();
      if (threadIdx.x == 0) {
        const double2 piv = df_load(M4[kc * b + kc]);
        inv_s = (piv.x != 0.0 || piv.y != 0.0) ? df_store(cdiv(cmk(1, 0), piv)) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      __syncthreads();
      const float4 inv = inv_s;
      for (int r = threadIdx.x; r < b; r += blockDim.x) fv[r] = r == kc ? make_float4(0.f, 0.f, 0.f, 0.f) : cdf_mul(M4[r * b + kc], inv);
      __syncthreads();
      const int wM = b - kc - 1, w = wM + b;  // columns kc+1..b-1 of M, all of X
      const float invw = 1.f / float(w);
      for (int e = threadIdx.x; e < (b - 1) * w; e += blockDim.x) {
        int j;
        int r = fdiv(e, invw, w, j);
        r += (r >= kc);
        if (j < wM) M4[r * b + kc + 1 + j] = cdf_fms(M4[r * b + kc + 1 + j], fv[r], M4[kc * b + kc + 1 + j]);
        else X4[r * b + (j - wM)] = cdf_fms(X4[r * b + (j - wM)], fv[r], X4[kc * b + (j - wM)]);
      }
      __syncthreads();
    }
    // X' = diag(M)^-1 X, then K = Hermitian part of i X' in FP32, V = I (double-float)
    for (int r = threadIdx.x; r < b; r += blockDim.x) {
      const double2 d = df_load(M4[r * b + r]);
      fv[r] = df_store(cdiv(cmk(1, 0), d));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x) X4[e] = cdf_mul(fv[e / b], X4[e]);
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const int r = e / b, q = e % b;
      const float4 xrq = X4[r * b + q], xqr = X4[q * b + r];
      // i X_rq = (-Im, Re); conj(i X_qr) = (-Im X_qr, -Re X_qr)
      const float re = 0.5f * (-(xrq.y + xrq.w) - (xqr.y + xqr.w));
      const float im = r == q ? 0.f : 0.5f * ((xrq.x + xrq.z) - (xqr.x + xqr.z));
      Kf[e] = make_float2(re, im);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < bb; e += blockDim.x) M4[e] = make_float4(e / b == e % b ? 1.f : 0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const int max_sweeps = kMaxSweeps;
    const bool conv = floquet_sweeps_df(Kf, M4, b, max_sweeps, wk);
    if (!conv) atomicOr(s.status, kNoConvergeFloquet);
    // Rayleigh quotients: Y = A_n V (into X's array), lam_r = sum_k conj(V_kr) Y_kr
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const int kr = e / b, r = e % b;
      CdfAcc a = {{0.f, 0.f}, {0.f, 0.f}};
      for (int l = 0; l < b; ++l) cdf_mac(a, Ug(kr, l), M4[l * b + r]);
      X4[e] = cdf_fin(a);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < b; r += blockDim.x) {
      CdfAcc a = {{0.f, 0.f}, {0.f, 0.f}};
      for (int kk = 0; kk < b; ++kk) {
        const float4 v = M4[kk * b + r];
        cdf_mac(a, make_float4(v.x, -v.y, v.z, -v.w), X4[kk * b + r]);
      }
      lam[r] = df_load(cdf_fin(a));
    }
    __syncthreads();
    if (pass == 1) break;
    if (threadIdx.x == 0) {
      double mind = 4.0;
      const double2 e2 = cmk(ca, sa);
      for (int r = 0; r < b; ++r) {
        const double2 w = cmul(e2, lam[r]);
        mind = fmin(mind, (1.0 + w.x) * (1.0 + w.x) + w.y * w.y);
      }
      done_s = conv && mind >= 0.0625;
      if (!done_s) {
        for (int r = 0; r < b; ++r) {
          const double th = atan2(lam[r].y, lam[r].x);
          int j = r;
          while (j > 0 && red[j - 1] > th) red[j] = red[j - 1], --j;
          red[j] = th;
        }
        double best = -1, mid = 0;
        for (int r = 0; r < b; ++r) {
          const double lo = red[r], hi = (r + 1 < b) ? red[r + 1] : red[0] + kPi2;
          if (hi - lo > best) best = hi - lo, mid = 0.5 * (lo + hi);
        }
        a_s = kPi - mid;
      }
    }
    __syncthreads();
    if (done_s) break;
  }
  for (int e = threadIdx.x; e < bb; e += blockDim.x) s.VF[at(bp + e, c, s.Cpad)] = df_load(M4[e]);
  for (int r = threadIdx.x; r < b; r += blockDim.x)
    s.L[at(bo + r, c, s.Cpad)] = cmk(log(hypot(lam[r].x, lam[r].y)), atan2(lam[r].y, lam[r].x));
}

// ------------------------------------------------------------------ mixed form, 4 x 4 tiles
// The mixed form's single-precision eigenframe with 4 x 4 output tiles per thread: 8 shared-memory loads per 16 complex multiply-adds (the 2 x 2 tiles of
// cta_mm_cplx_regs take 4 per 4), one tile per thread (blocks up to 74: at most 19 x 19
// tiles).  Same operands and the same sum per output element, in the same order.
__host__ __device__ constexpr int big4_tiles(int m, int n) { return ((m + 3) / 4) * ((n + 3) / 4); }
__host__ __device__ constexpr int big4_threads(int m, int n) { return (big4_tiles(m, n) + 31) / 32 * 32; }

// acc (this thread's tile; zero when it has none) = op(A) B, op = ^H if CONJ_A
template <bool CONJ_A>
__device__ __forceinline__ void cta_mm_cplx4(const float2 *A, int lda, const float2 *B, int ldb, int m, int n, int k,
                                             float2 (&acc)[4][4]) {
  const int tm = (m + 3) / 4, tn = (n + 3) / 4, t = threadIdx.x;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = make_float2(0.f, 0.f);
  if (t >= tm * tn) return;
  const int i0 = (t / tn) * 4, j0 = (t % tn) * 4;
  int ii[4], jj[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) ii[a] = min(i0 + a, m - 1), jj[a] = min(j0 + a, n - 1);
  for (int l = 0; l < k; ++l) {
    float2 av[4], bv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) av[a] = CONJ_A ? cconj(A[l * lda + ii[a]]) : A[ii[a] * lda + l];
#pragma unroll
    for (int b = 0; b < 4; ++b) bv[b] = B[l * ldb + jj[b]];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = cfma(av[a], bv[b], acc[a][b]);
  }
}
template <class F>
__device__ __forceinline__ void cta_tiles4_store(int m, int n, const float2 (&acc)[4][4], F f) {
  const int tm = (m + 3) / 4, tn = (n + 3) / 4, t = threadIdx.x;
  if (t >= tm * tn) return;
  const int i0 = (t / tn) * 4, j0 = (t % tn) * 4;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
      if (i0 + a < m && j0 + b < n) f(i0 + a, j0 + b, acc[a][b]);
}

// One CTA per crystallite: W_i = A_{i+1} V_F for i < n (mixed form: high parts of the
// double-float A, single-precision V and W), 4 x 4 tiles.
__global__ void __launch_bounds__(384) k_big_eigframe4(DevSys s, int k) {
  extern __shared__ __align__(16) unsigned char bsr4[];
  const int c = blockIdx.x;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  float2 *Vs = reinterpret_cast<float2 *>(bsr4), *As = Vs + bb;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) Vs[e] = cvt<float2>(s.VF[at(bp + e, c, s.Cpad)]);
  float2 acc[4][4];
  for (int i = 0; i < s.n; ++i) {
    const float4 *Ab4 = reinterpret_cast<const float4 *>(s.A + size_t(i) * s.S2 * s.Cpad);
    float2 *Wb = s.Wf + size_t(i) * s.S2 * s.Cpad;
    for (int e = threadIdx.x; e < bb; e += blockDim.x) {
      const float4 v = Ab4[big_at(s, b, bp, e, c)];
      As[e] = make_float2(v.x, v.y);
    }
    __syncthreads();
    cta_mm_cplx4<false>(As, b, Vs, b, b, b, b, acc);
    cta_tiles4_store(b, b, acc, [&](int r, int q, float2 v) { Wb[big_at(s, b, bp, r * b + q, c)] = v; });
    __syncthreads();
  }
}
