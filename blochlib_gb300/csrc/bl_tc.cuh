// Tensor-core (tcgen05) kernels of the mixed form, included by bl_engine.cu after bl_big.cuh.
//
// Exact-slice products (the Ozaki scheme on BF16 tensor cores).  A real matrix X with
// |x| <= 1 is split into four BF16 slices at their natural scale,
//     x = 2^-8 (q0 + 2^-8 q1 + 2^-16 q2 + 2^-24 q3),   q_j integers, |q_j| <= 256,
// each exact in BF16.  The product of two such matrices is the sum over slice pairs (s, t)
// of 2^-16 2^-8(s+t) q_s t_t.  With FP32 accumulation in tensor memory (TMEM):
//   level 0  (s + t = 0): integer sums below 2^17 for rows and columns of unit norm: exact;
//   level 1  (s + t = 1): multiples of 2^-8 below 2^12: exact;
//   levels 2 and 3 share one accumulator (multiples of 2^-24 of size ~2^3): its rounding is
//            below 2^-36 of the product;
//   levels 4 and up are dropped: below 2^-32.
// A unitary product therefore carries ~2^-32 relative error (double-float carries 2^-48),
// and a chain of n ~ 200 of them stays far inside the mixed form's 1e-6 FID bar (a numpy
// emulation of this exact scheme on 5- and 7-spin systems: 2.6e-9 and 2.7e-9 against FP64).
// The products run on the BF16 tensor pipe (about 2.25 PFLOP/s dense) instead of the FP32
// pipe, 10 slice pairs per real product.
//
// Slice tiles.  A b x b matrix (b <= kMaxB) is held as 4 planes (levels) of R x R BF16,
// R = up16(b), zero outside b x b, in the K-major canonical layout without swizzle: core
// matrices of 8 rows x 16 bytes; the K-adjacent core matrix 128 bytes on (leading byte
// offset), the next 8-row group R * 16 + 16 bytes on (stride byte offset; the 16 bytes of
// padding put the 8-row groups on different shared-memory banks, so that an epilogue lane
// per row stores whole 16-byte core-matrix rows without bank conflicts).  The matrices of
// the step exponential are symmetric, so one tile serves as either MMA operand.
//
// tcgen05 usage (PTX ISA, sm_100a family): one elected thread issues tcgen05.mma with
// 128-row tiles (cta_group::1, kind::f16, BF16 x BF16 -> FP32); an M = 128 MMA reads 128
// rows of its A tile, and rows past R fall into whatever follows (their products land in
// accumulator rows that are never read; the kernels keep memory after every tile).
// tcgen05.commit arrives on an mbarrier; every warp reads its 32-lane quarter of the
// accumulators with tcgen05.ld (four warps per quarter, on alternate 8-column chunks).
// Every wait is bounded (1 s): on a time-out the kernel sets kTcTimeout in the status word,
// waits (bounded) once more, frees its TMEM and returns.
// (bl_engine.cu includes <cuda_bf16.h> and <cstdint> at file scope.)

namespace tc {

constexpr int kTcThreads = 512;          // 16 warps: four per TMEM lane quarter
constexpr int kMaxB = kMaxBigBlock;      // largest block on these kernels (up16 = 80)
// smallest block on these kernels: below it the per-item costs (TMEM allocation, H assembly,
// one synchronised epilogue per product) outweigh the products, and the double-float kernels
// are faster (b = 28: the tensor-core step takes 3x the double-float step's time per item;
// with the stacked kernels, moving c3's 35-blocks here took its 512-system batch from 57.0
// to 54.2 FIDs/s)
constexpr int kMinB = 40;
constexpr unsigned long long kWaitNs = 1000000000ull;  // an mbarrier wait gives up after 1 s

__device__ __forceinline__ uint32_t saddr(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

__host__ __device__ constexpr int up16(int x) { return (x + 15) / 16 * 16; }
// bytes of one plane (R x R BF16 with padded 8-row groups) and of one 4-level tile
__host__ __device__ constexpr int sbo_bytes(int R) { return R * 16 + 16; }
__host__ __device__ constexpr size_t plane_bytes(int b) { return size_t(up16(b) / 8) * sbo_bytes(up16(b)); }
__host__ __device__ constexpr size_t tile_bytes(int b) { return 4 * plane_bytes(b); }
// bytes an M = 128 MMA may read past the end of an A tile
__host__ __device__ constexpr size_t overread_bytes(int b) {
  return size_t((128 - up16(b)) / 8) * sbo_bytes(up16(b));
}
// the step's output per (crystallite, step): 4 planes of C = cos X, then 4 planes of S = sin X
__host__ __device__ constexpr size_t slab_bytes(int b) { return 2 * tile_bytes(b); }
// element offset (BF16 units) of (r, k) in a plane of row length R
__device__ __forceinline__ int tix(int r, int k, int R) {
  return (r >> 3) * (R * 8 + 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

// Shared-memory matrix descriptor of a plane (start >> 4 in bits 0-13, leading byte offset
// >> 4 in 16-29, stride byte offset >> 4 in 32-45, version 1 at bit 46, no swizzle).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, int R) {
  return uint64_t((addr & 0x3FFFF) >> 4) | (uint64_t(128 >> 4) << 16) | (uint64_t(sbo_bytes(R) >> 4) << 32) |
         (1ull << 46);
}
// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits
// 7-9, 10-12 = 1), optional negation of A (bit 13), both K-major, N >> 3 in bits 17-22,
// M >> 4 in bits 24-28 (M = 128).
__host__ __device__ constexpr uint32_t idesc_bf16(int N, bool negA) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (negA ? (1u << 13) : 0u) | (uint32_t(N >> 3) << 17) |
         (uint32_t(128 >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(mbar))
               : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(mbar)));
  asm volatile("fence.mbarrier_init.release.cluster;");
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the mbarrier's phase `parity`: each try_wait suspends the warp in hardware for up
// to 20 us (no issue slots spent polling); gives up after kWaitNs.  True once it completed.
__device__ __forceinline__ bool wait_parity(uint64_t *mbar, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(saddr(mbar)), "r"(parity), "r"(20000u)
        : "memory");
    if (done) return true;
    if (gtimer() - t0 > kWaitNs) return false;
  }
}
// One thread: expect `bytes` on the mbarrier and start a bulk copy global -> shared of
// `bytes` (16-byte aligned addresses, a multiple of 16 bytes) that completes on it.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(mbar)), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
      "l"(src), "r"(bytes), "r"(saddr(mbar))
      : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// warp-wide: allocate ncols TMEM columns (a power of two >= 32); the base lands in *dst
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, int ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free(uint32_t base, int ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols));
}
// warp-wide: 8 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__host__ __device__ constexpr int pow2_cols(int c) {
  return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

// Four natural-scale slices of the double-float x = hi + lo (|x| <= ~1), as floats (each an
// integer times 2^-8j, exact in BF16).  Each residual d_j is exact (a rounded multiple of the
// previous one's ulp, below 1/2 in size); lo enters every stage through one FMA.
__device__ __forceinline__ void slice4f(float hi, float lo, float (&q)[4]) {
  const float q0 = rintf(hi * 256.f);
  const float d0 = __fmaf_rn(hi, 256.f, -q0);
  const float q1 = rintf(__fmaf_rn(lo, 65536.f, d0 * 256.f));
  const float d1 = __fmaf_rn(d0, 256.f, -q1);
  const float q2 = rintf(__fmaf_rn(lo, 16777216.f, d1 * 256.f));
  const float d2 = __fmaf_rn(d1, 256.f, -q2);
  const float q3 = rintf(__fmaf_rn(lo, 4294967296.f, d2 * 256.f));
  q[0] = q0, q[1] = q1 * 0x1p-8f, q[2] = q2 * 0x1p-16f, q[3] = q3 * 0x1p-24f;
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {  // a in the low half (lower address)
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&v);
}
// Slices of 8 consecutive elements (one core-matrix row) stored as one 16-byte vector per
// plane: planes at base + l * plane_elems (BF16 units), row offset o (a multiple of 8).
__device__ __forceinline__ void store_row8(__nv_bfloat16 *base, int plane_elems, int o, const float (&hi)[8],
                                           const float (&lo)[8]) {
  float q[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) slice4f(hi[j], lo[j], q[j]);
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    uint4 v;
    v.x = pack_bf16(q[0][l], q[1][l]);
    v.y = pack_bf16(q[2][l], q[3][l]);
    v.z = pack_bf16(q[4][l], q[5][l]);
    v.w = pack_bf16(q[6][l], q[7][l]);
    *reinterpret_cast<uint4 *>(base + size_t(l) * plane_elems + o) = v;
  }
}
// (hi, lo) of a + b + c for FP32 a, b (exact sums) and c: Knuth's two-sum twice
__device__ __forceinline__ float2 sum3(float a, float b, float c) {
  float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  const float s2 = __fadd_rn(s, c);
  bb = __fsub_rn(s2, s);
  e = __fadd_rn(e, __fadd_rn(__fsub_rn(s, __fsub_rn(s2, bb)), __fsub_rn(c, bb)));
  const float h = __fadd_rn(s2, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, s2)));
}

// Issues the 10 slice pairs of one real product into the three accumulators at TMEM column
// `col` (level 0, 1, 2+3 at col, col + R, col + 2R): A tile planes at a (plane stride pl
// bytes), B tile planes at b, R = up16(b) output columns, R / 16 K steps.  `accumulate`
// adds to what the accumulators hold instead of starting them.
__device__ __forceinline__ void issue_product(uint32_t tmem, uint32_t col, uint32_t a, uint32_t plA, uint32_t b,
                                              uint32_t plB, int R, bool negA, bool accumulate) {
  const uint32_t id = idesc_bf16(R, negA);
  const int sp[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3}, tp[10] = {0, 1, 0, 2, 1, 0, 3, 2, 1, 0};
  const int lev[10] = {0, 1, 1, 2, 2, 2, 2, 2, 2, 2};
#pragma unroll
  for (int q = 0; q < 10; ++q) {
    const uint32_t d = tmem + col + uint32_t(lev[q] * R);
    const bool first = !accumulate && (q == 0 || q == 1 || q == 3);
    const uint32_t a0 = a + uint32_t(sp[q]) * plA, b0 = b + uint32_t(tp[q]) * plB;
    for (int kk = 0; kk < R / 16; ++kk)
      mma(d, sdesc(a0 + kk * 256, R), sdesc(b0 + kk * 256, R), id, (first && kk == 0) ? 0u : 1u);
  }
}
__device__ __forceinline__ void issue_product(uint32_t tmem, uint32_t col, uint32_t a, uint32_t b, uint32_t pl,
                                              int R, bool negA, bool accumulate) {
  issue_product(tmem, col, a, pl, b, pl, R, negA, accumulate);
}

// -1 / (k (k + 1)) as double-float for the Horner steps (k = 1 .. 31), folded at compile time
// into constant memory (k is the same in every thread), so that no epilogue divides in FP64
#define BL_HC(k) dfv_const(-1.0 / (double(k) * double((k) + 1)))
__constant__ float2 kHornerCoef[32] = {BL_HC(1),  BL_HC(1),  BL_HC(2),  BL_HC(3),  BL_HC(4),  BL_HC(5),  BL_HC(6),
                                       BL_HC(7),  BL_HC(8),  BL_HC(9),  BL_HC(10), BL_HC(11), BL_HC(12), BL_HC(13),
                                       BL_HC(14), BL_HC(15), BL_HC(16), BL_HC(17), BL_HC(18), BL_HC(19), BL_HC(20),
                                       BL_HC(21), BL_HC(22), BL_HC(23), BL_HC(24), BL_HC(25), BL_HC(26), BL_HC(27),
                                       BL_HC(28), BL_HC(29), BL_HC(30), BL_HC(31)};
#undef BL_HC
__device__ __forceinline__ float2 horner_coef(int k) { return kHornerCoef[k < 1 ? 1 : (k > 31 ? 31 : k)]; }

// Taylor degree of the tensor-core step: the smallest K with x^(K+1)/(K+1)! <= 2^-35 (x <= 1):
// the exact-slice products carry ~2^-32 each, so a tighter series buys nothing
__device__ __forceinline__ int taylor_degree_tc(float x) {
  constexpr float thr[14] = {7.62939453125e-06f, 0.00055894250f, 0.0051409141f, 0.020352899f, 0.052506585f,
                             0.10562547f,        0.18141945f,    0.27994921f,   0.40028685f,  0.54099275f,
                             0.70041794f,        0.87688129f,    1.0687663f,    1.2745689f};
  int K = 15;
#pragma unroll
  for (int j = 13; j >= 0; --j)
    if (x <= thr[j]) K = j + 1;
  return K;
}

}  // namespace tc

enum { kTcTimeout = 64 };  // status bit: a tensor-core wait ran out

// A stacked tile: 128 rows (two R-row halves, the rest zero or unused) of the no-swizzle
// K-major slice layout, four planes of 16 row groups each.
__host__ __device__ constexpr size_t tc_stk_plane_bytes(int b) { return size_t(16) * tc::sbo_bytes(tc::up16(b)); }

// The step's prologue (every thread): the term coefficients into fk, H_i (double-float) into
// H, row sums of |H| into red, then the scale, squarings and Taylor degree into scl, nsq and
// nterms.  The block's operator non-zeros (CSR rows bp .. bp + bb) are first copied into
// `stage` (tiles that are free until X is sliced): coalesced, independent loads, after which
// each entry's walk over its terms (36 on a diagonal of eight coupled spins) reads shared
// memory instead of waiting on L2.
__device__ __forceinline__ void tc_step_prologue(const DevSys &s, int k, int c, int i, float2 *fk, float *red,
                                                 float2 *H, unsigned char *stage, size_t stage_bytes, float2 &scl,
                                                 int &nsq, int &nterms) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  {  // term coefficients (double-float pairs from k_coef)
    const float2 *fk2 = reinterpret_cast<const float2 *>(s.fk);
    for (int kk = tid; kk < s.nint; kk += tc::kTcThreads) fk[kk] = fk2[at(i * s.nint + kk, c, s.Cpad)];
  }
  __syncthreads();
  const float2 *Hcb = s.Hc_df + bp;
  {
    const int j0 = s.tk_ptr[bp], nz = s.tk_ptr[bp + bb] - j0;
    const size_t need = size_t(2 * bb + 1 + nz) * sizeof(int) + size_t(nz) * sizeof(float2) + 16;
    if (need <= stage_bytes) {
      int *sp = reinterpret_cast<int *>(stage);
      float2 *sv = reinterpret_cast<float2 *>(sp + ((2 * bb + 1 + nz + 3) & ~3));
      int *so = sp + bb + 1, *st = so + bb;
      // unrolled so that each thread's loads are in flight together (they do not depend on
      // one another); Hc goes straight into H, so the walk below touches no global memory
#pragma unroll 8
      for (int x = tid; x <= bb; x += tc::kTcThreads) sp[x] = s.tk_ptr[bp + x] - j0;
#pragma unroll 8
      for (int x = tid; x < bb; x += tc::kTcThreads) so[x] = s.tk_order[bp + x];
#pragma unroll 8
      for (int x = tid; x < nz; x += tc::kTcThreads) st[x] = s.tk_term[j0 + x], sv[x] = s.tk_val[j0 + x];
#pragma unroll 8
      for (int e = tid; e < bb; e += tc::kTcThreads) H[e] = Hcb[e];
      __syncthreads();
      // elements by descending term count: the 32 lanes of a warp walk similar lengths (the
      // diagonal, with a term for every interaction, together)
      for (int x = tid; x < bb; x += tc::kTcThreads) {
        const int e = so[x];
        float2 h = H[e];
        for (int j = sp[e]; j < sp[e + 1]; ++j) h = dfv_add(h, dfv_mul(fk[st[j]], sv[j]));
        H[e] = h;
      }
    } else {
      for (int e = tid; e < bb; e += tc::kTcThreads) {
        float2 h = Hcb[e];
        for (int j = s.tk_ptr[bp + e]; j < s.tk_ptr[bp + e + 1]; ++j)
          h = dfv_add(h, dfv_mul(fk[s.tk_term[j]], s.tk_val[j]));
        H[e] = h;
      }
    }
  }
  __syncthreads();
  // row sums of |H| (a warp per row, lanes over the columns), then their maximum: the norm
  for (int p = warp; p < b; p += tc::kTcThreads / 32) {
    float rs = 0.f;
    for (int q = lane; q < b; q += 32) rs += fabsf(H[p * b + q].x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);
    if (lane == 0) red[p] = rs;
  }
  __syncthreads();
  if (warp == 0) {
    float nrm = 0.f;
    for (int p = lane; p < b; p += 32) nrm = fmaxf(nrm, red[p]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nrm = fmaxf(nrm, __shfl_xor_sync(0xffffffffu, nrm, o));
    if (lane == 0) {
      nrm *= float(s.tau * kPi2) * (1.f + 1e-6f);
      int sq = 0;
      if (nrm > 1.f) {
        frexpf(nrm, &sq);  // nrm < 2^sq
        sq = min(sq, 60);
      }
      scl = make_float2(ldexpf(s.tpdf.x, -sq), ldexpf(s.tpdf.y, -sq));
      nsq = sq;
      nterms = tc::taylor_degree_tc(ldexpf(nrm, -sq));
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ step exponential
// One CTA per (crystallite, step) of a large block b <= tc::kMaxB of the mixed form (no rf
// schedule): H_i in double-float from k_coef's coefficients (as k_big_step_df),
// X = 2 pi tau H / 2^sq with ||X||_inf <= 1, and
//     C = cos X = sum_j (-1)^j Y^j / (2j)!,  S = sin X = X sum_j (-1)^j Y^j / (2j+1)!,  Y = X^2,
// to the degree K that taylor_degree_tc gives at 2^-35, each by Horner's rule
//     T <- I - Y T / (k (k + 1))
// on the tensor cores; the C and S chains run in two groups of 8 warps with their own
// accumulator sets, named barriers and MMA-issuing threads, so that one chain's epilogue
// runs while the other's products (and epilogue) run.  Then sq squarings
// (C, S) <- (C^2 - S^2, 2 C S) and the slices of U = C - i S go to the step's slab.
// Shared memory: four tiles (X, Y, T_C, T_S), then the over-read margin.
__host__ __device__ constexpr size_t tc_step_smem(int b) {
  return 4 * tc::tile_bytes(b) + tc::overread_bytes(b) + 1024;
}

__global__ void __launch_bounds__(tc::kTcThreads, 1) k_tc_step(DevSys s, int k, unsigned char *slab0) {
  using tc::kTcThreads;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ float2 fk[kMaxInt];
  __shared__ float red[tc::kMaxB];
  __shared__ float2 scl;
  __shared__ int nsq, nterms, gfail[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c = blockIdx.x % s.C, i = blockIdx.x / s.C;
  if (tid < 2) gfail[tid] = 0;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  const int R = tc::up16(b), pe = int(tc::plane_bytes(b) / 2);  // plane stride in BF16 units
  const int ncols = tc::pow2_cols(6 * R);
  unsigned char *base = tsm + ((1024 - (tc::saddr(tsm) & 1023)) & 1023);
  __nv_bfloat16 *Bf[4];
  uint32_t ba[4];
  for (int t = 0; t < 4; ++t) {
    Bf[t] = reinterpret_cast<__nv_bfloat16 *>(base + t * tc::tile_bytes(b));
    ba[t] = tc::saddr(Bf[t]);
  }
  if (warp == 0) tc::tmem_alloc(&tbase, ncols);
  if (tid == 0) tc::mbar_init(&mbar[0]), tc::mbar_init(&mbar[1]);
  // H (double-float) into the fourth tile as scratch, the other three as the staging area
  float2 *H = reinterpret_cast<float2 *>(Bf[3]);
  tc_step_prologue(s, k, c, i, fk, red, H, reinterpret_cast<unsigned char *>(Bf[0]), 3 * tc::tile_bytes(b), scl, nsq,
                   nterms);
  const int sq = nsq, K = nterms;
  const int mC = K / 2, mS = (K - 1) / 2;  // C to X^(2 mC), S to X^(2 mS + 1)
  {  // X slices into the first tile: one 8-column row chunk per thread and iteration, rows
     // fastest (a warp's 16-byte row stores fill whole row groups: no bank conflicts), H read
     // down its columns (H is symmetric, its (r, q) and (q, r) sums alike), contiguous
    const float2 sc = scl;
    const int nch = R * (R / 8);
    for (int t = tid; t < nch; t += kTcThreads) {
      const int r = t % R, c0 = (t / R) * 8;
      float hi[8], lo[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int q = c0 + j;
        float2 x = make_float2(0.f, 0.f);
        if (r < b && q < b) x = dfv_mul(sc, H[q * b + r]);
        hi[j] = x.x, lo[j] = x.y;
      }
      tc::store_row8(Bf[0], pe, tc::tix(r, c0, R), hi, lo);
    }
  }
  tc::fence_smem_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tbase;
  const uint32_t pl = uint32_t(tc::plane_bytes(b));
  const uint32_t set_col[2] = {0u, uint32_t(3 * R)};
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  const int q4 = warp & 3;  // this warp's TMEM lane quarter
  // Epilogue of accumulator set `set` over this thread's row and its 8-column chunks
  // (chunk index part, part + nparts, ...): out = diag I + coef P with
  // P = 2^-16 (acc0 + acc1 + acc23), or with `second` P = P_set0 - P_set1 (the squaring's
  // C^2 - S^2); slices into tile dst, zero padding.
  auto epilogue = [&](int set, float2 coef, float diag, bool second, __nv_bfloat16 *dst, int part, int nparts) {
    const int r = 32 * q4 + lane;
    if (32 * q4 >= R) return;  // warp-uniform: no stored row in this lane quarter
    for (int c0 = 8 * part; c0 < R; c0 += 8 * nparts) {
      float a0[8], a1[8], a2[8], b0[8], b1[8], b2[8];
      const uint32_t ta = tmem + (uint32_t(32 * q4) << 16) + set_col[set] + uint32_t(c0);
      tc::ld8(ta, a0);
      tc::ld8(ta + uint32_t(R), a1);
      tc::ld8(ta + uint32_t(2 * R), a2);
      if (second) {
        const uint32_t tb = tmem + (uint32_t(32 * q4) << 16) + set_col[1] + uint32_t(c0);
        tc::ld8(tb, b0);
        tc::ld8(tb + uint32_t(R), b1);
        tc::ld8(tb + uint32_t(2 * R), b2);
      }
      tc::wait_ld();
      if (r < R) {
        float hi[8], lo[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int q = c0 + j;
          float2 v = make_float2(0.f, 0.f);
          if (r < b && q < b) {
            const float2 p = tc::sum3(a0[j], a1[j], a2[j]);
            v = make_float2(p.x * 0x1p-16f, p.y * 0x1p-16f);
            if (second) {
              const float2 p2 = tc::sum3(b0[j], b1[j], b2[j]);
              v = dfv_add(v, make_float2(-p2.x * 0x1p-16f, -p2.y * 0x1p-16f));
            }
            v = dfv_mul(coef, v);
            if (r == q) v = dfv_add(v, make_float2(diag, 0.f));
          }
          hi[j] = v.x, lo[j] = v.y;
        }
        tc::store_row8(dst, pe, tc::tix(r, c0, R), hi, lo);
      }
    }
  };
  auto identity = [&](__nv_bfloat16 *dst) {  // the identity tile (C = I when mC == 0)
    const int nch = R * (R / 8);
    for (int t = tid; t < nch; t += kTcThreads) {
      const int r = t / (R / 8), c0 = (t % (R / 8)) * 8;
      float hi[8], lo[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) hi[j] = (r < b && r == c0 + j) ? 1.f : 0.f, lo[j] = 0.f;
      tc::store_row8(dst, pe, tc::tix(r, c0, R), hi, lo);
    }
  };
  auto sync_all = [&]() {  // epilogue writes -> the next MMAs, whole CTA
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  };
  auto wait_all = [&](int set) -> bool {
    const bool done = tc::wait_parity(&mbar[set], phase[set]);
    phase[set] ^= 1u;
    const bool all = __syncthreads_and(done);
    tc::fence_after();
    return all;
  };
  auto hcoef = [](int kk) { return tc::horner_coef(kk); };  // -1/(k(k+1)), double-float
  __nv_bfloat16 *X = Bf[0], *Y = Bf[1], *TC = Bf[2], *TS = Bf[3];
  const uint32_t aX = ba[0], aY = ba[1], aTC = ba[2], aTS = ba[3];
  // Y = X X, then the innermost Horner terms straight from Y (all 16 warps)
  if (tid == 0) {
    tc::issue_product(tmem, set_col[0], aX, aX, pl, R, false, false);
    tc::commit(&mbar[0]);
  }
  if (!wait_all(0)) ok = false;
  if (ok) {
    epilogue(0, make_float2(1.f, 0.f), 0.f, false, Y, warp >> 2, 4);
    if (mC >= 1) epilogue(0, hcoef(2 * mC - 1), 1.f, false, TC, warp >> 2, 4);
    else identity(TC);
    if (mS >= 1) epilogue(0, hcoef(2 * mS), 1.f, false, TS, warp >> 2, 4);
    sync_all();
  }
  // The two Horner chains, each in its own group of 8 warps (two per lane quarter) with its
  // own named barrier and MMA-issuing thread, so that their epilogues and products overlap:
  //   group 0: T_C <- I - Y T_C / ((2j-1) 2j) for j = mC-1..1 (set 0), C = T_C;
  //   group 1: T_S <- I - Y T_S / (2j (2j+1)) for j = mS-1..1 (set 1), then S = X T_S into
  //            X's tile (S = X when mS == 0).
  const int grp = warp >> 3, gpart = (warp >> 2) & 1, gbar = 1 + grp;
  const int leader = grp * (kTcThreads / 2);
  auto sync_grp = [&]() {
    tc::fence_smem_async();
    tc::fence_before();
    asm volatile("bar.sync %0, %1;" ::"r"(gbar), "r"(kTcThreads / 2) : "memory");
    tc::fence_after();
  };
  auto wait_grp = [&](int set) -> bool {
    const bool done = tc::wait_parity(&mbar[set], phase[set]);
    phase[set] ^= 1u;
    if (!done) gfail[grp] = 1;
    asm volatile("bar.sync %0, %1;" ::"r"(gbar), "r"(kTcThreads / 2) : "memory");
    tc::fence_after();
    return gfail[grp] == 0;
  };
  if (ok) {
    const int set = grp;
    __nv_bfloat16 *T = grp == 0 ? TC : TS;
    const uint32_t aT = grp == 0 ? aTC : aTS;
    int j = grp == 0 ? mC - 1 : mS - 1;
    while (j >= 1) {
      if (tid == leader) tc::issue_product(tmem, set_col[set], aY, aT, pl, R, false, false), tc::commit(&mbar[set]);
      if (!wait_grp(set)) break;
      epilogue(set, hcoef(grp == 0 ? 2 * j - 1 : 2 * j), 1.f, false, T, gpart, 2);
      --j;
      sync_grp();
    }
    if (grp == 1 && mS >= 1 && gfail[1] == 0) {
      if (tid == leader) tc::issue_product(tmem, set_col[1], aX, aTS, pl, R, false, false), tc::commit(&mbar[1]);
      if (wait_grp(1)) {
        epilogue(1, make_float2(1.f, 0.f), 0.f, false, X, gpart, 2);
        sync_grp();
      }
    }
  }
  sync_all();
  if (gfail[0] || gfail[1]) ok = false;
  // each group advanced only its own barrier's phase: both from the products committed
  phase[0] = uint32_t(1 + max(mC - 1, 0)) & 1u;
  phase[1] = uint32_t(max(mS - 1, 0) + (mS >= 1 ? 1 : 0)) & 1u;
  __nv_bfloat16 *Ct = TC, *St = X;
  uint32_t aC = aTC, aS = aX;
  // squarings: C' = C^2 - S^2 (sets 0 and 1), S' = 2 C S (set 0), into the two free tiles
  for (int t = 0; ok && t < sq; ++t) {
    __nv_bfloat16 *fr[2] = {nullptr, nullptr};
    uint32_t fa[2] = {0u, 0u};
    int nf = 0;
    for (int u = 0; u < 4; ++u)
      if (Bf[u] != Ct && Bf[u] != St && nf < 2) fr[nf] = Bf[u], fa[nf] = ba[u], ++nf;
    if (tid == 0) {
      tc::issue_product(tmem, set_col[0], aC, aC, pl, R, false, false);
      tc::commit(&mbar[0]);
      tc::issue_product(tmem, set_col[1], aS, aS, pl, R, false, false);
      tc::commit(&mbar[1]);
    }
    const bool w0 = wait_all(0), w1 = wait_all(1);
    if (!w0 || !w1) {
      ok = false;
      break;
    }
    epilogue(0, make_float2(1.f, 0.f), 0.f, true, fr[0], warp >> 2, 4);
    sync_all();
    if (tid == 0) tc::issue_product(tmem, set_col[0], aC, aS, pl, R, false, false), tc::commit(&mbar[0]);
    if (!wait_all(0)) {
      ok = false;
      break;
    }
    epilogue(0, make_float2(2.f, 0.f), 0.f, false, fr[1], warp >> 2, 4);
    sync_all();
    Ct = fr[0], aC = fa[0], St = fr[1], aS = fa[1];
  }
  if (ok && tid == 0) {  // real products issued: Y, the two chains, X S', 3 per squaring
    const int nprod = 1 + max(mC - 1, 0) + max(mS - 1, 0) + (mS >= 1 ? 1 : 0) + 3 * sq;
    atomicAdd(s.tc_flops, 20ull * (unsigned long long)nprod * (unsigned long long)(b * b * b));
  }
  if (ok) {  // the slab: C tile, then S tile (U = C - i S), 16-byte coalesced copies
    uint4 *dst = reinterpret_cast<uint4 *>(slab0 + (size_t(c) * s.n + i) * tc::slab_bytes(b));
    const int nv = int(tc::tile_bytes(b) / 16);
    const uint4 *cs = reinterpret_cast<const uint4 *>(Ct), *ss = reinterpret_cast<const uint4 *>(St);
    for (int v = tid; v < nv; v += kTcThreads) dst[v] = cs[v], dst[nv + v] = ss[v];
  } else {
    if (tid == 0) atomicOr(s.status, kTcTimeout);
    tc::wait_parity(&mbar[0], phase[0]);  // bounded: let MMAs in flight drain before TMEM is freed
    tc::wait_parity(&mbar[1], phase[1]);
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_free(tmem, ncols);
}

// ------------------------------------------------------------------ step exponential, stacked
// The same step for blocks with up16(b) = R <= 64, with both halves of the M = 128 tile
// holding rows.  X is sliced into both halves of a stacked tile XS, so that Y = XS X puts
// Y's rows in lanes m and R + m; the two Horner chains run as one, T = [T_C; T_S] stacked,
// T <- [I + c_C Y T_C; I + c_S Y T_S] from the single product T Y (T_C, T_S and Y are
// polynomials in Y and commute), the sine series carried to the same number of terms as the
// cosine (one more than it needs); S = T_S X from the same stacked T.  Every TMEM lane
// quarter holds rows for each epilogue.  C and S end in R-row tiles, where the squarings
// (as in k_tc_step) and the slab copy take them.  Shared memory: XS and T (stacked), two
// R-row tiles (Y, then C; H's scratch, then S), the over-read margin of an R-row A tile.
__host__ __device__ constexpr size_t tc_step_stk_smem(int b) {
  return 8 * tc_stk_plane_bytes(b) + 2 * tc::tile_bytes(b) + tc::overread_bytes(b) + 1024;
}

__global__ void __launch_bounds__(tc::kTcThreads, 1) k_tc_step_stk(DevSys s, int k, unsigned char *slab0) {
  using tc::kTcThreads;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ float2 fk[kMaxInt];
  __shared__ float red[tc::kMaxB];
  __shared__ float2 scl;
  __shared__ int nsq, nterms;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c = blockIdx.x % s.C, i = blockIdx.x / s.C;
  const int b = s.bs[k];
  const int R = tc::up16(b);
  const int pe = int(tc::plane_bytes(b) / 2), peS = int(tc_stk_plane_bytes(b) / 2);  // BF16 units
  const uint32_t pl = uint32_t(tc::plane_bytes(b)), plS = uint32_t(tc_stk_plane_bytes(b));
  const int ncols = tc::pow2_cols(6 * R);
  unsigned char *base = tsm + ((1024 - (tc::saddr(tsm) & 1023)) & 1023);
  __nv_bfloat16 *XS = reinterpret_cast<__nv_bfloat16 *>(base);
  __nv_bfloat16 *T = reinterpret_cast<__nv_bfloat16 *>(base + 4 * plS);
  __nv_bfloat16 *Yt = reinterpret_cast<__nv_bfloat16 *>(base + 8 * plS);
  __nv_bfloat16 *Wt = reinterpret_cast<__nv_bfloat16 *>(base + 8 * plS + tc::tile_bytes(b));
  const uint32_t aXS = tc::saddr(XS), aT = tc::saddr(T), aY = tc::saddr(Yt), aW = tc::saddr(Wt);
  if (warp == 0) tc::tmem_alloc(&tbase, ncols);
  if (tid == 0) tc::mbar_init(&mbar[0]), tc::mbar_init(&mbar[1]);
  // H into Wt as scratch; XS, T and Yt as the staging area
  float2 *H = reinterpret_cast<float2 *>(Wt);
  tc_step_prologue(s, k, c, i, fk, red, H, base, 8 * plS + tc::tile_bytes(b), scl, nsq, nterms);
  const int sq = nsq, K = nterms;
  const int mC = K / 2;  // C to X^(2 mC), S to X^(2 mC + 1)
  {  // X slices into both halves of XS: one 8-column row chunk per thread and iteration, rows
     // fastest, H read down its columns (as in k_tc_step)
    const float2 sc = scl;
    const int nch = R * (R / 8);
    for (int t = tid; t < nch; t += kTcThreads) {
      const int r = t % R, c0 = (t / R) * 8;
      float hi[8], lo[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int q = c0 + j;
        float2 x = make_float2(0.f, 0.f);
        if (r < b && q < b) x = dfv_mul(sc, H[q * b + r]);
        hi[j] = x.x, lo[j] = x.y;
      }
      tc::store_row8(XS, peS, tc::tix(r, c0, R), hi, lo);
      tc::store_row8(XS, peS, tc::tix(R + r, c0, R), hi, lo);
    }
  }
  tc::fence_smem_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tbase;
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  const int q4 = warp & 3, part = warp >> 2;  // lane quarter; 8-column chunks part, part+4, ...
  const int L = 32 * q4 + lane;                // TMEM lane: row L of the top half or L - R of the bottom
  const bool bot = L >= R, live = L < 2 * R;
  const int m = bot ? L - R : L;
  struct Out {
    __nv_bfloat16 *dst;
    int pe, row0;
    float2 coef;
    float diag;
  };
  // Epilogue of a stacked product (accumulator set 0): each live lane's row P (2^-16 times
  // the three accumulator levels, double-float) goes out as coef P + diag I into the outputs
  // of its half, as slices (row row0 + m of dst, plane stride pe), zero padding.
  auto epi = [&](const Out *o0, int n0, const Out *o1, int n1) {
    if (32 * q4 >= 2 * R) return;  // warp-uniform: no stacked row in this lane quarter
    const Out *o = bot ? o1 : o0;
    const int no = bot ? n1 : n0;
    for (int c0 = 8 * part; c0 < R; c0 += 32) {
      float a0[8], a1[8], a2[8];
      const uint32_t ta = tmem + (uint32_t(32 * q4) << 16) + uint32_t(c0);
      tc::ld8(ta, a0);
      tc::ld8(ta + uint32_t(R), a1);
      tc::ld8(ta + uint32_t(2 * R), a2);
      tc::wait_ld();
      if (!live || no == 0) continue;
      float2 P[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 p = tc::sum3(a0[j], a1[j], a2[j]);
        P[j] = (m < b && c0 + j < b) ? make_float2(p.x * 0x1p-16f, p.y * 0x1p-16f) : make_float2(0.f, 0.f);
      }
      for (int u = 0; u < no; ++u) {
        float hi[8], lo[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int q = c0 + j;
          float2 v = make_float2(0.f, 0.f);
          if (m < b && q < b) {
            v = dfv_mul(o[u].coef, P[j]);
            if (m == q) v = dfv_add(v, make_float2(o[u].diag, 0.f));
          }
          hi[j] = v.x, lo[j] = v.y;
        }
        tc::store_row8(o[u].dst, o[u].pe, tc::tix(o[u].row0 + m, c0, R), hi, lo);
      }
    }
  };
  auto sync_all = [&]() {  // epilogue writes -> the next MMAs, whole CTA
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  };
  auto wait_all = [&](int set) -> bool {
    const bool done = tc::wait_parity(&mbar[set], phase[set]);
    phase[set] ^= 1u;
    const bool all = __syncthreads_and(done);
    tc::fence_after();
    return all;
  };
  const float2 one = make_float2(1.f, 0.f), zero = make_float2(0.f, 0.f);
  // Y = X X (top and bottom halves alike); Y to Yt (when a chain step follows), the first
  // Horner terms T_C = I + c Y (to T, or straight to Yt as C when no chain step follows) and
  // T_S = I + c' Y (to T's bottom half); c = 0 when the series stops at the identity
  if (tid == 0) {
    tc::issue_product(tmem, 0, aXS, plS, aXS, plS, R, false, false);
    tc::commit(&mbar[0]);
  }
  if (!wait_all(0)) ok = false;
  if (ok) {
    const float2 cC = mC >= 1 ? tc::horner_coef(2 * mC - 1) : zero, cS = mC >= 1 ? tc::horner_coef(2 * mC) : zero;
    const Out top2[2] = {{Yt, pe, 0, one, 0.f}, {T, peS, 0, cC, 1.f}};
    const Out top1[1] = {{Yt, pe, 0, cC, 1.f}};
    const Out bot1[1] = {{T, peS, R, cS, 1.f}};
    if (mC >= 2) epi(top2, 2, bot1, 1);
    else epi(top1, 1, bot1, 1);
    sync_all();
  }
  // the chains: T <- [I + c_(2j-1) T_C Y; I + c_(2j) T_S Y] for j = mC-1 .. 1; the last
  // T_C (= C) goes to Yt, free once its product has run
  for (int j = mC - 1; ok && j >= 1; --j) {
    if (tid == 0) {
      tc::issue_product(tmem, 0, aT, plS, aY, pl, R, false, false);
      tc::commit(&mbar[0]);
    }
    if (!wait_all(0)) {
      ok = false;
      break;
    }
    const Out top[1] = {{j > 1 ? T : Yt, j > 1 ? peS : pe, 0, tc::horner_coef(2 * j - 1), 1.f}};
    const Out btm[1] = {{T, peS, R, tc::horner_coef(2 * j), 1.f}};
    epi(top, 1, btm, 1);
    sync_all();
  }
  // S = T_S X (the bottom half of T times X, X from XS's top half) into Wt
  if (ok) {
    if (tid == 0) {
      tc::issue_product(tmem, 0, aT, plS, aXS, plS, R, false, false);
      tc::commit(&mbar[0]);
    }
    if (!wait_all(0)) ok = false;
    if (ok) {
      const Out btm[1] = {{Wt, pe, 0, one, 0.f}};
      epi(nullptr, 0, btm, 1);
      sync_all();
    }
  }
  // squarings on R-row tiles: C' = C^2 - S^2 (sets 0 and 1), S' = 2 C S (set 0)
  __nv_bfloat16 *Bf[4] = {Yt, Wt, XS, reinterpret_cast<__nv_bfloat16 *>(base + tc::tile_bytes(b))};
  const uint32_t ba[4] = {aY, aW, aXS, aXS + uint32_t(tc::tile_bytes(b))};
  __nv_bfloat16 *Ct = Yt, *St = Wt;
  uint32_t aC = aY, aS = aW;
  const uint32_t set_col[2] = {0u, uint32_t(3 * R)};
  auto epi_sq = [&](int set, float2 coef, bool second, __nv_bfloat16 *dst) {
    if (32 * q4 >= R) return;  // warp-uniform
    const int r = 32 * q4 + lane;
    for (int c0 = 8 * part; c0 < R; c0 += 32) {
      float a0[8], a1[8], a2[8], b0[8], b1[8], b2[8];
      const uint32_t ta = tmem + (uint32_t(32 * q4) << 16) + set_col[set] + uint32_t(c0);
      tc::ld8(ta, a0);
      tc::ld8(ta + uint32_t(R), a1);
      tc::ld8(ta + uint32_t(2 * R), a2);
      if (second) {
        const uint32_t tb = tmem + (uint32_t(32 * q4) << 16) + set_col[1] + uint32_t(c0);
        tc::ld8(tb, b0);
        tc::ld8(tb + uint32_t(R), b1);
        tc::ld8(tb + uint32_t(2 * R), b2);
      }
      tc::wait_ld();
      if (r < R) {
        float hi[8], lo[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int q = c0 + j;
          float2 v = make_float2(0.f, 0.f);
          if (r < b && q < b) {
            const float2 p = tc::sum3(a0[j], a1[j], a2[j]);
            v = make_float2(p.x * 0x1p-16f, p.y * 0x1p-16f);
            if (second) {
              const float2 p2 = tc::sum3(b0[j], b1[j], b2[j]);
              v = dfv_add(v, make_float2(-p2.x * 0x1p-16f, -p2.y * 0x1p-16f));
            }
            v = dfv_mul(coef, v);
          }
          hi[j] = v.x, lo[j] = v.y;
        }
        tc::store_row8(dst, pe, tc::tix(r, c0, R), hi, lo);
      }
    }
  };
  for (int t = 0; ok && t < sq; ++t) {
    __nv_bfloat16 *fr[2] = {nullptr, nullptr};
    uint32_t fa[2] = {0u, 0u};
    int nf = 0;
    for (int u = 0; u < 4; ++u)
      if (Bf[u] != Ct && Bf[u] != St && nf < 2) fr[nf] = Bf[u], fa[nf] = ba[u], ++nf;
    if (tid == 0) {
      tc::issue_product(tmem, set_col[0], aC, aC, pl, R, false, false);
      tc::commit(&mbar[0]);
      tc::issue_product(tmem, set_col[1], aS, aS, pl, R, false, false);
      tc::commit(&mbar[1]);
    }
    const bool w0 = wait_all(0), w1 = wait_all(1);
    if (!w0 || !w1) {
      ok = false;
      break;
    }
    epi_sq(0, one, true, fr[0]);
    sync_all();
    if (tid == 0) tc::issue_product(tmem, set_col[0], aC, aS, pl, R, false, false), tc::commit(&mbar[0]);
    if (!wait_all(0)) {
      ok = false;
      break;
    }
    epi_sq(0, make_float2(2.f, 0.f), false, fr[1]);
    sync_all();
    Ct = fr[0], aC = fa[0], St = fr[1], aS = fa[1];
  }
  if (ok && tid == 0) {  // real products: Y, two per chain step, T_S X, 3 per squaring
    const int nprod = 1 + 2 * max(mC - 1, 0) + 1 + 3 * sq;
    atomicAdd(s.tc_flops, 20ull * (unsigned long long)nprod * (unsigned long long)(b * b * b));
  }
  if (ok) {  // the slab: C tile, then S tile (U = C - i S), 16-byte coalesced copies
    uint4 *dst = reinterpret_cast<uint4 *>(slab0 + (size_t(c) * s.n + i) * tc::slab_bytes(b));
    const int nv = int(tc::tile_bytes(b) / 16);
    const uint4 *cs = reinterpret_cast<const uint4 *>(Ct), *ss = reinterpret_cast<const uint4 *>(St);
    for (int v = tid; v < nv; v += kTcThreads) dst[v] = cs[v], dst[nv + v] = ss[v];
  } else {
    if (tid == 0) atomicOr(s.status, kTcTimeout);
    tc::wait_parity(&mbar[0], phase[0]);  // bounded: let MMAs in flight drain before TMEM is freed
    tc::wait_parity(&mbar[1], phase[1]);
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_free(tmem, ncols);
}

// ------------------------------------------------------------------ Dyson product
// One CTA per crystallite: A_{i+1} = U_i A_i for i < n, large block k of the mixed form.
// The product is formed transposed, A_{i+1}^T = A_i^T U_i (U_i = C - i S is symmetric):
//   re = Ar^T C + Ai^T S,   im = Ai^T C - Ar^T S   (the minus by the negate-A bit),
// so that the epilogue lane of column m of A_{i+1} stores row m of the next A_i^T tile as
// whole 16-byte core-matrix rows.  U_i's slab (written by k_tc_step) arrives by a bulk copy
// that overlaps the previous step's epilogue.  A_{i+1} also goes to s.A as double-float
// (float4 re.hi, im.hi, re.lo, im.lo; crystallite-major per block, big_at, so that the lanes'
// stores are contiguous) for the eigenframe and the Floquet step.  Shared memory: the A^T tiles (re, im), the U slab (C, S), the margin.
__host__ __device__ constexpr size_t tc_dyson_smem(int b) {
  return 4 * tc::tile_bytes(b) + tc::overread_bytes(b) + 1024;
}

__global__ void __launch_bounds__(tc::kTcThreads, 1) k_tc_dyson(DevSys s, int k, const unsigned char *slab0) {
  using tc::kTcThreads;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t mbar[2];  // 0: MMAs done, 1: U slab arrived
  const int c = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int b = s.bs[k], bp = s.bpoff[k];
  const int R = tc::up16(b), pe = int(tc::plane_bytes(b) / 2);
  const int ncols = tc::pow2_cols(6 * R);
  unsigned char *base = tsm + ((1024 - (tc::saddr(tsm) & 1023)) & 1023);
  __nv_bfloat16 *Ar = reinterpret_cast<__nv_bfloat16 *>(base);
  __nv_bfloat16 *Ai = reinterpret_cast<__nv_bfloat16 *>(base + tc::tile_bytes(b));
  unsigned char *Us = base + 2 * tc::tile_bytes(b);  // C tile, then S tile
  const uint32_t slab = uint32_t(tc::slab_bytes(b));
  const unsigned char *src = slab0 + size_t(c) * s.n * tc::slab_bytes(b);
  {  // A_0^T = I: zero both A tiles, 256 (= 1 at natural scale) on the level-0 real diagonal
    uint4 *z = reinterpret_cast<uint4 *>(base);
    const int n16 = int(2 * tc::tile_bytes(b) / 16);
    for (int e = tid; e < n16; e += kTcThreads) z[e] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  for (int r = tid; r < b; r += kTcThreads) Ar[tc::tix(r, r, R)] = __float2bfloat16_rn(256.f);
  if (warp == 0) tc::tmem_alloc(&tbase, ncols);
  if (tid == 0) {
    tc::mbar_init(&mbar[0]), tc::mbar_init(&mbar[1]);
    tc::bulk_load(Us, src, slab, &mbar[1]);
  }
  tc::fence_smem_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tbase;
  const uint32_t aAr = tc::saddr(Ar), aAi = tc::saddr(Ai), aC = tc::saddr(Us);
  const uint32_t aS = aC + uint32_t(tc::tile_bytes(b)), pl = uint32_t(tc::plane_bytes(b));
  const int q4 = warp & 3, part = warp >> 2;  // lane quarter; 8-column chunks part, part+4, ...
  float4 *A4 = reinterpret_cast<float4 *>(s.A);
  uint32_t ph[2] = {0u, 0u};
  bool ok = true;
  for (int i = 0; i < s.n; ++i) {
    {  // U_i's slab must have landed
      const bool got = tc::wait_parity(&mbar[1], ph[1]);
      ph[1] ^= 1u;
      if (!__syncthreads_and(got)) {
        ok = false;
        break;
      }
    }
    if (tid == 0) {
      tc::fence_after();
      tc::issue_product(tmem, 0, aAr, aC, pl, R, false, false);                // re  = Ar^T C
      tc::issue_product(tmem, 0, aAi, aS, pl, R, false, true);                 // re += Ai^T S
      tc::issue_product(tmem, uint32_t(3 * R), aAi, aC, pl, R, false, false);  // im  = Ai^T C
      tc::issue_product(tmem, uint32_t(3 * R), aAr, aS, pl, R, true, true);    // im -= Ar^T S
      tc::commit(&mbar[0]);
    }
    {
      const bool done = tc::wait_parity(&mbar[0], ph[0]);
      ph[0] ^= 1u;
      if (!__syncthreads_and(done)) {
        ok = false;
        break;
      }
      tc::fence_after();
    }
    // U_{i+1} streams in while the epilogue runs (the products no longer read the slab)
    if (tid == 0 && i + 1 < s.n) tc::bulk_load(Us, src + size_t(i + 1) * slab, slab, &mbar[1]);
    // epilogue: lane m = column m of A_{i+1}, 8 rows n at a time
    float4 *Ab = A4 + size_t(i) * s.S2 * s.Cpad;
    const int m = 32 * q4 + lane;
    if (32 * q4 < R) {
      for (int c0 = 8 * part; c0 < R; c0 += 32) {
        float r0[8], r1[8], r2[8], i0[8], i1[8], i2[8];
        const uint32_t ta = tmem + (uint32_t(32 * q4) << 16) + uint32_t(c0);
        tc::ld8(ta, r0);
        tc::ld8(ta + uint32_t(R), r1);
        tc::ld8(ta + uint32_t(2 * R), r2);
        tc::ld8(ta + uint32_t(3 * R), i0);
        tc::ld8(ta + uint32_t(4 * R), i1);
        tc::ld8(ta + uint32_t(5 * R), i2);
        tc::wait_ld();
        if (m < R) {
          float rh[8], rl[8], ih[8], il[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = c0 + j;
            float2 re = make_float2(0.f, 0.f), im = re;
            if (m < b && n < b) {
              const float2 pr = tc::sum3(r0[j], r1[j], r2[j]), pi = tc::sum3(i0[j], i1[j], i2[j]);
              re = make_float2(pr.x * 0x1p-16f, pr.y * 0x1p-16f);
              im = make_float2(pi.x * 0x1p-16f, pi.y * 0x1p-16f);
              Ab[big_at(s, b, bp, n * b + m, c)] = make_float4(re.x, im.x, re.y, im.y);
            }
            rh[j] = re.x, rl[j] = re.y, ih[j] = im.x, il[j] = im.y;
          }
          const int o = tc::tix(m, c0, R);
          tc::store_row8(Ar, pe, o, rh, rl);
          tc::store_row8(Ai, pe, o, ih, il);
        }
      }
    }
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
  }
  if (ok && tid == 0)  // 4 real products per step
    atomicAdd(s.tc_flops + 1, 80ull * (unsigned long long)s.n * (unsigned long long)(b * b * b));
  if (!ok) {
    if (tid == 0) atomicOr(s.status, kTcTimeout);
    tc::wait_parity(&mbar[0], ph[0]);  // bounded: let MMAs and the copy in flight drain
    tc::wait_parity(&mbar[1], ph[1]);
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_free(tmem, ncols);
}

// ------------------------------------------------------------------ Dyson product, stacked
// The same product for blocks with up16(b) = R <= 64, with both halves of the M = 128 tile
// holding rows: A1 = [Ar^T; Ai^T] and A2 = [Ai^T; -Ar^T] (R rows each, rows 2R.. zero), so
//   D = A1 C + A2 S = [Ar^T C + Ai^T S; Ai^T C - Ar^T S] = [re; im]
// in two stacked real products (20 slice pairs) instead of four, and every TMEM lane
// quarter holds rows for the epilogue: lane m < R is row m of re, lane R + m row m of im.
// Each epilogue lane writes its row's slices into both stacked tiles (negated in A2's lower
// half) and its half of the double-float A_{i+1} element (re: .x and .z, im: .y and .w of the
// float4 re.hi, im.hi, re.lo, im.lo).  Shared memory: A1, A2 (128 rows each), the U slab.
__host__ __device__ constexpr size_t tc_dyson_stk_smem(int b) {
  return 2 * 4 * tc_stk_plane_bytes(b) + tc::slab_bytes(b) + 1024;
}

__global__ void __launch_bounds__(tc::kTcThreads, 1) k_tc_dyson_stk(DevSys s, int k, const unsigned char *slab0) {
  using tc::kTcThreads;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t mbar[2];  // 0: MMAs done, 1: U slab arrived
  const int c = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int b = s.bs[k], bp = s.bpoff[k];
  const int R = tc::up16(b);
  const int peA = int(tc_stk_plane_bytes(b) / 2);  // stacked plane stride, BF16 units
  const int ncols = tc::pow2_cols(3 * R);
  unsigned char *base = tsm + ((1024 - (tc::saddr(tsm) & 1023)) & 1023);
  __nv_bfloat16 *A1 = reinterpret_cast<__nv_bfloat16 *>(base);
  __nv_bfloat16 *A2 = reinterpret_cast<__nv_bfloat16 *>(base + 4 * tc_stk_plane_bytes(b));
  unsigned char *Us = base + 8 * tc_stk_plane_bytes(b);  // C tile, then S tile
  const uint32_t slab = uint32_t(tc::slab_bytes(b));
  const unsigned char *src = slab0 + size_t(c) * s.n * tc::slab_bytes(b);
  {  // A_0^T = I: A1 = [I; 0], A2 = [0; -I] (256 = 1 at natural scale, level-0 plane)
    uint4 *z = reinterpret_cast<uint4 *>(base);
    const int n16 = int(8 * tc_stk_plane_bytes(b) / 16);
    for (int e = tid; e < n16; e += kTcThreads) z[e] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  for (int r = tid; r < b; r += kTcThreads) {
    A1[tc::tix(r, r, R)] = __float2bfloat16_rn(256.f);
    A2[tc::tix(R + r, r, R)] = __float2bfloat16_rn(-256.f);
  }
  if (warp == 0) tc::tmem_alloc(&tbase, ncols);
  if (tid == 0) {
    tc::mbar_init(&mbar[0]), tc::mbar_init(&mbar[1]);
    tc::bulk_load(Us, src, slab, &mbar[1]);
  }
  tc::fence_smem_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tbase;
  const uint32_t aA1 = tc::saddr(A1), aA2 = tc::saddr(A2), aC = tc::saddr(Us);
  const uint32_t aS = aC + uint32_t(tc::tile_bytes(b)), plB = uint32_t(tc::plane_bytes(b));
  const uint32_t plA = uint32_t(tc_stk_plane_bytes(b));
  const int q4 = warp & 3, part = warp >> 2;  // lane quarter; 8-column chunks part, part+4, ...
  const int L = 32 * q4 + lane;               // TMEM lane: re row L (L < R) or im row L - R
  const bool is_im = L >= R, live = L < 2 * R;
  const int m = is_im ? L - R : L;
  float *Af = reinterpret_cast<float *>(s.A);
  uint32_t ph[2] = {0u, 0u};
  bool ok = true;
  for (int i = 0; i < s.n; ++i) {
    {  // U_i's slab must have landed
      const bool got = tc::wait_parity(&mbar[1], ph[1]);
      ph[1] ^= 1u;
      if (!__syncthreads_and(got)) {
        ok = false;
        break;
      }
    }
    if (tid == 0) {
      tc::fence_after();
      tc::issue_product(tmem, 0, aA1, plA, aC, plB, R, false, false);  // [Ar^T C; Ai^T C]
      tc::issue_product(tmem, 0, aA2, plA, aS, plB, R, false, true);   // + [Ai^T S; -Ar^T S]
      tc::commit(&mbar[0]);
    }
    {
      const bool done = tc::wait_parity(&mbar[0], ph[0]);
      ph[0] ^= 1u;
      if (!__syncthreads_and(done)) {
        ok = false;
        break;
      }
      tc::fence_after();
    }
    // U_{i+1} streams in while the epilogue runs (the products no longer read the slab)
    if (tid == 0 && i + 1 < s.n) tc::bulk_load(Us, src + size_t(i + 1) * slab, slab, &mbar[1]);
    float *Ab = Af + size_t(i) * s.S2 * s.Cpad * 4;
    if (32 * q4 < 2 * R) {
      for (int c0 = 8 * part; c0 < R; c0 += 32) {
        float v0[8], v1[8], v2[8];
        const uint32_t ta = tmem + (uint32_t(32 * q4) << 16) + uint32_t(c0);
        tc::ld8(ta, v0);
        tc::ld8(ta + uint32_t(R), v1);
        tc::ld8(ta + uint32_t(2 * R), v2);
        tc::wait_ld();
        if (live) {
          float h[8], l[8], nh[8], nl[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = c0 + j;
            float2 v = make_float2(0.f, 0.f);
            if (m < b && n < b) {
              const float2 p = tc::sum3(v0[j], v1[j], v2[j]);
              v = make_float2(p.x * 0x1p-16f, p.y * 0x1p-16f);
              float *e = Ab + 4 * big_at(s, b, bp, n * b + m, c) + (is_im ? 1 : 0);
              e[0] = v.x, e[2] = v.y;
            }
            h[j] = v.x, l[j] = v.y, nh[j] = -v.x, nl[j] = -v.y;
          }
          // re row m: A1 row m, A2 row R + m negated; im row m: A1 row R + m, A2 row m
          tc::store_row8(A1, peA, tc::tix(is_im ? R + m : m, c0, R), h, l);
          if (is_im) tc::store_row8(A2, peA, tc::tix(m, c0, R), h, l);
          else tc::store_row8(A2, peA, tc::tix(R + m, c0, R), nh, nl);
        }
      }
    }
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
  }
  if (ok && tid == 0)  // 4 real products per step
    atomicAdd(s.tc_flops + 1, 80ull * (unsigned long long)s.n * (unsigned long long)(b * b * b));
  if (!ok) {
    if (tid == 0) atomicOr(s.status, kTcTimeout);
    tc::wait_parity(&mbar[0], ph[0]);  // bounded: let MMAs and the copy in flight drain
    tc::wait_parity(&mbar[1], ph[1]);
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 0) tc::tmem_free(tmem, ncols);
}
