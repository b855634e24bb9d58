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
// pipe, 10 slice pairs x 4 real products per complex product.
//
// tcgen05 usage (PTX ISA, sm_100a family): one elected thread issues tcgen05.mma with
// 128-row tiles (cta_group::1, kind::f16, BF16 x BF16 -> FP32) whose operands sit in shared
// memory in the K-major canonical layout without swizzle; tcgen05.commit arrives on an
// mbarrier; every warp then reads its 32-lane quarter of the accumulators with tcgen05.ld.
// Every wait is bounded: on a time-out the kernel sets kTcTimeout in the status word,
// waits (bounded) once more for its own MMAs, frees its TMEM and returns.
// (bl_engine.cu includes <cuda_bf16.h> and <cstdint> at file scope.)

namespace tc {

constexpr int kTcThreads = 256;                // 8 warps: two per TMEM lane quarter
constexpr int kMaxB = kMaxBigBlock;            // largest block: 6 accumulators of up16(74) = 80 columns
constexpr int kEPT = (kMaxB * kMaxB + kTcThreads - 1) / kTcThreads;  // U elements per thread
constexpr long kWaitLimit = 1L << 26;          // mbarrier polls before a time-out

__device__ __forceinline__ uint32_t saddr(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Element (r, k) of a rows x K BF16 operand tile, K-major without swizzle: core matrices of
// 8 rows x 16 bytes, the K-adjacent core matrix 128 bytes on (leading byte offset), the next
// 8-row group K * 16 bytes on (stride byte offset).
__host__ __device__ __forceinline__ int kmaj(int r, int k, int K) {
  return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}
// Shared-memory matrix descriptor of such a tile (tcgen05 layout: start >> 4 in bits 0-13,
// leading byte offset >> 4 in 16-29, stride byte offset >> 4 in 32-45, version 1 at bit 46,
// swizzle mode 0 in bits 61-63).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, int K) {
  return uint64_t((addr & 0x3FFFF) >> 4) | (uint64_t(128 >> 4) << 16) | (uint64_t((K * 16) >> 4) << 32) |
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
// Polls the mbarrier's phase `parity` at most kWaitLimit times; true once it completed.
__device__ __forceinline__ bool wait_parity(uint64_t *mbar, uint32_t parity) {
  uint32_t done = 0;
  for (long it = 0; it < kWaitLimit && !done; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(saddr(mbar)), "r"(parity)
        : "memory");
  }
  return done != 0;
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

__host__ __device__ constexpr int up16(int x) { return (x + 15) / 16 * 16; }
__host__ __device__ constexpr int up8(int x) { return (x + 7) / 8 * 8; }
// TMEM columns for the six accumulators (level 0, 1, 2+3; real and imaginary), rounded up
// to the power of two tcgen05.alloc takes
__host__ __device__ constexpr int tmem_cols(int b) {
  return 6 * up16(b) <= 32 ? 32 : 6 * up16(b) <= 64 ? 64 : 6 * up16(b) <= 128 ? 128 : 6 * up16(b) <= 256 ? 256 : 512;
}
// Shared memory of k_tc_dyson: 8 U slices (4 levels x re/im, up8(b) rows) and 8 A slices
// (up16(b) rows), both up16(b) wide in K, plus 1 KB for alignment.  An M = 128 MMA reads
// 128 rows of a U slice; rows past up8(b) fall into the following slices (their products
// land in accumulator rows >= b, which are never read), and the 8 A slices behind the last
// U slice always cover that reach (8 up16(b) >= 128 - up8(b)).
__host__ __device__ constexpr size_t dyson_smem(int b) {
  return size_t(2) * 8 * (size_t(up8(b)) + size_t(up16(b))) * size_t(up16(b)) + 1024;
}

// Four natural-scale BF16 slices of the double-float x = hi + lo (|x| <= ~1).  Each residual
// d_j is exact (a rounded multiple of the previous one's ulp, below 1/2 in size); lo enters
// every stage through one FMA.
__device__ __forceinline__ void slice4(float hi, float lo, __nv_bfloat16 &s0, __nv_bfloat16 &s1,
                                       __nv_bfloat16 &s2, __nv_bfloat16 &s3) {
  const float q0 = rintf(hi * 256.f);
  const float d0 = __fmaf_rn(hi, 256.f, -q0);
  const float q1 = rintf(__fmaf_rn(lo, 65536.f, d0 * 256.f));
  const float d1 = __fmaf_rn(d0, 256.f, -q1);
  const float q2 = rintf(__fmaf_rn(lo, 16777216.f, d1 * 256.f));
  const float d2 = __fmaf_rn(d1, 256.f, -q2);
  const float q3 = rintf(__fmaf_rn(lo, 4294967296.f, d2 * 256.f));
  s0 = __float2bfloat16_rn(q0);
  s1 = __float2bfloat16_rn(q1 * 0x1p-8f);
  s2 = __float2bfloat16_rn(q2 * 0x1p-16f);
  s3 = __float2bfloat16_rn(q3 * 0x1p-24f);
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

}  // namespace tc

enum { kTcTimeout = 64 };  // status bit: a tensor-core wait ran out

// One CTA per crystallite: A_{i+1} = U_i A_i for i < n on the tensor cores, the large block k
// (b <= tc::kMaxB) of the mixed form, U and A as double-float (float4 re.hi, im.hi, re.lo,
// im.lo in the [item][c] layout).  Per step: the elected thread issues the 10 slice pairs x 4
// real products (Cr = Ur Ar - Ui Ai, Ci = Ur Ai + Ui Ar; the minus by the descriptor's
// negate-A bit) into the six accumulators and commits; meanwhile every thread loads its part
// of U_{i+1} into registers; after the commit's barrier, the epilogue forms A_{i+1} =
// 2^-16 (acc0 + acc1 + acc23) in double-float, stores it and writes its slices (the next
// step's B operand, transposed: row = column of A) into shared memory, and the prefetched
// U_{i+1} is sliced into the A operand.
__global__ void __launch_bounds__(tc::kTcThreads, 1) k_tc_dyson(DevSys s, int k) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ uint32_t tbase;
  __shared__ __align__(8) uint64_t mbar;
  const int c = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int b = s.bs[k], bp = s.bpoff[k], bb = b * b;
  const int Kp = up16(b), Np = Kp, Mr = up8(b), ncols = tmem_cols(b);
  unsigned char *base = tsm + ((1024 - (saddr(tsm) & 1023)) & 1023);
  __nv_bfloat16 *Us = reinterpret_cast<__nv_bfloat16 *>(base);  // [level][re, im] Mr x Kp
  __nv_bfloat16 *As = Us + 8 * Mr * Kp;                            // [level][re, im] Np x Kp
  const int us_sz = Mr * Kp, as_sz = Np * Kp;
  // zero both operand sets (K and N padding stays zero), A_0 = I
  {
    uint4 *z = reinterpret_cast<uint4 *>(base);
    const int n16 = (8 * (us_sz + as_sz) * 2) / 16;
    for (int e = tid; e < n16; e += kTcThreads) z[e] = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  for (int r = tid; r < b; r += kTcThreads) As[kmaj(r, r, Kp)] = __float2bfloat16_rn(256.f);
  if (warp == 0) tmem_alloc(&tbase, ncols);
  if (tid == 0) mbar_init(&mbar);
  // U_0 slices
  const float4 *U4 = reinterpret_cast<const float4 *>(s.U);
  float4 ureg[kEPT];
  auto load_u = [&](int i) {
    const float4 *Ub = U4 + size_t(i) * s.S2 * s.Cpad;
#pragma unroll
    for (int j = 0; j < kEPT; ++j) {
      const int e = tid + j * kTcThreads;
      if (e < bb) ureg[j] = Ub[at(bp + e, c, s.Cpad)];
    }
  };
  auto store_u = [&]() {
#pragma unroll
    for (int j = 0; j < kEPT; ++j) {
      const int e = tid + j * kTcThreads;
      if (e < bb) {
        const int r = e / b, q = e - r * b, o = kmaj(r, q, Kp);
        const float4 u = ureg[j];
        slice4(u.x, u.z, Us[o], Us[2 * us_sz + o], Us[4 * us_sz + o], Us[6 * us_sz + o]);
        slice4(u.y, u.w, Us[us_sz + o], Us[3 * us_sz + o], Us[5 * us_sz + o], Us[7 * us_sz + o]);
      }
    }
  };
  load_u(0);
  store_u();
  fence_smem_async();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tbase;
  const uint32_t ua = saddr(Us), aa = saddr(As);
  const uint32_t idp = idesc_bf16(Np, false), idn = idesc_bf16(Np, true);
  const int q4 = warp & 3, half = warp >> 2, hcols = Np / 2;
  float4 *A4 = reinterpret_cast<float4 *>(s.A);
  bool ok = true;
  for (int i = 0; i < s.n; ++i) {
    if (tid == 0) {
      // U slice (level l, part p) at ua + (2l + p) us_sz * 2 bytes; A slice likewise
      auto gemm = [&](uint32_t col, int ul, int up, int al, int ap, bool neg, bool first) {
        const uint32_t u0 = ua + uint32_t((2 * ul + up) * us_sz * 2), a0 = aa + uint32_t((2 * al + ap) * as_sz * 2);
        for (int kk = 0; kk < Kp / 16; ++kk)
          mma(tmem + col, sdesc(u0 + kk * 256, Kp), sdesc(a0 + kk * 256, Kp), neg ? idn : idp,
              (first && kk == 0) ? 0u : 1u);
      };
      auto pair = [&](int lev, int us_, int at_, bool first) {
        const uint32_t cre = uint32_t(2 * lev * Np), cim = uint32_t((2 * lev + 1) * Np);
        gemm(cre, us_, 0, at_, 0, false, first);
        gemm(cre, us_, 1, at_, 1, true, false);
        gemm(cim, us_, 0, at_, 1, false, first);
        gemm(cim, us_, 1, at_, 0, false, false);
      };
      pair(0, 0, 0, true);
      pair(1, 0, 1, true);
      pair(1, 1, 0, false);
      pair(2, 0, 2, true);
      pair(2, 1, 1, false);
      pair(2, 2, 0, false);
      pair(2, 0, 3, false);
      pair(2, 1, 2, false);
      pair(2, 2, 1, false);
      pair(2, 3, 0, false);
      commit(&mbar);
    }
    if (i + 1 < s.n) load_u(i + 1);  // overlaps the MMAs
    const bool done = wait_parity(&mbar, uint32_t(i & 1));
    if (!__syncthreads_and(done)) {
      ok = false;
      break;
    }
    fence_after();
    // epilogue: this thread's row r of A_{i+1}, columns of its half
    const int r = 32 * q4 + lane;
    float4 *Ab = A4 + size_t(i) * s.S2 * s.Cpad;
    if (32 * q4 < b) {
      for (int c0 = half * hcols; c0 < (half + 1) * hcols; c0 += 8) {
        float a0r[8], a0i[8], a1r[8], a1i[8], a2r[8], a2i[8];
        const uint32_t ta = tmem + (uint32_t(32 * q4) << 16) + uint32_t(c0);
        ld8(ta, a0r);
        ld8(ta + uint32_t(Np), a0i);
        ld8(ta + uint32_t(2 * Np), a1r);
        ld8(ta + uint32_t(3 * Np), a1i);
        ld8(ta + uint32_t(4 * Np), a2r);
        ld8(ta + uint32_t(5 * Np), a2i);
        wait_ld();
        if (r < b) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = c0 + j;
            if (col < b) {
              const float2 re = sum3(a0r[j], a1r[j], a2r[j]), im = sum3(a0i[j], a1i[j], a2i[j]);
              const float rh = re.x * 0x1p-16f, rl = re.y * 0x1p-16f, ih = im.x * 0x1p-16f, il = im.y * 0x1p-16f;
              Ab[at(bp + r * b + col, c, s.Cpad)] = make_float4(rh, ih, rl, il);
              const int o = kmaj(col, r, Kp);  // B operand: row = column of A, K = row of A
              slice4(rh, rl, As[o], As[2 * as_sz + o], As[4 * as_sz + o], As[6 * as_sz + o]);
              slice4(ih, il, As[as_sz + o], As[3 * as_sz + o], As[5 * as_sz + o], As[7 * as_sz + o]);
            }
          }
        }
      }
    }
    if (i + 1 < s.n) store_u();
    fence_smem_async();
    fence_before();
    __syncthreads();
    fence_after();
  }
  if (!ok) {
    if (tid == 0) atomicOr(s.status, kTcTimeout);
    wait_parity(&mbar, 0);  // bounded: let any MMA still in flight drain before TMEM is freed
    wait_parity(&mbar, 1);
    fence_before();
    __syncthreads();
    fence_after();
  }
  if (warp == 0) tmem_free(tmem, ncols);
}
