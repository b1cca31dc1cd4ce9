// ibl_tc.cu -- precision path: the GGX prefilter and the irradiance
// convolution as dense contractions on the sm_103a tensor cores (tcgen05,
// BF16 hi/lo operands, FP32 accumulation in TMEM, FP64 weight normalisation).
//
// What is computed (the quadrature the FP64 oracle states):
//   prefilter(n) = sum_t L_t w(n,t) / sum_t w(n,t),
//     w = D_GGX(n.h; a2 = r^2) * max(0, n.w_t) * Omega_t,  n.h = sqrt((1 + n.w_t)/2)
//   irradiance(n) = (1/pi) sum_t L_t max(0, n.w_t) Omega_t
// over the texels t of a chosen source level S of the env chain (box
// averages of level 0), at the reference's texel-corner output directions.
// The planner (althea_ibl_tc_plan) picks S per mip from a measured error
// table so the result stays within 1e-3 of the same sum over level 0.
// Outputs of at most kNarrowMax texels (the roughest mips) are summed on the
// CUDA cores instead (narrow_kernel): as GEMMs they are a few rows by a few
// columns, which the tensor cores would spend almost entirely on padding.
//
// Structure.  On an equirect map the weight of output texel (i, x) for source
// texel (j, y) depends only on (i, j, d = y - s*x), s = W_src / W_out, through
// c = cos p_i cos q_j cos(2 pi (d + 0.5) / W_src) + sin p_i sin q_j.  Pick a
// phase count g and a column step m with 8 g = s m (g = 1, m = 8/s for s <= 8;
// g = s/8, m = 1 for s >= 8) and split each source row into g phase rows
// P_ph[u] = L_j[g u + ph] (length krow = ws / g).  For the output columns
// x = x0 + m (n0 + n):
//   out[i, x] = sum_{j, ph, k} A[i, (j, ph, k)] * B[(j, ph, k), n],
//   A = w_ij(g ((k - (s/g) x0) mod krow) + ph),  B[k, n] = P_ph[(8 n + k + 8 n0) mod krow],
// a GEMM with M = 128 output rows (TMEM lanes), N = up to 128 columns n and
// K = (j, ph, k).  B is a Hankel matrix (rows 8 elements = 16 bytes apart),
// which the K-major no-swizzle UMMA layout expresses directly (LBO = 16 B,
// SBO = 128 B): the radiance operand is read straight from a staged row.
// The column residue x0 shifts the weights, not the row, so every staged row
// is the phase row rotated by a multiple of 16 bytes: TMA bulk copies.
//
// Kernel (warp-specialised, one CTA per SM, 640 threads):
//   warps 0-15  weight producers: generate A (hi and lo BF16) for one K = 32
//               stage and write it straight into TMEM with tcgen05.st (four
//               stages in flight), so no shared-memory bandwidth goes to A;
//   warps 16-18 one thread each issues the MMAs of one colour channel (A from
//               TMEM, B from shared memory).  A single issuing thread cannot
//               keep the tensor core busy: on sm_103a one thread issues a
//               tcgen05.mma about every 64 cycles, while an N = 64 MMA
//               executes in 32;
//   warp 19     one thread stages the Hankel radiance rows with TMA bulk
//               copies (up to four slots in flight).
// Unpaired outputs of 33 to 64 rows run as column tiles instead: the staged
// Hankel is the A operand (M = 128 output columns) and the weights, written
// by the producers to shared memory, the B operand (N = 64 rows).
// Each CTA owns at most kMaxK = 32768 of K (the source rows are split over the
// grid to guarantee it), so each accumulator is one tensor-core FP32
// accumulation chain of bounded length; the producer warps move it to the
// partial sums at the end.  32768 against 16384: half the partial sums to
// write and add again, 3 % faster bakes, the worst error over the production
// test unchanged (mean errors of the 1024x512 and 512x256 mips up by 2e-5 to
// 4e-5).  All hand-offs are mbarriers; every wait is bounded by the global
// timer and an abort flag, after which the kernel records an error, waits
// (bounded) for its own MMAs and copies, frees its TMEM and returns.
// A bake runs every CTA of its contractions as work items of one queue launch
// (contract_queue_kernel); a batch, those of every probe in one persistent
// kernel (contract_persistent_kernel).  Either way one CTA per SM pulls
// items largest first, so a job is split only to bound K per CTA.
//
// Precision.  Radiance and weights are each split x = hi + lo (hi = bf16(x),
// lo = bf16(x - hi)); three MMAs per channel (hi*hi + hi*lo + lo*hi) give
// products to ~2^-17 relative.  BF16 shares FP32's exponent range, so
// 1e6-bright suns need no scaling.  The weight sum of each output row is
// taken in FP64 (FP32 within one source phase row) by the producers.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "althea_ibl.h"
#include "ibl_device.cuh"
#include "ibl_internal.h"

namespace ibl {
namespace tc {

constexpr int kM = 128;           // output rows per CTA (TMEM lanes)
constexpr int kKS = 32;           // K per pipeline stage (two K = 16 MMAs)
constexpr int kStages = 4;        // A stages in TMEM
constexpr int kNBMax = 128;       // MMA N (columns) per CTA
constexpr int kACol = 3 * kNBMax; // first A stage column (accumulators before it)
constexpr int kTmemCols = 512;
constexpr int kProducerWarps = 16;  // four per TMEM lane quarter, 8 K each per stage
constexpr int kMmaWarp0 = 16;       // MMA issuers: one per colour channel
constexpr int kMmaWarps = 3;
constexpr int kLoaderWarp = 19;
constexpr int kThreads = 32 * (kLoaderWarp + 1);
static_assert(kMmaWarp0 == kProducerWarps && kLoaderWarp == kMmaWarp0 + kMmaWarps, "warp roles");
static_assert(kACol + kStages * kKS <= kTmemCols, "TMEM columns");
constexpr int kMaxSlots = 4;      // staged radiance rows in flight
constexpr int kMaxK = 32768;      // K per CTA: one TMEM accumulation chain
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
constexpr uint32_t kSleepNs = 200000;  // longest hardware suspension per try (0.2 ms)
constexpr float kPiF = 3.14159265358979f;
constexpr int kSmemLimit = 232448;  // opt-in shared memory per block
constexpr int kCtN = 64;            // column tiles: weight rows (MMA N)

// ---- PTX wrappers -------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy (16-byte aligned addresses, size a multiple of
// 16), completion counted on the mbarrier's transaction count.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait that lets the hardware suspend the thread until the phase
// completes or `ns` nanoseconds pass, so waiting warps do not take issue
// slots from the working ones.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: false when the abort flag is up or after `limit_ns` (which
// raises the flag so every other role stops too).
__device__ __forceinline__ bool wait_bar_for(uint64_t* bar, uint32_t parity, volatile int* abort,
                                             unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait_sleep(bar, parity, kSleepNs)) return true;
    if (*abort) return false;
    if (global_ns() - t0 > limit_ns) {
      *abort = 1;
      return false;
    }
  }
}
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort) {
  return wait_bar_for(bar, parity, abort, kWaitNs);
}

// Self-test of the bounded wait: an mbarrier that nothing completes is waited
// on with a short limit; the wait must give up, raise the abort flag and let
// the kernel report through an error word and return.
__global__ void wait_selftest_kernel(int* result, unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  __shared__ int abort_sh;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  abort_sh = 0;
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const unsigned long long t0 = global_ns();
  const bool completed = wait_bar_for(&bar, 0u, &abort_sh, limit_ns);
  const unsigned long long waited = global_ns() - t0;
  result[0] = completed ? 0 : 1;        // 1: the wait gave up
  result[1] = abort_sh;                 // 1: the abort flag went up
  result[2] = (int)(waited / 1000000);  // milliseconds waited
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  // tcgen05 shared-memory matrix descriptor, no swizzle:
  // [0,14) addr>>4, [16,30) LBO>>4, [32,46) SBO>>4, [46,48) version = 1,
  // [49,52) base offset = 0, [52] LBO mode = 0, [61,64) layout = 0 (none).
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) |                    // D format F32
         (1u << 7) | (1u << 10) |       // A, B format BF16
         ((uint32_t)(n >> 3) << 17) |   // N / 8
         ((uint32_t)(m >> 4) << 24);    // M / 16
}

// One K = 32 stage of one channel, hi/lo split, then a commit to `bar`:
//   D += Ahi*Bhi + Ahi*Blo + Alo*Bhi  for K = 0..15 and 16..31
// A: TMEM columns a (hi, K 0..15 at +0, 16..31 at +8; lo at +16 / +24);
// B: descriptors bh/bl (hi/lo plane) and bh2/bl2 (the same 16 K further).
// One asm block so the six MMAs leave the issuing thread back to back: any
// instruction between two tcgen05.mma adds to the per-MMA issue time.
__device__ __forceinline__ void mma_stage_ts(uint32_t d, uint32_t a, uint64_t bh, uint64_t bl,
                                             uint64_t bh2, uint64_t bl2, uint32_t idesc,
                                             uint32_t accumulate, uint64_t* bar) {
  asm volatile(
      "{\n .reg .pred p, t;\n .reg .b32 a8, a16, a24;\n"
      " setp.ne.b32 p, %7, 0;\n setp.eq.b32 t, %7, %7;\n"
      " add.u32 a8, %1, 8;\n add.u32 a16, %1, 16;\n add.u32 a24, %1, 24;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %6, p;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %3, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a16], %2, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a8], %4, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a8], %5, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a24], %4, %6, t;\n"
      " tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%8];\n}\n" ::"r"(d),
      "r"(a), "l"(bh), "l"(bl), "l"(bh2), "l"(bl2), "r"(idesc), "r"(accumulate),
      "r"((uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

// A K = 64 stage with the weights as BF16 hi only (two products per K = 16):
//   D += Ahi*Bhi + Ahi*Blo  for K = 16t .. 16t + 15, t = 0..3,
// A at TMEM columns a + 8t (hi only: 64 K in 32 columns), B descriptors
// bh + 2t / bl + 2t (16-byte units).  Without the lo half of the weights a
// stage of 64 K fits the TMEM of a 32 K hi/lo stage, which halves the
// producers' per-stage hand-off work per weight.  The weight sum is taken
// over the same rounded weights, so the normalised result is an exact
// weighted average with BF16 weights.
__device__ __forceinline__ void mma_stage64_ts2(uint32_t d, uint32_t a, uint64_t bh, uint64_t bl,
                                                uint32_t idesc, uint32_t accumulate,
                                                uint64_t* bar) {
  asm volatile(
      "{\n .reg .pred p, t;\n .reg .b32 a8, a16, a24;\n .reg .b64 h2, l2, h4, l4, h6, l6;\n"
      " setp.ne.b32 p, %5, 0;\n setp.eq.b32 t, %5, %5;\n"
      " add.u32 a8, %1, 8;\n add.u32 a16, %1, 16;\n add.u32 a24, %1, 24;\n"
      " add.u64 h2, %2, 2;\n add.u64 l2, %3, 2;\n add.u64 h4, %2, 4;\n"
      " add.u64 l4, %3, 4;\n add.u64 h6, %2, 6;\n add.u64 l6, %3, 6;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %4, p;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %3, %4, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a8], h2, %4, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a8], l2, %4, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a16], h4, %4, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a16], l4, %4, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a24], h6, %4, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [a24], l6, %4, t;\n"
      " tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%6];\n}\n" ::"r"(d),
      "r"(a), "l"(bh), "l"(bl), "r"(idesc), "r"(accumulate),
      "r"((uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

// Column tiles (both operands in shared memory): one K = 32 stage of one
// channel, hi/lo split, then a commit to `bar`:
//   D += Lhi*Whi + Lhi*Wlo + Llo*Whi  for K = 0..15 and 16..31
// A = radiance descriptors ah/al (hi/lo plane, the next K = 16 at +2 units of
// 16 bytes), B = weight descriptors bh/bl (the next K = 16 at +bk units).
__device__ __forceinline__ void mma_stage_ss(uint32_t d, uint64_t ah, uint64_t al, uint64_t bh,
                                             uint64_t bl, uint32_t bk, uint32_t idesc,
                                             uint32_t accumulate, uint64_t* bar) {
  asm volatile(
      "{\n .reg .pred p, t;\n .reg .b64 bk64, ah2, al2, bh2, bl2;\n"
      " setp.ne.b32 p, %7, 0;\n setp.eq.b32 t, %7, %7;\n cvt.u64.u32 bk64, %5;\n"
      " add.u64 ah2, %1, 2;\n add.u64 al2, %2, 2;\n add.u64 bh2, %3, bk64;\n"
      " add.u64 bl2, %4, bk64;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %3, %6, p;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %4, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %2, %3, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], ah2, bh2, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], ah2, bl2, %6, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], al2, bh2, %6, t;\n"
      " tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%8];\n}\n" ::"r"(d),
      "l"(ah), "l"(al), "l"(bh), "l"(bl), "r"(bk), "r"(idesc), "r"(accumulate),
      "r"((uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

// Column tiles, a K = 64 stage with the weights as BF16 hi only:
//   D += Lhi*Whi + Llo*Whi  for K = 16t .. 16t + 15, t = 0..3
// (A at +2t units, B at +t bk units).
__device__ __forceinline__ void mma_stage64_ss2(uint32_t d, uint64_t ah, uint64_t al, uint64_t bh,
                                                uint32_t bk, uint32_t idesc, uint32_t accumulate,
                                                uint64_t* bar) {
  asm volatile(
      "{\n .reg .pred p, t;\n .reg .b64 bk64, a1, a2, a3, l1, l2, l3, b1, b2, b3;\n"
      " setp.ne.b32 p, %6, 0;\n setp.eq.b32 t, %6, %6;\n cvt.u64.u32 bk64, %4;\n"
      " add.u64 a1, %1, 2;\n add.u64 a2, %1, 4;\n add.u64 a3, %1, 6;\n"
      " add.u64 l1, %2, 2;\n add.u64 l2, %2, 4;\n add.u64 l3, %2, 6;\n"
      " add.u64 b1, %3, bk64;\n add.u64 b2, b1, bk64;\n add.u64 b3, b2, bk64;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %3, %5, p;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %2, %3, %5, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], a1, b1, %5, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], l1, b1, %5, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], a2, b2, %5, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], l2, b2, %5, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], a3, b3, %5, t;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], l3, b3, %5, t;\n"
      " tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%7];\n}\n" ::"r"(d),
      "l"(ah), "l"(al), "l"(bh), "r"(bk), "r"(idesc), "r"(accumulate),
      "r"((uint32_t)__cvta_generic_to_shared(bar))
      : "memory");
}

// Hardware reciprocal approximation (one MUFU operation, ~1 ulp).
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_st4(uint32_t taddr, const uint32_t* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr),
               "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3])
               : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
      : "memory");
}

__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- job description --------------------------------------------------------------
struct Job {
  const __nv_bfloat16* src;  // 6 planes (R hi, R lo, G hi, G lo, B hi, B lo) as
                             // [plane][hs][g][krow] (g = 1: the level itself)
  int ws, hs;                // source level size
  int wo, ho;                // output size
  int s, g, m;               // s = ws / wo; 8 g = s m
  int krow, kpad;            // phase row length ws / g, padded to a multiple of kKS
  int nres, nb, nblk;        // columns per residue x0, MMA N, column blocks per residue
  int rlen;                  // staged row length (bf16 elements, multiple of 8)
  int nslots;                // staged rows in flight (2..kMaxSlots)
  int kind;                  // 0 = GGX prefilter, 1 = irradiance
  float a2;                  // roughness^2
  int ksplit;                // source rows are split over this many CTAs
  const float* cos_d;        // [ws]  cos(2 pi (d + 0.5) / ws)
  const float* src_rows;     // [hs][3]  cos q, sin q, Omega
  const float* out_rows;     // [ho][2]  cos p, sin p
  float* partial;            // [ksplit][3][wo][ho]
  double* wsum_part;         // [ksplit][ho]  (kind 0)
  int* error;                // set when a bounded wait gave up
  int out_half;              // 1: outputs are RGBA16F (8-byte texels), else RGBA32F
  int two_prod;              // 1: BF16 hi weights only (two products per channel), weight
                             // sum over the rounded weights; 0: hi/lo weights (three)
  // A second output of the same geometry (same source level, phase count,
  // columns) in the same CTA: they share every radiance operand, only the
  // weights differ.  Row tiles: TMEM lanes 64-127, so that two outputs of
  // <= 64 rows fill one M = 128 tile.
  // K interleave (row tiles of <= 32 rows): every lane quarter holds the same
  // rows and owns every fourth K stage (stage slot q), so the weight work of
  // one quarter spreads over the four SM sub-partitions; the CTA adds the
  // quarters' sums before writing one partial per split.
  // Visible offsets: vis[tile * hs + j] = half-width (in phase-row units) of
  // the window of column offsets around 0 where some output row of row tile
  // `tile` sees source row j above its horizon (max(0, n.w) > 0); -1 when no
  // row of the tile sees row j at all; >= krow when all offsets are needed.
  // Outside the window every weight of the tile is exactly 0, so those K
  // stages are skipped.  A margin of two texels covers the FP32 evaluation.
  const int* vis;
  int kinter;                // 1 or 4
  int nparts;                // partial sums the finish adds: ksplit
  int pair;                  // 1: a second output (ho_b rows) is contracted too
  int ho_b, kind_b;
  float a2_b;
  const float* out_rows_b;   // [ho_b][2]
  float* partial_b;          // [ksplit][3][wo][ho_b]
  double* wsum_part_b;       // [ksplit][ho_b]  (kind_b 0)
  // Column tiles (unpaired outputs of 33 to 64 rows): the staged radiance
  // Hankel is the A operand (M = 128 output columns, nb = 128) and the
  // weights the B operand (N = kCtN = 64 rows), written by the producers to
  // shared memory.
  int ct;
  // Weight sums of a cosine (kind 1) output too -- an irradiance from which a
  // roughness-1 mip is derived (wsum1: the first output; wsum1_b: the second
  // of a pair).
  int wsum1, wsum1_b;
};

// Weight stages of a column-tile CTA: K-major, no swizzle; per stage and
// plane, KS/8 groups of 8 K, each kCtN rows x 16 bytes (row i at
// (i / 8) 128 + (i % 8) 16).  Three products: hi and lo planes of 32 K; two
// products: the hi plane of 64 K.  Either way 128 kCtN bytes per stage.
__host__ __device__ inline size_t ct_stage_bytes(const Job& J) { return (size_t)128 * kCtN; }

struct SmemPlan {
  size_t slots, cosd, bst, total;
};

__host__ __device__ inline SmemPlan smem_plan(const Job& J) {
  SmemPlan p;
  p.slots = 0;
  p.cosd = p.slots + (size_t)J.nslots * 6 * J.rlen * 2;
  const size_t end = p.cosd + (size_t)J.g * J.kpad * 4;
  p.bst = (end + 127) & ~(size_t)127;
  p.total = J.ct ? p.bst + kStages * ct_stage_bytes(J) : end;
  return p;
}

// K chunks (of ks) of a source row that hold visible offsets: [0, ca) and
// [cb, kchunks), from the window half-width uh (see Job::vis).  The window is
// |u| <= uh around the CTA's column shift sh < 8, i.e. k in [-uh, uh + 8)
// modulo krow.
__host__ __device__ __forceinline__ void visible_chunks(int uh, int krow, int ks, int kchunks,
                                                        int& ca, int& cb) {
  if (uh < 0) {  // no row of the tile sees this source row
    ca = 0;
    cb = kchunks;
  } else if (uh >= krow) {
    ca = cb = kchunks;
  } else {
    const int a = (uh + 8 + ks - 1) / ks, b = (krow - uh) / ks;
    ca = a < kchunks ? a : kchunks;
    cb = b > ca ? b : ca;
  }
}

// Shared state of one contraction CTA: the barriers, the abort flag and the
// producers' weight sums.
struct CtaShared {
  uint64_t a_full[kStages], a_empty[kStages];
  uint64_t slot_full[kMaxSlots], slot_empty[kMaxSlots];
  uint64_t done_bar;
  int abort;
  double wsum[kProducerWarps / 4][kM];
};

// Bounded wait for a barrier phase that is known to complete (the arrivals
// are already in flight); false after kWaitNs.
__device__ __forceinline__ bool settle(uint64_t* bar, uint32_t parity) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > kWaitNs) return false;
  return true;
}

// Eight weights of one output row at K = kb .. kb + 7 of phase row cdrow:
// w = k1 c D(c) (GGX, D = 1 / (alpha + beta c)^2) or k1 c (cosine), c =
// ccq cos_d + ssq, clamped at 0 and zero past krow; packed FP32x2 arithmetic.
__device__ __forceinline__ __nv_bfloat162 bf16_zero2() { return __float2bfloat162_rn(0.0f); }

// CLAMP = false leaves the negative weights (beyond a row's horizon) to the
// caller, which clamps them after rounding to BF16 (two per instruction).
template <bool CLAMP = true>
__device__ __forceinline__ void weights8(const float* cdrow, int kb, int krow, float2 ccq2,
                                         float2 ssq2, float2 k12, float2 alpha2, float2 beta2,
                                         bool ggx, float2 (&w)[4]) {
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const float4 cd = *reinterpret_cast<const float4*>(cdrow + kb + 4 * e);
    const float2 c01 = __ffma2_rn(ccq2, make_float2(cd.x, cd.y), ssq2);
    const float2 c23 = __ffma2_rn(ccq2, make_float2(cd.z, cd.w), ssq2);
    if (ggx) {
      const float2 d01 = __ffma2_rn(c01, beta2, alpha2);
      const float2 d23 = __ffma2_rn(c23, beta2, alpha2);
      const float2 q01 = __fmul2_rn(d01, d01), q23 = __fmul2_rn(d23, d23);
      const float2 r01 = make_float2(rcp_approx(q01.x), rcp_approx(q01.y));
      const float2 r23 = make_float2(rcp_approx(q23.x), rcp_approx(q23.y));
      w[2 * e] = __fmul2_rn(__fmul2_rn(k12, c01), r01);
      w[2 * e + 1] = __fmul2_rn(__fmul2_rn(k12, c23), r23);
    } else {
      w[2 * e] = __fmul2_rn(k12, c01);
      w[2 * e + 1] = __fmul2_rn(k12, c23);
    }
  }
  if (CLAMP) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      w[e].x = fmaxf(w[e].x, 0.0f);
      w[e].y = fmaxf(w[e].y, 0.0f);
    }
  }
  if (kb + 8 > krow) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (kb + u >= krow) {
        if (u & 1)
          w[u >> 1].y = 0.0f;
        else
          w[u >> 1].x = 0.0f;
      }
  }
}

// Hankel row loader (one thread): for every source row of split `split`
// with a visible chunk and every phase, slot[p][t] = P_ph[(t + 8 n0) mod
// krow], t < rlen, by bulk copies completing on slot_full.  Waits (bounded)
// for its last copies before returning.
__device__ __forceinline__ void load_rows(const Job& job, __nv_bfloat16* slots,
                                          uint64_t* slot_full, uint64_t* slot_empty, int split,
                                          int ks, int kchunks, const int* vis_row, int n0,
                                          volatile int* abort_flag) {
  const int u0 = (8 * n0) % job.krow;
  long long row_id = 0;
  bool ok = true;
  for (int j = split; j < job.hs && ok; j += job.ksplit) {
    int ca, cb;
    visible_chunks(vis_row[j], job.krow, ks, kchunks, ca, cb);
    if (ca + kchunks - cb == 0) continue;  // no visible offset: the row is not staged
    for (int ph = 0; ph < job.g && ok; ++ph, ++row_id) {
      const int slot = (int)(row_id % job.nslots);
      const long long use = row_id / job.nslots;
      if (use >= 1 && !wait_bar(&slot_empty[slot], (uint32_t)((use - 1) & 1), abort_flag)) {
        ok = false;
        break;
      }
      __nv_bfloat16* dst = slots + (size_t)slot * 6 * job.rlen;
      mbar_expect_tx(&slot_full[slot], (uint32_t)(6 * job.rlen * 2));
      for (int p = 0; p < 6; ++p) {
        const __nv_bfloat16* srcrow =
            job.src + (((size_t)p * job.hs + j) * job.g + ph) * job.krow;
        int t = 0, u = u0;
        while (t < job.rlen) {
          const int len = min(job.krow - u, job.rlen - t);
          bulk_g2s(dst + (size_t)p * job.rlen + t, srcrow + u, (uint32_t)(len * 2),
                   &slot_full[slot]);
          t += len;
          u = 0;
        }
      }
    }
  }
  // After an abort, copies may still be in flight: they land before the CTA
  // exits (in a normal run the MMA threads have already seen every fill).
  for (long long r = row_id > job.nslots ? row_id - job.nslots : 0; r < row_id; ++r) {
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(&slot_full[r % job.nslots], (uint32_t)((r / job.nslots) & 1)))
      if (global_ns() - t0 > kWaitNs) break;
  }
}

// An MMA issuer's end: every MMA it issued has completed (done_bar, which
// every issuer commits to) and the arrivals of its last commits on the stage
// and slot barriers have landed, so that nothing is in flight on them.
__device__ __forceinline__ void issuer_drain(CtaShared& sh, uint32_t gidx, uint32_t row_id,
                                             int nslots, bool ok, volatile int* abort_flag) {
  mma_commit(&sh.done_bar);
  if (!settle(&sh.done_bar, 0u)) *abort_flag = 1;
  for (uint32_t st = 0; ok && st < (uint32_t)kStages && st < gidx; ++st) {
    const uint32_t last = st + kStages * ((gidx - 1 - st) / kStages);
    if (!settle(&sh.a_empty[st], (last / kStages) & 1u)) *abort_flag = 1;
  }
  const uint32_t ns_ = (uint32_t)nslots;
  for (uint32_t sl = 0; ok && sl < ns_ && sl < row_id; ++sl) {
    const uint32_t last = sl + ns_ * ((row_id - 1 - sl) / ns_);
    if (!settle(&sh.slot_empty[sl], (last / ns_) & 1u)) *abort_flag = 1;
  }
}

// Invalidates every barrier of a quiescent CTA (thread 0), for the next item.
__device__ __forceinline__ void inval_barriers(CtaShared& sh) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_inval(&sh.a_full[s]);
      mbar_inval(&sh.a_empty[s]);
    }
    for (int s = 0; s < kMaxSlots; ++s) {
      mbar_inval(&sh.slot_full[s]);
      mbar_inval(&sh.slot_empty[s]);
    }
    mbar_inval(&sh.done_bar);
  }
}

// One work item of a contraction: output rows bx * 128 .., column block by,
// source rows of split bz (an item of a bake's queue launch or of a batch's
// persistent kernel: the same body, so the same bits).  Each CTA sums at most kMaxK of K in
// one TMEM accumulation chain per channel.  The caller holds all 512 TMEM
// columns at `tmem`.  Returns false when a bounded wait gave up (the job's
// error word is set).  Otherwise every barrier is quiescent and invalidated
// on return, so the CTA may run another item.
template <int KIND, bool TWO>
__device__ __forceinline__ bool contract_cta(const Job& job, int bx, int by, int bz,
                                             uint32_t tmem, unsigned char* smem,
                                             CtaShared& sh) {
  uint64_t* const a_full = sh.a_full;
  uint64_t* const a_empty = sh.a_empty;
  uint64_t* const slot_full = sh.slot_full;
  uint64_t* const slot_empty = sh.slot_empty;
  uint64_t& done_bar = sh.done_bar;
  int& abort_sh = sh.abort;
  double(*wsum_sh)[kM] = sh.wsum;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i0 = bx * kM;
  const int x0 = by / job.nblk;
  const int n0 = (by - x0 * job.nblk) * job.nb;
  const int split = bz;
  const SmemPlan sp = smem_plan(job);
  __nv_bfloat16* slots = reinterpret_cast<__nv_bfloat16*>(smem + sp.slots);
  float* cosd_sm = reinterpret_cast<float*>(smem + sp.cosd);
  volatile int* abort_flag = &abort_sh;

  // Producer warps only for lane quarters that hold output rows (four per
  // quarter); the others have nothing to generate and stay out of the loop.
  // quarters 0-1 hold rows of the first output and 2-3 of the second (pair),
  // or all four the first output's rows i0 ..
  const bool kint = job.kinter > 1;
  auto quarter_live = [&](int q) -> bool {
    if (kint) return true;
    if (job.pair) return q < 2 ? 32 * q < job.ho : 32 * (q - 2) < job.ho_b;
    return i0 + 32 * q < job.ho;
  };
  int live_count = 0;
  for (int q = 0; q < 4; ++q) live_count += quarter_live(q) ? 1 : 0;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      // arrivals per stage: the four warps of every live quarter, or of the
      // owning quarter alone (K interleave)
      mbar_init(&a_full[s], kint ? 4 : 4 * live_count);
      mbar_init(&a_empty[s], kMmaWarps);
    }
    for (int s = 0; s < kMaxSlots; ++s) {
      mbar_init(&slot_full[s], 1);
      mbar_init(&slot_empty[s], kMmaWarps);
    }
    mbar_init(&done_bar, kMmaWarps);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // cos of the column offsets in phase order, shifted by this CTA's column
  // residue: cosd_sm[ph][k] = cos_d[g ((k - (s/g) x0) mod krow) + ph]
  {
    const int sh = (job.s / job.g) * x0 % job.krow;
    for (int e = tid; e < job.g * job.kpad; e += kThreads) {
      int ph = e / job.kpad, k = e - ph * job.kpad;
      int kk = k - sh;
      if (kk < 0) kk += job.krow;
      cosd_sm[e] = k < job.krow ? job.cos_d[job.g * kk + ph] : 0.0f;
    }
  }
  // generic shared-memory writes of a previous work item (the K-interleave
  // reduction) come before this item's bulk copies into the same bytes
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (kint) {
    // K interleave: a quarter's lanes in the three stage slots it does not
    // own stay zero, so the MMAs of other quarters' stages add nothing there
    if (warp < kProducerWarps) {
      const int q = warp & 3, h = warp >> 2;
      const uint32_t zero[4] = {0u, 0u, 0u, 0u};
      const uint32_t base = tmem + ((uint32_t)(32 * q) << 16);
      for (int st = 0; st < kStages; ++st) {
        if (st == q) continue;
        const uint32_t col = (uint32_t)(kACol + st * kKS + 4 * h);
        tmem_st4(base + col, zero);
        tmem_st4(base + col + 16, zero);
      }
      tmem_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }

  // This CTA's source rows: j = split, split + ksplit, ... (round robin, so
  // every split holds the same mix of latitudes and the visible-offset
  // windows cost every CTA about the same).
  const int jstep = job.ksplit;
  // K per pipeline stage: 64 with hi-only weights (two products), else 32
  constexpr int KS = TWO ? 64 : kKS;
  constexpr int KW = KS / 4;   // K per producer warp and stage
  constexpr int NG = KW / 8;   // groups of 8 K per producer warp and stage
  const int kchunks = job.kpad / KS;
  // stages this CTA runs: the visible chunks of each of its source rows
  const int* vis_row = job.vis + (size_t)bx * job.hs;
  long long total = 0;
  for (int j = split; j < job.hs; j += jstep) {
    int ca, cb;
    visible_chunks(vis_row[j], job.krow, KS, kchunks, ca, cb);
    total += (long long)job.g * (ca + kchunks - cb);
  }
  const bool want_wsum = (KIND == 0 || job.wsum1) && by == 0;
  const bool want_wsum_b = job.pair && (job.kind_b == 0 || job.wsum1_b) && by == 0;

  if (warp < kProducerWarps) {
    // ---- weight producers: rows 32q + lane, K sub-range [8h, 8h + 8) of each stage
    const int q = warp & 3, h = warp >> 2;
    const int row = 32 * q + lane;
    const bool live = quarter_live(q);
    // second output of a pair in quarters 2-3 (its own rows, kind, roughness)
    const bool second = job.pair && q >= 2;
    const int gi = kint ? lane : (second ? row - 64 : i0 + row);
    const int ho_here = second ? job.ho_b : job.ho;
    const float* orows = second ? job.out_rows_b : job.out_rows;
    const bool ggx = second ? job.kind_b == 0 : KIND == 0;
    const bool want = second ? want_wsum_b : want_wsum;
    float cp = 0.0f, sp_ = 0.0f;
    if (gi < ho_here) {
      cp = orows[2 * gi];
      sp_ = orows[2 * gi + 1];
    }
    const float a2 = second ? job.a2_b : job.a2;
    const float alpha = 0.5f * (1.0f + a2), beta = 0.5f * (a2 - 1.0f), ka = a2 / kPiF;
    const float2 alpha2 = make_float2(alpha, alpha), beta2 = make_float2(beta, beta);
    const float2 minus1 = make_float2(-1.0f, -1.0f);
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    double wacc = 0.0;
    uint32_t gidx = 0;
    int pending = -1;  // stage whose stores are issued but not yet published
    bool ok = true;
    for (int j = split; live && j < job.hs && ok; j += jstep) {
      int ca, cb;
      visible_chunks(vis_row[j], job.krow, KS, kchunks, ca, cb);
      const int nvis = ca + kchunks - cb;
      const float cq = job.src_rows[3 * j], sq = job.src_rows[3 * j + 1];
      const float om = job.src_rows[3 * j + 2];
      const float ccq = cp * cq, ssq = sp_ * sq;
      const float k1 = ggx ? ka * om : om;
      const float2 ccq2 = make_float2(ccq, ccq), ssq2 = make_float2(ssq, ssq);
      const float2 k12 = make_float2(k1, k1);
      for (int ph = 0; ph < job.g && ok; ++ph) {
        const float* cdrow = cosd_sm + ph * job.kpad;
        float2 rowsum2 = make_float2(0.0f, 0.0f);
        for (int v = 0; v < nvis; ++v, ++gidx) {
          const int kc = v < ca ? v : cb + (v - ca);
          const int st = (int)(gidx & (kStages - 1));
          const uint32_t use = gidx / kStages;
          if (kint && st != q) continue;  // another quarter's stage
          uint32_t hw[4 * NG], lw[4];
          if (live) {
#pragma unroll
           for (int gq = 0; gq < NG; ++gq) {
            const int kb = kc * KS + KW * h + 8 * gq;
            float2 w[4];
            weights8<!TWO>(cdrow, kb, job.krow, ccq2, ssq2, k12, alpha2, beta2, ggx, w);
            __nv_bfloat162 h2s[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              __nv_bfloat162 h2 = __floats2bfloat162_rn(w[e].x, w[e].y);
              if (TWO) h2 = __hmax2(h2, bf16_zero2());  // max(bf16(w), 0) = bf16(max(w, 0))
              h2s[e] = h2;
              hw[4 * gq + e] = *reinterpret_cast<const uint32_t*>(&h2);
              if (!TWO) {
                const float2 lo = __ffma2_rn(__bfloat1622float2(h2), minus1, w[e]);
                const __nv_bfloat162 l2 = __floats2bfloat162_rn(lo.x, lo.y);
                lw[e] = *reinterpret_cast<const uint32_t*>(&l2);
              }
            }
            if (want) {
              if (TWO) {  // the weights the MMAs use
#pragma unroll
                for (int e = 0; e < 4; ++e) w[e] = __bfloat1622float2(h2s[e]);
              }
              rowsum2 = __fadd2_rn(__fadd2_rn(rowsum2, w[0]), __fadd2_rn(__fadd2_rn(w[1], w[2]), w[3]));
            }
           }
          }
          // Software pipeline: the previous stage's TMEM stores landed while
          // this stage's weights were computed; publish that stage now.
          if (pending >= 0) {
            if (live) tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&a_full[pending]);
            pending = -1;
          }
          if (use >= 1 && !wait_bar(&a_empty[st], (uint32_t)((use - 1) & 1), abort_flag)) {
            ok = false;
            break;
          }
          if (live) {
            if (TWO) {
              // hi only, K 16t .. 16t + 15 at stage column 8t: this warp's 16 K
              tmem_st8(lane_base + (uint32_t)(kACol + st * kKS + 8 * h), hw);
            } else {
              const uint32_t col = (uint32_t)(kACol + st * kKS + 4 * h);
              tmem_st4(lane_base + col, hw);
              tmem_st4(lane_base + col + 16, lw);
            }
          }
          if (kint) {
            // publish at once: the next stage this quarter owns is four away
            tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&a_full[st]);
          } else {
            pending = st;
          }
        }
        wacc += (double)(rowsum2.x + rowsum2.y);
      }
    }
    if (live) tmem_wait_st();
    if (pending >= 0) {
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&a_full[pending]);
    }
    wsum_sh[h][row] = wacc;
  } else if (warp < kMmaWarp0 + kMmaWarps) {
    // ---- MMA issuers: one thread per colour channel -----------------------------
    // (two issuers per channel, on column halves, measured slower)
    const int ch = warp - kMmaWarp0;
    if (lane == 0 && total > 0) {
      const uint32_t idesc = idesc_bf16(kM, job.nb);
      // B descriptors differ only in the start-address field (16-byte units;
      // every staged address stays below 2^18 bytes, so no carry out of it).
      const uint64_t bdesc0 = smem_desc(smem_u32(slots), 16, 128);
      const uint32_t r8 = (uint32_t)(job.rlen >> 3);
      const uint32_t d = tmem + (uint32_t)(ch * job.nb);
      // this issuer's hi plane rows within a slot, in 16-byte units
      const uint32_t plane16 = 2u * (uint32_t)ch * r8;
      const uint32_t slot16 = 6u * r8;
      uint32_t gidx = 0, row_id = 0;
      bool ok = true;
      for (int j = split; j < job.hs && ok; j += jstep) {
        int ca, cb;
        visible_chunks(vis_row[j], job.krow, KS, kchunks, ca, cb);
        const int nvis = ca + kchunks - cb;
        if (nvis == 0) continue;  // not staged by the loader either
        for (int ph = 0; ph < job.g && ok; ++ph, ++row_id) {
          const uint32_t slot = row_id % (uint32_t)job.nslots;
          if (!wait_bar(&slot_full[slot], (row_id / (uint32_t)job.nslots) & 1u, abort_flag)) {
            ok = false;
            break;
          }
          const uint64_t dbh_row = bdesc0 + (uint64_t)(slot * slot16 + plane16);
          for (int v = 0; v < nvis; ++v, ++gidx) {
            const int kc = v < ca ? v : cb + (v - ca);
            const uint64_t dbh = dbh_row + (uint64_t)(kc * (KS * 2 / 16));
            const uint32_t st = gidx & (kStages - 1);
            if (!wait_bar(&a_full[st], (gidx / kStages) & 1u, abort_flag)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a_hi = tmem + (uint32_t)kACol + st * kKS;
            if (TWO)
              mma_stage64_ts2(d, a_hi, dbh, dbh + r8, idesc, gidx != 0, &a_empty[st]);
            else
              mma_stage_ts(d, a_hi, dbh, dbh + r8, dbh + 2, dbh + 2 + r8, idesc, gidx != 0,
                           &a_empty[st]);
          }
          // the row's slot is free once its MMAs are done
          if (ok) mma_commit(&slot_empty[slot]);
        }
      }
      // every MMA issued by all issuers has completed before the accumulators
      // are read and TMEM is released; the barriers are quiescent
      issuer_drain(sh, gidx, row_id, job.nslots, ok, abort_flag);
    }
  } else if (warp == kLoaderWarp && lane == 0) {
    // ---- Hankel row loader ----
    load_rows(job, slots, slot_full, slot_empty, split, KS, kchunks, vis_row, n0, abort_flag);
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const bool failed = abort_sh != 0;
  if (failed) {
    if (tid == 0) atomicExch(job.error, 1);
  } else if (kint) {
    // K interleave: the four lane quarters hold the same output rows and
    // every fourth K stage.  Their sums are added here, in quarter order, so
    // one partial sum per split is written (shared memory is free again: the
    // loader has seen its last copy land).
    const int ncol = 3 * job.nb;
    float* red = reinterpret_cast<float*>(smem);  // [quarter][column][lane]
    if (warp < kProducerWarps) {
      const int q = warp & 3;
      for (int c0 = 16 * (warp >> 2); c0 < ncol; c0 += 16 * (kProducerWarps / 4)) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int u = 0; u < 16; ++u) red[((size_t)q * ncol + c0 + u) * 32 + lane] = v[u];
      }
    }
    __syncthreads();
    for (int e = tid; e < ncol * 32; e += kThreads) {
      const int col = e >> 5, r = e & 31, ch = col / job.nb, n = col - ch * job.nb;
      const int x = x0 + job.m * (n0 + n);
      if (r < job.ho && n0 + n < job.nres && x < job.wo) {
        const size_t c = (size_t)col * 32 + r, qs = (size_t)ncol * 32;
        const float sum = ((red[c] + red[qs + c]) + red[2 * qs + c]) + red[3 * qs + c];
        job.partial[(((size_t)split * 3 + ch) * job.wo + x) * job.ho + r] =
            total > 0 ? sum : 0.0f;
      }
    }
    if (tid < 32 && want_wsum && tid < job.ho) {
      double ws = 0.0;
      for (int q = 0; q < 4; ++q)
        for (int hh = 0; hh < kProducerWarps / 4; ++hh) ws += wsum_sh[hh][32 * q + tid];
      job.wsum_part[(size_t)split * job.ho + tid] = ws;
    }
  } else {
    const int q = warp & 3;
    if (warp < kProducerWarps && quarter_live(q)) {
      // accumulators -> partial sums (lane = output row, column = (channel, n));
      // the four warps of a lane quarter take every fourth 16-column chunk
      const bool second = job.pair && q >= 2;
      const int gi = second ? 32 * (q - 2) + lane : i0 + 32 * q + lane;
      const int ho_here = second ? job.ho_b : job.ho;
      float* part = second ? job.partial_b : job.partial;
      const int slot_split = split;
      for (int c0 = 16 * (warp >> 2); c0 < 3 * job.nb; c0 += 16 * (kProducerWarps / 4)) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int col = c0 + u, ch = col / job.nb, n = col - ch * job.nb;
          const int x = x0 + job.m * (n0 + n);
          if (gi < ho_here && n0 + n < job.nres && x < job.wo)
            part[(((size_t)slot_split * 3 + ch) * job.wo + x) * ho_here + gi] =
                total > 0 ? v[u] : 0.0f;
        }
      }
    }
    if (tid < kM) {
      const bool second = job.pair && tid >= 64;
      const int gi = second ? tid - 64 : i0 + tid;
      const int slot_split = split;
      if (second ? (want_wsum_b && gi < job.ho_b) : (want_wsum && gi < job.ho)) {
        double ws = 0.0;
        for (int hh = 0; hh < kProducerWarps / 4; ++hh) ws += wsum_sh[hh][tid];
        if (second)
          job.wsum_part_b[(size_t)split * job.ho_b + gi] = ws;
        else
          job.wsum_part[(size_t)slot_split * job.ho + gi] = ws;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (failed) return false;
  // quiescent: every arrival has landed (the MMA issuers settled the last
  // phases), so the barriers can be invalidated for the next work item
  inval_barriers(sh);
  return true;
}

// One CTA of a column-tile contraction (Job::ct): output columns n0 ..
// n0 + 127 of residue x0 (column block by), every row of the output, source
// rows of split bz.  A = the staged Hankel
// rows (M = 128 columns: the descriptor of the row tiles' B), B = the weights
// of the kCtN rows in shared memory; accumulator lane = column, TMEM column =
// channel * kCtN + row.  Producer warps form G groups, group g owning the
// stage slots st with st % G == g; each warp writes 8 K of 32 rows per stage
// (one 16-byte store per lane).  Same contract as contract_cta: false when a bounded wait
// gave up, else every barrier quiescent and invalidated.
template <int KIND, bool TWO>
__device__ __forceinline__ bool contract_cta_ct(const Job& job, int by, int bz, uint32_t tmem,
                                                unsigned char* smem, CtaShared& sh) {
  uint64_t* const a_full = sh.a_full;
  uint64_t* const a_empty = sh.a_empty;
  uint64_t* const slot_full = sh.slot_full;
  uint64_t* const slot_empty = sh.slot_empty;
  double* const wsum_sh = &sh.wsum[0][0];  // [producer warp][lane]
  static_assert(sizeof(CtaShared::wsum) >= sizeof(double) * kProducerWarps * 32, "weight sums");

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x0 = by / job.nblk;
  const int n0 = (by - x0 * job.nblk) * kM;
  const int split = bz;
  const SmemPlan sp = smem_plan(job);
  __nv_bfloat16* slots = reinterpret_cast<__nv_bfloat16*>(smem + sp.slots);
  float* cosd_sm = reinterpret_cast<float*>(smem + sp.cosd);
  unsigned char* bst = smem + sp.bst;
  volatile int* abort_flag = &sh.abort;

  constexpr int KS = TWO ? 64 : kKS;  // K per stage
  constexpr int KG = KS / 8;          // groups of 8 K per stage
  constexpr int N = kCtN;             // weight rows (MMA N)
  constexpr int R = N / 32;           // row groups of 32 lanes
  constexpr int T = R * KG;           // producer tasks per stage: 8 or 16
  constexpr int G = kProducerWarps / T;  // producer groups: 2 or 1
  constexpr int TW = T;               // warps per group, one task each
  static_assert(kProducerWarps % T == 0 && kStages % G == 0, "producer groups");
  constexpr uint32_t stage_bytes = 128u * N;
  constexpr uint32_t group_bytes = 16u * N;               // 8 K of all N rows
  constexpr uint32_t plane_bytes = (uint32_t)KG * group_bytes;  // lo plane after hi

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&a_full[s], TW);  // the warps of the owning group
      mbar_init(&a_empty[s], kMmaWarps);  // the issuers' commits
    }
    for (int s = 0; s < kMaxSlots; ++s) {
      mbar_init(&slot_full[s], 1);
      mbar_init(&slot_empty[s], kMmaWarps);
    }
    mbar_init(&sh.done_bar, kMmaWarps);
    sh.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  {
    const int shf = (job.s / job.g) * x0 % job.krow;
    for (int e = tid; e < job.g * job.kpad; e += kThreads) {
      int ph = e / job.kpad, k = e - ph * job.kpad;
      int kk = k - shf;
      if (kk < 0) kk += job.krow;
      cosd_sm[e] = k < job.krow ? job.cos_d[job.g * kk + ph] : 0.0f;
    }
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  const int jstep = job.ksplit;
  const int kchunks = job.kpad / KS;
  const int* vis_row = job.vis;  // the one row tile
  long long total = 0;
  for (int j = split; j < job.hs; j += jstep) {
    int ca, cb;
    visible_chunks(vis_row[j], job.krow, KS, kchunks, ca, cb);
    total += (long long)job.g * (ca + kchunks - cb);
  }
  const bool by0 = by == 0;

  if (warp < kProducerWarps) {
    // ---- weight producers: B row i = 32 rg + lane, 8 K (group kg) of the stage
    const int gw = warp / TW, wi = warp - gw * TW;
    const int rg = wi % R, kg = wi / R;
    const int i = 32 * rg + lane;  // output row
    const bool real = i < job.ho;
    float cp = 0.0f, sp_ = 0.0f;
    if (real) {
      cp = job.out_rows[2 * i];
      sp_ = job.out_rows[2 * i + 1];
    }
    const float a2 = job.a2;
    constexpr bool ggx = KIND == 0;
    const bool want = real && (ggx || job.wsum1) && by0;
    const float alpha = 0.5f * (1.0f + a2), beta = 0.5f * (a2 - 1.0f), ka = a2 / kPiF;
    const float2 alpha2 = make_float2(alpha, alpha), beta2 = make_float2(beta, beta);
    const float2 minus1 = make_float2(-1.0f, -1.0f);
    const uint32_t row_off = (uint32_t)((i >> 3) * 128 + (i & 7) * 16);
    double wacc = 0.0;
    uint32_t gidx = 0;
    bool ok = true;
    for (int j = split; j < job.hs && ok; j += jstep) {
      int ca, cb;
      visible_chunks(vis_row[j], job.krow, KS, kchunks, ca, cb);
      const int nvis = ca + kchunks - cb;
      const float cq = job.src_rows[3 * j], sq = job.src_rows[3 * j + 1];
      const float om = job.src_rows[3 * j + 2];
      const float ccq = cp * cq, ssq = sp_ * sq;
      const float k1 = real ? (ggx ? ka * om : om) : 0.0f;  // padded rows: zero weights
      const float2 ccq2 = make_float2(ccq, ccq), ssq2 = make_float2(ssq, ssq);
      const float2 k12 = make_float2(k1, k1);
      for (int ph = 0; ph < job.g && ok; ++ph) {
        const float* cdrow = cosd_sm + ph * job.kpad;
        float2 rowsum2 = make_float2(0.0f, 0.0f);
        for (int v = 0; v < nvis; ++v, ++gidx) {
          const int st = (int)(gidx & (kStages - 1));
          if (st % G != gw) continue;  // another group's stage slot
          const uint32_t use = gidx / kStages;
          const int kc = v < ca ? v : cb + (v - ca);
          uint32_t hw[4], lw[4];
          {
            float2 w[4];
            weights8(cdrow, kc * KS + 8 * kg, job.krow, ccq2, ssq2, k12, alpha2, beta2, ggx, w);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 h2 = __floats2bfloat162_rn(w[e].x, w[e].y);
              hw[e] = *reinterpret_cast<const uint32_t*>(&h2);
              if (TWO) {
                w[e] = __bfloat1622float2(h2);  // the weight the MMAs use
              } else {
                const float2 lo = __ffma2_rn(__bfloat1622float2(h2), minus1, w[e]);
                const __nv_bfloat162 l2 = __floats2bfloat162_rn(lo.x, lo.y);
                lw[e] = *reinterpret_cast<const uint32_t*>(&l2);
              }
            }
            if (want)
              rowsum2 = __fadd2_rn(__fadd2_rn(rowsum2, w[0]), __fadd2_rn(__fadd2_rn(w[1], w[2]), w[3]));
          }
          if (use >= 1 && !wait_bar(&a_empty[st], (uint32_t)((use - 1) & 1), abort_flag)) {
            ok = false;
            break;
          }
          {
            unsigned char* g8 = bst + (size_t)st * stage_bytes + row_off + (size_t)kg * group_bytes;
            *reinterpret_cast<uint4*>(g8) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            if (!TWO)
              *reinterpret_cast<uint4*>(g8 + plane_bytes) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
          }
          // the stores are read by the tensor cores (async proxy)
          fence_async_smem();
          __syncwarp();
          if (lane == 0) mbar_arrive(&a_full[st]);
        }
        wacc += (double)(rowsum2.x + rowsum2.y);
      }
    }
    wsum_sh[warp * 32 + lane] = wacc;
  } else if (warp < kMmaWarp0 + kMmaWarps) {
    // ---- MMA issuers: one thread per colour channel ------------------------------
    const int ch = warp - kMmaWarp0;
    if (lane == 0 && total > 0) {
      const uint32_t idesc = idesc_bf16(kM, N);
      // descriptors differ only in the start-address field (16-byte units;
      // every address stays below 2^18 bytes, so no carry out of it)
      const uint64_t adesc0 = smem_desc(smem_u32(slots), 16, 128);
      const uint64_t bdesc0 = smem_desc(smem_u32(bst), group_bytes, 128);
      const uint32_t r8 = (uint32_t)(job.rlen >> 3);
      const uint32_t plane16 = 2u * (uint32_t)ch * r8;  // this channel's hi plane
      const uint32_t slot16 = 6u * r8;
      const uint32_t stage16 = stage_bytes >> 4, lo16 = plane_bytes >> 4;
      const uint32_t bk = 2u * (group_bytes >> 4);  // B units per K = 16
      const uint32_t d = tmem + (uint32_t)(ch * N);
      uint32_t gidx = 0, row_id = 0;
      bool ok = true;
      for (int j = split; j < job.hs && ok; j += jstep) {
        int ca, cb;
        visible_chunks(vis_row[j], job.krow, KS, kchunks, ca, cb);
        const int nvis = ca + kchunks - cb;
        if (nvis == 0) continue;  // not staged by the loader either
        for (int ph = 0; ph < job.g && ok; ++ph, ++row_id) {
          const uint32_t slot = row_id % (uint32_t)job.nslots;
          if (!wait_bar(&slot_full[slot], (row_id / (uint32_t)job.nslots) & 1u, abort_flag)) {
            ok = false;
            break;
          }
          const uint64_t arow = adesc0 + (uint64_t)(slot * slot16 + plane16);
          for (int v = 0; v < nvis; ++v, ++gidx) {
            const int kc = v < ca ? v : cb + (v - ca);
            const uint32_t st = gidx & (kStages - 1);
            if (!wait_bar(&a_full[st], (gidx / kStages) & 1u, abort_flag)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t ah = arow + (uint64_t)(kc * (KS * 2 / 16));
            const uint64_t bh = bdesc0 + (uint64_t)(st * stage16);
            if (TWO)
              mma_stage64_ss2(d, ah, ah + r8, bh, bk, idesc, gidx != 0, &a_empty[st]);
            else
              mma_stage_ss(d, ah, ah + r8, bh, bh + lo16, bk, idesc, gidx != 0, &a_empty[st]);
          }
          if (ok) mma_commit(&slot_empty[slot]);  // the row's slot is free once its MMAs are done
        }
      }
      issuer_drain(sh, gidx, row_id, job.nslots, ok, abort_flag);
    }
  } else if (warp == kLoaderWarp && lane == 0) {
    // ---- Hankel row loader (rows of 8 * 128 + kpad elements) ----
    load_rows(job, slots, slot_full, slot_empty, split, KS, kchunks, vis_row, n0, abort_flag);
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const bool failed = sh.abort != 0;
  if (failed) {
    if (tid == 0) atomicExch(job.error, 1);
  } else {
    if (warp < kProducerWarps) {
      // accumulators -> partial sums: lane quarter q holds columns 32 q ..;
      // its four warps take every fourth 16-column chunk (16 rows of one channel)
      const int q = warp & 3;
      const int n = 32 * q + lane;
      const int x = x0 + job.m * (n0 + n);
      const bool col_ok = n0 + n < job.nres && x < job.wo;
      for (int c0 = 16 * (warp >> 2); c0 < 3 * N; c0 += 16 * (kProducerWarps / 4)) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
        const int ch = c0 / N, i0 = c0 - ch * N;
        if (!col_ok) continue;
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int i = i0 + u;
          const float val = total > 0 ? v[u] : 0.0f;
          if (i < job.ho) job.partial[(((size_t)split * 3 + ch) * job.wo + x) * job.ho + i] = val;
        }
      }
    }
    if ((KIND == 0 || job.wsum1) && by0 && tid < job.ho) {
      // weight sums of row i: the warps of row group i / 32, in warp order
      const int i = tid, rg = i >> 5, l = i & 31;
      double ws = 0.0;
      for (int w = 0; w < kProducerWarps; ++w)
        if ((w % TW) % R == rg) ws += wsum_sh[w * 32 + l];  // every group, in warp order
      job.wsum_part[(size_t)split * job.ho + i] = ws;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (failed) return false;
  inval_barriers(sh);
  return true;
}

// TMEM for a contraction CTA: all 512 columns, allocated by warp 0.
__device__ __forceinline__ uint32_t tmem_alloc_all(uint32_t* slot) {
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(slot)),
                 "r"((uint32_t)kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return *slot;
}

__device__ __forceinline__ void tmem_free_all(uint32_t tmem) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)kTmemCols));
}

// One work item: the CTA (bx, by, bz) of the grid a job would have as a
// launch of its own -- the row tile bx (row tiles; column tiles have one),
// the column block and residue by, the split bz -- run on this CTA, with all
// of TMEM at `tmem` and the job's record in shared memory.
__device__ __forceinline__ bool run_item(const Job& job, int bx, int by, int bz, uint32_t tmem,
                                         unsigned char* smem, CtaShared& sh) {
  if (job.ct) {
    if (job.kind == 1) return contract_cta_ct<1, false>(job, by, bz, tmem, smem, sh);
    if (job.two_prod) return contract_cta_ct<0, true>(job, by, bz, tmem, smem, sh);
    return contract_cta_ct<0, false>(job, by, bz, tmem, smem, sh);
  }
  if (job.kind == 1) return contract_cta<1, false>(job, bx, by, bz, tmem, smem, sh);
  if (job.two_prod) return contract_cta<0, true>(job, bx, by, bz, tmem, smem, sh);
  return contract_cta<0, false>(job, bx, by, bz, tmem, smem, sh);
}

__device__ __forceinline__ void copy_job(Job& dst, const Job& src) {
  static_assert(sizeof(Job) % 8 == 0, "job copy in 8-byte words");
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(&src);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
  for (int e = threadIdx.x; e < (int)(sizeof(Job) / 8); e += blockDim.x) d[e] = s[e];
}

// The contractions of one bake as one queue: job k owns items
// [begin[k], begin[k + 1]), item = bx + gx (by + gy bz) within the job.  The
// jobs come in the order of their items' K, largest first, and one CTA per SM
// pulls items from a counter until the queue is empty: the jobs need no
// splits to fill the GPU on their own, and no launch waits for another's tail.
constexpr int kMaxQueueJobs = ALTHEA_IBL_MAX_MIPS + 1;
struct QueueArgs {
  Job jobs[kMaxQueueJobs];
  int begin[kMaxQueueJobs + 1];
  int gx[kMaxQueueJobs], gy[kMaxQueueJobs];
  int n;
};
static_assert(sizeof(QueueArgs) <= 4096, "queue arguments fit the kernel parameter space");

__global__ void __launch_bounds__(kThreads, 1)
    contract_queue_kernel(const __grid_constant__ QueueArgs a, unsigned int* __restrict__ next) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ CtaShared sh;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int item_sh;
  __shared__ __align__(16) Job job_sh;
  const uint32_t tmem = tmem_alloc_all(&tmem_base_sh);
  for (;;) {
    if (threadIdx.x == 0) item_sh = (int)atomicAdd(next, 1u);
    __syncthreads();
    const int it = item_sh;
    if (it >= a.begin[a.n]) break;
    int k = 0;
    while (k + 1 < a.n && it >= a.begin[k + 1]) ++k;
    copy_job(job_sh, a.jobs[k]);
    __syncthreads();
    const int local = it - a.begin[k], gx = a.gx[k], gy = a.gy[k];
    const bool ok = run_item(job_sh, local % gx, (local / gx) % gy, local / (gx * gy), tmem,
                             smem, sh);
    if (!ok) break;  // uniform: every thread read the same abort flag
    __syncthreads();  // item_sh and job_sh are rewritten next
  }
  tmem_free_all(tmem);
}

// One CTA of some job of a batch.
struct WorkItem {
  int job;         // index into the job table
  int bx, by, bz;  // row tile, column block and split within the job
};

// The persistent contraction kernel of a batch: one CTA per SM (each holds
// all of TMEM for its lifetime), pulling (job, tile, column block, split)
// work items from a queue in the order given (largest first) until it is
// empty.  Each item runs exactly the body that the probe's single bake runs
// for it (contract_queue_kernel), so the results are the same bits.  A CTA whose bounded wait gave up stops
// taking items (the job's error word is set).
__global__ void __launch_bounds__(kThreads, 1)
    contract_persistent_kernel(const Job* __restrict__ jobs, const WorkItem* __restrict__ items,
                               int nitems, unsigned int* __restrict__ next) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ CtaShared sh;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int item_sh;
  __shared__ __align__(16) Job job_sh;
  const uint32_t tmem = tmem_alloc_all(&tmem_base_sh);
  for (;;) {
    if (threadIdx.x == 0) item_sh = (int)atomicAdd(next, 1u);
    __syncthreads();
    const int it = item_sh;
    if (it >= nitems) break;
    const WorkItem wi = items[it];
    copy_job(job_sh, jobs[wi.job]);
    __syncthreads();
    const bool ok = run_item(job_sh, wi.bx, wi.by, wi.bz, tmem, smem, sh);
    if (!ok) break;  // uniform: every thread read the same abort flag
    __syncthreads();  // item_sh and job_sh are rewritten next
  }
  tmem_free_all(tmem);
}

// ---- narrow outputs on the CUDA cores ----------------------------------------------
// An output of at most kNarrowMax texels and kNarrowMaxW columns (the
// roughest mips) is a GEMM with M and N of a few rows and columns against a K
// of a whole source level: on the tensor cores most of each MMA would be
// padding.  These sum the same quadrature on the CUDA cores, sharing weights:
// the weight of output (i, x) and source (j, y) depends on (i, j) and the
// column offset t = (y - s x) mod ws only.  A block takes one output row i and
// a band of source rows; per source row it stages the row and the ws weights
// of row i (computed once, with their sum, which is the same for every x).
// Lanes are output columns (x = lane mod wo; with wo < 32 the lanes of one x
// split the columns further): each walks source columns y, reading the staged
// texel L[y] (one address per warp, a broadcast) and the weight W[t].  The
// weights are stored skewed, W[t] at t + t / s, which puts the lanes' t
// (s apart) in different banks.  FP32 within a row, FP64 across rows, a fixed
// order across warps; bands are combined by narrow_finish_kernel.  Measured
// on a 2048-wide source: 16x8 in 129 us (the tensor path: 334 us), 8x4 in
// 81 us (414 us); a 32x16 output took 405 us here against 323 us on the
// tensor cores, hence the 128-texel limit.
constexpr int kNarrowMax = 128;
constexpr int kNarrowMaxW = 32;
constexpr int kNarrowThreads = 256;
constexpr int kNarrowWarps = kNarrowThreads / 32;
struct NarrowJob {
  const float4* src;        // source level, RGBA32F, ws x hs
  int ws, hs, wo, ho;
  int s;                    // ws / wo
  int ksplit;               // bands of source rows
  float a2;
  const float* cos_d;       // [ws]  cos(2 pi (d + 0.5) / ws)
  const float* src_rows;    // [hs][3]  cos q, sin q, Omega
  const float* out_rows;    // [ho][2]  cos p, sin p
  double* partial;          // [ksplit][wo * ho][4]  R, G, B, weight sum
};

// Dynamic shared memory of narrow_kernel: the staged row (ws float4), the
// skewed weights (ws + wo floats), the cos table (ws floats), both float
// arrays rounded up to a multiple of 4, and the per-lane FP64 sums of the
// final reduction (8 warps x 32 lanes x 3).
__host__ __device__ inline size_t narrow_smem_bytes(int ws, int wo) {
  const size_t wsk = (size_t)((ws + wo + 3) & ~3), cdn = (size_t)((ws + 3) & ~3);
  return (size_t)ws * 16 + (wsk + cdn) * 4 + (size_t)kNarrowThreads * 3 * 8;
}

template <int KIND>
__device__ __forceinline__ void narrow_block(const NarrowJob& J, int i, int band) {
  extern __shared__ __align__(16) unsigned char nsm[];
  const int ws = J.ws, wo = J.wo, s = J.s;
  float4* row = reinterpret_cast<float4*>(nsm);        // staged L_j
  float* Wsk = reinterpret_cast<float*>(row + ws);      // weights of (i, j), skewed
  float* cd = Wsk + ((ws + wo + 3) & ~3);               // cos_d
  double* fin = reinterpret_cast<double*>(cd + ((ws + 3) & ~3));  // [256][3]
  __shared__ float red[kNarrowWarps];
  __shared__ double wsum_sh;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // lane -> (output column x, sub-range r of the warp's source columns)
  const int R = 32 / wo, x = lane % wo, r = lane / wo;
  const bool lane_live = r < R;
  // this lane's source columns: warp range split into R contiguous pieces
  const int wy0 = warp * ws / kNarrowWarps, wy1 = (warp + 1) * ws / kNarrowWarps;
  const int y0 = wy0 + r * (wy1 - wy0) / R, y1 = wy0 + (r + 1) * (wy1 - wy0) / R;
  for (int t = tid; t < ws; t += kNarrowThreads) cd[t] = J.cos_d[t];
  const float cp = J.out_rows[2 * i], sp = J.out_rows[2 * i + 1];
  const float alpha = 0.5f * (1.0f + J.a2), beta = 0.5f * (J.a2 - 1.0f), ka = J.a2 / kPiF;
  const int j_per = (J.hs + J.ksplit - 1) / J.ksplit;
  const int j0 = band * j_per, j1 = min(J.hs, j0 + j_per);
  const int sx = (int)(((long long)s * x) % ws);
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, wsum = 0.0;
  for (int j = j0; j < j1; ++j) {
    __syncthreads();  // the previous row and weights are no longer read
    const float4* srow = J.src + (size_t)j * ws;
    for (int y = tid; y < ws; y += kNarrowThreads) row[y] = srow[y];
    const float cq = J.src_rows[3 * j], sq = J.src_rows[3 * j + 1], om = J.src_rows[3 * j + 2];
    const float A = cp * cq, B = sp * sq, k1 = KIND == 0 ? ka * om : om;
    float part = 0.0f;
    for (int t = tid; t < ws; t += kNarrowThreads) {
      const float c = fmaf(A, cd[t], B);
      float wgt;
      if (KIND == 0) {
        const float d = fmaf(c, beta, alpha);
        wgt = k1 * c * rcp_approx(d * d);
      } else {
        wgt = k1 * c;
      }
      wgt = fmaxf(wgt, 0.0f);
      Wsk[t + t / s] = wgt;
      part += wgt;
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (tid == 0) {
      float rs = 0.0f;
      for (int w = 0; w < kNarrowWarps; ++w) rs += red[w];
      wsum += rs;
    }
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
    if (lane_live) {
      // segments of y that stay inside one block of s weights
      for (int yc = y0; yc < y1;) {
        int t0 = yc - sx;
        if (t0 < 0) t0 += ws;
        const int seg = min(y1 - yc, s - t0 % s);
        const float* wp = Wsk + t0 + t0 / s;
        const float4* lp = row + yc;
#pragma unroll 4
        for (int k = 0; k < seg; ++k) {
          const float w = wp[k];
          const float4 L = lp[k];
          s0 = fmaf(w, L.x, s0);
          s1 = fmaf(w, L.y, s1);
          s2 = fmaf(w, L.z, s2);
        }
        yc += seg;
      }
    }
    a0 += s0;
    a1 += s1;
    a2 += s2;
  }
  // every (warp, r) holds a partial sum of its columns for output x
  fin[3 * tid] = a0;
  fin[3 * tid + 1] = a1;
  fin[3 * tid + 2] = a2;
  if (tid == 0) wsum_sh = wsum;
  __syncthreads();
  if (tid < wo) {
    double t0 = 0.0, t1 = 0.0, t2 = 0.0;
    for (int w = 0; w < kNarrowWarps; ++w)
      for (int rr = 0; rr < R; ++rr) {
        const int src_t = 32 * w + rr * wo + tid;
        t0 += fin[3 * src_t];
        t1 += fin[3 * src_t + 1];
        t2 += fin[3 * src_t + 2];
      }
    double* dst = J.partial + ((size_t)band * wo * J.ho + (size_t)i * wo + tid) * 4;
    dst[0] = t0;
    dst[1] = t1;
    dst[2] = t2;
    dst[3] = wsum_sh;
  }
}

// Output row i, band of source rows `band`: grid (ho, ksplit).
template <int KIND>
__global__ void __launch_bounds__(kNarrowThreads) narrow_kernel(const NarrowJob J) {
  narrow_block<KIND>(J, blockIdx.x, blockIdx.y);
}

// The narrow jobs of many probes (one kind) in one launch: block b is block
// b - begins[k] = band * ho + i of job k.  Dynamic shared memory: the largest
// job's.
template <int KIND>
__global__ void __launch_bounds__(kNarrowThreads)
    narrow_batch_kernel(const NarrowJob* __restrict__ jobs, const long long* __restrict__ begins,
                        int njobs) {
  const int k = find_range(begins, njobs, blockIdx.x);
  const NarrowJob& J = jobs[k];
  const int local = (int)((long long)blockIdx.x - begins[k]);
  narrow_block<KIND>(J, local % J.ho, local / J.ho);
}

// One warp per output texel o: the splits in a fixed order (lane k takes k,
// k + 32, ...; then a fixed shuffle tree), normalised, written.
__device__ __forceinline__ void narrow_finish_warp(const NarrowJob& J, int kind,
                                                   void* __restrict__ out, long long pitch,
                                                   int out_half, int o) {
  const int lane = threadIdx.x & 31;
  const int n_out = J.wo * J.ho;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k = lane; k < J.ksplit; k += 32) {
    const double* p = J.partial + ((size_t)k * n_out + o) * 4;
    for (int c = 0; c < 4; ++c) t[c] += p[c];
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int c = 0; c < 4; ++c) t[c] += __shfl_down_sync(0xffffffffu, t[c], off);
  if (lane != 0) return;
  const double norm = kind == 1 ? (1.0 / 3.14159265358979323846) : (1.0 / t[3]);
  const float r = (float)(t[0] * norm), g = (float)(t[1] * norm), b = (float)(t[2] * norm);
  const int x = o % J.wo, i = o / J.wo;
  if (out_half) {
    const __half2 rg = __floats2half2_rn(r, g), ba = __floats2half2_rn(b, 1.0f);
    uint2 v;
    v.x = *reinterpret_cast<const uint32_t*>(&rg);
    v.y = *reinterpret_cast<const uint32_t*>(&ba);
    reinterpret_cast<uint2*>(out)[(long long)i * pitch + x] = v;
  } else {
    reinterpret_cast<float4*>(out)[(long long)i * pitch + x] = make_float4(r, g, b, 1.0f);
  }
}

__global__ void narrow_finish_kernel(const NarrowJob J, int kind, void* __restrict__ out,
                                     long long pitch, int out_half) {
  narrow_finish_warp(J, kind, out, pitch, out_half, blockIdx.x);
}

// A narrow output of a batch: its job, kind and destination.
struct NarrowOut {
  NarrowJob J;
  int kind;
  void* out;
  long long pitch;
  int out_half;
};

// Every narrow output of a batch: block b (one warp) is texel b - begins[k]
// of output k.
__global__ void narrow_finish_batch_kernel(const NarrowOut* __restrict__ outs,
                                           const long long* __restrict__ begins, int n) {
  const int k = find_range(begins, n, blockIdx.x);
  const NarrowOut& o = outs[k];
  narrow_finish_warp(o.J, o.kind, o.out, o.pitch, o.out_half,
                     (int)((long long)blockIdx.x - begins[k]));
}

// Direction tables in FP64, stored as FP32: cos of the column offsets
// (2 pi (d + 0.5) / ws), source rows (cos q, sin q, solid angle) and output
// rows (cos p, sin p at texel corners).  One launch for every job of a bake:
// blockIdx.y selects the job.
constexpr int kMaxTcJobs = ALTHEA_IBL_MAX_MIPS + 1;
struct TableArgs {
  int ws[kMaxTcJobs], hs[kMaxTcJobs], ho[kMaxTcJobs];
  float* cosd[kMaxTcJobs];
  float* srows[kMaxTcJobs];
  float* orows[kMaxTcJobs];
  // visible-offset windows (tensor jobs only; vis null otherwise): row tiles of
  // kM rows, or one tile holding rows 0..ho-1 and a paired second output's
  // rows 0..ho_b-1
  int* vis[kMaxTcJobs];
  int ntiles[kMaxTcJobs], ho_b[kMaxTcJobs], g[kMaxTcJobs], krow[kMaxTcJobs];
};
constexpr int kMaxTiles = 512;  // row tiles of an output (65536 rows / kM)

// Half-width of the visible offset window for output rows [ia, ib] (texel
// corners of an ho-row output) against source row q.  c = cos p cos q cos D +
// sin p sin q > 0 needs cos D > X = -tan p tan q.  The kernels evaluate c in
// FP32 from FP32 tables, within about 4 2^-24 (cos p cos q + |sin p sin q|)
// of its value, so a weight can come out positive wherever cos D >
// X' = X - 1e-6 (1 + |X|).  X' grows with X and X is monotonic in p, so the
// tile's end rows bound it.  The window |t + 0.5| <= T = acos(X') ws / 2 pi
// (+ 2 texels) in phase-row units u (t = g u + ph).  -1: X' > 1 for every
// row (every weight of the tile for this source row is exactly 0); >= krow:
// every offset.
__host__ __device__ inline int visible_halfwidth_sc(double sq, double cq, double spa,
                                                    double cpa, double spb, double cpb, int ws,
                                                    int g, int krow) {
  const double pi = 3.14159265358979323846;
  // X = -tan p tan q at the two end rows (cos p = 6e-17 at a pole corner: finite)
  double xmin = fmin(-(spa * sq) / (cpa * cq), -(spb * sq) / (cpb * cq));
  xmin -= 1e-6 * (1.0 + fabs(xmin));
  if (xmin > 1.0) return -1;
  const double a = acos(fmax(-1.0, xmin));
  const double T = a * ws / (2.0 * pi) + 2.0;  // texels, two-texel margin
  const double uh = ceil((T + 0.5 + g) / g) + 1.0;
  return uh * 2.0 + 8.0 >= (double)krow ? krow : (int)uh;
}

// The same from the rows' indices (the host-side planning statistics).
__host__ __device__ inline int visible_halfwidth(double q, int ia, int ib, int ho, int ws, int g,
                                                 int krow) {
  const double pi = 3.14159265358979323846;
  const double pa = pi * ((double)ia / ho - 0.5), pb = pi * ((double)ib / ho - 0.5);
  return visible_halfwidth_sc(sin(q), cos(q), sin(pa), cos(pa), sin(pb), cos(pb), ws, g, krow);
}

__global__ void tables_kernel(const TableArgs a) {
  const double pi = 3.14159265358979323846;
  const int jb = blockIdx.y;
  const int ws = a.ws[jb], hs = a.hs[jb], ho = a.ho[jb];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ws) a.cosd[jb][t] = (float)cos(2.0 * pi * (t + 0.5) / ws);
  if (t < hs) {
    double q = pi * ((t + 0.5) / hs - 0.5);
    double q0 = pi * ((double)t / hs - 0.5), q1 = pi * ((double)(t + 1) / hs - 0.5);
    a.srows[jb][3 * t] = (float)cos(q);
    a.srows[jb][3 * t + 1] = (float)sin(q);
    a.srows[jb][3 * t + 2] = (float)((2.0 * pi / ws) * (sin(q1) - sin(q0)));
  }
  if (t < ho) {
    double p = pi * ((double)t / ho - 0.5);
    a.orows[jb][2 * t] = (float)cos(p);
    a.orows[jb][2 * t + 1] = (float)sin(p);
  }
  if (!a.vis[jb]) return;
  // sin and cos of the tiles' end rows, once per block: [tile][end][sin, cos];
  // the entry after the last tile is a pair's second output
  __shared__ double endrows[kMaxTiles + 1][2][2];
  const int ntiles = a.ntiles[jb];
  for (int e = threadIdx.x; e < 2 * (ntiles + 1); e += blockDim.x) {
    const int tile = e >> 1, end = e & 1;
    double p;
    if (tile < ntiles) {
      const int ia = tile * kM, ib = min(ho, ia + kM) - 1;
      p = pi * ((double)(end ? ib : ia) / ho - 0.5);
    } else {
      const int hb = a.ho_b[jb] > 0 ? a.ho_b[jb] : 1;
      p = pi * ((double)(end ? hb - 1 : 0) / hb - 0.5);
    }
    endrows[tile][end][0] = sin(p);
    endrows[tile][end][1] = cos(p);
  }
  __syncthreads();
  if (t < hs) {
    const double q = pi * ((t + 0.5) / hs - 0.5), sq = sin(q), cq = cos(q);
    for (int tile = 0; tile < ntiles; ++tile) {
      int uh = visible_halfwidth_sc(sq, cq, endrows[tile][0][0], endrows[tile][0][1],
                                    endrows[tile][1][0], endrows[tile][1][1], ws, a.g[jb],
                                    a.krow[jb]);
      if (a.ho_b[jb] > 0)  // a pair: the union with the second output's rows
        uh = max(uh, visible_halfwidth_sc(sq, cq, endrows[ntiles][0][0], endrows[ntiles][0][1],
                                          endrows[ntiles][1][0], endrows[ntiles][1][1], ws,
                                          a.g[jb], a.krow[jb]));
      a.vis[jb][(size_t)tile * hs + t] = uh;
    }
  }
}

// One RGBA32F source row -> 6 bf16 planes (R hi, R lo, G hi, G lo, B hi, B lo) in
// phase order: out[plane][j][ph][u] = split(src[j][g u + ph]), for every phase
// count g the plan uses on this level (the row is read and split once).  Block
// per source row; the row is split into shared memory, then written out
// contiguously once per g.  Dynamic shared memory: 6 * ws bf16.
constexpr int kMaxRowsOut = 8;
struct RowsArgs {
  const float4* src;
  int ws, hs, n;
  int g[kMaxRowsOut];
  __nv_bfloat16* out[kMaxRowsOut];
};

// The staged row in shared memory: element x of a plane at x + 2 (x / 64).
// The phase-row pass below has lane c read elements 4 g c + ph, 4 g apart:
// unswizzled that is a 2g-word stride (a 16-way bank conflict at g = 8, 32-way
// from g = 16); the extra word every 64 elements spreads the lanes over
// distinct banks for g <= 16 (two-way at g = 32).
__host__ __device__ constexpr int rows_swz(int x) { return x + 2 * (x >> 6); }
__host__ __device__ constexpr int rows_plane(int ws) { return rows_swz(ws) + 2; }
constexpr int rows_smem_bytes(int ws) { return 6 * rows_plane(ws) * 2; }

__device__ __forceinline__ void rows_block(const RowsArgs& a, int j) {
  extern __shared__ __nv_bfloat16 row_sm[];
  const float4* __restrict__ src = a.src;
  const int ws = a.ws, hs = a.hs, pl = rows_plane(ws);
  for (int x = threadIdx.x; x < ws; x += blockDim.x) {
    const float4 v = src[(size_t)j * ws + x];
    const float c[3] = {v.x, v.y, v.z};
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const __nv_bfloat16 h = __float2bfloat16_rn(c[ch]);
      row_sm[(2 * ch) * pl + rows_swz(x)] = h;
      row_sm[(2 * ch + 1) * pl + rows_swz(x)] = __float2bfloat16_rn(c[ch] - __bfloat162float(h));
    }
  }
  __syncthreads();
  // Phase rows are krow (a multiple of 8) long: each thread writes four
  // consecutive elements of one phase row at a time (8-byte stores).
  for (int q = 0; q < a.n; ++q) {
    const int g = a.g[q], krow = ws / g, quads = krow >> 2;
    __nv_bfloat16* __restrict__ out = a.out[q];
    for (int p = 0; p < 6; ++p) {
      const __nv_bfloat16* rp = row_sm + p * pl;
      __nv_bfloat16* op = out + ((size_t)p * hs + j) * ws;
      for (int ph = 0; ph < g; ++ph) {
        for (int c = threadIdx.x; c < quads; c += blockDim.x) {
          const int u = 4 * c;
          __nv_bfloat162 v01, v23;
          v01.x = rp[rows_swz(g * u + ph)];
          v01.y = rp[rows_swz(g * (u + 1) + ph)];
          v23.x = rp[rows_swz(g * (u + 2) + ph)];
          v23.y = rp[rows_swz(g * (u + 3) + ph)];
          uint2 w;
          w.x = *reinterpret_cast<const uint32_t*>(&v01);
          w.y = *reinterpret_cast<const uint32_t*>(&v23);
          *reinterpret_cast<uint2*>(op + ph * krow + u) = w;
        }
      }
    }
  }
}

__global__ void rows_kernel(const RowsArgs a) { rows_block(a, blockIdx.x); }

// The split passes of many levels (of many probes) in one launch: block b is
// source row b - begins[k] of level job k.  Dynamic shared memory: the widest
// level's.
__global__ void rows_batch_kernel(const RowsArgs* __restrict__ jobs,
                                  const long long* __restrict__ begins, int njobs) {
  const int k = find_range(begins, njobs, blockIdx.x);
  rows_block(jobs[k], (int)((long long)blockIdx.x - begins[k]));
}

// Sum the K splits (FP32, fixed order), normalise by the FP64 weight sum,
// write RGBA32F or RGBA16F.  A block of 8 warps covers 32 slots of four
// consecutive output rows (slot = (column, row quad), quads fastest: the
// partial sums are [split][channel][x][row], rows fastest, so a warp reads
// contiguous float4s); warp w adds the splits k = w, w + 8, ... (two in
// flight), and warp 0 combines the eight in order.  Rows of outputs whose
// height is not a multiple of 4 are read one by one.  FP64 is used only for
// the weight sums and the final normalisation.
constexpr int kFinishRows = 4;   // output rows per slot
constexpr int kFinishWarps = 8;
constexpr int kFinishThreads = 32 * kFinishWarps;

__device__ __forceinline__ void store_texel(void* out, long long pitch, int i, int x, int half,
                                            float r, float g, float b) {
  if (half) {
    const __half2 rg = __floats2half2_rn(r, g), ba = __floats2half2_rn(b, 1.0f);
    uint2 v;
    v.x = *reinterpret_cast<const uint32_t*>(&rg);
    v.y = *reinterpret_cast<const uint32_t*>(&ba);
    reinterpret_cast<uint2*>(out)[(long long)i * pitch + x] = v;
  } else {
    reinterpret_cast<float4*>(out)[(long long)i * pitch + x] = make_float4(r, g, b, 1.0f);
  }
}

// What the finish of one contracted output reads.
struct FinishJob {
  const float* partial;      // [nparts][3][wo][ho]
  const double* wsum_part;   // [nparts][ho] (kind 0, or a kind 1 output with a derived mip)
  int wo, ho, nparts, kind, out_half;
  // An irradiance's derived roughness-1 mip: texel (x / df, i / df) for
  // every x and i divisible by df is the normalised cosine sum there.
  void* dout;
  long long dpitch;
  int df;
};

__device__ __forceinline__ void finish_block(const FinishJob& job, void* __restrict__ out,
                                             long long pitch, long long slot0) {
  __shared__ float red[kFinishWarps][3][kFinishRows][32];
  __shared__ double redw[kFinishWarps][kFinishRows][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int quads = (job.ho + kFinishRows - 1) / kFinishRows;
  const long long slot = slot0 + lane;
  const bool live = slot < (long long)quads * job.wo;
  const int x = live ? (int)(slot / quads) : 0, quad = live ? (int)(slot % quads) : 0;
  const int i0 = quad * kFinishRows;
  const size_t plane = (size_t)job.wo * job.ho;
  const bool vec = (job.ho % kFinishRows) == 0;
  float s[3][kFinishRows];
  double sw[kFinishRows];
#pragma unroll
  for (int r = 0; r < kFinishRows; ++r) {
    s[0][r] = s[1][r] = s[2][r] = 0.0f;
    sw[r] = 0.0;
  }
  const float* base = job.partial + (size_t)x * job.ho + i0;
  const bool sums = job.kind == 0 || job.df > 0;  // weight sums to read
  if (live && vec) {
    constexpr int kU = 1;
    for (int k0 = w; k0 < job.nparts; k0 += kU * kFinishWarps) {
      float4 v[kU][3];
      double2 wv[kU][2];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int k = k0 + u * kFinishWarps;
        if (k < job.nparts) {
          const float* p = base + (size_t)k * 3 * plane;
#pragma unroll
          for (int c = 0; c < 3; ++c) v[u][c] = *reinterpret_cast<const float4*>(p + c * plane);
          if (sums) {
            const double* wp = job.wsum_part + (size_t)k * job.ho + i0;
            wv[u][0] = *reinterpret_cast<const double2*>(wp);
            wv[u][1] = *reinterpret_cast<const double2*>(wp + 2);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (k0 + u * kFinishWarps < job.nparts) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            s[c][0] += v[u][c].x;
            s[c][1] += v[u][c].y;
            s[c][2] += v[u][c].z;
            s[c][3] += v[u][c].w;
          }
          if (sums) {
            sw[0] += wv[u][0].x;
            sw[1] += wv[u][0].y;
            sw[2] += wv[u][1].x;
            sw[3] += wv[u][1].y;
          }
        }
      }
    }
  } else if (live) {
    for (int k = w; k < job.nparts; k += kFinishWarps) {
      const float* p = base + (size_t)k * 3 * plane;
#pragma unroll
      for (int r = 0; r < kFinishRows; ++r) {
        if (i0 + r < job.ho) {
#pragma unroll
          for (int c = 0; c < 3; ++c) s[c][r] += p[c * plane + r];
          if (sums) sw[r] += job.wsum_part[(size_t)k * job.ho + i0 + r];
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kFinishRows; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) red[w][c][r][lane] = s[c][r];
    redw[w][r][lane] = sw[r];
  }
  __syncthreads();
  if (w != 0 || !live) return;
#pragma unroll
  for (int r = 0; r < kFinishRows; ++r) {
    if (i0 + r >= job.ho) break;
    float t0 = 0.0f, t1 = 0.0f, t2 = 0.0f;
    double tw = 0.0;
    for (int ww = 0; ww < kFinishWarps; ++ww) {
      t0 += red[ww][0][r][lane];
      t1 += red[ww][1][r][lane];
      t2 += red[ww][2][r][lane];
      tw += redw[ww][r][lane];
    }
    const double norm = job.kind == 1 ? (1.0 / 3.14159265358979323846) : (1.0 / tw);
    store_texel(out, pitch, i0 + r, x, job.out_half, (float)(t0 * norm), (float)(t1 * norm),
                (float)(t2 * norm));
    if (job.df > 0 && x % job.df == 0 && (i0 + r) % job.df == 0) {
      const double dn = 1.0 / tw;
      store_texel(job.dout, job.dpitch, (i0 + r) / job.df, x / job.df, job.out_half,
                  (float)(t0 * dn), (float)(t1 * dn), (float)(t2 * dn));
    }
  }
}

// Every tensor job's finish in one launch: block b belongs to the job k with
// begin[k] <= b < begin[k + 1] and covers 32 slots (four rows, one column) of it.
constexpr int kMaxFinishJobs = ALTHEA_IBL_MAX_MIPS + 1;
struct FinishArgs {
  FinishJob job[kMaxFinishJobs];
  void* out[kMaxFinishJobs];
  long long pitch[kMaxFinishJobs];
  int begin[kMaxFinishJobs + 1];
  int n;
};

__global__ void __launch_bounds__(kFinishThreads, 4) finish_all_kernel(
    const __grid_constant__ FinishArgs a) {
  const int b = blockIdx.x;
  int k = 0;
  while (k + 1 < a.n && b >= a.begin[k + 1]) ++k;
  finish_block(a.job[k], a.out[k], a.pitch[k], (long long)(b - a.begin[k]) * 32);
}

// A contracted output of a batch: its job and destination.
struct FinishOut {
  FinishJob job;
  void* out;
  long long pitch;
};

// Every contracted output of a batch: block b is block b - begins[k] (32
// slots) of output k.
__global__ void __launch_bounds__(kFinishThreads, 4)
    finish_batch_kernel(const FinishOut* __restrict__ outs, const long long* __restrict__ begins,
                        int n) {
  __shared__ FinishOut o;
  __shared__ long long slot0;
  if (threadIdx.x == 0) {
    const int k = find_range(begins, n, blockIdx.x);
    o = outs[k];
    slot0 = ((long long)blockIdx.x - begins[k]) * 32;
  }
  __syncthreads();
  finish_block(o.job, o.out, o.pitch, slot0);
}

}  // namespace tc
}  // namespace ibl

// =====================================================================================
// Host side: planning, workspace layout, launches.
// =====================================================================================
using namespace ibl;
using namespace ibl::tc;

namespace {

// Source level per output mip / irradiance: the coarsest level whose max
// relative error against the level-0 FP64 quadrature stays within 1e-3 on a
// 4096x2048 map with 1e6 suns -- checked on every texel within 5 degrees of a
// sun, the u = 0 seam, the pole rows and 1024 random texels per output --
// expressed as the angular size of a source texel relative to the env:
// level = log2(W / target).  The error grows with the roughness for a given
// source width (a 1024-wide source: 1.8e-4 at r = 0.14, 6.5e-4 at 0.29, 7.6e-4
// at 0.375, 9.6e-4 at 0.5 and 1.1e-3 at 0.43 on a 2048-wide map), hence the
// finer source above r = 0.40; roughness 0.875 from a 512-wide source
// reached 3.6e-3.
int planned_level(int w, int ow, float roughness, bool irradiance) {
  // target source width by role (for a 4096-wide env: irradiance and rough
  // mips at level 1, glossy mips at level 2).
  int target;
  if (irradiance)
    target = 2048;
  else if (roughness <= 0.40f)
    target = 1024;
  else
    target = 2048;
  // Scale with the env: the error depends on the angular size of a texel.
  int level = 0;
  while ((w >> (level + 1)) >= target && level + 1 < 15) ++level;
  // never coarser than the output itself
  while (level > 0 && (w >> level) < ow) --level;
  return level;
}

struct LevelPlanes {
  int level, g, ws, hs;
  size_t offset;  // byte offset of the 6 planes (phase order for g) in the workspace
};

struct JobPlan {
  Job J;
  int level = -1;  // index into TcPlan::levels; -1 = roughness 0 (plain path)
  bool narrow = false;  // summed on the CUDA cores (narrow_kernel)
  int src_level = 0;    // chain level of a narrow job's source
  int pair_with = -1;   // a second job run in this job's lanes 64-127
  bool paired = false;  // this job runs inside another's launch (finish only)
  size_t cosd_off = 0, rows_off = 0, orows_off = 0, partial_off = 0,
         wsum_off = 0, vis_off = 0;
  void* out = nullptr;   // the output image and its pitch (texels), set at setup
  long long pitch = 0;
  int finish_slot = -1;  // this job's entry in the finish arguments
  // A roughness-1 GGX mip is the irradiance's normalised cosine sum (D = 1/pi):
  // written by the irradiance's finish at every derived_factor-th texel, no
  // work of its own.
  bool derived = false;
  int derived_factor = 0;
};

struct TcPlan {
  std::vector<JobPlan> jobs;
  std::vector<LevelPlanes> levels;
  size_t total = 0;
};

// One planned precision bake with every pointer set (tc_setup), launched in
// phases: prep (split planes, tables, CUDA-core outputs), contractions,
// finish (split sums, roughness-0 mips).
struct TcBake {
  TcPlan P;
  const float* chain = nullptr;
  int w = 0, h = 0, n = 0;
  althea_ibl_mip_target mips[ALTHEA_IBL_MAX_MIPS];
  int out_half = 0;
  char* base = nullptr;
  ChainTable tab;
  FinishArgs fa;
  int finish_blocks = 0;
  std::vector<int> launch_jobs;  // P.jobs run by a contraction launch (not paired, not narrow)
};

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

int level_index(TcPlan& P, int w, int h, int level, int g, size_t& off) {
  for (size_t k = 0; k < P.levels.size(); ++k)
    if (P.levels[k].level == level && P.levels[k].g == g) return (int)k;
  LevelPlanes L;
  L.level = level;
  L.g = g;
  L.ws = level_dim(w, level);
  L.hs = level_dim(h, level);
  L.offset = off;
  off = al256(off + (size_t)6 * L.ws * L.hs * 2);
  P.levels.push_back(L);
  return (int)P.levels.size() - 1;
}

// Glossy mips at most this rough, on a source level the planner chose, take
// the two-product split (BF16 hi weights, the weight sum over the rounded
// weights).  The rounding of the weights is then an error of its own, up to
// 2^-9 per weight, correlated over a sun's texels: measured against the FP64
// quadrature over level 0 on the 4096x2048 map with 1e6 suns (seeds 0-2,
// every texel within 5 degrees of a sun, seams, poles and 512 random texels),
// mip 1 (roughness 1/8 from a 1024-wide level) reaches 5.4e-4 with it against
// 1.8e-4 without, and mip 2 (roughness 1/4, same level) 5.7e-4 against
// 2.6e-4 over seeds 0-4 (the batch probes' mip 1 of roughness 1/4, and the
// 512x256 probe's at every texel, are in the GPU tests).  The rougher mips
// already carry up to 7.6e-4 from their source level and keep three products.
constexpr float kTwoProdMaxRoughness = 0.25f;

// Adds a contraction job (mip or irradiance) to the plan.
int add_job(TcPlan& P, int w, int h, int ow, int oh, float roughness, int kind, int level,
            bool planned, size_t& off) {
  JobPlan jp;
  Job& J = jp.J;
  memset(&J, 0, sizeof(J));
  J.ws = level_dim(w, level);
  J.hs = level_dim(h, level);
  J.wo = ow;
  J.ho = oh;
  J.s = J.ws / ow;
  if (8 % J.s == 0) {
    J.g = 1;
    J.m = 8 / J.s;
  } else if (J.s % 8 == 0) {
    J.g = J.s / 8;
    J.m = 1;
  } else {
    J.g = J.s;
    J.m = 8;
  }
  J.kind = kind;
  J.a2 = roughness * roughness;
  J.two_prod = planned && kind == 0 && roughness <= kTwoProdMaxRoughness ? 1 : 0;
  if (ow * oh <= kNarrowMax && ow <= kNarrowMaxW && 32 % ow == 0) {
    // CUDA-core job: one block per (output row, band of source rows), about
    // four blocks per SM
    int ks = (4 * 152 + oh - 1) / oh;
    if (ks > J.hs) ks = J.hs;
    J.ksplit = ks;
    jp.narrow = true;
    jp.level = -2;
    jp.src_level = level;
    jp.cosd_off = off;
    off = al256(off + (size_t)J.ws * 4);
    jp.rows_off = off;
    off = al256(off + (size_t)J.hs * 12);
    jp.orows_off = off;
    off = al256(off + (size_t)oh * 8);
    jp.partial_off = off;
    off = al256(off + (size_t)ks * ow * oh * 4 * 8);
    P.jobs.push_back(jp);
    return ALTHEA_IBL_OK;
  }
  const int li = level_index(P, w, h, level, J.g, off);
  J.krow = J.ws / J.g;
  {
    const int ks = J.two_prod ? 2 * kKS : kKS;  // K per pipeline stage of the kernel variant
    J.kpad = ((J.krow + ks - 1) / ks) * ks;
  }
  J.nres = (ow + J.m - 1) / J.m;
  J.nb = ((J.nres + 15) / 16) * 16;
  if (J.nb > kNBMax) J.nb = kNBMax;
  J.nblk = (J.nres + J.nb - 1) / J.nb;
  J.rlen = ((8 * J.nb + J.kpad + 7) / 8) * 8;
  J.kind = kind;
  J.a2 = roughness * roughness;
  // Staged rows are rotations of a phase row by multiples of 8 elements, copied
  // by TMA in 16-byte units.
  if (J.krow % 8 != 0)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                     "tensor path: a %dx%d output against a %d-wide level has phase rows of "
                     "%d texels (needs a multiple of 8)",
                     ow, oh, J.ws, J.krow);
  for (J.nslots = kMaxSlots; J.nslots > 2; --J.nslots)
    if (smem_plan(J).total + 4096 <= (size_t)kSmemLimit) break;
  if (smem_plan(J).total + 4096 > (size_t)kSmemLimit || rows_smem_bytes(J.ws) > kSmemLimit)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                     "tensor path: a %dx%d output against a %d-wide level needs too much "
                     "shared memory",
                     ow, oh, J.ws);
  // Split the source rows so that no CTA sums more than kMaxK of K (one
  // source row at least: a phase row longer than kMaxK is one chain).  No
  // more: the contractions of a bake run as one queue of work items (and a
  // batch's as one persistent kernel), so a job need not fill the GPU alone.
  // An FP32 tensor-core chain of K = 32768 (2048 MMAs) adds up to about
  // 1.3e-4 of rounding against the FP64 quadrature at the same level
  // (measured: 1.26e-4 on a 128x64 mip at K = 32768, 1.14e-4 on a 24x12 one
  // at K = 14,600), well within the 1e-3 of the precision path.  Planned and
  // caller-named levels split alike, so the two bake the same levels
  // bit-identically.
  int rows_max = kMaxK / (J.g * J.kpad);
  if (rows_max < 1) rows_max = 1;
  int ks = (J.hs + rows_max - 1) / rows_max;
  if (ks > J.hs) ks = J.hs;
  if (ks < 1) ks = 1;
  J.ksplit = ks;
  J.kinter = 1;
  J.nparts = ks;
  // one partial sum per split
  const int parts = ks;
  jp.level = li;
  jp.cosd_off = off;
  off = al256(off + (size_t)J.ws * 4);
  jp.rows_off = off;
  off = al256(off + (size_t)J.hs * 12);
  jp.orows_off = off;
  off = al256(off + (size_t)oh * 8);
  jp.partial_off = off;
  off = al256(off + (size_t)parts * 3 * ow * oh * 4);
  jp.wsum_off = off;
  off = al256(off + (size_t)parts * oh * 8);
  jp.vis_off = off;  // one window per (row tile, source row)
  off = al256(off + (size_t)((oh + kM - 1) / kM) * J.hs * 4);
  P.jobs.push_back(jp);
  return ALTHEA_IBL_OK;
}

// Widest contracted output (mips with roughness > 0 and the irradiance): the
// widths the kernels have been run and checked at.
constexpr int kMaxTcWidth = 1024;

int make_plan(int w, int h, const althea_ibl_mip_target* mips, int n, const int* levels,
              int irr_w, int irr_h, int irr_level, TcPlan& P) {
  size_t off = 256;  // the error flag (byte 0) and the queue counter (byte 128) first
  // A source level named by the caller must exist in the chain (the planner's
  // own choices always do).
  const int nlevels = chain_levels(w, h);
  // The irradiance's level, and whether it is contracted on the tensor cores:
  // a roughness-1 mip on the same level whose texel corners are a subset of
  // the irradiance's is derived from it.  With a2 = 1 the GGX weight is
  // D cos Omega = cos Omega / pi, the irradiance's weight over pi, so the mip
  // is the irradiance's sum over its weight sum: the same quadrature.
  const int irr_lv = irr_w > 0 ? (irr_level >= 0 ? irr_level : planned_level(w, irr_w, 1.0f, true))
                               : -1;
  const bool irr_tensor =
      irr_w > 0 && !(irr_w * irr_h <= kNarrowMax && irr_w <= kNarrowMaxW && 32 % irr_w == 0);
  bool any_derived = false;
  for (int m = 0; m < n; ++m) {
    if (mips[m].roughness == 0.0f) {  // a delta: handled by the plain path
      P.jobs.push_back(JobPlan{});
      continue;
    }
    const bool planned = !(levels && levels[m] >= 0);
    int lv = planned ? planned_level(w, mips[m].width, mips[m].roughness, false) : levels[m];
    if (mips[m].roughness == 1.0f && irr_tensor && lv == irr_lv && irr_w % mips[m].width == 0 &&
        irr_h % mips[m].height == 0 && irr_w / mips[m].width == irr_h / mips[m].height) {
      JobPlan d;
      d.level = -3;
      d.derived = true;
      d.derived_factor = irr_w / mips[m].width;
      P.jobs.push_back(d);
      any_derived = true;
      continue;
    }
    if (lv >= nlevels)
      return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                       "tensor path: mip %d source level %d; the chain has levels 0..%d", m, lv,
                       nlevels - 1);
    int ws = level_dim(w, lv);
    if (ws < mips[m].width || ws % mips[m].width != 0 || mips[m].width > kMaxTcWidth ||
        mips[m].height > 65536)
      return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                       "tensor path: mip %d (%dx%d) cannot contract against level %d", m,
                       mips[m].width, mips[m].height, lv);
    int st = add_job(P, w, h, mips[m].width, mips[m].height, mips[m].roughness, 0, lv, planned,
                     off);
    if (st) return st;
  }
  if (irr_w > 0) {
    int lv = irr_level >= 0 ? irr_level : planned_level(w, irr_w, 1.0f, true);
    if (lv >= nlevels)
      return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                       "tensor path: irradiance source level %d; the chain has levels 0..%d", lv,
                       nlevels - 1);
    int ws = level_dim(w, lv);
    if (ws < irr_w || ws % irr_w != 0 || irr_w > kMaxTcWidth)
      return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "tensor path: irradiance %dx%d vs level %d",
                       irr_w, irr_h, lv);
    int st = add_job(P, w, h, irr_w, irr_h, 1.0f, 1, lv, irr_level < 0, off);
    if (st) return st;
    if (any_derived) P.jobs.back().J.wsum1 = 1;
  }
  // Pair tensor jobs of at most 64 rows that share every radiance operand
  // (same source level and phase decomposition, same columns): one launch
  // runs both, the second in TMEM lanes 64-127.
  for (size_t a = 0; a < P.jobs.size(); ++a) {
    JobPlan& A = P.jobs[a];
    if (A.level < 0 || A.narrow || A.paired || A.pair_with >= 0 || A.J.ho > 64) continue;
    for (size_t b = a + 1; b < P.jobs.size(); ++b) {
      JobPlan& B = P.jobs[b];
      if (B.level != A.level || B.narrow || B.paired || B.pair_with >= 0 || B.J.ho > 64)
        continue;
      const Job &x = A.J, &y = B.J;
      if (x.ws != y.ws || x.hs != y.hs || x.wo != y.wo || x.g != y.g || x.m != y.m ||
          x.krow != y.krow || x.kpad != y.kpad || x.nres != y.nres || x.nb != y.nb ||
          x.nblk != y.nblk || x.rlen != y.rlen || x.nslots != y.nslots ||
          x.ksplit != y.ksplit || x.two_prod != y.two_prod)
        continue;
      A.pair_with = (int)b;
      B.paired = true;
      break;
    }
  }
  // Unpaired tensor outputs of 33 to 64 rows: column tiles.  An M = 128 tile
  // of their rows would be half or more padding; their columns fill it
  // instead (the operands swap roles: N = 64 rows).  With both operands in
  // shared memory the MMAs read 4 KB of radiance per K = 16 whatever N is,
  // which only pays at N = 64 (about 6 KB per 37-cycle MMA, near the
  // shared-memory rate): smaller outputs keep row tiles (pairs, K
  // interleave).  Same grid and splits (one row tile; column blocks of 128
  // either way), so the workspace layout is unchanged.
  for (auto& jp : P.jobs) {
    if (jp.level < 0 || jp.narrow || jp.paired || jp.pair_with >= 0 || jp.J.ho <= 32 ||
        jp.J.ho > 64)
      continue;
    Job& J = jp.J;
    J.ct = 1;
    J.nb = kM;
    J.nblk = (J.nres + kM - 1) / kM;
    J.rlen = 8 * kM + J.kpad;
    for (J.nslots = kMaxSlots; J.nslots > 2; --J.nslots)
      if (smem_plan(J).total + 4096 <= (size_t)kSmemLimit) break;
    if (smem_plan(J).total + 4096 > (size_t)kSmemLimit)
      return set_error(ALTHEA_IBL_ERR_UNSUPPORTED,
                       "tensor path: a %dx%d output against a %d-wide level needs too much "
                       "shared memory",
                       J.wo, J.ho, J.ws);
  }
  // Unpaired tensor outputs of at most 32 rows: K interleave over the four
  // lane quarters.
  // (The K interleave runs the 32 K hi/lo stages: such an output keeps three
  // products; its kpad, a multiple of 64 if it had two, is still a multiple
  // of 32.)
  for (auto& jp : P.jobs)
    if (jp.level >= 0 && !jp.narrow && !jp.paired && jp.pair_with < 0 && jp.J.ho <= 32) {
      jp.J.kinter = 4;
      jp.J.nparts = jp.J.ksplit;
      jp.J.two_prod = 0;
    }
  P.total = off;
  return ALTHEA_IBL_OK;
}

}  // namespace

extern "C" int althea_ibl_tc_stats(int w, int h, const althea_ibl_mip_target* mips, int n,
                                   const int* levels, int irr_w, int irr_h, int irr_level,
                                   althea_ibl_tc_work* out) {
  if (!out) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "tc stats: null output");
  memset(out, 0, sizeof(*out));
  if (check_env(w, h)) return ALTHEA_IBL_ERR_INVALID_ARGUMENT;
  if (n < 0 || n > ALTHEA_IBL_MAX_MIPS || (n > 0 && !mips))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "tc stats: %d mips (0..%d, non-null)", n,
                     ALTHEA_IBL_MAX_MIPS);
  TcPlan P;
  int st = make_plan(w, h, mips, n, levels, irr_w, irr_h, irr_level, P);
  if (st) return st;
  const double pi = 3.14159265358979323846;
  for (const JobPlan& jp : P.jobs) {
    const Job& J = jp.J;
    if (jp.level < 0 && !jp.narrow) continue;  // roughness 0: the delta pass
    const double dense = (double)J.ho * J.wo * J.hs * J.ws;
    if (jp.narrow) {
      out->cuda_core_pairs += dense;
      continue;
    }
    out->dense_pairs += dense;
    if (jp.paired) continue;  // contracted inside its partner's launch
    out->tensor_launches = 1;  // one queue launch for every contraction
    const bool pair = jp.pair_with >= 0;
    const int ho_b = pair ? P.jobs[jp.pair_with].J.ho : 0;
    const int KS = J.two_prod ? 2 * kKS : kKS;
    const int kchunks = J.kpad / KS, products = J.two_prod ? 2 : 3;
    const int ntiles = (J.ho + kM - 1) / kM, gy = J.m * J.nblk;
    // flops of one stage's MMAs: 3 channels x products x K/16 MMAs of M = 128,
    // K = 16 and N = nb (row tiles) or kCtN (column tiles)
    const double stage_flops = 3.0 * products * (KS / 16) * 2.0 * kM * (J.ct ? kCtN : J.nb) * 16;
    for (int tile = 0; tile < ntiles; ++tile) {
      const int ia = tile * kM, ib = std::min(J.ho, ia + kM) - 1;
      const int rows = ib - ia + 1 + ho_b;
      for (int j = 0; j < J.hs; ++j) {
        const double q = pi * ((j + 0.5) / J.hs - 0.5);
        int uh = visible_halfwidth(q, ia, ib, J.ho, J.ws, J.g, J.krow);
        if (pair) uh = std::max(uh, visible_halfwidth(q, 0, ho_b - 1, ho_b, J.ws, J.g, J.krow));
        int ca, cb;
        visible_chunks(uh, J.krow, KS, kchunks, ca, cb);
        const int nvis = ca + kchunks - cb;
        out->tensor_flops += (double)gy * J.g * nvis * stage_flops;
        out->visible_pairs += (double)rows * J.wo * J.g * std::min(J.krow, nvis * KS);
      }
    }
  }
  return ALTHEA_IBL_OK;
}

extern "C" size_t althea_ibl_tc_workspace_size(int w, int h, const althea_ibl_mip_target* mips,
                                               int n, const int* levels, int irr_w, int irr_h,
                                               int irr_level) {
  return tc_workspace_bytes(w, h, mips, n, levels, irr_w, irr_h, irr_level);
}

extern "C" int althea_ibl_tc_plan(int w, int h, const althea_ibl_mip_target* mips, int n,
                                  int irr_w, int* levels_out, int* irr_level_out) {
  if (check_env(w, h)) return ALTHEA_IBL_ERR_INVALID_ARGUMENT;
  if (n < 0 || n > ALTHEA_IBL_MAX_MIPS || (n > 0 && (!mips || !levels_out)))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "tensor plan: %d mips (0..%d, non-null)",
                     n, ALTHEA_IBL_MAX_MIPS);
  for (int m = 0; m < n; ++m)
    levels_out[m] = mips[m].roughness == 0.0f
                        ? -1
                        : planned_level(w, mips[m].width, mips[m].roughness, false);
  if (irr_level_out) *irr_level_out = irr_w > 0 ? planned_level(w, irr_w, 1.0f, true) : -1;
  return ALTHEA_IBL_OK;
}

namespace ibl {

int tc_setup(const float* chain, int w, int h, const althea_ibl_mip_target* mips, int n,
             const int* levels, float* irr_out, int irr_w, int irr_h, size_t irr_pitch,
             int irr_level, void* ws, size_t ws_bytes, int out_format, TcBake& B) {
  int st = check_env(w, h);
  if (st) return st;
  if (out_format != ALTHEA_IBL_FORMAT_RGBA32F && out_format != ALTHEA_IBL_FORMAT_RGBA16F)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "tensor path: output format %d",
                     out_format);
  B.out_half = out_format == ALTHEA_IBL_FORMAT_RGBA16F;
  const size_t texel = B.out_half ? 8 : 16;
  if (!chain || ((uintptr_t)chain) % 16 || n < 0 || n > ALTHEA_IBL_MAX_MIPS || (n && !mips))
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "tensor path: chain/mips");
  for (int m = 0; m < n; ++m) {
    st = check_image(mips[m].out_dev, mips[m].width, mips[m].height, mips[m].pitch_bytes, texel,
                     "tc mip");
    if (st) return st;
  }
  if (irr_out) {
    st = check_image(irr_out, irr_w, irr_h, irr_pitch, texel, "tc irradiance");
    if (st) return st;
  }
  TcPlan& P = B.P;
  st = make_plan(w, h, mips, n, levels, irr_out ? irr_w : 0, irr_h, irr_level, P);
  if (st) return st;
  if (!ws || ws_bytes < P.total || ((uintptr_t)ws) % 256)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT,
                     "tensor path workspace needs %zu bytes (256-byte aligned)", P.total);
  B.chain = chain;
  B.w = w;
  B.h = h;
  B.n = n;
  for (int m = 0; m < n; ++m) B.mips[m] = mips[m];
  B.base = static_cast<char*>(ws);
  make_table(w, h, &B.tab);
  char* base = B.base;
  // Every pointer of every job, and the finish arguments.
  memset(&B.fa, 0, sizeof(B.fa));
  B.finish_blocks = 0;
  B.launch_jobs.clear();
  for (size_t k = 0; k < P.jobs.size(); ++k) {
    JobPlan& jp = P.jobs[k];
    if (jp.derived) {  // written by the irradiance's finish
      jp.out = mips[k].out_dev;
      jp.pitch = (long long)(mips[k].pitch_bytes / texel);
      continue;
    }
    if (jp.level < 0 && !jp.narrow) continue;  // roughness 0: the delta pass
    Job& J = jp.J;
    J.cos_d = reinterpret_cast<float*>(base + jp.cosd_off);
    J.src_rows = reinterpret_cast<float*>(base + jp.rows_off);
    J.out_rows = reinterpret_cast<float*>(base + jp.orows_off);
    void* out = nullptr;
    long long pitch = 0;
    if ((int)k < n) {
      out = mips[k].out_dev;
      pitch = (long long)(mips[k].pitch_bytes / texel);
    } else {
      out = irr_out;
      pitch = (long long)(irr_pitch / texel);
    }
    jp.out = out;
    jp.pitch = pitch;
    if (jp.narrow) continue;
    const LevelPlanes& L = P.levels[jp.level];
    J.src = reinterpret_cast<const __nv_bfloat16*>(base + L.offset);
    J.partial = reinterpret_cast<float*>(base + jp.partial_off);
    J.wsum_part = reinterpret_cast<double*>(base + jp.wsum_off);
    J.error = reinterpret_cast<int*>(base);
    J.out_half = B.out_half;
    if (B.fa.n >= kMaxFinishJobs)
      return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "tc: too many jobs");
    B.fa.out[B.fa.n] = out;
    B.fa.pitch[B.fa.n] = pitch;
    B.fa.begin[B.fa.n] = B.finish_blocks;
    B.finish_blocks +=
        (int)(((long long)((J.ho + kFinishRows - 1) / kFinishRows) * J.wo + 31) / 32);
    jp.finish_slot = B.fa.n++;
    if (jp.paired) continue;  // contracted inside its partner's launch
    J.vis = reinterpret_cast<const int*>(base + jp.vis_off);
    J.pair = 0;
    if (jp.pair_with >= 0) {
      const JobPlan& bp = P.jobs[jp.pair_with];
      J.pair = 1;
      J.ho_b = bp.J.ho;
      J.kind_b = bp.J.kind;
      J.wsum1_b = bp.J.wsum1;
      J.a2_b = bp.J.a2;
      J.out_rows_b = reinterpret_cast<const float*>(base + bp.orows_off);
      J.partial_b = reinterpret_cast<float*>(base + bp.partial_off);
      J.wsum_part_b = reinterpret_cast<double*>(base + bp.wsum_off);
    }
    B.launch_jobs.push_back((int)k);
  }
  // the paired jobs' pointers are set above too: every job's finish record
  for (const JobPlan& jp : P.jobs)
    if (jp.finish_slot >= 0) {
      FinishJob& f = B.fa.job[jp.finish_slot];
      f.partial = jp.J.partial;
      f.wsum_part = jp.J.wsum_part;
      f.wo = jp.J.wo;
      f.ho = jp.J.ho;
      f.nparts = jp.J.nparts;
      f.kind = jp.J.kind;
      f.out_half = jp.J.out_half;
      f.dout = nullptr;
      f.dpitch = 0;
      f.df = 0;
    }
  // a derived roughness-1 mip rides on the irradiance's finish (the last job)
  for (const JobPlan& jp : P.jobs)
    if (jp.derived && P.jobs.back().finish_slot >= 0) {
      FinishJob& f = B.fa.job[P.jobs.back().finish_slot];
      f.dout = jp.out;
      f.dpitch = jp.pitch;
      f.df = jp.derived_factor;
    }
  B.fa.begin[B.fa.n] = B.finish_blocks;
  return ALTHEA_IBL_OK;
}

// The split passes of a bake: one per source level, writing every phase
// decomposition of it (up to kMaxRowsOut per pass).
std::vector<RowsArgs> rows_jobs(const TcBake& B) {
  const TcPlan& P = B.P;
  std::vector<RowsArgs> out;
  std::vector<char> done(P.levels.size(), 0);
  for (size_t a0 = 0; a0 < P.levels.size(); ++a0) {
    if (done[a0]) continue;
    const LevelPlanes& L = P.levels[a0];
    RowsArgs ra;
    memset(&ra, 0, sizeof(ra));
    ra.src = reinterpret_cast<const float4*>(B.chain) + B.tab.off[L.level];
    ra.ws = L.ws;
    ra.hs = L.hs;
    for (size_t a1 = a0; a1 < P.levels.size() && ra.n < kMaxRowsOut; ++a1) {
      if (done[a1] || P.levels[a1].level != L.level) continue;
      ra.g[ra.n] = P.levels[a1].g;
      ra.out[ra.n] = reinterpret_cast<__nv_bfloat16*>(B.base + P.levels[a1].offset);
      ++ra.n;
      done[a1] = 1;
    }
    out.push_back(ra);
  }
  return out;
}

// Direction tables and visible-offset windows of every job of a bake, one
// launch (FP64 transcendentals spread over many SMs).  They depend on the
// sizes only.
int tc_launch_tables(const TcBake& B, cudaStream_t s) {
  const TcPlan& P = B.P;
  TableArgs ta;
  memset(&ta, 0, sizeof(ta));
  int nt = 0, nmax = 1;
  for (size_t k = 0; k < P.jobs.size(); ++k) {
    const JobPlan& jp = P.jobs[k];
    if (jp.level < 0 && !jp.narrow) continue;
    const Job& J = jp.J;
    ta.ws[nt] = J.ws;
    ta.hs[nt] = J.hs;
    ta.ho[nt] = J.ho;
    ta.cosd[nt] = const_cast<float*>(J.cos_d);
    ta.srows[nt] = const_cast<float*>(J.src_rows);
    ta.orows[nt] = const_cast<float*>(J.out_rows);
    if (!jp.narrow && !jp.paired) {  // a tensor launch: its visible-offset windows
      ta.vis[nt] = const_cast<int*>(J.vis);
      ta.ntiles[nt] = (J.ho + kM - 1) / kM;
      ta.ho_b[nt] = jp.pair_with >= 0 ? P.jobs[jp.pair_with].J.ho : 0;
      ta.g[nt] = J.g;
      ta.krow[nt] = J.krow;
    }
    nmax = std::max(nmax, std::max(J.ws, std::max(J.hs, J.ho)));
    ++nt;
  }
  if (nt > 0) tables_kernel<<<dim3((nmax + 31) / 32, nt), 32, 0, s>>>(ta);
  return cuda_status(cudaGetLastError(), "tc tables launch");
}

// The CUDA-core job of a narrow output.
NarrowJob narrow_job(const TcBake& B, const JobPlan& jp) {
  const Job& J = jp.J;
  NarrowJob nj;
  nj.src = reinterpret_cast<const float4*>(B.chain) + B.tab.off[jp.src_level];
  nj.ws = J.ws;
  nj.hs = J.hs;
  nj.wo = J.wo;
  nj.ho = J.ho;
  nj.s = J.ws / J.wo;
  nj.ksplit = J.ksplit;
  nj.a2 = J.a2;
  nj.cos_d = J.cos_d;
  nj.src_rows = J.src_rows;
  nj.out_rows = J.out_rows;
  nj.partial = reinterpret_cast<double*>(B.base + jp.partial_off);
  return nj;
}

int tc_launch_narrow(const TcBake& B, cudaStream_t ns);

// Error flag, split planes and tables; with `narrow`, the CUDA-core outputs
// too (on the side stream when there is one, returned in *ns_out).
int tc_launch_prep(TcBake& B, cudaStream_t s, const SideStream* side, cudaStream_t* ns_out,
                   bool narrow = true, bool tables = true) {
  const TcPlan& P = B.P;
  *ns_out = s;
  cudaError_t e = cudaMemsetAsync(B.base, 0, 256, s);
  if (e != cudaSuccess) return cuda_status(e, "tc error flag");
  for (const RowsArgs& ra : rows_jobs(B)) {
    const int sm = rows_smem_bytes(ra.ws);
    if (sm > 48 * 1024) {
      e = cudaFuncSetAttribute(rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      if (e != cudaSuccess) return cuda_status(e, "tc rows smem attribute");
    }
    rows_kernel<<<ra.hs, 256, sm, s>>>(ra);
  }
  if (tables) {
    const int r = tc_launch_tables(B, s);
    if (r) return r;
  }
  // The outputs summed on the CUDA cores and the roughness-0 mips go to the
  // side stream when there is one (they need the tables and the chain,
  // nothing else of the tensor path), where they fill the gaps between the
  // contraction launches.
  bool any_side = false;
  for (int k = 0; k < (int)P.jobs.size(); ++k)
    any_side |= P.jobs[k].narrow || (k < B.n && P.jobs[k].level < 0 && !P.jobs[k].derived);
  if (!narrow) return cuda_status(cudaGetLastError(), "tensor path prep launch");
  cudaStream_t ns = s;
  if (side && any_side) {
    e = cudaEventRecord(side->fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side->stream, side->fork, 0);
    if (e != cudaSuccess) return cuda_status(e, "tc side-stream fork");
    ns = side->stream;
  }
  *ns_out = ns;
  const int r = tc_launch_narrow(B, ns);
  if (r) return r;
  // Roughness-0 mips are a delta (no contraction): the reflected sample itself.
  for (int m = 0; m < B.n; ++m) {
    if (P.jobs[m].level >= 0 || P.jobs[m].narrow || P.jobs[m].derived) continue;
    const int st = launch_delta_mip(B.chain, B.w, B.h, &B.mips[m], B.out_half, ns);
    if (st) return st;
  }
  return ALTHEA_IBL_OK;
}

// The outputs summed on the CUDA cores (after the prep launches' tables).
int tc_launch_narrow(const TcBake& B, cudaStream_t ns) {
  cudaError_t e;
  for (const JobPlan& jp : B.P.jobs) {
    if (!jp.narrow) continue;
    const Job& J = jp.J;
    const NarrowJob nj = narrow_job(B, jp);
    // dynamic part; with the 8 KB static reduction buffer it can pass the
    // 48 KB default, so the limit is always raised to what this job needs
    const int smem = (int)narrow_smem_bytes(J.ws, J.wo);
    const dim3 grid(J.ho, J.ksplit);
    if (J.kind == 0) {
      e = cudaFuncSetAttribute(narrow_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               smem);
      if (e != cudaSuccess) return cuda_status(e, "tc narrow smem attribute");
      narrow_kernel<0><<<grid, kNarrowThreads, smem, ns>>>(nj);
    } else {
      e = cudaFuncSetAttribute(narrow_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               smem);
      if (e != cudaSuccess) return cuda_status(e, "tc narrow smem attribute");
      narrow_kernel<1><<<grid, kNarrowThreads, smem, ns>>>(nj);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "tc narrow launch");
    narrow_finish_kernel<<<J.wo * J.ho, 32, 0, ns>>>(nj, J.kind, jp.out, jp.pitch, B.out_half);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "tc narrow finish launch");
  }
  return cuda_status(cudaGetLastError(), "tensor path prep launch");
}

// Dynamic shared memory of a contraction CTA of job J: its staging slots,
// cos table and (column tiles) weight stages, at least 120 KB so that no two
// CTAs share an SM (each allocates all of TMEM), and room for a K
// interleave's quarter sums.
int contract_smem(const Job& J) {
  int smem = (int)smem_plan(J).total;
  if (smem < 120 * 1024) smem = 120 * 1024;
  if (J.kinter > 1 && smem < 4 * 3 * J.nb * 32 * 4) smem = 4 * 3 * J.nb * 32 * 4;
  return smem;
}

// K one item of job J sums: its source rows times the phase rows' length.
long long item_k(const Job& J) { return (long long)((J.hs + J.ksplit - 1) / J.ksplit) * J.g * J.kpad; }

// Every contraction of the bake: one queue launch (contract_queue_kernel).
// The queue's counter sits in the workspace's first 256 bytes, which the prep
// zeroes with the error flag.
int tc_launch_contract(const TcBake& B, cudaStream_t s) {
  if (B.launch_jobs.empty()) return ALTHEA_IBL_OK;
  std::vector<int> order = B.launch_jobs;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return item_k(B.P.jobs[a].J) > item_k(B.P.jobs[c].J);
  });
  if ((int)order.size() > kMaxQueueJobs)
    return set_error(ALTHEA_IBL_ERR_UNSUPPORTED, "tc: %d contraction jobs", (int)order.size());
  QueueArgs qa;
  memset(&qa, 0, sizeof(qa));
  int items = 0, smem = 0;
  for (int k : order) {
    const Job& J = B.P.jobs[k].J;
    const int gx = J.ct ? 1 : (J.ho + kM - 1) / kM, gy = J.m * J.nblk;
    qa.jobs[qa.n] = J;
    qa.gx[qa.n] = gx;
    qa.gy[qa.n] = gy;
    qa.begin[qa.n] = items;
    items += gx * gy * J.ksplit;
    smem = std::max(smem, contract_smem(J));
    ++qa.n;
  }
  qa.begin[qa.n] = items;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(contract_queue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
  if (e != cudaSuccess) return cuda_status(e, "tc queue setup");
  unsigned int* next = reinterpret_cast<unsigned int*>(B.base + 128);
  contract_queue_kernel<<<std::min(std::max(sms, 1), items), kThreads, smem, s>>>(qa, next);
  return cuda_status(cudaGetLastError(), "tc contraction launch");
}

int tc_launch_finish(TcBake& B, cudaStream_t s, cudaStream_t ns, const SideStream* side) {
  cudaError_t e;
  if (B.fa.n > 0) {
    finish_all_kernel<<<B.finish_blocks, kFinishThreads, 0, s>>>(B.fa);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e, "tc finish launch");
  }
  if (ns != s) {  // join the side stream
    e = cudaEventRecord(side->join, ns);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, side->join, 0);
    if (e != cudaSuccess) return cuda_status(e, "tc side-stream join");
  }
  return cuda_status(cudaGetLastError(), "tensor path launch");
}

int tc_bake(const float* chain, int w, int h, const althea_ibl_mip_target* mips, int n,
            const int* levels, float* irr_out, int irr_w, int irr_h, size_t irr_pitch,
            int irr_level, void* ws, size_t ws_bytes, int out_format, cudaStream_t stream,
            const SideStream* side, bool tables, const cudaEvent_t* timing) {
  ibl::NvtxRange nvtx_range("precision bake");
  TcBake B;
  int st = tc_setup(chain, w, h, mips, n, levels, irr_out, irr_w, irr_h, irr_pitch, irr_level,
                    ws, ws_bytes, out_format, B);
  if (st) return st;
  cudaStream_t ns = stream;
  st = tc_launch_prep(B, stream, side, &ns, true, tables);
  if (!st && timing) st = cuda_status(cudaEventRecord(timing[0], stream), "timing event");
  if (!st) st = tc_launch_contract(B, stream);
  if (!st && timing) st = cuda_status(cudaEventRecord(timing[1], stream), "timing event");
  if (!st) st = tc_launch_finish(B, stream, ns, side);
  return st;
}

size_t tc_workspace_bytes(int w, int h, const althea_ibl_mip_target* mips, int n,
                          const int* levels, int irr_w, int irr_h, int irr_level) {
  if (check_env(w, h)) return 0;
  if (n < 0 || n > ALTHEA_IBL_MAX_MIPS || (n > 0 && !mips)) {
    set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "tensor path: %d mips (0..%d, non-null)", n,
              ALTHEA_IBL_MAX_MIPS);
    return 0;
  }
  TcPlan P;
  if (make_plan(w, h, mips, n, levels, irr_w, irr_h, irr_level, P)) return 0;
  return P.total;
}

// ---- precision batches: one persistent contraction for every probe --------------
// A device job table with its block offsets: job k owns blocks
// [begins[k], begins[k + 1]) of one launch.
template <typename T>
struct DevTable {
  T* jobs = nullptr;
  long long* begins = nullptr;
  int n = 0;
  long long blocks = 0;
  int smem = 0;  // dynamic shared memory of the launch (the largest job's)
};

struct TcBatch {
  std::vector<TcBake*> bakes;   // one per probe
  Job* d_jobs = nullptr;        // every contraction launch of every probe
  WorkItem* d_items = nullptr;  // every CTA of those launches, largest first
  unsigned int* d_next = nullptr;
  int* d_error = nullptr;       // set by any work item whose bounded wait gave up
  int nitems = 0, njobs = 0, smem = 0, ctas = 0;
  // the rest of every probe's bake, one launch per kind of work
  DevTable<RowsArgs> rows;
  DevTable<NarrowJob> narrow[2];  // GGX, cosine
  DevTable<NarrowOut> narrow_out;
  DevTable<FinishOut> finish;
  DevTable<DeltaJob> delta;
  std::vector<void*> allocs;
};

void tc_batch_destroy(TcBatch* b) {
  if (!b) return;
  for (TcBake* B : b->bakes) delete B;
  for (void* p : b->allocs) cudaFree(p);
  delete b;
}

namespace {

// Copies a host job table and its block offsets to the device.
template <typename T>
cudaError_t upload(TcBatch* b, const std::vector<T>& jobs, const std::vector<long long>& blocks,
                   DevTable<T>& t) {
  t.n = (int)jobs.size();
  if (t.n == 0) return cudaSuccess;
  std::vector<long long> begins(jobs.size());
  long long acc = 0;
  for (size_t k = 0; k < jobs.size(); ++k) {
    begins[k] = acc;
    acc += blocks[k];
  }
  t.blocks = acc;
  cudaError_t e = cudaMalloc(&t.jobs, sizeof(T) * jobs.size());
  if (e == cudaSuccess) b->allocs.push_back(t.jobs);
  if (e == cudaSuccess) e = cudaMalloc(&t.begins, sizeof(long long) * begins.size());
  if (e == cudaSuccess) b->allocs.push_back(t.begins);
  if (e == cudaSuccess)
    e = cudaMemcpy(t.jobs, jobs.data(), sizeof(T) * jobs.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(t.begins, begins.data(), sizeof(long long) * begins.size(),
                   cudaMemcpyHostToDevice);
  return e;
}

}  // namespace

int tc_batch_create(const TcBatchProbe* probes, int n, int out_format, cudaStream_t st,
                    TcBatch** out) {
  *out = nullptr;
  TcBatch* b = new (std::nothrow) TcBatch();
  if (!b) return set_error(ALTHEA_IBL_ERR_OUT_OF_MEMORY, "host allocation");
  std::vector<Job> jobs;
  struct Cand {
    WorkItem wi;
    long long k;  // K this CTA sums (its source rows x phase rows), for the order
  };
  std::vector<Cand> items;
  std::vector<RowsArgs> rows;
  std::vector<NarrowJob> narrow[2];
  std::vector<NarrowOut> nouts;
  std::vector<FinishOut> fins;
  std::vector<DeltaJob> deltas;
  std::vector<long long> rows_blk, narrow_blk[2], nout_blk, fin_blk, delta_blk;
  for (int i = 0; i < n; ++i) {
    const TcBatchProbe& p = probes[i];
    TcBake* B = new (std::nothrow) TcBake();
    if (!B) {
      tc_batch_destroy(b);
      return set_error(ALTHEA_IBL_ERR_OUT_OF_MEMORY, "host allocation");
    }
    b->bakes.push_back(B);
    int r = tc_setup(p.chain, p.w, p.h, p.mips.data(), (int)p.mips.size(), nullptr, p.irr,
                     p.irr_w, p.irr_h, p.irr_pitch, -1, p.ws, p.ws_bytes, out_format, *B);
    // the tables depend on the sizes only: computed once, here
    if (!r) r = tc_launch_tables(*B, st);
    if (r) {
      tc_batch_destroy(b);
      return r;
    }
    for (int k : B->launch_jobs) {
      const Job& J = B->P.jobs[k].J;
      const int jid = (int)jobs.size();
      jobs.push_back(J);
      b->smem = std::max(b->smem, contract_smem(J));
      const int gx = J.ct ? 1 : (J.ho + kM - 1) / kM, gy = J.m * J.nblk, gz = J.ksplit;
      for (int bz = 0; bz < gz; ++bz) {
        const long long rws = (J.hs - bz + gz - 1) / gz;  // rows bz, bz + gz, ...
        for (int by = 0; by < gy; ++by)
          for (int bx = 0; bx < gx; ++bx)
            items.push_back(Cand{WorkItem{jid, bx, by, bz}, rws * J.g * J.kpad});
      }
    }
    for (const RowsArgs& ra : rows_jobs(*B)) {
      rows.push_back(ra);
      rows_blk.push_back(ra.hs);
      b->rows.smem = std::max(b->rows.smem, rows_smem_bytes(ra.ws));
    }
    for (const JobPlan& jp : B->P.jobs) {
      if (!jp.narrow) continue;
      const int kind = jp.J.kind;
      const NarrowJob nj = narrow_job(*B, jp);
      narrow[kind].push_back(nj);
      narrow_blk[kind].push_back((long long)nj.ho * nj.ksplit);
      b->narrow[kind].smem = std::max(b->narrow[kind].smem, (int)narrow_smem_bytes(nj.ws, nj.wo));
      nouts.push_back(NarrowOut{nj, kind, jp.out, jp.pitch, B->out_half});
      nout_blk.push_back((long long)nj.wo * nj.ho);
    }
    for (int k = 0; k < B->fa.n; ++k) {
      fins.push_back(FinishOut{B->fa.job[k], B->fa.out[k], B->fa.pitch[k]});
      fin_blk.push_back(B->fa.begin[k + 1] - B->fa.begin[k]);
    }
    for (int m = 0; m < B->n; ++m) {
      if (B->P.jobs[m].level >= 0 || B->P.jobs[m].narrow || B->P.jobs[m].derived)
        continue;  // roughness 0 only
      const althea_ibl_mip_target& t = B->mips[m];
      DeltaJob d;
      d.chain = B->chain;
      d.w = B->w;
      d.h = B->h;
      d.out = t.out_dev;
      d.pitch = (long long)(t.pitch_bytes / (B->out_half ? 8 : 16));
      d.ow = t.width;
      d.oh = t.height;
      d.out_half = B->out_half;
      d.blocks_x = (t.width + 31) / 32;
      deltas.push_back(d);
      delta_blk.push_back((long long)d.blocks_x * ((t.height + 7) / 8));
    }
  }
  std::stable_sort(items.begin(), items.end(),
                   [](const Cand& a, const Cand& c) { return a.k > c.k; });
  std::vector<WorkItem> wi(items.size());
  for (size_t k = 0; k < items.size(); ++k) wi[k] = items[k].wi;
  b->njobs = (int)jobs.size();
  b->nitems = (int)wi.size();
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->ctas = sms > 0 ? sms : 1;
  auto track = [&](void* p) { b->allocs.push_back(p); };
  if (e == cudaSuccess && b->njobs > 0) e = cudaMalloc(&b->d_jobs, sizeof(Job) * jobs.size());
  if (e == cudaSuccess && b->d_jobs) track(b->d_jobs);
  if (e == cudaSuccess && b->nitems > 0)
    e = cudaMalloc(&b->d_items, sizeof(WorkItem) * wi.size());
  if (e == cudaSuccess && b->d_items) track(b->d_items);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_next, sizeof(unsigned int));
  if (e == cudaSuccess) track(b->d_next);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_error, sizeof(int));
  if (e == cudaSuccess) track(b->d_error);
  if (e == cudaSuccess) e = cudaMemset(b->d_error, 0, sizeof(int));
  for (Job& J : jobs) J.error = b->d_error;  // one status word for the whole batch
  if (e == cudaSuccess && b->njobs > 0)
    e = cudaMemcpy(b->d_jobs, jobs.data(), sizeof(Job) * jobs.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && b->nitems > 0)
    e = cudaMemcpy(b->d_items, wi.data(), sizeof(WorkItem) * wi.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = upload(b, rows, rows_blk, b->rows);
  for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind)
    e = upload(b, narrow[kind], narrow_blk[kind], b->narrow[kind]);
  if (e == cudaSuccess) e = upload(b, nouts, nout_blk, b->narrow_out);
  if (e == cudaSuccess) e = upload(b, fins, fin_blk, b->finish);
  if (e == cudaSuccess) e = upload(b, deltas, delta_blk, b->delta);
  if (e == cudaSuccess && b->smem > 0)
    e = cudaFuncSetAttribute(contract_persistent_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, b->smem);
  if (e == cudaSuccess && b->rows.smem > 48 * 1024)
    e = cudaFuncSetAttribute(rows_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             b->rows.smem);
  if (e == cudaSuccess && b->narrow[0].n)
    e = cudaFuncSetAttribute(narrow_batch_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             b->narrow[0].smem);
  if (e == cudaSuccess && b->narrow[1].n)
    e = cudaFuncSetAttribute(narrow_batch_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             b->narrow[1].smem);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the tables are in place
  if (e != cudaSuccess) {
    tc_batch_destroy(b);
    return cuda_status(e, "precision batch plan");
  }
  *out = b;
  return ALTHEA_IBL_OK;
}

int tc_batch_items(const TcBatch* b) { return b ? b->nitems : 0; }

int tc_batch_error(const TcBatch* b, cudaStream_t st) {
  int flag = 0;
  cudaError_t e = cudaMemcpyAsync(&flag, b->d_error, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "precision batch status");
  if (flag)
    return set_error(ALTHEA_IBL_ERR_CUDA, "precision batch: a bounded wait timed out");
  return ALTHEA_IBL_OK;
}

int tc_batch_run(TcBatch* b, cudaStream_t st, cudaStream_t side, cudaEvent_t fork_ev,
                 cudaEvent_t join_ev) {
  ibl::NvtxRange nvtx_range("precision batch");
  // The CUDA-core work (narrow outputs, roughness-0 mips) needs the chain and
  // the tables only: it runs on the side stream beside the split passes and
  // the contraction.
  cudaError_t e = cudaEventRecord(fork_ev, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork_ev, 0);
  if (e != cudaSuccess) return cuda_status(e, "precision batch fork");
  if (b->rows.n)
    rows_batch_kernel<<<(unsigned)b->rows.blocks, 256, b->rows.smem, st>>>(
        b->rows.jobs, b->rows.begins, b->rows.n);
  if (b->nitems > 0) {
    e = cudaMemsetAsync(b->d_next, 0, sizeof(unsigned int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_error, 0, sizeof(int), st);
    if (e == cudaSuccess) {
      contract_persistent_kernel<<<b->ctas, kThreads, b->smem, st>>>(b->d_jobs, b->d_items,
                                                                     b->nitems, b->d_next);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess && b->finish.n)
    finish_batch_kernel<<<(unsigned)b->finish.blocks, kFinishThreads, 0, st>>>(
        b->finish.jobs, b->finish.begins, b->finish.n);
  if (e == cudaSuccess && b->narrow[0].n)
    narrow_batch_kernel<0><<<(unsigned)b->narrow[0].blocks, kNarrowThreads, b->narrow[0].smem,
                             side>>>(b->narrow[0].jobs, b->narrow[0].begins, b->narrow[0].n);
  if (e == cudaSuccess && b->narrow[1].n)
    narrow_batch_kernel<1><<<(unsigned)b->narrow[1].blocks, kNarrowThreads, b->narrow[1].smem,
                             side>>>(b->narrow[1].jobs, b->narrow[1].begins, b->narrow[1].n);
  if (e == cudaSuccess && b->narrow_out.n)
    narrow_finish_batch_kernel<<<(unsigned)b->narrow_out.blocks, 32, 0, side>>>(
        b->narrow_out.jobs, b->narrow_out.begins, b->narrow_out.n);
  if (e == cudaSuccess) e = cudaGetLastError();
  int r = e == cudaSuccess ? ALTHEA_IBL_OK : cuda_status(e, "precision batch launch");
  if (!r) r = launch_delta_batch(b->delta.jobs, b->delta.begins, b->delta.n, b->delta.blocks, side);
  // join (also after an error, so that a stream capture can end cleanly)
  e = cudaEventRecord(join_ev, side);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st, join_ev, 0);
  if (r) return r;
  return cuda_status(e, "precision batch join");
}

}  // namespace ibl

extern "C" int althea_ibl_tc_wait_selftest(unsigned long long limit_ns, int* waited_ms,
                                           void* stream) {
  if (limit_ns == 0 || limit_ns > 1000000000ull)
    return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "wait self-test: limit 1 ns .. 1 s");
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, 3 * sizeof(int));
  if (e != cudaSuccess) return cuda_status(e, "wait self-test buffer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int h[3] = {0, 0, 0};
  e = cudaMemsetAsync(d, 0, 3 * sizeof(int), s);
  if (e == cudaSuccess) {
    wait_selftest_kernel<<<1, 32, 0, s>>>(d, limit_ns);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, "wait self-test");
  if (waited_ms) *waited_ms = h[2];
  if (h[0] != 1 || h[1] != 1)
    return set_error(ALTHEA_IBL_ERR_CUDA, "wait self-test: the wait did not give up (%d, %d)",
                     h[0], h[1]);
  return ALTHEA_IBL_OK;
}

extern "C" int althea_ibl_bake_tc(const float* chain, int w, int h,
                                  const althea_ibl_mip_target* mips, int n, const int* levels,
                                  float* irr_out, int irr_w, int irr_h, size_t irr_pitch,
                                  int irr_level, void* ws, size_t ws_bytes, void* stream) {
  return tc_bake(chain, w, h, mips, n, levels, irr_out, irr_w, irr_h, irr_pitch, irr_level, ws,
                 ws_bytes, ALTHEA_IBL_FORMAT_RGBA32F, (cudaStream_t)stream);
}

extern "C" int althea_ibl_bake_tc_ex(const float* chain, int w, int h,
                                     const althea_ibl_mip_target* mips, int n, const int* levels,
                                     void* irr_out, int irr_w, int irr_h, size_t irr_pitch,
                                     int irr_level, void* ws, size_t ws_bytes, int out_format,
                                     void* stream) {
  return tc_bake(chain, w, h, mips, n, levels, static_cast<float*>(irr_out), irr_w, irr_h,
                 irr_pitch, irr_level, ws, ws_bytes, out_format, (cudaStream_t)stream);
}

extern "C" int althea_ibl_tc_error(const void* ws, void* stream) {
  if (!ws) return set_error(ALTHEA_IBL_ERR_INVALID_ARGUMENT, "null workspace");
  int flag = 0;
  cudaError_t e = cudaMemcpyAsync(&flag, ws, sizeof(int), cudaMemcpyDeviceToHost,
                                  (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "tc status");
  if (flag) return set_error(ALTHEA_IBL_ERR_CUDA, "tensor path: a bounded wait timed out");
  return ALTHEA_IBL_OK;
}
