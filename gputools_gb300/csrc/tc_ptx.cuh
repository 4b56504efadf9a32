// tc_ptx.cuh -- inline-PTX wrappers for Blackwell (sm_103a) tensor-core
// kernels: mbarriers, TMA tensor loads, tcgen05 MMA / TMEM, and bounded waits.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace gt {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Streaming store (evict-first in L2): outputs written once, so that they do
// not push the operands a kernel re-reads out of L2.
__device__ __forceinline__ void st_stream(float *p, float v) {
  asm volatile("st.global.cs.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// try_wait with a suspend-time hint: a waiting thread sleeps until the phase
// completes or `hint_ns` passes, instead of polling and taking issue slots
// from the warps that do the work.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity,
                                                    uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Non-blocking test of the phase (mbarrier.test_wait never suspends; a
// try_wait may suspend until the phase completes, whatever its hint).
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr uint32_t kSleepHintNs = 100000;  // 0.1 ms: well inside every wait limit

// Bounded-wait settings of a launch: the device error word a CTA sets when
// one of its waits gives up, the limit of each wait, and the sleep hint (0
// for limits too short for a suspending wait: those waits poll).
struct WaitCfg {
  int *err;
  uint64_t limit_ns;
  uint32_t hint_ns;
};

// Waits for the phase of `bar` with the given parity.  Gives up (returns
// false) after `limit_ns` or as soon as *abort becomes non-zero, so a kernel
// never spins forever on a barrier that will not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort,
                                          uint64_t limit_ns, uint32_t hint_ns = kSleepHintNs) {
  if (hint_ns == 0) {
    // a short limit: poll without suspending, so that the limit holds
    const uint64_t t0 = globaltimer_ns();
    while (true) {
      if (mbar_test_wait(bar, parity)) return true;
      if (*abort) return false;
      if (globaltimer_ns() - t0 > limit_ns) return false;
    }
  }
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait_sleep(bar, parity, hint_ns)) return true;
    if (*abort) return false;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort,
                                          const WaitCfg &wc) {
  return mbar_wait(bar, parity, abort, wc.limit_ns, wc.hint_ns);
}

// Bounded wait that ignores the abort flag (used to drain in-flight work).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
}

// ---------------------------------------------------------------- TMA
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int32_t c0, int32_t c1, int32_t c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---------------------------------------------------------------- tcgen05
// Whole warp: allocate `ncols` TMEM columns, address written to *dst (smem).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, bf16 x bf16 -> f32, one thread issues.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on `bar` once every tcgen05 operation issued so far by this thread
// has completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 32 TMEM lanes x 32 consecutive columns -> 32 registers per thread
// (thread i of the warp reads lane base+i).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 32 TMEM lanes x 8 consecutive columns -> 8 registers per thread, without
// the wait: several loads may be in flight before one tmem_wait_ld().
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 32 TMEM lanes x 16 consecutive columns -> 16 registers per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Hardware square root approximation (sqrt.approx.ftz.f32; relative error
// about 2^-23), for epilogues whose inputs are already rounded to float.
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Hardware reciprocal square root approximation (rsqrt.approx.ftz.f32).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Shared-memory matrix descriptor of a K-major bf16 tile whose rows are
// `row_bytes` (128 -> SWIZZLE_128B, 64 -> SWIZZLE_64B) and whose 8-row
// groups are dense (stride 8 * row_bytes).  The tile must start on an
// 8 * row_bytes boundary.
__device__ __forceinline__ uint64_t smem_desc_kmajor(uint32_t saddr, int row_bytes) {
  const uint64_t sbo = uint64_t(8 * row_bytes) >> 4;
  const uint64_t layout = row_bytes == 128 ? 2ull : 4ull;  // SWIZZLE_128B / SWIZZLE_64B
  uint64_t d = 0;
  d |= uint64_t((saddr & 0x3FFFFu) >> 4);  // start address
  d |= uint64_t(1) << 16;                  // leading byte offset (unused for swizzled K-major)
  d |= sbo << 32;                          // stride byte offset
  d |= uint64_t(1) << 46;                  // descriptor version (tcgen05)
  d |= layout << 61;
  return d;
}

// Instruction descriptor: kind::f16, D = f32, A and B K-major and of the same
// 16-bit type (ab_fmt 0: fp16, 1: bf16).
__host__ __device__ constexpr uint32_t idesc_f32acc(int M, int N, uint32_t ab_fmt) {
  return (1u << 4)                    // D format f32
         | (ab_fmt << 7)              // A format
         | (ab_fmt << 10)             // B format
         | (uint32_t(N >> 3) << 17)   // N / 8
         | (uint32_t(M >> 4) << 24);  // M / 16
}

// Operand encodings of the split planes (the values of enum gt_gram_path):
//   bf16x3  two bf16 parts (hi, lo), products hi.hi + hi.lo + lo.hi
//   bf16x6  three bf16 parts, the six products of total order <= 2
//   f16x3   two fp16 parts of the value times a power of two chosen so that
//           the largest magnitude lies in [2^14, 2^15); hi carries 11 bits and
//           lo the next 11, so the three products keep ~2^-22 per element
//           at the cost of bf16x3.
constexpr int KIND_BF16X3 = 0, KIND_BF16X6 = 1, KIND_F16X3 = 3;
// The error-free fixed-point split (gram_exact.cu) has its own kernel.
constexpr int KIND_F16X6 = 4;

template <int KIND>
struct Kind {
  static constexpr int NSPLIT = KIND == KIND_BF16X6 ? 3 : 2;
  static constexpr bool F16 = KIND == KIND_F16X3;
  static constexpr uint32_t AB_FMT = F16 ? 0u : 1u;
};

// Split of v into the parts of KIND, as raw 16-bit patterns; each part is the
// round-to-nearest of the remainder of the previous ones (every remainder is
// exact in float).  For f16x3, v must already carry its power-of-two scale.
template <int KIND>
__device__ __forceinline__ void split_parts(float v, uint16_t (&p)[3]) {
  float rem = v;
  if (Kind<KIND>::F16) {
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const __half h = __float2half_rn(rem);
      p[i] = __half_as_ushort(h);
      rem -= __half2float(h);
    }
    p[2] = 0;
  } else {
#pragma unroll
    for (int i = 0; i < 3; i++) {
      if (i < Kind<KIND>::NSPLIT) {
        const __nv_bfloat16 h = __float2bfloat16_rn(rem);
        p[i] = __bfloat16_as_ushort(h);
        rem -= __bfloat162float(h);
      } else {
        p[i] = 0;
      }
    }
  }
}

// Power of two 2^e, e in [-126, 127], built from its exponent bits.
__device__ __forceinline__ float exp2i(int e) { return __uint_as_float(uint32_t(e + 127) << 23); }

// Scale exponent that brings the largest magnitude m of a row into
// [2^14, 2^15) for the f16x3 encoding (0 for m = 0 or non-finite m).
__device__ __forceinline__ int f16_scale_exp(float m) {
  if (!(m > 0.f) || !(m <= 3.4e38f)) return 0;
  const int e = int((__float_as_uint(m) >> 23) & 255u) - 127;  // floor(log2 m), normal m
  int s = 14 - e;
  return s > 126 ? 126 : (s < -126 ? -126 : s);
}

}  // namespace tc
}  // namespace gt
