// Device helpers shared by the tcgen05 kernels (split-TF32 GEMMs): mbarriers with bounded waits,
// TMEM allocation, tcgen05.mma / commit / ld, shared-memory and instruction descriptors, and the
// FP64 <-> split-TF32 conversions.
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "common.cuh"

namespace tc {

constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
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

// Bounded wait: false (and an error code recorded) when the budget runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) {
      atomicExch(err, code);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
  const uint64_t addr = (uint64_t)(smem_u32(p) & 0x3FFFF) >> 4;
  return addr | (1ull << 16) | (64ull << 32) | (1ull << 46) | (2ull << 61);
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t make_idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// hi + lo <- hi + lo + x with hi + x split error-free (Knuth's TwoSum; the _rn intrinsics keep the
// compiler from reassociating it)
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float t = __fadd_rn(hi, x);
  const float z = __fsub_rn(t, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(x, z));
  hi = t;
  lo = __fadd_rn(lo, e);
}

// FP32 -> FP64 by integer operations (exact for normal numbers, infinities and NaNs; FP32
// subnormals, below 1.2e-38, become signed zeros, as the split-TF32 operands already do)
__device__ __forceinline__ double f32_to_f64(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t e = (u >> 23) & 0xFFu;
  uint64_t bits = (uint64_t)(u >> 31) << 63;
  const uint64_t mant = (uint64_t)(u & 0x7FFFFFu) << 29;
  if (e == 0xFFu) bits |= (0x7FFull << 52) | mant;
  else if (e != 0u) bits |= ((uint64_t)(e + 896u) << 52) | mant;
  return __longlong_as_double((long long)bits);
}

// x -> tf32(x) + tf32(remainder). One conversion from FP64 (the FP64 pipe issues 64 times fewer
// lanes per clock than FP32 here); the remainder is taken from the FP32 value, exactly: the bits
// of x below FP32's 24 lie beneath the 22 that hi + lo keep.
__device__ __forceinline__ void split_tf32(double x, float& hi, float& lo) {
  const float xf = __double2float_rn(x);
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(xf));
  const float rem = __fsub_rn(xf, __uint_as_float(h));
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(rem));
  hi = __uint_as_float(h);
  lo = __uint_as_float(l);
}

__device__ __forceinline__ bool finite_f64(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7FF) != 0x7FF;
}


}  // namespace tc
