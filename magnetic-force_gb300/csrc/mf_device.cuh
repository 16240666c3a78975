// mf_device.cuh -- sm_103a device helpers: bulk-copy staging through mbarriers,
// approximate reciprocal square root, compensated summation.
//
// Every spin-wait here is bounded.  A wait that runs out returns false; the
// caller records MF_DEVERR_* in the launch's error word and leaves the kernel
// after draining its own copies, so a stuck copy can never hang the GPU.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mfgb {

// Device-side error codes written to the error word a launch is given.
enum : int {
  MF_DEVERR_NONE = 0,
  MF_DEVERR_STAGE_TIMEOUT = 1,   // a source tile never arrived in shared memory
  MF_DEVERR_DRAIN_TIMEOUT = 2,   // copies still in flight when leaving after an error
};

// Try-wait iterations before a staging wait gives up.  Each try_wait blocks
// for a hardware-defined slice (~microseconds), so this bounds a wait at well
// under a second.
constexpr uint32_t kWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make mbarrier initialisation visible to the async (bulk-copy) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared, completion signalled on `bar` as tx bytes.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
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

// Bounded wait for phase `parity` of `bar`: at most `limit` try-waits.
// Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Try-waits of a staging wait: the default bound, or, with the debug setting
// a launch carries (mf_debug_stage_wait_limit), debug - 1 of them.  Drains
// after an error always wait with the default bound.
__device__ __forceinline__ uint32_t stage_wait_limit(uint32_t debug) { return debug ? debug - 1 : kWaitLimit; }

// Asynchronous 16-byte copy global -> shared (L2 only), grouped per thread:
// cp_async_commit closes the thread's current group, cp_async_wait<N> waits
// until at most N of its groups are in flight.  Other threads see the data
// after a barrier that includes them (__syncwarp / __syncthreads).  Both
// addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// rsqrt.approx.ftz.f32: hardware reciprocal square root (MUFU), relative error
// below 2^-22 per the PTX ISA.  rsqrt(+0) = +inf, which callers never feed
// into a product that survives (near pairs take the exact branch).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Knuth's two-sum: s + e == a + b exactly (round-to-nearest, no FMA
// contraction: the intrinsics pin each operation to one rounding).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Running compensated accumulator: adds one block-sum `x` to (s, c).
__device__ __forceinline__ void comp_add(float& s, float& c, float x) {
  float t, e;
  two_sum(s, x, t, e);
  s = t;
  c = __fadd_rn(c, e);
}

// Packed FP32 pairs (PTX .f32x2, sm_100 and later): one instruction applies
// the operation to both halves, so the FMA pipe does the same work with half
// the issue slots.  Rounding is round-to-nearest per half, as for FFMA.
__device__ __forceinline__ unsigned long long f2_bits(float2 a) {
  return (static_cast<unsigned long long>(__float_as_uint(a.y)) << 32) | __float_as_uint(a.x);
}
__device__ __forceinline__ float2 f2_from(unsigned long long r) {
  return make_float2(__uint_as_float(unsigned(r & 0xffffffffull)), __uint_as_float(unsigned(r >> 32)));
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
  return f2_from(r);
}
__device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(r);
}
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(r);
}
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(r);
}
__device__ __forceinline__ float2 f2_dup(float v) { return make_float2(v, v); }

// Packed 4-wide particle record (x, y, z, pad): 16 B for FP32, 32 B for FP64,
// so a tile of them is one contiguous, 16-byte-aligned bulk copy.
struct alignas(32) dbl4 {
  double x, y, z, w;
};
template <class Real>
struct Vec4T;
template <>
struct Vec4T<float> {
  using type = float4;
};
template <>
struct Vec4T<double> {
  using type = dbl4;
};

}  // namespace mfgb
