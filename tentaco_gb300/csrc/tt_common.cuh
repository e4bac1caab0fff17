// tt_common.cuh -- device helpers shared by the sm_103a kernels of libtentaco_gb300.
//
// Memory access discipline on GB300 (HBM3e, 129 MB L2 over two dies):
//  * CSF streams (crd, vals) are read once per call: 128-bit loads that do not
//    allocate in L1 and are marked evict_first in L2, so they do not push the
//    factor matrices out of L2.
//  * Factor-row gathers are marked evict_last in L2: the factors are the only
//    data re-read across the call, and keeping them L2-resident is what bounds
//    the random-gather cost.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

namespace tt {

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization starts (its blocks become resident) once every block of the
// previous kernel on the stream has exited, without the launch gap, and waits here
// until that kernel's memory operations are visible.  Launched without the
// attribute, it returns at once.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Storage precisions: which of values / factors are held in 16 bits.
//   kFP32  values FP32, factors FP32
//   kBF16  values BF16, factors BF16 (power-of-two per-column scales)
//   kBF16F values FP32, factors BF16
//   kFP16  values FP16, factors FP16 (power-of-two per-column scales that put
//          each column's max in [2^14, 2^15), so the 11-bit significand is used
//          over the whole column and nothing overflows)
//   kFX16  the leaf-level factor as 16-bit fixed point (kI16: each column scaled so
//          its max maps to 32767, then each row by a power of two so its largest
//          entry lies in [16384, 32767]); the values FP32, each multiplied by its
//          leaf row's power of two (exact); the other factors FP32 (small, they stay
//          in L2).  Strip walk only.
enum Prec : int { kFP32 = 0, kBF16 = 1, kBF16F = 2, kFP16 = 3, kFX16 = 4 };
// Element kinds of one stored array.  kI16: a 16-bit integer q in [-32767, 32767]
// stored offset-binary (q + 32768), value = q / scale.
enum Kind : int { kF32 = 0, kB16 = 1, kH16 = 2, kI16 = 3 };
// Kind of the (leaf-level) factors and of the values.
__host__ __device__ constexpr int fac_kind(int prec) {
  return prec == kFP32 ? kF32 : prec == kFP16 ? kH16 : prec == kFX16 ? kI16 : kB16;
}
__host__ __device__ constexpr int val_kind(int prec) { return prec == kBF16 ? kB16 : prec == kFP16 ? kH16 : kF32; }

// ---------------------------------------------------------------------------
// L2 cache policies (createpolicy, sm_80+).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_normal() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// ---------------------------------------------------------------------------
// Streaming loads (read-only, no L1 allocation, L2 evict_first).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int4 ld_stream_i4(const int32_t* p, uint64_t pol) {
  int4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ float4 ld_stream_f4(const float* p, uint64_t pol) {
  float4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
// 16 bytes of a stream that the lane's neighbour reads the other half sector of
// in its next load: L1 allocation kept, L2 evict_first.
__device__ __forceinline__ uint4 ld_stream_l1_u4(const void* p, uint64_t pol) {
  uint4 r;
  asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
// 32 bytes of a stream (p 32-byte aligned): one 256-bit load (sm_100 and later).
__device__ __forceinline__ void ld_stream_l1_v8(const void* p, uint64_t pol, uint32_t (&r)[8]) {
  asm volatile("ld.global.nc.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "l"(p), "l"(pol));
}
__device__ __forceinline__ uint2 ld_stream_u2(const void* p, uint64_t pol) {
  uint2 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
               : "=r"(r.x), "=r"(r.y)
               : "l"(p), "l"(pol));
  return r;
}

// ---------------------------------------------------------------------------
// Gather loads (read-only, L2 evict_last).  Widths 2..16 bytes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 ld_gather_16(const void* p, uint64_t pol) {
  uint4 r;
  asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ uint2 ld_gather_8(const void* p, uint64_t pol) {
  uint2 r;
  asm volatile("ld.global.nc.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
               : "=r"(r.x), "=r"(r.y)
               : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ uint32_t ld_gather_4(const void* p, uint64_t pol) {
  uint32_t r;
  asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ uint32_t ld_gather_2(const void* p, uint64_t pol) {
  unsigned short r;
  asm volatile("ld.global.nc.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(r) : "l"(p), "l"(pol));
  return (uint32_t)r;
}

// Same gathers without allocating in L1 (rows gathered once per nonzero rarely hit L1).
__device__ __forceinline__ uint4 ld_gather_16_na(const void* p, uint64_t pol) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ uint2 ld_gather_8_na(const void* p, uint64_t pol) {
  uint2 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
               : "=r"(r.x), "=r"(r.y)
               : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ uint32_t ld_gather_4_na(const void* p, uint64_t pol) {
  uint32_t r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  return r;
}
__device__ __forceinline__ uint32_t ld_gather_2_na(const void* p, uint64_t pol) {
  unsigned short r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(r) : "l"(p), "l"(pol));
  return (uint32_t)r;
}

// ---------------------------------------------------------------------------
// mbarrier and TMA (cp.async.bulk.tensor) helpers.  Addresses are 32-bit shared
// addresses; the tensor map lives in kernel parameter space (__grid_constant__).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// Make barrier initialisation visible to the async proxy (the TMA unit).
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Order this thread's earlier shared-memory accesses before later async-proxy writes.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// One bounded probe of the barrier's phase with the given parity (true: completed).
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Nanoseconds of the GPU's global timer (bounds every wait on a barrier).
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for the barrier phase with the given parity, at most limit_ns; true: completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}
// Four rows (y0..y3) of a 2-D tensor map, columns from x, into shared memory at dst
// (contiguous, 4 x box-width elements), completing `bytes` on the barrier.
__device__ __forceinline__ void tma_gather4(uint32_t dst, const void* tmap, int x, int y0, int y1, int y2, int y3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
      ::"r"(dst), "l"(tmap), "r"(x), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(bar)
      : "memory");
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (cp.async, 16 bytes, L2 only).  Nothing is
// held in registers while a copy is in flight, so a block can have thousands of
// row gathers outstanding.  src_bytes < 16 reads only that many bytes and
// zero-fills the rest (ragged ends of caller-owned arrays).
// ---------------------------------------------------------------------------
// (No L2 cache-policy operand: in cp.async's operand list a lone fourth operand
// is the source size, so only the plain and the 32-bit source-size forms are used.)
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* src, uint64_t pol) {
  (void)pol;
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16_part(void* smem_dst, const void* src, int src_bytes) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// CPT consecutive entries of a row held in shared memory, stored as KIND, as floats.
template <int KIND, int CPT>
__device__ __forceinline__ void smem_row(const unsigned char* row, int q, float (&v)[CPT]);

// BF16 -> FP32 is exact: the bf16 bits are the high half of the fp32 bits.
__device__ __forceinline__ float bf16lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

__device__ __forceinline__ float h16lo(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w & 0xffffu))); }
__device__ __forceinline__ float h16hi(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w >> 16))); }

// Both halves of a packed word as floats (FP16: one packed conversion, no masking).
template <int KIND>
__device__ __forceinline__ float2 pair16(uint32_t w) {
  if constexpr (KIND == kB16) {
    return make_float2(bf16lo(w), bf16hi(w));
  } else {
    __half2 h;
    memcpy(&h, &w, 4);
    return __half22float2(h);
  }
}

// Mixed-precision FMA (sm_100 and later): 16-bit operands, FP32 addend and
// result, one rounding.  The product of two FP16 (or two BF16) numbers is exact
// in FP32, so acc = fma(a, b, acc) equals fmaf on the operands converted to FP32;
// no conversion instructions are issued.
//   mfma2<KIND, HV>: a0 += lo(d) * v.half[HV], a1 += hi(d) * v.half[HV]
//   mfma1<KIND, HV>: a0 += lo(d) * v.half[HV]
template <int KIND, int HV>
__device__ __forceinline__ void mfma2(float& a0, float& a1, uint32_t d, uint32_t v) {
  if constexpr (KIND == kB16) {
    if constexpr (HV == 0)
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %2;\n\tmov.b32 {vl, vh}, %3;\n\t"
          "fma.rn.f32.bf16 %0, dl, vl, %0;\n\tfma.rn.f32.bf16 %1, dh, vl, %1;\n\t}"
          : "+f"(a0), "+f"(a1) : "r"(d), "r"(v));
    else
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %2;\n\tmov.b32 {vl, vh}, %3;\n\t"
          "fma.rn.f32.bf16 %0, dl, vh, %0;\n\tfma.rn.f32.bf16 %1, dh, vh, %1;\n\t}"
          : "+f"(a0), "+f"(a1) : "r"(d), "r"(v));
  } else {
    if constexpr (HV == 0)
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %2;\n\tmov.b32 {vl, vh}, %3;\n\t"
          "fma.rn.f32.f16 %0, dl, vl, %0;\n\tfma.rn.f32.f16 %1, dh, vl, %1;\n\t}"
          : "+f"(a0), "+f"(a1) : "r"(d), "r"(v));
    else
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %2;\n\tmov.b32 {vl, vh}, %3;\n\t"
          "fma.rn.f32.f16 %0, dl, vh, %0;\n\tfma.rn.f32.f16 %1, dh, vh, %1;\n\t}"
          : "+f"(a0), "+f"(a1) : "r"(d), "r"(v));
  }
}
template <int KIND, int HV>
__device__ __forceinline__ void mfma1(float& a0, uint32_t d, uint32_t v) {
  if constexpr (KIND == kB16) {
    if constexpr (HV == 0)
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %1;\n\tmov.b32 {vl, vh}, %2;\n\t"
          "fma.rn.f32.bf16 %0, dl, vl, %0;\n\t}" : "+f"(a0) : "r"(d), "r"(v));
    else
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %1;\n\tmov.b32 {vl, vh}, %2;\n\t"
          "fma.rn.f32.bf16 %0, dl, vh, %0;\n\t}" : "+f"(a0) : "r"(d), "r"(v));
  } else {
    if constexpr (HV == 0)
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %1;\n\tmov.b32 {vl, vh}, %2;\n\t"
          "fma.rn.f32.f16 %0, dl, vl, %0;\n\t}" : "+f"(a0) : "r"(d), "r"(v));
    else
      asm("{\n\t.reg .b16 dl, dh, vl, vh;\n\tmov.b32 {dl, dh}, %1;\n\tmov.b32 {vl, vh}, %2;\n\t"
          "fma.rn.f32.f16 %0, dl, vh, %0;\n\t}" : "+f"(a0) : "r"(d), "r"(v));
  }
}

// Exact products of the 16-bit halves of two packed words: (lo(c) * lo(d),
// hi(c) * hi(d)) in FP32 by the mixed-precision FMA with a zero addend (two
// 11-bit or 8-bit significands multiply exactly into FP32's 24 bits).
template <int KIND>
__device__ __forceinline__ float2 hprod2(uint32_t c, uint32_t d) {
  float p0, p1;
  if constexpr (KIND == kB16)
    asm("{\n\t.reg .b16 cl, ch, dl, dh;\n\tmov.b32 {cl, ch}, %2;\n\tmov.b32 {dl, dh}, %3;\n\t"
        "fma.rn.f32.bf16 %0, cl, dl, 0f00000000;\n\tfma.rn.f32.bf16 %1, ch, dh, 0f00000000;\n\t}"
        : "=f"(p0), "=f"(p1) : "r"(c), "r"(d));
  else
    asm("{\n\t.reg .b16 cl, ch, dl, dh;\n\tmov.b32 {cl, ch}, %2;\n\tmov.b32 {dl, dh}, %3;\n\t"
        "fma.rn.f32.f16 %0, cl, dl, 0f00000000;\n\tfma.rn.f32.f16 %1, ch, dh, 0f00000000;\n\t}"
        : "=f"(p0), "=f"(p1) : "r"(c), "r"(d));
  return make_float2(p0, p1);
}
// Exact product of one 16-bit half of each of two words (HC of c, HD of d).
template <int KIND, int HC, int HD>
__device__ __forceinline__ float hprod1(uint32_t c, uint32_t d) {
  const unsigned short a = (unsigned short)(HC ? c >> 16 : c), b = (unsigned short)(HD ? d >> 16 : d);
  float p;
  if constexpr (KIND == kB16)
    asm("fma.rn.f32.bf16 %0, %1, %2, 0f00000000;" : "=f"(p) : "h"(a), "h"(b));
  else
    asm("fma.rn.f32.f16 %0, %1, %2, 0f00000000;" : "=f"(p) : "h"(a), "h"(b));
  return p;
}

// Packed FP32 arithmetic (sm_100 and later): two lanes of FP32 per instruction,
// each rounded like its scalar form.  The FMA pipe's throughput is the same;
// the issue slots are halved.
//   ffma2: (a0, a1) += (b0, b1) * (c0, c1)
__device__ __forceinline__ void ffma2(float& a0, float& a1, float b0, float b1, float c0, float c1) {
  asm("{\n\t.reg .b64 ra, rb, rc;\n\tmov.b64 ra, {%0, %1};\n\tmov.b64 rb, {%2, %3};\n\tmov.b64 rc, {%4, %5};\n\t"
      "fma.rn.f32x2 ra, rb, rc, ra;\n\tmov.b64 {%0, %1}, ra;\n\t}"
      : "+f"(a0), "+f"(a1) : "f"(b0), "f"(b1), "f"(c0), "f"(c1));
}
//   fmul2: (b0, b1) * (c0, c1)
__device__ __forceinline__ float2 fmul2(float b0, float b1, float c0, float c1) {
  float r0, r1;
  asm("{\n\t.reg .b64 rr, rb, rc;\n\tmov.b64 rb, {%2, %3};\n\tmov.b64 rc, {%4, %5};\n\t"
      "mul.rn.f32x2 rr, rb, rc;\n\tmov.b64 {%0, %1}, rr;\n\t}"
      : "=f"(r0), "=f"(r1) : "f"(b0), "f"(b1), "f"(c0), "f"(c1));
  return make_float2(r0, r1);
}

// 16-bit fixed point (offset-binary halves) to FP32: the half placed in the
// mantissa of 2^23 gives the float 2^23 + u exactly; subtracting 2^23 + 2^15
// leaves q exactly.  One integer op per half, one packed subtraction per pair.
__device__ __forceinline__ float2 i16pair(uint32_t w) {
  uint32_t lo, hi;
  asm("prmt.b32 %0, %1, 0x4B000000, 0x7510;" : "=r"(lo) : "r"(w));
  asm("prmt.b32 %0, %1, 0x4B000000, 0x7532;" : "=r"(hi) : "r"(w));
  float r0, r1;
  asm("{\n\t.reg .b64 ra, rk;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rk, {%4, %4};\n\t"
      "sub.rn.f32x2 ra, ra, rk;\n\tmov.b64 {%0, %1}, ra;\n\t}"
      : "=f"(r0), "=f"(r1) : "f"(__uint_as_float(lo)), "f"(__uint_as_float(hi)), "f"(8421376.0f));
  return make_float2(r0, r1);
}
__device__ __forceinline__ float i16lo(uint32_t w) { return __uint_as_float(0x4B000000u | (w & 0xffffu)) - 8421376.0f; }
__device__ __forceinline__ float i16hi(uint32_t w) { return __uint_as_float(0x4B000000u | (w >> 16)) - 8421376.0f; }

template <int KIND>
__device__ __forceinline__ float lo16(uint32_t w) { return KIND == kB16 ? bf16lo(w) : KIND == kI16 ? i16lo(w) : h16lo(w); }
template <int KIND>
__device__ __forceinline__ float hi16(uint32_t w) { return KIND == kB16 ? bf16hi(w) : KIND == kI16 ? i16hi(w) : h16hi(w); }

// Load CPT consecutive entries starting at element offset `off` of a row-major
// array stored as KIND, as floats (gather path: L2 evict_last).
template <int KIND, int CPT>
__device__ __forceinline__ void row_load(const void* base, int64_t off, uint64_t pol, float (&v)[CPT]) {
  if constexpr (KIND == kF32) {
    const float* p = static_cast<const float*>(base) + off;
    if constexpr (CPT == 8) {
      uint4 a = ld_gather_16(p, pol), b = ld_gather_16(p + 4, pol);
      v[0] = __uint_as_float(a.x); v[1] = __uint_as_float(a.y); v[2] = __uint_as_float(a.z); v[3] = __uint_as_float(a.w);
      v[4] = __uint_as_float(b.x); v[5] = __uint_as_float(b.y); v[6] = __uint_as_float(b.z); v[7] = __uint_as_float(b.w);
    } else if constexpr (CPT == 4) {
      uint4 a = ld_gather_16(p, pol);
      v[0] = __uint_as_float(a.x); v[1] = __uint_as_float(a.y); v[2] = __uint_as_float(a.z); v[3] = __uint_as_float(a.w);
    } else if constexpr (CPT == 2) {
      uint2 a = ld_gather_8(p, pol);
      v[0] = __uint_as_float(a.x); v[1] = __uint_as_float(a.y);
    } else {
      v[0] = __uint_as_float(ld_gather_4(p, pol));
    }
  } else {
    const uint16_t* p = static_cast<const uint16_t*>(base) + off;
    if constexpr (CPT == 8) {
      uint4 a = ld_gather_16(p, pol);
      v[0] = lo16<KIND>(a.x); v[1] = hi16<KIND>(a.x); v[2] = lo16<KIND>(a.y); v[3] = hi16<KIND>(a.y);
      v[4] = lo16<KIND>(a.z); v[5] = hi16<KIND>(a.z); v[6] = lo16<KIND>(a.w); v[7] = hi16<KIND>(a.w);
    } else if constexpr (CPT == 4) {
      uint2 a = ld_gather_8(p, pol);
      v[0] = lo16<KIND>(a.x); v[1] = hi16<KIND>(a.x); v[2] = lo16<KIND>(a.y); v[3] = hi16<KIND>(a.y);
    } else if constexpr (CPT == 2) {
      uint32_t a = ld_gather_4(p, pol);
      v[0] = lo16<KIND>(a); v[1] = hi16<KIND>(a);
    } else {
      v[0] = lo16<KIND>(ld_gather_2(p, pol));
    }
  }
}

template <int KIND, int CPT>
__device__ __forceinline__ void smem_row(const unsigned char* row, int q, float (&v)[CPT]) {
  if constexpr (KIND == kF32) {
    const float* p = reinterpret_cast<const float*>(row) + q * CPT;
    if constexpr (CPT == 8) {
      const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else if constexpr (CPT == 4) {
      const float4 a = *reinterpret_cast<const float4*>(p);
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    } else if constexpr (CPT == 2) {
      const float2 a = *reinterpret_cast<const float2*>(p);
      v[0] = a.x; v[1] = a.y;
    } else {
      v[0] = p[0];
    }
  } else {
    const uint16_t* p = reinterpret_cast<const uint16_t*>(row) + q * CPT;
    if constexpr (CPT == 8) {
      const uint4 a = *reinterpret_cast<const uint4*>(p);
      v[0] = lo16<KIND>(a.x); v[1] = hi16<KIND>(a.x); v[2] = lo16<KIND>(a.y); v[3] = hi16<KIND>(a.y);
      v[4] = lo16<KIND>(a.z); v[5] = hi16<KIND>(a.z); v[6] = lo16<KIND>(a.w); v[7] = hi16<KIND>(a.w);
    } else if constexpr (CPT == 4) {
      const uint2 a = *reinterpret_cast<const uint2*>(p);
      v[0] = lo16<KIND>(a.x); v[1] = hi16<KIND>(a.x); v[2] = lo16<KIND>(a.y); v[3] = hi16<KIND>(a.y);
    } else if constexpr (CPT == 2) {
      const uint32_t a = *reinterpret_cast<const uint32_t*>(p);
      v[0] = lo16<KIND>(a); v[1] = hi16<KIND>(a);
    } else {
      v[0] = lo16<KIND>((uint32_t)p[0]);
    }
  }
}

// Largest x in [lo, hi] with a[x] <= t, given a[lo] <= t (a non-decreasing).
template <typename IdxT>
__device__ __forceinline__ int64_t search_le(const IdxT* a, int64_t lo, int64_t hi, int64_t t) {
  while (lo < hi) {
    int64_t mid = lo + ((hi - lo + 1) >> 1);
    if ((int64_t)a[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace tt
