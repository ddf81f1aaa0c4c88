// tcgen05 / TMA / mbarrier helpers shared by the tensor-core MTTKRP kernels (inline PTX).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "ptg.h"

namespace ptg {
namespace tc {

constexpr uint32_t kSpinLimit = 1u << 26;   // polls before a bounded wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; false when it gave up (or another role already gave up).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && *abort) return false;
  }
  return false;
}

// Bounded wait that does not stop on the abort word (for the final drains).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Bounded wait with the poll limit given by the launch (a limit of 0 gives up at once).
__device__ __forceinline__ bool mbar_wait_lim(uint64_t *bar, uint32_t parity, volatile int *abort, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && *abort) return false;
  }
  return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
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

// Shared-memory matrix descriptor (tcgen05): start, leading/stride byte offsets, fixed
// version bits 46-48 = 0b001, 128-byte swizzle (layout type 2 in bits 61-63).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// The same descriptor without its start address: the start field (bits 0-13, address >> 4)
// is ORed in by the caller, and stepping the start by b bytes adds b >> 4 (no carry: shared
// addresses are below 2^18).
__device__ __forceinline__ uint64_t smem_desc_sw128_hi(uint32_t lbo, uint32_t sbo) {
  return ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46) |
         ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// FP8 x FP8 -> FP32 (kind::f8f6f4; the operand formats are in the instruction descriptor)
__device__ __forceinline__ void umma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Two FP32 values rounded to nearest e4m3 (saturating at +-448): lo in bits 0-7, hi in 8-15.
__device__ __forceinline__ uint32_t e4m3x2_rn(float lo, float hi) {
  uint16_t r;
  asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;" : "=h"(r) : "f"(hi), "f"(lo));
  return r;
}
// The two e4m3 values of bits 0-7 (x) and 8-15 (y), exactly, as FP32.
__device__ __forceinline__ float2 e4m3x2_to_f32(uint32_t v) {
  uint32_t h2;
  asm("cvt.rn.f16x2.e4m3x2 %0, %1;" : "=r"(h2) : "h"((uint16_t)v));
  float2 f;
  asm("{\n .reg .f16 a, b;\n mov.b32 {a, b}, %2;\n cvt.f32.f16 %0, a;\n cvt.f32.f16 %1, b;\n}\n"
      : "=f"(f.x), "=f"(f.y)
      : "r"(h2));
  return f;
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// One side of a Khatri-Rao row: the factors whose mixed-radix digits make up `lin`.
struct KrDevTc {
  int n;
  uint32_t ext[PTG_MAX_ORDER];
  uint32_t valid[PTG_MAX_ORDER];
  const float *fac[PTG_MAX_ORDER];
};

// Khatri-Rao values of one side for linear index `lin`, 8 consecutive columns from c.
__device__ __forceinline__ void kr8(const KrDevTc &s, uint32_t lin, int R, int c, float *v) {
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = 1.0f;
  for (int f = 0; f < s.n; ++f) {
    const uint32_t e = s.ext[f];
    const uint32_t d = lin % e;
    lin /= e;
    if (d >= s.valid[f]) {
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = 0.0f;
      return;
    }
    const float *row = s.fac[f] + (size_t)d * R;
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] *= (c + j < R) ? __ldg(row + c + j) : 0.0f;
  }
}

// The same product for 4 consecutive columns from c.
__device__ __forceinline__ void kr4(const KrDevTc &s, uint32_t lin, int R, int c, float *v) {
#pragma unroll
  for (int j = 0; j < 4; ++j) v[j] = 1.0f;
  for (int f = 0; f < s.n; ++f) {
    const uint32_t e = s.ext[f];
    const uint32_t d = lin % e;
    lin /= e;
    if (d >= s.valid[f]) {
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = 0.0f;
      return;
    }
    const float *row = s.fac[f] + (size_t)d * R;
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] *= (c + j < R) ? __ldg(row + c + j) : 0.0f;
  }
}

// The rows of the first two factors of one side for the digits of `lin` (null when the side
// has fewer factors), and whether every digit lies within its factor's valid rows (a padded
// mode-0 index makes the Khatri-Rao value zero; its row address then points at row 0, so no
// load leaves the factor).  Kept in registers: no per-thread arrays.
struct KrRows2 {
  const float *r0, *r1;
  bool ok;
};
__device__ __forceinline__ KrRows2 kr_rows2(const KrDevTc &s, uint32_t lin, int R) {
  KrRows2 o{nullptr, nullptr, true};
  for (int f = 0; f < s.n; ++f) {
    const uint32_t e = s.ext[f];
    const uint32_t d = lin % e;
    lin /= e;
    const bool in = d < s.valid[f];
    o.ok = o.ok && in;
    const float *p = s.fac[f] + (size_t)(in ? d : 0u) * R;
    if (f == 0) o.r0 = p;
    else if (f == 1) o.r1 = p;
  }
  return o;
}

// W consecutive values of a factor row from column c (0 beyond R; 1 when row is null, the
// neutral factor of an empty side).  vec: R % 4 == 0 and 16-byte aligned rows, so float4.
template <int W>
__device__ __forceinline__ void kr_load(const float *row, int R, int c, bool vec, float *t) {
  if (vec) {
#pragma unroll
    for (int q = 0; q < W / 4; ++q) {
      float4 x = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
      if (row) x = (c + 4 * q < R) ? __ldg(reinterpret_cast<const float4 *>(row + c + 4 * q))
                                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      t[4 * q] = x.x;
      t[4 * q + 1] = x.y;
      t[4 * q + 2] = x.z;
      t[4 * q + 3] = x.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < W; ++j) t[j] = row ? ((c + j < R) ? __ldg(row + c + j) : 0.0f) : 1.0f;
  }
}

// Factors 2, 3, ... of one side multiplied into v (a side has more than two factors only
// for orders >= 4 on the before side or >= 5 on the after side).
template <int W>
__device__ __forceinline__ void kr_tail(const KrDevTc &s, uint32_t lin, int R, int c, bool vec, float *v) {
  for (int f = 0; f < s.n; ++f) {
    const uint32_t e = s.ext[f];
    const uint32_t d = lin % e;
    lin /= e;
    if (f < 2) continue;
    float t[W];
    kr_load<W>(s.fac[f] + (size_t)(d < s.valid[f] ? d : 0u) * R, R, c, vec, t);
#pragma unroll
    for (int j = 0; j < W; ++j) v[j] *= t[j];
  }
}

// Khatri-Rao values of columns [c, c + W) for the K row (lin_a on the "after" side, lin_b on
// the "before" side when use_b): (1 * a_0 * a_1 ...) * (1 * b_0 * b_1 ...), the order of kr8.
// The first two factors of each side are loaded before any product is formed, so a 3- or
// 4-way contraction pays one memory round trip per call.
template <int W>
__device__ __forceinline__ void kr_pair(const KrDevTc &A, uint32_t lin_a, const KrDevTc &B, uint32_t lin_b,
                                        bool use_b, int R, int c, bool vec, float *v) {
  const KrRows2 ra = kr_rows2(A, lin_a, R);
  KrRows2 rb{nullptr, nullptr, true};
  if (use_b) rb = kr_rows2(B, lin_b, R);
  float a0[W], a1[W], b0[W], b1[W];
  kr_load<W>(ra.r0, R, c, vec, a0);
  kr_load<W>(ra.r1, R, c, vec, a1);
  kr_load<W>(rb.r0, R, c, vec, b0);
  kr_load<W>(rb.r1, R, c, vec, b1);
#pragma unroll
  for (int j = 0; j < W; ++j) {
    a0[j] = ra.r1 ? a0[j] * a1[j] : a0[j];
    b0[j] = rb.r1 ? b0[j] * b1[j] : b0[j];
  }
  if (A.n > 2) kr_tail<W>(A, lin_a, R, c, vec, a0);
  if (use_b && B.n > 2) kr_tail<W>(B, lin_b, R, c, vec, b0);
  const bool ok = ra.ok && rb.ok;
#pragma unroll
  for (int j = 0; j < W; ++j) v[j] = ok ? (use_b ? a0[j] * b0[j] : a0[j]) : 0.0f;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    cudaGetLastError();
  });
  return fn;
}

}  // namespace tc
}  // namespace ptg
