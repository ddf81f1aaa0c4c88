// FP8 (e4m3) tensor storage with per-slab scales, and its MTTKRP on the tensor cores.
//
// Storage.  Entry x of slab s (the index of the last mode) is stored as the e4m3 code of
// float(x) / scale_s, where scale_s = 2^k is the smallest power of two with
// max_slab |x| <= 448 * 2^k.  The rounding is stochastic: x/scale lies between two
// neighbours of the e4m3 grid, and it goes up with probability equal to its distance from
// the lower one (in units of the spacing), decided by a 24-bit hash of the entry's position
// in the FP64 source.  The stored tensor is then an unbiased copy of the data:
// E[stored] = float(x), so <X_stored, Y> estimates <X, Y> without the drift that
// round-to-nearest at 3 mantissa bits would leave in the ALS cost.
//
// Contraction.  The same [P, Q, S] view as the BF16 kernel (ptg_mttkrp_tc.cu), on
// tcgen05.mma kind::f8f6f4 (E4M3 x E4M3 -> FP32), one TMA tile of 128 x 128 codes
// (16 KB) per K-block.  The Khatri-Rao operand is built in shared memory as two e4m3 parts
// per value, hi = rn(v) and lo = rn(16 (v - hi)), stacked along N (N = 2 x rank padded to
// 16), so the MMA returns X.hi and X.lo and the epilogue forms X.hi + X.lo / 16: about
// eight significant bits per Khatri-Rao value, like BF16.  Before rounding, column r of
// the Khatri-Rao tile is multiplied by c_r = 2^k chosen from the factor columns' maxima
// (f8_colscale_kernel) so that every value stays within e4m3's normal range, and, for the
// modes whose contraction runs over the last mode, by the slab's scale; the epilogue
// divides by c_r (and multiplies by the slab scale when the slab index is the output row).
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "ptg_internal.h"
#include "ptg_tcgen05.h"

namespace ptg {

// ------------------------------------------------------------------------------------
// Encoding
// ------------------------------------------------------------------------------------

// splitmix64 finaliser of position idx, top 24 bits: the dither of that entry's rounding.
__device__ __forceinline__ uint32_t f8_dither(uint64_t idx) {
  uint64_t z = idx * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (uint32_t)(z >> 40);
}

// e4m3 code of v (|v| <= 448), stochastically rounded with the 24-bit dither u.  Every
// step is exact in FP32: the spacing is a power of two, so y = |v| / spacing, its
// fractional part t and t * 2^24 carry no rounding.
__device__ __forceinline__ uint32_t f8_encode_sr(float v, uint32_t u) {
  const uint32_t vb = __float_as_uint(v);
  const float a = fabsf(v);
  float inv_sp, sp;
  if (a < 0.015625f) {   // below 2^-6: the subnormal grid, spacing 2^-9
    inv_sp = 512.0f;
    sp = 0.001953125f;
  } else {
    const int e = (int)((__float_as_uint(a) >> 23) & 0xFF) - 127;   // -6 .. 8
    inv_sp = __uint_as_float((uint32_t)(127 - (e - 3)) << 23);
    sp = __uint_as_float((uint32_t)(127 + (e - 3)) << 23);
  }
  const float y = a * inv_sp;
  const float fl = floorf(y);
  const float q = ((y - fl) * 16777216.0f > (float)u) ? fl + 1.0f : fl;
  const float r = q * sp;   // an e4m3 value, 0 .. 448
  uint32_t code;
  if (r < 0.015625f) {
    code = (uint32_t)(r * 512.0f);   // 0 .. 7 (8 is 2^-6, written by the normal branch)
  } else {
    const uint32_t rb = __float_as_uint(r);
    code = ((((rb >> 23) & 0xFF) - 127 + 7) << 3) | ((rb >> 20) & 7);
  }
  return code | ((vb >> 24) & 0x80);
}

// Exact FP32 value of an e4m3 code.
__device__ __forceinline__ float f8_decode(uint32_t c) {
  const int e = (c >> 3) & 15, m = c & 7;
  const float mag = e == 0 ? (float)m * 0.001953125f : __uint_as_float((uint32_t)(e - 7 + 127) << 23) * (1.0f + m * 0.125f);
  return (c & 0x80) ? -mag : mag;
}

// Exponent k of the slab scale 2^k: the smallest k with max <= 448 * 2^k (448 = 0.875 * 2^9).
__device__ __forceinline__ int f8_scale_exp(double mx) {
  if (!(mx > 0.0)) return 0;
  int E;
  const double f = frexp(mx, &E);   // mx = f * 2^E, f in [0.5, 1)
  int k = (f <= 0.875) ? E - 9 : E - 8;
  return max(-126, min(127, k));
}

namespace {

constexpr int kF8EncThreads = 256;

__device__ __forceinline__ void f8_flush_max(double m, int64_t slab, unsigned long long *slab_bits) {
  __shared__ double red[kF8EncThreads / 32];
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = red[0];
    for (int w = 1; w < kF8EncThreads / 32; ++w) b = fmax(b, red[w]);
    // |x| >= 0: the bit patterns of non-negative doubles order like the values
    atomicMax(slab_bits + slab, (unsigned long long)__double_as_longlong(b));
  }
  __syncthreads();
}

// Max |x| of every slab met by fibres [fiber0, fiber0 + nfib) of an FP64 ColMajor source
// (fibre = one mode-0 column, slab = fibre / fibres_per_slab).  Each block takes a
// contiguous run of fibres, so it meets few slabs and flushes once per slab.
__global__ void __launch_bounds__(kF8EncThreads)
f8_slab_max_kernel(const double *__restrict__ src, int64_t I0, int64_t fiber0, int64_t nfib, int64_t fps,
                   unsigned long long *__restrict__ slab_bits) {
  const int64_t per = (nfib + gridDim.x - 1) / gridDim.x;
  const int64_t f_begin = (int64_t)blockIdx.x * per, f_end = min(nfib, f_begin + per);
  double m = 0.0;
  int64_t cur = -1;
  for (int64_t f = f_begin; f < f_end; ++f) {
    const int64_t slab = (fiber0 + f) / fps;
    if (slab != cur) {
      if (cur >= 0) f8_flush_max(m, cur, slab_bits);
      cur = slab;
      m = 0.0;
    }
    const double *s = src + f * I0;
    for (int64_t i = threadIdx.x; i < I0; i += blockDim.x) m = fmax(m, fabs(__ldg(s + i)));
  }
  if (cur >= 0) f8_flush_max(m, cur, slab_bits);
}

// Encode fibres [fiber0, fiber0 + nfib): codes (mode 0 padded to pI0 with zero codes),
// the slab scales, the optional FP32 copy, and FP64 partial sums of squares of the source
// (as FP32 values, like the other storage types) and of the stored values.  Four
// consecutive entries per thread, written as one 32-bit word.
__global__ void __launch_bounds__(kF8EncThreads)
f8_encode_kernel(const double *__restrict__ src, int64_t I0, int64_t pI0, int64_t fiber0, int64_t nfib, int64_t fps,
                 const unsigned long long *__restrict__ slab_bits, uint8_t *__restrict__ dst,
                 float *__restrict__ dst32, float *__restrict__ scales, double *__restrict__ part) {
  double s64 = 0.0, sst = 0.0;
  for (int64_t f = blockIdx.x; f < nfib; f += gridDim.x) {
    const int64_t gf = fiber0 + f;
    const int64_t slab = gf / fps;
    const int k = f8_scale_exp(__longlong_as_double((long long)slab_bits[slab]));
    const float sc = ldexpf(1.0f, k), inv = ldexpf(1.0f, -k);
    if (threadIdx.x == 0 && gf % fps == 0) scales[slab] = sc;
    const double *s = src + f * I0;
    uint8_t *d = dst + gf * pI0;
    float *d32 = dst32 ? dst32 + gf * pI0 : nullptr;
    for (int64_t i0 = 4 * (int64_t)threadIdx.x; i0 < pI0; i0 += 4 * (int64_t)blockDim.x) {
      uint32_t word = 0;
      float p64 = 0.0f, pst = 0.0f;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t i = i0 + j;
        const double x = i < I0 ? __ldcs(s + i) : 0.0;
        const float xf = (float)x;
        uint32_t code = 0;
        if (i < I0) code = f8_encode_sr(xf * inv, f8_dither((uint64_t)(gf * I0 + i)));
        const float back = f8_decode(code) * sc;
        p64 = fmaf(xf, xf, p64);
        pst = fmaf(back, back, pst);
        word |= code << (8 * j);
        if (d32) d32[i] = xf;
      }
      *reinterpret_cast<uint32_t *>(d + i0) = word;
      s64 += (double)p64;
      sst += (double)pst;
    }
  }
  __shared__ double r64[kF8EncThreads / 32], rst[kF8EncThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s64 += __shfl_down_sync(0xffffffffu, s64, o);
    sst += __shfl_down_sync(0xffffffffu, sst, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r64[threadIdx.x >> 5] = s64;
    rst[threadIdx.x >> 5] = sst;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kF8EncThreads / 32; ++w) {
      a += r64[w];
      b += rst[w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

}  // namespace

int f8_slab_max_launch(const double *src, int64_t I0, int64_t fiber0, int64_t nfib, int64_t fps,
                       unsigned long long *slab_bits, int sm_count, cudaStream_t s) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)sm_count * 8, nfib));
  f8_slab_max_kernel<<<blocks, kF8EncThreads, 0, s>>>(src, I0, fiber0, nfib, fps, slab_bits);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

int f8_encode_launch(const double *src, int64_t I0, int64_t pI0, int64_t fiber0, int64_t nfib, int64_t fps,
                     const unsigned long long *slab_bits, uint8_t *dst, float *dst32, float *scales, double *part,
                     int blocks, cudaStream_t s) {
  f8_encode_kernel<<<blocks, kF8EncThreads, 0, s>>>(src, I0, pI0, fiber0, nfib, fps, slab_bits, dst, dst32,
                                                     scales, part);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

// ------------------------------------------------------------------------------------
// MTTKRP
// ------------------------------------------------------------------------------------
namespace {

using namespace tc;

constexpr int F8_BM = 128;          // q rows per tile (MMA M)
constexpr int F8_BK = 128;          // contraction elements per K-block (one 128-byte row)
constexpr int F8_MAX_STAGES = 6;    // X tile ring (measured faster than 8 to 10)
constexpr int F8_GROUP = 2;         // K-blocks per group, modes n >= 1 (measured: 2 beats 1 and 4)
constexpr int F8_MAX_KSTAGES = 4;   // Khatri-Rao tile ring: two groups
constexpr int F8_THREADS = 320;     // producer, MMA issuer, 8 Khatri-Rao builder warps
constexpr int F8_BUILDERS = 256;
constexpr int F8_ATILE = F8_BM * F8_BK;   // 16 KB
constexpr int F8_WORK_WORDS = 2 * PTG_MAX_ORDER * 128 + 32;   // column maxima + ticket

struct F8Params {
  int64_t P, Q, S;
  int64_t kblocks_total, kblocks_per_split, pblocks;
  int qtiles, mt_per_cta;
  int RP;        // rank padded to a multiple of 16
  int N;         // MMA N = 2 RP: the hi columns, then the lo columns
  int R;
  int mmajor;
  int stages, kstages;
  int group;                 // G: K-blocks per group; the q-tiles are the outer loop of a group
  uint32_t tmem_cols;
  uint32_t spin;             // poll limit of every bounded wait
  int vec4;                  // factor rows are read as float4 (R % 4 == 0, 16-byte aligned)
  KrDevTc before, after;
  const float *slab_scale;   // scale of each index of the last mode
  int64_t slab_div;          // slab = lin / slab_div, lin = s (slab_in_q == 0) or q
  int slab_in_q;
  const float *col_scale;    // c_r, [R]
  float *partial;            // [nsplit][Q][RP]
  int *err;
  const int *skip;
};

// c_r = 2^k with (prod_f max_i |A_f(i, r)|) * smax * c_r in (128, 256]: the largest
// scaled Khatri-Rao value then rounds to at most 256 < 448.  Column maxima are gathered
// with integer atomics on the float bits (non-negative floats order like unsigned ints);
// the last block to finish turns them into c_r and zeroes the work words for the next
// launch.
__global__ void f8_colscale_kernel(KrDevTc before, KrDevTc after, int R, float smax, unsigned *work,
                                   float *col_scale, const int *skip) {
  if (skip && *skip) return;
  __shared__ unsigned cm[2 * PTG_MAX_ORDER][128];
  __shared__ bool last;
  const int nf = before.n + after.n;
  for (int i = threadIdx.x; i < nf * 128; i += blockDim.x) cm[i / 128][i % 128] = 0u;
  __syncthreads();
  for (int f = 0; f < nf; ++f) {
    const KrDevTc &sd = f < before.n ? before : after;
    const int fi = f < before.n ? f : f - before.n;
    const float *A = sd.fac[fi];
    const int64_t n = (int64_t)sd.valid[fi] * R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      atomicMax(&cm[f][i % R], __float_as_uint(fabsf(__ldg(A + i))));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nf * R; i += blockDim.x) atomicMax(&work[(i / R) * 128 + i % R], cm[i / R][i % R]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&work[2 * PTG_MAX_ORDER * 128], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    double m = smax;
    for (int f = 0; f < nf; ++f) m *= (double)__uint_as_float(atomicOr(&work[f * 128 + r], 0u));
    int k = 0;
    if (m > 0.0 && isfinite(m)) {
      int E;
      const double fr = frexp(m, &E);
      k = (fr == 0.5) ? 9 - E : 8 - E;
      k = max(-120, min(120, k));
    }
    col_scale[r] = ldexpf(1.0f, k);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nf * 128; i += blockDim.x) work[i] = 0u;
  if (threadIdx.x == 0) work[2 * PTG_MAX_ORDER * 128] = 0u;
}

__device__ __forceinline__ uint32_t f8_kr_off(int n, int k) {
  return (uint32_t)((n >> 3) * 1024 + (n & 7) * 128 + ((((k >> 4) ^ (n & 7)) & 7) << 4) + (k & 15));
}

__global__ void __launch_bounds__(F8_THREADS, 1)
mttkrp_f8_kernel(const __grid_constant__ CUtensorMap tmap, const F8Params prm) {
  if (prm.skip && *prm.skip) return;   // before any barrier or TMEM allocation
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int N = prm.N, RP = prm.RP;
  const int STAGES = prm.stages, KSTAGES = prm.kstages, G = prm.group;
  const int KTILE = N * 128;   // N rows of 128 bytes
  uint8_t *aring = base;
  uint8_t *kring = aring + STAGES * F8_ATILE;
  uint64_t *bars = (uint64_t *)(kring + KSTAGES * KTILE);
  uint64_t *full_a = bars, *empty_a = bars + F8_MAX_STAGES;
  uint64_t *full_k = empty_a + F8_MAX_STAGES, *empty_k = full_k + F8_MAX_KSTAGES;
  uint64_t *done = empty_k + F8_MAX_KSTAGES;
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  float *cs = (float *)(tmem_slot + 4);   // c_r, then 1 / c_r (2 x 128 floats)

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qgroup = blockIdx.x, split = blockIdx.y;
  const int qt0 = qgroup * prm.mt_per_cta;
  const int nqt = min(prm.mt_per_cta, prm.qtiles - qt0);
  const int64_t kb0 = (int64_t)split * prm.kblocks_per_split;
  const int64_t kb1 = min(prm.kblocks_total, kb0 + prm.kblocks_per_split);
  const int nkb = kb1 > kb0 ? (int)(kb1 - kb0) : 0;
  const uint32_t spin = prm.spin;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full_a[i], 1);
      mbar_init(&empty_a[i], 1);
    }
    for (int i = 0; i < KSTAGES; ++i) {
      mbar_init(&full_k[i], F8_BUILDERS);
      mbar_init(&empty_k[i], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = threadIdx.x; i < 128; i += blockDim.x) {
    const float c = i < prm.R ? __ldg(prm.col_scale + i) : 1.0f;
    cs[i] = c;
    cs[128 + i] = 1.0f / c;   // exact: c is a power of two
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(prm.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  // idesc: D=F32 (bit 4), A=E4M3 (bits 7-9 = 0), B=E4M3 (bits 10-12 = 0), A major (bit 15),
  // N>>3 (17-22), M>>4 (24-28)
  const uint32_t idesc =
      (1u << 4) | ((uint32_t)prm.mmajor << 15) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(F8_BM >> 4) << 24);

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0 && nkb > 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued[F8_MAX_STAGES] = {0};   // loads issued into each stage
      bool ok = true;
      // K-block t covers s in [t BK, t BK + BK) (mode 0), else slab t / pblocks, p from
      // (t % pblocks) BK; the coordinates step along a group without dividing
      const int pend = (int)(prm.pblocks * F8_BK);
      if (G == 1) {   // one K-block at a time (this loop form issues fastest; see the issuer)
        for (int kb = 0; kb < nkb && ok; ++kb) {
          const int64_t t = kb0 + kb;
          for (int m = 0; m < nqt; ++m) {
            if (!mbar_wait_lim(&empty_a[stage], phase ^ 1, abort_flag, spin)) {
              ok = false;
              break;
            }
            mbar_expect_tx(&full_a[stage], F8_ATILE);
            uint8_t *dst = aring + stage * F8_ATILE;
            const int q = (qt0 + m) * F8_BM;
            if (prm.mmajor) {
              tma_load_2d(dst, &tmap, &full_a[stage], q, (int)(t * F8_BK));
            } else {
              const int s = (int)(t / prm.pblocks);
              const int p0 = (int)((t % prm.pblocks) * F8_BK);
              tma_load_3d(dst, &tmap, &full_a[stage], p0, q, s);
            }
            ++issued[stage];
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      for (int g0 = 0; G > 1 && g0 < nkb && ok; g0 += G) {
        const int gn = min(G, nkb - g0);
        const int64_t tg = kb0 + g0;
        int sg, pg = 0;
        if (prm.mmajor) {
          sg = (int)(tg * F8_BK);
        } else {
          sg = (int)(tg / prm.pblocks);
          pg = (int)((tg - (int64_t)sg * prm.pblocks) * F8_BK);
        }
        for (int m = 0; m < nqt && ok; ++m) {
          const int q = (qt0 + m) * F8_BM;
          int s = sg, p = pg;
          for (int j = 0; j < gn; ++j) {
            if (!mbar_wait_lim(&empty_a[stage], phase ^ 1, abort_flag, spin)) {
              ok = false;
              break;
            }
            mbar_expect_tx(&full_a[stage], F8_ATILE);
            uint8_t *dst = aring + stage * F8_ATILE;
            if (prm.mmajor) {
              tma_load_2d(dst, &tmap, &full_a[stage], q, s);
              s += F8_BK;
            } else {
              tma_load_3d(dst, &tmap, &full_a[stage], p, q, s);
              p += F8_BK;
              if (p == pend) {
                p = 0;
                ++s;
              }
            }
            ++issued[stage];
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      if (!ok) {
        *abort_flag = 1;
        atomicExch(prm.err, PTG_ERR_TIMEOUT);
        // a stage holds at most one load in flight (the next one waits for its release),
        // the last one issued into it: wait for it so no copy lands after the CTA exits
        for (int s = 0; s < STAGES; ++s)
          if (issued[s] > 0) mbar_wait_bounded(&full_a[s], (uint32_t)((issued[s] - 1) & 1));
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0, kst = 0;
      uint32_t phase = 0, kphase = 0;
      bool ok = true;
      // descriptors: a constant high word and the start address >> 4, stepped per K = 32 codes
      // (32 bytes along a K-major row, or 32 rows of 128 bytes of the MN-major tile: 4 groups
      // of 8 rows, 1024 bytes apart)
      const uint64_t a_hi = prm.mmajor ? smem_desc_sw128_hi(8192, 1024) : smem_desc_sw128_hi(16, 1024);
      const uint64_t b_hi = smem_desc_sw128_hi(16, 1024);
      const uint32_t a_step = prm.mmajor ? (4096u >> 4) : (32u >> 4);
      const uint32_t a_lo0 = smem_u32(aring) >> 4, k_lo0 = smem_u32(kring) >> 4;
      if (G == 1) {
        // one K-block at a time, descriptors built next to each MMA: measured faster than the
        // group loop below with G = 1 (the issuing thread is the busiest role of the kernel)
        for (int kb = 0; kb < nkb && ok; ++kb) {
          if (!mbar_wait_lim(&full_k[kst], kphase, abort_flag, spin)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t kaddr = smem_u32(kring + kst * KTILE);
          for (int m = 0; m < nqt; ++m) {
            if (!mbar_wait_lim(&full_a[stage], phase, abort_flag, spin)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t aaddr = smem_u32(aring + stage * F8_ATILE);
#pragma unroll
            for (int kk = 0; kk < F8_BK / 32; ++kk) {
              const uint64_t ad = prm.mmajor ? smem_desc_sw128(aaddr + kk * 4096, 8192, 1024)
                                             : smem_desc_sw128(aaddr + kk * 32, 16, 1024);
              const uint64_t bd = smem_desc_sw128(kaddr + kk * 32, 16, 1024);
              umma_f8(tmem_base + (uint32_t)(m * N), ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            }
            umma_commit(&empty_a[stage]);
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          umma_commit(&empty_k[kst]);
          if (++kst == KSTAGES) {
            kst = 0;
            kphase ^= 1;
          }
        }
      }
      // a group's Khatri-Rao tiles sit in ring slots kst .. kst + gn - 1: the ring holds a
      // whole number of groups, so a group never wraps around its end
      for (int g0 = 0; G > 1 && g0 < nkb && ok; g0 += G) {
        const int gn = min(G, nkb - g0);
        for (int j = 0; j < gn && ok; ++j) ok = mbar_wait_lim(&full_k[kst + j], kphase, abort_flag, spin);
        if (!ok) break;
        tc_fence_after();
        for (int m = 0; m < nqt && ok; ++m) {
          const uint32_t d_tmem = tmem_base + (uint32_t)(m * N);
          for (int j = 0; j < gn; ++j) {
            if (!mbar_wait_lim(&full_a[stage], phase, abort_flag, spin)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t ad = a_hi | (uint64_t)(a_lo0 + (uint32_t)stage * (F8_ATILE >> 4));
            const uint64_t bd = b_hi | (uint64_t)(k_lo0 + (uint32_t)(kst + j) * (uint32_t)(KTILE >> 4));
            umma_f8(d_tmem, ad, bd, idesc, (g0 | j) != 0 ? 1u : 0u);
#pragma unroll
            for (int kk = 1; kk < F8_BK / 32; ++kk)
              umma_f8(d_tmem, ad + kk * a_step, bd + kk * (32u >> 4), idesc, 1u);
            umma_commit(&empty_a[stage]);
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
        if (!ok) break;
        for (int j = 0; j < gn; ++j) umma_commit(&empty_k[kst + j]);
        kst += G;
        if (kst == KSTAGES) {
          kst = 0;
          kphase ^= 1;
        }
      }
      if (!ok) {
        *abort_flag = 1;
        atomicExch(prm.err, PTG_ERR_TIMEOUT);
      }
      umma_commit(done);   // arrives once every MMA issued above has completed
      // TMEM is released after the final barrier: the MMAs must have finished by then
      mbar_wait_bounded(done, 0);
    }
  } else {
    // ---------------- Khatri-Rao builders (256 threads: each K row by two threads) ----------------
    const int k = (threadIdx.x - 64) & (F8_BK - 1);
    const int part = (threadIdx.x - 64) >> 7;   // 16-column chunks part, part + 2, ...
    const bool drains = warp < 6;               // warps 2..5 cover the four TMEM lane quarters
    int kst = 0;
    uint32_t kphase = 0;
    // slab and p-block of K-block kb0 + kb (modes n >= 1), stepped without dividing
    int64_t sl = kb0 / prm.pblocks;
    int pb = (int)(kb0 - sl * prm.pblocks);
    for (int kb = 0; kb < nkb; ++kb) {
      if (!mbar_wait_lim(&empty_k[kst], kphase ^ 1, abort_flag, spin)) {
        *abort_flag = 1;
        atomicExch(prm.err, PTG_ERR_TIMEOUT);
        break;
      }
      const int64_t t = kb0 + kb;
      uint8_t *kt = kring + kst * KTILE;
      bool valid;
      uint32_t lin_b = 0, lin_a;
      if (prm.mmajor) {
        const int64_t s = t * F8_BK + k;
        valid = s < prm.S;
        lin_a = (uint32_t)s;
      } else {
        const int64_t p = (int64_t)pb * F8_BK + k;
        valid = p < prm.P;
        lin_a = (uint32_t)sl;
        lin_b = (uint32_t)p;
      }
      const float row_sc = (valid && !prm.slab_in_q) ? __ldg(prm.slab_scale + (int64_t)lin_a / prm.slab_div) : 1.0f;
      for (int c = 16 * part; c < RP; c += 32) {
        float v[16];
        if (valid) {
          kr_pair<16>(prm.after, lin_a, prm.before, lin_b, !prm.mmajor, prm.R, c, prm.vec4 != 0, v);
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const float a0 = v[j] * row_sc * cs[c + j], a1 = v[j + 1] * row_sc * cs[c + j + 1];
          const uint32_t hi = e4m3x2_rn(a0, a1);
          const float2 hb = e4m3x2_to_f32(hi);
          // a - hi is exact (hi is a's nearest e4m3 neighbour); x16 keeps lo off the subnormals
          const uint32_t lo = e4m3x2_rn((a0 - hb.x) * 16.0f, (a1 - hb.y) * 16.0f);
          kt[f8_kr_off(c + j, k)] = (uint8_t)(hi & 0xFF);
          kt[f8_kr_off(c + j + 1, k)] = (uint8_t)(hi >> 8);
          kt[f8_kr_off(RP + c + j, k)] = (uint8_t)(lo & 0xFF);
          kt[f8_kr_off(RP + c + j + 1, k)] = (uint8_t)(lo >> 8);
        }
      }
      fence_async_smem();
      mbar_arrive(&full_k[kst]);
      if (++pb == prm.pblocks) {
        pb = 0;
        ++sl;
      }
      if (++kst == KSTAGES) {
        kst = 0;
        kphase ^= 1;
      }
    }
    // ---------------- epilogue: TMEM -> partials ----------------
    const bool have = drains && (nkb > 0) && mbar_wait_lim(done, 0, abort_flag, spin) && !*abort_flag;
    tc_fence_after();
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    for (int m = 0; drains && m < nqt; ++m) {
      const int64_t q = (int64_t)(qt0 + m) * F8_BM + row;
      float *dst = prm.partial + ((int64_t)split * prm.Q + q) * RP;
      const float qsc = (prm.slab_in_q && q < prm.Q) ? __ldg(prm.slab_scale + q / prm.slab_div) : 1.0f;
      for (int c0 = 0; c0 < RP; c0 += 16) {
        float vh[16], vl[16];
        if (have) {
          const uint32_t ta = tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(m * N + c0);
          tmem_ld16(ta, vh);
          tmem_ld16(ta + (uint32_t)RP, vl);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) vh[i] = vl[i] = 0.0f;
        }
        if (q < prm.Q) {
          float o[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) o[i] = fmaf(vl[i], 0.0625f, vh[i]) * cs[128 + c0 + i] * qsc;
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4 *>(dst + c0 + i) = make_float4(o[i], o[i + 1], o[i + 2], o[i + 3]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(prm.tmem_cols)
                 : "memory");
  }
}

__global__ void f8_reduce_kernel(const float *__restrict__ partial, int nsplit, int64_t Q, int RP, int64_t q_write,
                                 int R, float *__restrict__ out, const int *skip) {
  if (skip && *skip) return;
  const int64_t n = q_write * R;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = idx / R;
    const int c = (int)(idx % R);
    out[idx] = sum_splits(partial + q * RP + c, Q * RP, nsplit);
  }
}

size_t f8_smem_bytes(int N, int stages, int kstages) {
  return 1024 /*alignment slack*/ + (size_t)stages * F8_ATILE + (size_t)kstages * N * 128 +
         sizeof(uint64_t) * (2 * F8_MAX_STAGES + 2 * F8_MAX_KSTAGES + 1) + 16 + 2 * 128 * sizeof(float);
}

}  // namespace

int f8_contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                          cudaStream_t stream) {
  if (t->dtype != PTG_FP8E4M3) return set_error(PTG_ERR_INVALID, "internal: the FP8 path needs FP8 storage");
  if (R > 128) return set_error(PTG_ERR_UNSUPPORTED, "FP8 MTTKRP: rank > 128");
  if (!t->f8_scales) return set_error(PTG_ERR_INVALID, "internal: FP8 tensor without slab scales");
  EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(PTG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const bool mmajor = (c.P == 1);
  if (mmajor && (c.Q % 16) != 0) return set_error(PTG_ERR_INVALID, "internal: Q must be a multiple of 16");
  if (!mmajor && (c.P % 16) != 0) return set_error(PTG_ERR_INVALID, "internal: P must be a multiple of 16");
  if (c.Q > 0x7fffffffLL || c.S > 0x7fffffffLL || c.P > 0x7fffffffLL)
    return set_error(PTG_ERR_UNSUPPORTED, "FP8 MTTKRP: extent exceeds 2^31");
  if (c.slab_div < 1) return set_error(PTG_ERR_INVALID, "internal: contraction without slab layout");
  if (!ctx->f8_work) {   // zero once; every launch of the column-scale kernel leaves it zero
    const size_t wb = F8_WORK_WORDS * sizeof(unsigned) + 128 * sizeof(float);
    PTG_TRY(ctx_malloc(ctx, &ctx->f8_work, wb, "FP8 work words"));
    PTG_CUDA(cudaMemsetAsync(ctx->f8_work, 0, wb, stream));
  }
  unsigned *work = (unsigned *)ctx->f8_work;
  float *col_scale = (float *)(work + F8_WORK_WORDS);

  F8Params prm{};
  prm.P = c.P;
  prm.Q = c.Q;
  prm.S = c.S;
  prm.RP = (R + 15) / 16 * 16;
  prm.N = 2 * prm.RP;
  prm.R = R;
  prm.mmajor = mmajor ? 1 : 0;
  prm.spin = spin_limit(ctx);
  auto cp = [](const KrSide &s) {
    KrDevTc d{};
    d.n = s.n;
    for (int i = 0; i < s.n; ++i) {
      d.ext[i] = (uint32_t)s.ext[i];
      d.valid[i] = (uint32_t)s.valid[i];
      d.fac[i] = s.fac[i];
    }
    return d;
  };
  prm.before = cp(c.before);
  prm.after = cp(c.after);
  prm.vec4 = kr_vec4_ok(c, R) ? 1 : 0;
  prm.slab_scale = t->f8_scales;
  prm.slab_div = c.slab_div;
  prm.slab_in_q = c.slab_in_q ? 1 : 0;
  prm.col_scale = col_scale;
  prm.qtiles = (int)((c.Q + F8_BM - 1) / F8_BM);
  int mt = std::max(1, 512 / prm.N);
  mt = std::min(mt, prm.qtiles);
  const int qgroups_min = (prm.qtiles + mt - 1) / mt;
  mt = (prm.qtiles + qgroups_min - 1) / qgroups_min;
  prm.mt_per_cta = mt;
  const int qgroups = (prm.qtiles + mt - 1) / mt;
  uint32_t cols = 32;
  while (cols < (uint32_t)(mt * prm.N)) cols <<= 1;
  prm.tmem_cols = cols;
  if (mmajor) {
    prm.pblocks = 1;
    prm.kblocks_total = (c.S + F8_BK - 1) / F8_BK;
  } else {
    prm.pblocks = (c.P + F8_BK - 1) / F8_BK;
    prm.kblocks_total = c.S * prm.pblocks;
  }
  int64_t nsplit = std::max<int64_t>(1, ctx->sm_count / qgroups);
  nsplit = std::min<int64_t>(nsplit, prm.kblocks_total);
  prm.kblocks_per_split = (prm.kblocks_total + nsplit - 1) / nsplit;
  nsplit = (prm.kblocks_total + prm.kblocks_per_split - 1) / prm.kblocks_per_split;
  // The rings take at most the shared memory that leaves room on the SM for the eigenvalue-
  // bound kernel beside it: an X ring of up to 6 stages and a Khatri-Rao ring of two groups
  // (a mode-0 K-block is one contiguous run of X: G = 1 there)
  const size_t budget = ctx->smem_beside_eigen;
  const int G = mmajor ? 1 : F8_GROUP;
  prm.group = G;
  prm.kstages = F8_MAX_KSTAGES;
  prm.stages = F8_MAX_STAGES;
  while (f8_smem_bytes(prm.N, prm.stages, prm.kstages) > budget && prm.stages > 3) --prm.stages;
  while (f8_smem_bytes(prm.N, prm.stages, prm.kstages) > ctx->smem_optin && prm.kstages > 2 && G == 1)
    --prm.kstages;
  const size_t smem = f8_smem_bytes(prm.N, prm.stages, prm.kstages);
  if (smem > ctx->smem_optin) return set_error(PTG_ERR_UNSUPPORTED, "FP8 MTTKRP: shared memory");

  CUtensorMap map;
  CUresult r;
  if (mmajor) {
    cuuint64_t gdim[2] = {(cuuint64_t)c.Q, (cuuint64_t)c.S};
    cuuint64_t gstride[1] = {(cuuint64_t)c.Q};
    cuuint32_t box[2] = {128, 128};
    cuuint32_t es[2] = {1, 1};
    r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, t->data, gdim, gstride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {
    cuuint64_t gdim[3] = {(cuuint64_t)c.P, (cuuint64_t)c.Q, (cuuint64_t)c.S};
    cuuint64_t gstride[2] = {(cuuint64_t)c.P, (cuuint64_t)c.P * c.Q};
    cuuint32_t box[3] = {128, 128, 1};
    cuuint32_t es[3] = {1, 1, 1};
    r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, t->data, gdim, gstride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  if (r != CUDA_SUCCESS) {
    char buf[128];
    snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return set_error(PTG_ERR_CUDA, buf);
  }
  const size_t part_bytes = (size_t)nsplit * c.Q * prm.RP * sizeof(float);
  PTG_TRY(ctx->scratch.ensure(part_bytes));
  prm.partial = reinterpret_cast<float *>(ctx->scratch.ptr);
  prm.err = ctx->dev_err;
  prm.skip = c.skip;

  const float smax = c.slab_in_q ? 1.0f : t->f8_scale_max;
  f8_colscale_kernel<<<32, 256, 0, stream>>>(prm.before, prm.after, R, smax, work, col_scale, c.skip);
  PTG_CUDA(cudaGetLastError());
  PTG_CUDA(cudaFuncSetAttribute(mttkrp_f8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PTG_CUDA(cudaFuncSetAttribute(mttkrp_f8_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared));
  dim3 grid((unsigned)qgroups, (unsigned)nsplit);
  mttkrp_f8_kernel<<<grid, F8_THREADS, smem, stream>>>(map, prm);
  PTG_CUDA(cudaGetLastError());
  const int64_t n = c.q_write * R;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
  f8_reduce_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(prm.partial, (int)nsplit, c.Q, prm.RP, c.q_write, R,
                                                            out, c.skip);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 3);
  return PTG_OK;
}

}  // namespace ptg
