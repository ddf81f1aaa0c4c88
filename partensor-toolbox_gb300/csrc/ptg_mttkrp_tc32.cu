// FP32-accurate dense MTTKRP on the tensor cores: tcgen05.mma kind::tf32 with a three-term
// split (Markidis et al. 2018, "NVIDIA tensor core programmability, performance & precision";
// the 3xTF32 scheme).  Every FP32 operand x is split into hi = x rounded to TF32 (10 mantissa
// bits) and lo = x - hi (exact in FP32); the product is accumulated as
//   hi_X hi_K + hi_X lo_K + lo_X hi_K
// in FP32 in TMEM (the dropped lo_X lo_K is below 2^-22 of |x k|, and lo itself enters as
// TF32, an error below 2^-22 of |x|), so the result carries FP32-level accuracy while the
// tensor is read once, in FP32.
//
// Same contraction as ptg_mttkrp.cu: the FP32 tensor viewed as [P, Q, S],
// out[q, r] = sum_{p,s} X[p,q,s] KRb[p,r] KRa[s,r].  One CTA per (q-group, K-split), 10 warps:
//   warp 0      TMA producer: 128 x 32 FP32 tiles of X (K-major, 128-byte swizzle, for
//               modes n >= 1; four 32 x 32 MN-major boxes for mode 0) into an 8-stage ring;
//   warps 6..9  split each staged tile into hi and lo K-major tiles (2-stage ring),
//               transposing mode-0 tiles on the way, and free the staging slot;
//   warp 1      TMEM allocation and the MMA issuer (one lane): per K-step of 8,
//               D[:, 0:2N] += A_hi [K_hi; K_lo]^T and D[:, 0:N] += A_lo K_hi^T
//               (M=128, N = R padded to 16), so A_hi is read once;
//   warps 2..5  Khatri-Rao tiles ([hi rows; lo rows], swizzled K-major) and the drains of
//               columns [0, N/2); warps 6..9 drain [N/2, N).
// The tensor cores' FP32 accumulation in TMEM is not round-to-nearest: it drifts low by about
// 2^-25 of the running sum per accumulate step, so a long chain carries a bias.  Every
// accumulator chain therefore spans T3_CHAIN K-blocks (16 accumulate steps); the builders drain
// it (the two column halves summed) into FP32 registers with round-to-nearest adds while the
// MMA fills the other of two TMEM accumulators, and write the register sums as split-K
// partials.  The builders and the splitters each keep half of the columns, so a CTA takes
// 128/N q-tiles (between 2 and 8) with 64 sums per thread.
// Every mbarrier wait is bounded: on timeout the kernel raises an error word, and returns
// after its MMAs completed and its TMEM was released.
#include <algorithm>
#include <cstdio>

#include "ptg_internal.h"
#include "ptg_tcgen05.h"

namespace ptg {
namespace {

using namespace tc;

constexpr int T3_BM = 128;                     // q rows per tile (MMA M)
constexpr int T3_BK = 32;                      // contraction elements per K-block (128-byte rows)
constexpr int T3_SSTAGES = 2;                  // split ring: hi and lo K-major tiles
constexpr int T3_KSTAGES = 2;                  // Khatri-Rao ring: [hi rows; lo rows]
constexpr int T3_TILE = T3_BM * T3_BK * 4;     // 16 KB
constexpr int T3_THREADS = 320;
constexpr uint32_t kTf32HiMask = 0xFFFFE000u;
// K-blocks per TMEM accumulator chain before it is drained into FP32 registers
constexpr int T3_CHAIN = 2;
// q-tiles per CTA: the drained sums (MT x N/2 floats per thread) stay in registers, and the
// two accumulators (2 x MT x 2N columns) fit the 512 columns of TMEM
template <int N>
struct T3Shape {
  static constexpr int MT = 128 / N > 8 ? 8 : 128 / N;
  static constexpr int HALF = N / 2;
  // staging stages: as many as leave room on the SM for the eigenvalue-bound kernel launched
  // beside this one (its 39 KB of shared memory; 228 KB per SM)
  static constexpr int XST = N <= 16 ? 7 : N <= 48 ? 6 : 5;
};

// Chain c's accumulator, columns [col0, col0 + HALF) of both halves, added into the sums of
// this thread's row (TMEM lanes 32 * quarter + lane); then the accumulator is released.
template <int N>
__device__ __forceinline__ bool t3_drain(float (&sum)[T3Shape<N>::MT][T3Shape<N>::HALF], int c, int nqt,
                                         uint32_t tmem_base, int quarter, int col0, uint64_t *acc_full,
                                         uint64_t *acc_empty, volatile int *abort_flag) {
  constexpr int MT = T3Shape<N>::MT, HALF = T3Shape<N>::HALF;
  const int buf = c & 1;
  if (!mbar_wait(&acc_full[buf], (c >> 1) & 1, abort_flag)) return false;
  tc_fence_after();
#pragma unroll
  for (int m = 0; m < MT; ++m) {
    if (m < nqt) {
#pragma unroll
      for (int c0 = 0; c0 < HALF; c0 += 8) {
        float v[8], w[8];
        const uint32_t ta =
            tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((buf * MT + m) * 2 * N + col0 + c0);
        tmem_ld8(ta, v);
        tmem_ld8(ta + (uint32_t)N, w);
#pragma unroll
        for (int i = 0; i < 8; ++i) sum[m][c0 + i] += v[i] + w[i];
      }
    }
  }
  tc_fence_before();
  mbar_arrive(&acc_empty[buf]);
  return true;
}

struct T3Params {
  int64_t P, Q, S;
  int64_t kblocks_total, kblocks_per_split, pblocks;
  int qtiles, mt_per_cta;
  int N;          // rank padded to a multiple of 16 (TMEM holds 2N columns per q-tile)
  int R;
  int mmajor;
  uint32_t tmem_cols;
  KrDevTc before, after;
  float *partial;  // [nsplit][Q][N]
  int *err;
  const int *skip;  // nonzero: return at once (Contraction::skip)
};

// x rounded to the nearest TF32 value (ties away from zero): exact in TF32, and lo = x - hi is
// exact in FP32 with |lo| <= 2^-11 |x| and no sign bias
__device__ __forceinline__ float tf32_hi(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & kTf32HiMask);
}

// Appends the factor rows whose mixed-radix digits make up `lin` (one side of a Khatri-Rao
// row); false when a digit falls in a padding slot (the row is zero).
__device__ __forceinline__ bool kr_rows(const KrDevTc &s, uint32_t lin, int R, const float **rows, int &n) {
  for (int f = 0; f < s.n; ++f) {
    const uint32_t e = s.ext[f];
    const uint32_t d = lin % e;
    lin /= e;
    if (d >= s.valid[f]) return false;
    rows[n++] = s.fac[f] + (size_t)d * R;
  }
  return true;
}

// byte offset of element (row, k) in a 128-byte-swizzled K-major FP32 tile (8-row atoms)
__device__ __forceinline__ uint32_t sw128_off(int row, int k) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 2) ^ (row & 7)) & 7) << 4) + (k & 3) * 4);
}

__device__ __forceinline__ void fail_timeout(volatile int *abort_flag, int *err) {
  *abort_flag = 1;
  atomicExch(err, PTG_ERR_TIMEOUT);
}

// At most 160 registers a thread: 320 x 160 leaves 14,336 of the SM's 65,536 for the
// eigenvalue-bound kernel's 256 threads beside it.
template <int N>
__global__ void __maxnreg__(160)
mttkrp_tc32_kernel(const __grid_constant__ CUtensorMap tmap, const T3Params prm) {
  constexpr int MT = T3Shape<N>::MT;
  constexpr int T3_XSTAGES = T3Shape<N>::XST;
  if (prm.skip && *prm.skip) return;   // before any barrier or TMEM allocation
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int KTILE = 2 * N * 128;                       // [hi rows 0..N-1; lo rows N..2N-1]
  uint8_t *xring = base;                                   // [T3_XSTAGES] staging tiles
  uint8_t *sring = xring + T3_XSTAGES * T3_TILE;           // [2]{hi, lo}
  uint8_t *kring = sring + T3_SSTAGES * 2 * T3_TILE;       // [2] Khatri-Rao tiles
  uint64_t *bars = (uint64_t *)(kring + T3_KSTAGES * KTILE);
  uint64_t *full_x = bars, *free_x = bars + T3_XSTAGES;
  uint64_t *full_s = bars + 2 * T3_XSTAGES, *empty_s = full_s + T3_SSTAGES;
  uint64_t *full_k = empty_s + T3_SSTAGES, *empty_k = full_k + T3_KSTAGES;
  uint64_t *acc_full = empty_k + T3_KSTAGES, *acc_empty = acc_full + 2;   // per accumulator
  uint64_t *done = acc_empty + 2;
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qgroup = blockIdx.x, split = blockIdx.y;
  const int qt0 = qgroup * prm.mt_per_cta;
  const int nqt = min(prm.mt_per_cta, prm.qtiles - qt0);
  const int64_t kb0 = (int64_t)split * prm.kblocks_per_split;
  const int64_t kb1 = min(prm.kblocks_total, kb0 + prm.kblocks_per_split);
  const int nkb = kb1 > kb0 ? (int)(kb1 - kb0) : 0;

  if (threadIdx.x == 0) {
    for (int i = 0; i < T3_XSTAGES; ++i) {
      mbar_init(&full_x[i], 1);
      mbar_init(&free_x[i], 128);
    }
    for (int i = 0; i < T3_SSTAGES; ++i) {
      mbar_init(&full_s[i], 128);
      mbar_init(&empty_s[i], 1);
    }
    for (int i = 0; i < T3_KSTAGES; ++i) {
      mbar_init(&full_k[i], 128);
      mbar_init(&empty_k[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&acc_full[i], 1);
      mbar_init(&acc_empty[i], 256);   // the builders and the splitters
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
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

  uint32_t issued[T3_XSTAGES] = {};   // TMA loads per stage (producer lane)
  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0 && nkb > 0) {
      int xs = 0;
      uint32_t xph = 0;
      for (int kb = 0; kb < nkb; ++kb) {
        const int64_t t = kb0 + kb;
        for (int m = 0; m < nqt; ++m) {
          if (!mbar_wait(&free_x[xs], xph ^ 1, abort_flag)) {
            fail_timeout(abort_flag, prm.err);
            goto producer_done;
          }
          mbar_expect_tx(&full_x[xs], T3_TILE);
          uint8_t *dst = xring + xs * T3_TILE;
          const int q = (qt0 + m) * T3_BM;
          if (prm.mmajor) {
            const int s0 = (int)(t * T3_BK);
#pragma unroll
            for (int j = 0; j < 4; ++j) tma_load_2d(dst + j * (T3_TILE / 4), &tmap, &full_x[xs], q + 32 * j, s0);
          } else {
            const int s = (int)(t / prm.pblocks);
            const int p0 = (int)((t % prm.pblocks) * T3_BK);
            tma_load_3d(dst, &tmap, &full_x[xs], p0, q, s);
          }
          ++issued[xs];
          if (++xs == T3_XSTAGES) {
            xs = 0;
            xph ^= 1;
          }
        }
      }
    producer_done:;
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    // per K-step of 8: D[:, 0:2N] += A_hi [K_hi; K_lo]^T, then D[:, 0:N] += A_lo K_hi^T; chain c
    // (K-blocks c*T3_CHAIN ..) accumulates into accumulator c & 1, which its drain must have
    // emptied (chain c - 2)
    if (lane == 0) {
      const uint32_t idesc2 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)((2 * N) >> 3) << 17) |
                              ((uint32_t)(T3_BM >> 4) << 24);
      const uint32_t idesc1 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
                              ((uint32_t)(T3_BM >> 4) << 24);
      int ss = 0, ks = 0;
      uint32_t sph = 0, kph = 0;
      bool ok = true;
      for (int kb = 0; kb < nkb && ok; ++kb) {
        const int c = kb / T3_CHAIN, cs = kb - c * T3_CHAIN, buf = c & 1;
        if (cs == 0 && c >= 2) {
          if (!mbar_wait(&acc_empty[buf], ((c >> 1) - 1) & 1, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
        }
        if (!mbar_wait(&full_k[ks], kph, abort_flag)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t kt = smem_u32(kring + ks * KTILE);
        for (int m = 0; m < nqt; ++m) {
          if (!mbar_wait(&full_s[ss], sph, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t ahi = smem_u32(sring + ss * 2 * T3_TILE), alo = ahi + (uint32_t)T3_TILE;
          const uint32_t d = tmem_base + (uint32_t)((buf * MT + m) * 2 * N);
#pragma unroll
          for (int kk = 0; kk < T3_BK / 8; ++kk) {
            const uint64_t adh = smem_desc_sw128(ahi + kk * 32, 16, 1024);
            const uint64_t adl = smem_desc_sw128(alo + kk * 32, 16, 1024);
            const uint64_t bd = smem_desc_sw128(kt + kk * 32, 16, 1024);   // 2N rows: hi then lo
            umma_tf32(d, adh, bd, idesc2, (cs > 0 || kk > 0) ? 1u : 0u);
            umma_tf32(d, adl, bd, idesc1, 1u);                              // first N rows: hi
          }
          umma_commit(&empty_s[ss]);
          if (++ss == T3_SSTAGES) {
            ss = 0;
            sph ^= 1;
          }
        }
        if (!ok) break;
        umma_commit(&empty_k[ks]);
        if (++ks == T3_KSTAGES) {
          ks = 0;
          kph ^= 1;
        }
        if (cs == T3_CHAIN - 1 || kb == nkb - 1) umma_commit(&acc_full[buf]);   // the chain is complete
      }
      if (!ok) fail_timeout(abort_flag, prm.err);
      umma_commit(done);   // arrives once every MMA issued above has completed
    }
  } else if (warp < 6) {
    // ---------------- Khatri-Rao builders and drains (128 threads) ----------------
    const int tb = threadIdx.x - 64;
    const int k = tb & 31, ng = tb >> 5;
    constexpr int cpg = N / 4;   // columns per group (>= 4)
    const int quarter = warp & 3;   // the TMEM lanes this warp may read: 32 * quarter ..
    constexpr int HALF = T3Shape<N>::HALF;
    float sum[MT][HALF];   // columns [0, HALF) of this thread's row
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int i = 0; i < HALF; ++i) sum[m][i] = 0.0f;
    bool alive = true;
    auto drain = [&](int c) {
      if (alive && !t3_drain<N>(sum, c, nqt, tmem_base, quarter, 0, acc_full, acc_empty, abort_flag)) {
        fail_timeout(abort_flag, prm.err);
        alive = false;
      }
    };
    int ks = 0;
    uint32_t kph = 0;
    for (int kb = 0; kb < nkb; ++kb) {
      if (!mbar_wait(&empty_k[ks], kph ^ 1, abort_flag)) {
        fail_timeout(abort_flag, prm.err);
        alive = false;
        break;
      }
      const int64_t t = kb0 + kb;
      uint8_t *kt = kring + ks * KTILE;
      // the factor rows of this thread's Khatri-Rao row, decoded once per K-block
      const float *rows[2 * PTG_MAX_ORDER];
      int nrows = 0;
      bool valid;
      if (prm.mmajor) {
        const int64_t s = t * T3_BK + k;
        valid = s < prm.S && kr_rows(prm.after, (uint32_t)s, prm.R, rows, nrows);
      } else {
        const int64_t s = t / prm.pblocks;
        const int64_t p = (t % prm.pblocks) * T3_BK + k;
        valid = p < prm.P && kr_rows(prm.after, (uint32_t)s, prm.R, rows, nrows) &&
                kr_rows(prm.before, (uint32_t)p, prm.R, rows, nrows);
      }
      const bool vec = (prm.R & 3) == 0;
      for (int c = ng * cpg; c < (ng + 1) * cpg; c += 4) {
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (valid && c < prm.R) {
          v[0] = v[1] = v[2] = v[3] = 1.0f;
#pragma unroll
          for (int f = 0; f < 2 * PTG_MAX_ORDER; ++f) {
            if (f >= nrows) break;
            if (vec) {
              const float4 w = __ldg(reinterpret_cast<const float4 *>(rows[f] + c));
              v[0] *= w.x;
              v[1] *= w.y;
              v[2] *= w.z;
              v[3] *= w.w;
            } else {
#pragma unroll
              for (int j = 0; j < 4; ++j) v[j] *= (c + j < prm.R) ? __ldg(rows[f] + c + j) : 0.0f;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float hi = tf32_hi(v[j]);
          *reinterpret_cast<float *>(kt + sw128_off(c + j, k)) = hi;
          *reinterpret_cast<float *>(kt + sw128_off(N + c + j, k)) = v[j] - hi;
        }
      }
      fence_async_smem();
      mbar_arrive(&full_k[ks]);
      if (++ks == T3_KSTAGES) {
        ks = 0;
        kph ^= 1;
      }
      // at the end of chain c, drain chain c - 1 (the MMA is filling chain c's accumulator)
      const int c = kb / T3_CHAIN;
      if ((kb - c * T3_CHAIN == T3_CHAIN - 1 || kb == nkb - 1) && c >= 1) drain(c - 1);
    }
    if (nkb > 0) drain((nkb - 1) / T3_CHAIN);
    // ---------------- the drained sums -> split-K partials ----------------
    const int row = quarter * 32 + lane;
#pragma unroll
    for (int m = 0; m < MT; ++m) {
      if (m >= nqt) continue;
      const int64_t q = (int64_t)(qt0 + m) * T3_BM + row;
      if (q >= prm.Q) continue;
      float *dst = prm.partial + ((int64_t)split * prm.Q + q) * N;
#pragma unroll
      for (int i = 0; i < HALF; i += 4)
        *reinterpret_cast<float4 *>(dst + i) = make_float4(sum[m][i], sum[m][i + 1], sum[m][i + 2], sum[m][i + 3]);
    }
  } else {
    // ---------------- X splitters (128 threads), and the drains of columns [N/2, N) ----------------
    const int ts = threadIdx.x - 192;
    const int quarter = warp & 3;
    constexpr int HALF = T3Shape<N>::HALF;
    float sum[MT][HALF];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
      for (int i = 0; i < HALF; ++i) sum[m][i] = 0.0f;
    bool alive = true;
    auto drain = [&](int c) {
      if (alive && !t3_drain<N>(sum, c, nqt, tmem_base, quarter, HALF, acc_full, acc_empty, abort_flag)) {
        fail_timeout(abort_flag, prm.err);
        alive = false;
      }
    };
    int xs = 0, ss = 0;
    uint32_t xph = 0, sph = 0;
    for (int kb = 0; kb < nkb; ++kb) {
      for (int m = 0; m < nqt; ++m) {
        if (!mbar_wait(&full_x[xs], xph, abort_flag) || !mbar_wait(&empty_s[ss], sph ^ 1, abort_flag)) {
          fail_timeout(abort_flag, prm.err);
          goto split_done;
        }
        {
          const uint8_t *stg = xring + xs * T3_TILE;
          uint8_t *hi = sring + ss * 2 * T3_TILE, *lo = hi + T3_TILE;
          if (!prm.mmajor) {
            // the staging tile is already the swizzled K-major layout: split chunk by chunk
#pragma unroll
            for (int i = 0; i < T3_TILE / 16 / 128; ++i) {
              const int ch = ts + 128 * i;
              const float4 v = *reinterpret_cast<const float4 *>(stg + ch * 16);
              const float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
              *reinterpret_cast<float4 *>(hi + ch * 16) = h;
              *reinterpret_cast<float4 *>(lo + ch * 16) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
            }
          } else {
            // four [32 s][32 q] boxes (q contiguous) -> K-major rows q, chunks of 4 s
            const int q = ts;
            const float *box = reinterpret_cast<const float *>(stg + (q >> 5) * (T3_TILE / 4));
#pragma unroll
            for (int sc = 0; sc < T3_BK / 4; ++sc) {
              float v[4], h[4];
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                v[i] = box[(sc * 4 + i) * 32 + (q & 31)];
                h[i] = tf32_hi(v[i]);
              }
              const uint32_t off = sw128_off(q, sc * 4);
              *reinterpret_cast<float4 *>(hi + off) = make_float4(h[0], h[1], h[2], h[3]);
              *reinterpret_cast<float4 *>(lo + off) = make_float4(v[0] - h[0], v[1] - h[1], v[2] - h[2], v[3] - h[3]);
            }
          }
        }
        fence_async_smem();
        mbar_arrive(&free_x[xs]);
        mbar_arrive(&full_s[ss]);
        if (++xs == T3_XSTAGES) {
          xs = 0;
          xph ^= 1;
        }
        if (++ss == T3_SSTAGES) {
          ss = 0;
          sph ^= 1;
        }
      }
      // at the end of chain c, drain chain c - 1 (the MMA is filling chain c's accumulator)
      const int c = kb / T3_CHAIN;
      if ((kb - c * T3_CHAIN == T3_CHAIN - 1 || kb == nkb - 1) && c >= 1) drain(c - 1);
    }
    alive = alive && !*abort_flag;
    if (nkb > 0) drain((nkb - 1) / T3_CHAIN);
  split_done:;
    const int row = quarter * 32 + lane;
#pragma unroll
    for (int m = 0; m < MT; ++m) {
      if (m >= nqt) continue;
      const int64_t q = (int64_t)(qt0 + m) * T3_BM + row;
      if (q >= prm.Q) continue;
      float *dst = prm.partial + ((int64_t)split * prm.Q + q) * N + HALF;
#pragma unroll
      for (int i = 0; i < HALF; i += 4)
        *reinterpret_cast<float4 *>(dst + i) = make_float4(sum[m][i], sum[m][i + 1], sum[m][i + 2], sum[m][i + 3]);
    }
  }
  // before TMEM is released and the CTA exits: every MMA has completed (the issuer's final
  // commit) and every TMA load this CTA issued has landed, waited for with a bound even
  // after an abort
  if (warp == 1 && lane == 0) mbar_wait_bounded(done, 0);
  if (warp == 0 && lane == 0) {
    for (int i = 0; i < T3_XSTAGES; ++i)
      if (issued[i]) mbar_wait_bounded(&full_x[i], (issued[i] - 1) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(prm.tmem_cols)
                 : "memory");
  }
}

__global__ void tc32_reduce_kernel(const float *__restrict__ partial, int nsplit, int64_t Q, int N,
                                   int64_t q_write, int R, float *__restrict__ out, const int *skip) {
  if (skip && *skip) return;
  const int64_t n = q_write * R;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = idx / R;
    const int c = (int)(idx % R);
    out[idx] = sum_splits(partial + q * N + c, Q * N, nsplit);
  }
}

size_t tc32_smem_bytes(int N) {
  const int xst = N == 16 ? T3Shape<16>::XST : N == 32 ? T3Shape<32>::XST : N == 48 ? T3Shape<48>::XST
                                                                                 : T3Shape<64>::XST;
  return 1024 /*alignment slack*/ + (size_t)xst * T3_TILE + (size_t)T3_SSTAGES * 2 * T3_TILE +
         (size_t)T3_KSTAGES * 2 * N * 128 +
         sizeof(uint64_t) * (2 * xst + 2 * T3_SSTAGES + 2 * T3_KSTAGES + 4 + 1) + 16;
}

}  // namespace

int tc32_contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                            cudaStream_t stream) {
  if (t->dtype != PTG_F32) return set_error(PTG_ERR_INVALID, "internal: the TF32-split path needs FP32 storage");
  if (R > 64) return set_error(PTG_ERR_UNSUPPORTED, "tensor-core FP32 MTTKRP: rank > 64");
  EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(PTG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const bool mmajor = (c.P == 1);
  if ((mmajor && (c.Q % 8) != 0) || (!mmajor && (c.P % 8) != 0))
    return set_error(PTG_ERR_INVALID, "internal: the contiguous extent must be a multiple of 8");
  if (c.Q > 0x7fffffffLL || c.S > 0x7fffffffLL || c.P > 0x7fffffffLL)
    return set_error(PTG_ERR_UNSUPPORTED, "tensor-core FP32 MTTKRP: extent exceeds 2^31");
  T3Params prm{};
  prm.P = c.P;
  prm.Q = c.Q;
  prm.S = c.S;
  prm.N = (R + 15) / 16 * 16;
  prm.R = R;
  prm.mmajor = mmajor ? 1 : 0;
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
  prm.qtiles = (int)((c.Q + T3_BM - 1) / T3_BM);
  const int mt_max = std::min(8, 128 / prm.N);   // T3Shape<N>::MT
  int mt = std::min(mt_max, prm.qtiles);
  const int qgroups_min = (prm.qtiles + mt - 1) / mt;
  mt = (prm.qtiles + qgroups_min - 1) / qgroups_min;   // balance q-tiles over the groups
  prm.mt_per_cta = mt;
  const int qgroups = (prm.qtiles + mt - 1) / mt;
  uint32_t cols = 32;   // two accumulators of MT q-tiles x 2N columns
  while (cols < (uint32_t)(2 * mt_max * 2 * prm.N)) cols <<= 1;
  prm.tmem_cols = cols;
  if (mmajor) {
    prm.pblocks = 1;
    prm.kblocks_total = (c.S + T3_BK - 1) / T3_BK;
  } else {
    prm.pblocks = (c.P + T3_BK - 1) / T3_BK;
    prm.kblocks_total = c.S * prm.pblocks;
  }
  int64_t nsplit = std::max<int64_t>(1, ctx->sm_count / qgroups);
  nsplit = std::min<int64_t>(nsplit, prm.kblocks_total);
  prm.kblocks_per_split = (prm.kblocks_total + nsplit - 1) / nsplit;
  nsplit = (prm.kblocks_total + prm.kblocks_per_split - 1) / prm.kblocks_per_split;
  if (nsplit > 65535) return set_error(PTG_ERR_UNSUPPORTED, "tensor-core FP32 MTTKRP: too many K-splits");

  // tensor map over the FP32 tensor
  CUtensorMap map;
  CUresult r;
  if (mmajor) {   // [S][Q], boxes of 32 q x 32 s (128-byte rows, no swizzle)
    cuuint64_t gdim[2] = {(cuuint64_t)c.Q, (cuuint64_t)c.S};
    cuuint64_t gstride[1] = {(cuuint64_t)c.Q * 4};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t es[2] = {1, 1};
    r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, t->data, gdim, gstride, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {        // [S][Q][P], boxes of 32 p x 128 q, 128-byte swizzle (the MMA's K-major layout)
    cuuint64_t gdim[3] = {(cuuint64_t)c.P, (cuuint64_t)c.Q, (cuuint64_t)c.S};
    cuuint64_t gstride[2] = {(cuuint64_t)c.P * 4, (cuuint64_t)c.P * c.Q * 4};
    cuuint32_t box[3] = {32, 128, 1};
    cuuint32_t es[3] = {1, 1, 1};
    r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, t->data, gdim, gstride, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  if (r != CUDA_SUCCESS) {
    char buf[128];
    snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return set_error(PTG_ERR_CUDA, buf);
  }
  const size_t part_bytes = (size_t)nsplit * c.Q * prm.N * sizeof(float);
  PTG_TRY(ctx->scratch.ensure(part_bytes));
  prm.partial = reinterpret_cast<float *>(ctx->scratch.ptr);
  prm.err = ctx->dev_err;
  prm.skip = c.skip;
  const size_t smem = tc32_smem_bytes(prm.N);
  if (smem > ctx->smem_optin) return set_error(PTG_ERR_UNSUPPORTED, "tensor-core FP32 MTTKRP: shared memory");
  auto kern = prm.N == 16 ? mttkrp_tc32_kernel<16>
              : prm.N == 32 ? mttkrp_tc32_kernel<32>
              : prm.N == 48 ? mttkrp_tc32_kernel<48>
                            : mttkrp_tc32_kernel<64>;
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared));
  dim3 grid((unsigned)qgroups, (unsigned)nsplit);
  kern<<<grid, T3_THREADS, smem, stream>>>(map, prm);
  PTG_CUDA(cudaGetLastError());
  const int64_t n = c.q_write * R;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
  tc32_reduce_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(prm.partial, (int)nsplit, c.Q, prm.N, c.q_write,
                                                              R, out, c.skip);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 2);
  return PTG_OK;
}

}  // namespace ptg
