// Dense MTTKRP on the 5th-generation tensor cores (tcgen05, kind::f16, BF16 x BF16 -> FP32).
//
// Same contraction as the CUDA-core kernel (ptg_mttkrp.cu): the BF16 tensor viewed as
// [P, Q, S], out[q, r] = sum_{p,s} X[p,q,s] KRb[p,r] KRa[s,r].  One CTA per SM, warp
// specialised:
//   warp 0      TMA producer: 128 x 64 BF16 tiles of X into a ring of shared-memory stages
//               (128-byte swizzle; K-major for modes n >= 1, MN-major for mode 0).  K-blocks
//               go in groups of G consecutive ones: within a group the q-tiles are the outer
//               loop, so each row of X is read as one run of G x 128 bytes (a mode-0 K-block
//               is already one contiguous run; there G = 1);
//   warp 1      allocates TMEM and issues tcgen05.mma (M=128, N=R padded to 16, K=16) from
//               one elected lane; each q-tile of the CTA accumulates in its own TMEM columns;
//   warps 2..9  build the R x 64 Khatri-Rao tile of every K-block in shared memory (BF16,
//               swizzled K-major; four threads per K row, one 8-column chunk each, the
//               factor rows of a chunk loaded together); warps 2..5 then drain TMEM
//               (tcgen05.ld) into the split-K partials.
// Every mbarrier wait is bounded: on timeout the kernel raises an error word and returns
// after releasing its TMEM.
#include <cuda.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "ptg_internal.h"
#include "ptg_tcgen05.h"

namespace ptg {
namespace {

using namespace tc;

constexpr int TC_BM = 128;         // q rows per tile (MMA M)
constexpr int TC_BK = 64;          // contraction elements per K-block (one 128-byte row)
constexpr int TC_MAX_STAGES = 8;   // X tile ring (fewer when the shared-memory budget is short)
constexpr int TC_GROUP = 2;        // K-blocks per group, modes n >= 1 (measured: 2 beats 1 and 4)
constexpr int TC_MAX_KSTAGES = 4;  // Khatri-Rao tile ring: two groups
constexpr int TC_THREADS = 320;    // producer, MMA issuer, 8 Khatri-Rao builder warps
constexpr int TC_BUILDERS = 256;
constexpr int TC_ATILE = TC_BM * TC_BK * 2;   // 16 KB

struct TcParams {
  int64_t P, Q, S;
  int64_t kblocks_total, kblocks_per_split, pblocks;
  int qtiles, mt_per_cta;
  int N;          // MMA N: rank padded to a multiple of 16
  int R;
  int mmajor;
  int stages;      // X ring stages
  int group;       // G: K-blocks per group
  int kstages;     // Khatri-Rao ring stages (a multiple of G, >= 2 G)
  uint32_t tmem_cols;
  uint32_t spin;   // poll limit of every bounded wait
  int vec4;        // factor rows are read as float4 (R % 4 == 0, 16-byte aligned)
  KrDevTc before, after;
  float *partial;  // [nsplit][Q][N]
  int *err;
  const int *skip;  // nonzero: return at once (Contraction::skip)
};

__global__ void __launch_bounds__(TC_THREADS, 1)
mttkrp_tc_kernel(const __grid_constant__ CUtensorMap tmap, const TcParams prm) {
  if (prm.skip && *prm.skip) return;   // before any barrier or TMEM allocation
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // 1024-byte aligned carve: A ring, K ring, barriers
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int N = prm.N;
  const int KTILE = N * 128;                       // R_pad rows of 128 bytes
  uint8_t *aring = base;
  const int STAGES = prm.stages, KSTAGES = prm.kstages, G = prm.group;
  uint8_t *kring = aring + STAGES * TC_ATILE;
  uint64_t *bars = (uint64_t *)(kring + KSTAGES * KTILE);
  uint64_t *full_a = bars, *empty_a = bars + TC_MAX_STAGES;
  uint64_t *full_k = empty_a + TC_MAX_STAGES, *empty_k = full_k + TC_MAX_KSTAGES;
  uint64_t *done = empty_k + TC_MAX_KSTAGES;
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
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full_a[i], 1);
      mbar_init(&empty_a[i], 1);
    }
    for (int i = 0; i < KSTAGES; ++i) {
      mbar_init(&full_k[i], TC_BUILDERS);
      mbar_init(&empty_k[i], 1);
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

  // idesc: D=F32 (bit 4), A=BF16 (bit 7), B=BF16 (bit 10), A major (bit 15), N>>3 (17-22), M>>4 (24-28)
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)prm.mmajor << 15) |
                         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0 && nkb > 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued[TC_MAX_STAGES] = {0};   // loads issued into each stage
      bool ok = true;
      // K-block t covers s in [t BK, t BK + BK) (mode 0), else slab t / pblocks, p from
      // (t % pblocks) BK; the coordinates step along a group without dividing
      const int pend = (int)(prm.pblocks * TC_BK);
      if (G == 1) {   // one K-block at a time (this loop form issues fastest; see the issuer)
        for (int kb = 0; kb < nkb && ok; ++kb) {
          const int64_t t = kb0 + kb;
          for (int m = 0; m < nqt; ++m) {
            if (!mbar_wait_lim(&empty_a[stage], phase ^ 1, abort_flag, prm.spin)) {
              ok = false;
              break;
            }
            mbar_expect_tx(&full_a[stage], TC_ATILE);
            uint8_t *dst = aring + stage * TC_ATILE;
            const int q = (qt0 + m) * TC_BM;
            if (prm.mmajor) {
              const int s0 = (int)(t * TC_BK);
              tma_load_2d(dst, &tmap, &full_a[stage], q, s0);
              tma_load_2d(dst + TC_ATILE / 2, &tmap, &full_a[stage], q + 64, s0);
            } else {
              const int s = (int)(t / prm.pblocks);
              const int p0 = (int)((t % prm.pblocks) * TC_BK);
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
          sg = (int)(tg * TC_BK);
        } else {
          sg = (int)(tg / prm.pblocks);
          pg = (int)((tg - (int64_t)sg * prm.pblocks) * TC_BK);
        }
        for (int m = 0; m < nqt && ok; ++m) {
          const int q = (qt0 + m) * TC_BM;
          int s = sg, p = pg;
          for (int j = 0; j < gn; ++j) {
            if (!mbar_wait_lim(&empty_a[stage], phase ^ 1, abort_flag, prm.spin)) {
              ok = false;
              break;
            }
            mbar_expect_tx(&full_a[stage], TC_ATILE);
            uint8_t *dst = aring + stage * TC_ATILE;
            if (prm.mmajor) {
              tma_load_2d(dst, &tmap, &full_a[stage], q, s);
              tma_load_2d(dst + TC_ATILE / 2, &tmap, &full_a[stage], q + 64, s);
              s += TC_BK;
            } else {
              tma_load_3d(dst, &tmap, &full_a[stage], p, q, s);
              p += TC_BK;
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
      }
      // a stage holds at most one load in flight (the next one waits for its release), the
      // last one issued into it: wait for each so no copy lands after the CTA has exited
      // (loads that were consumed completed long ago and return at once)
      for (int s = 0; s < STAGES; ++s)
        if (issued[s] > 0) mbar_wait_bounded(&full_a[s], (uint32_t)((issued[s] - 1) & 1));
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0, kst = 0;
      uint32_t phase = 0, kphase = 0;
      bool ok = true;
      // descriptors: a constant high word and the start address >> 4, stepped per K = 16
      const uint64_t a_hi = prm.mmajor ? smem_desc_sw128_hi(TC_ATILE / 2, 1024) : smem_desc_sw128_hi(16, 1024);
      const uint64_t b_hi = smem_desc_sw128_hi(16, 1024);
      const uint32_t a_step = prm.mmajor ? (2048u >> 4) : (32u >> 4);
      const uint32_t a_lo0 = smem_u32(aring) >> 4, k_lo0 = smem_u32(kring) >> 4;
      if (G == 1) {
        // one K-block at a time, descriptors built next to each MMA: measured faster than the
        // group loop below with G = 1 (the issuing thread is the busiest role of the kernel)
        for (int kb = 0; kb < nkb && ok; ++kb) {
          if (!mbar_wait_lim(&full_k[kst], kphase, abort_flag, prm.spin)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t kaddr = smem_u32(kring + kst * KTILE);
          for (int m = 0; m < nqt; ++m) {
            if (!mbar_wait_lim(&full_a[stage], phase, abort_flag, prm.spin)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t aaddr = smem_u32(aring + stage * TC_ATILE);
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk) {
              const uint64_t ad = prm.mmajor ? smem_desc_sw128(aaddr + kk * 2048, TC_ATILE / 2, 1024)
                                             : smem_desc_sw128(aaddr + kk * 32, 16, 1024);
              const uint64_t bd = smem_desc_sw128(kaddr + kk * 32, 16, 1024);
              umma_bf16(tmem_base + (uint32_t)(m * N), ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
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
        for (int j = 0; j < gn && ok; ++j)
          ok = mbar_wait_lim(&full_k[kst + j], kphase, abort_flag, prm.spin);
        if (!ok) break;
        tc_fence_after();
        for (int m = 0; m < nqt && ok; ++m) {
          const uint32_t d_tmem = tmem_base + (uint32_t)(m * N);
          for (int j = 0; j < gn; ++j) {
            if (!mbar_wait_lim(&full_a[stage], phase, abort_flag, prm.spin)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t ad = a_hi | (uint64_t)(a_lo0 + (uint32_t)stage * (TC_ATILE >> 4));
            const uint64_t bd = b_hi | (uint64_t)(k_lo0 + (uint32_t)(kst + j) * (uint32_t)(KTILE >> 4));
            umma_bf16(d_tmem, ad, bd, idesc, (g0 | j) != 0 ? 1u : 0u);
#pragma unroll
            for (int kk = 1; kk < TC_BK / 16; ++kk)
              umma_bf16(d_tmem, ad + kk * a_step, bd + kk * (32u >> 4), idesc, 1u);
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
    // ---------------- Khatri-Rao builders (256 threads) ----------------
    const int tb = threadIdx.x - 64;
    const int k = tb & 63, part = tb >> 6;   // four threads per K row: 8-column chunks part, part + 4, ...
    const bool drains = warp < 6;            // warps 2..5 cover the four TMEM lane quarters
    int kst = 0;
    uint32_t kphase = 0;
    // slab and p-block of K-block kb0 + kb (modes n >= 1), stepped without dividing
    int64_t sl = kb0 / prm.pblocks;
    int pb = (int)(kb0 - sl * prm.pblocks);
    for (int kb = 0; kb < nkb; ++kb) {
      if (!mbar_wait_lim(&empty_k[kst], kphase ^ 1, abort_flag, prm.spin)) {
        *abort_flag = 1;
        atomicExch(prm.err, PTG_ERR_TIMEOUT);
        break;
      }
      const int64_t t = kb0 + kb;
      uint8_t *kt = kring + kst * KTILE;
      // linear indices of this thread's row of the K-block
      bool valid;
      uint32_t lin_b = 0, lin_a;
      if (prm.mmajor) {
        const int64_t s = t * TC_BK + k;
        valid = s < prm.S;
        lin_a = (uint32_t)s;
      } else {
        const int64_t p = (int64_t)pb * TC_BK + k;
        valid = p < prm.P;
        lin_a = (uint32_t)sl;
        lin_b = (uint32_t)p;
      }
      // the thread's 8-column chunks, the loads of a chunk's factor rows issued together
      for (int c = 8 * part; c < N; c += 32) {
        float va[8];
        if (valid) {
          kr_pair<8>(prm.after, lin_a, prm.before, lin_b, !prm.mmajor, prm.R, c, prm.vec4 != 0, va);
        } else {
#pragma unroll
          for (int j = 0; j < 8; ++j) va[j] = 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int n = c + j;
          const uint32_t off = (uint32_t)((n >> 3) * 1024 + (n & 7) * 128 + ((((k >> 3) ^ (n & 7)) & 7) << 4) +
                                          (k & 7) * 2);
          *reinterpret_cast<__nv_bfloat16 *>(kt + off) = __float2bfloat16_rn(va[j]);
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
    const bool have = drains && (nkb > 0) && mbar_wait_lim(done, 0, abort_flag, prm.spin) && !*abort_flag;
    tc_fence_after();
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    for (int m = 0; drains && m < nqt; ++m) {
      const int64_t q = (int64_t)(qt0 + m) * TC_BM + row;
      float *dst = prm.partial + ((int64_t)split * prm.Q + q) * N;
      for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        if (have) {
          tmem_ld16(tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(m * N + c0), v);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = 0.0f;
        }
        if (q < prm.Q) {
#pragma unroll
          for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4 *>(dst + c0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
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

__global__ void tc_reduce_kernel(const float *__restrict__ partial, int nsplit, int64_t Q, int N, int64_t q_write,
                                 int R, float *__restrict__ out, const int *skip) {
  if (skip && *skip) return;
  const int64_t n = q_write * R;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = idx / R;
    const int c = (int)(idx % R);
    out[idx] = sum_splits(partial + q * N + c, Q * N, nsplit);
  }
}

size_t tc_smem_bytes(int N, int stages, int kstages) {
  return 1024 /*alignment slack*/ + (size_t)stages * TC_ATILE + (size_t)kstages * N * 128 +
         sizeof(uint64_t) * (2 * TC_MAX_STAGES + 2 * TC_MAX_KSTAGES + 1) + 16;
}

}  // namespace

int tc_contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                          cudaStream_t stream) {
  if (t->dtype != PTG_BF16) return set_error(PTG_ERR_INVALID, "internal: tcgen05 path needs BF16 storage");
  if (R > 128) return set_error(PTG_ERR_UNSUPPORTED, "tcgen05 MTTKRP: rank > 128");
  EncodeTiledFn enc = encode_fn();
  if (!enc) return set_error(PTG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const bool mmajor = (c.P == 1);
  if (mmajor && (c.Q % 8) != 0) return set_error(PTG_ERR_INVALID, "internal: Q must be a multiple of 8");
  if (c.Q > 0x7fffffffLL || c.S > 0x7fffffffLL || c.P > 0x7fffffffLL)
    return set_error(PTG_ERR_UNSUPPORTED, "tcgen05 MTTKRP: extent exceeds 2^31");
  TcParams prm{};
  prm.P = c.P;
  prm.Q = c.Q;
  prm.S = c.S;
  prm.N = (R + 15) / 16 * 16;
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
  prm.qtiles = (int)((c.Q + TC_BM - 1) / TC_BM);
  int mt = std::max(1, 512 / prm.N);
  mt = std::min(mt, prm.qtiles);
  const int qgroups_min = (prm.qtiles + mt - 1) / mt;
  // balance q-tiles over the groups
  mt = (prm.qtiles + qgroups_min - 1) / qgroups_min;
  prm.mt_per_cta = mt;
  const int qgroups = (prm.qtiles + mt - 1) / mt;
  uint32_t cols = 32;
  while (cols < (uint32_t)(mt * prm.N)) cols <<= 1;
  prm.tmem_cols = cols;
  if (mmajor) {
    prm.pblocks = 1;
    prm.kblocks_total = (c.S + TC_BK - 1) / TC_BK;
  } else {
    prm.pblocks = (c.P + TC_BK - 1) / TC_BK;
    prm.kblocks_total = c.S * prm.pblocks;
  }
  int64_t nsplit = std::max<int64_t>(1, ctx->sm_count / qgroups);
  nsplit = std::min<int64_t>(nsplit, prm.kblocks_total);
  prm.kblocks_per_split = (prm.kblocks_total + nsplit - 1) / nsplit;
  nsplit = (prm.kblocks_total + prm.kblocks_per_split - 1) / prm.kblocks_per_split;

  // tensor map over the BF16 tensor
  CUtensorMap map;
  CUresult r;
  if (mmajor) {
    cuuint64_t gdim[2] = {(cuuint64_t)c.Q, (cuuint64_t)c.S};
    cuuint64_t gstride[1] = {(cuuint64_t)c.Q * 2};
    cuuint32_t box[2] = {64, 64};
    cuuint32_t es[2] = {1, 1};
    r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, t->data, gdim, gstride, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {
    cuuint64_t gdim[3] = {(cuuint64_t)c.P, (cuuint64_t)c.Q, (cuuint64_t)c.S};
    cuuint64_t gstride[2] = {(cuuint64_t)c.P * 2, (cuuint64_t)c.P * c.Q * 2};
    cuuint32_t box[3] = {64, 128, 1};
    cuuint32_t es[3] = {1, 1, 1};
    r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, t->data, gdim, gstride, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  if (r != CUDA_SUCCESS) {
    char buf[128];
    snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return set_error(PTG_ERR_CUDA, buf);
  }
  // scratch: split-K partials
  const size_t part_bytes = (size_t)nsplit * c.Q * prm.N * sizeof(float);
  PTG_TRY(ctx->scratch.ensure(part_bytes));
  prm.partial = reinterpret_cast<float *>(ctx->scratch.ptr);
  prm.err = ctx->dev_err;
  prm.skip = c.skip;
  // The rings take at most the shared memory that leaves room on the SM for the eigenvalue-
  // bound kernel beside it: an X ring of up to 8 stages (more measured no faster) and a
  // Khatri-Rao ring of two groups
  const size_t budget = ctx->smem_beside_eigen;
  prm.group = mmajor ? 1 : TC_GROUP;
  prm.kstages = TC_MAX_KSTAGES;
  int stages = TC_MAX_STAGES;
  while (stages > 4 && tc_smem_bytes(prm.N, stages, prm.kstages) > budget) --stages;
  prm.stages = stages;
  const size_t smem = tc_smem_bytes(prm.N, prm.stages, prm.kstages);
  if (smem > ctx->smem_optin) return set_error(PTG_ERR_UNSUPPORTED, "tcgen05 MTTKRP: shared memory");
  auto kern = mttkrp_tc_kernel;
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // the largest carveout, which the eigenvalue-bound kernel beside it asks for too
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                cudaSharedmemCarveoutMaxShared));
  dim3 grid((unsigned)qgroups, (unsigned)nsplit);
  kern<<<grid, TC_THREADS, smem, stream>>>(map, prm);
  PTG_CUDA(cudaGetLastError());
  const int64_t n = c.q_write * R;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
  tc_reduce_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(prm.partial, (int)nsplit, c.Q, prm.N, c.q_write, R,
                                                            out, c.skip);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 2);
  return PTG_OK;
}

}  // namespace ptg
