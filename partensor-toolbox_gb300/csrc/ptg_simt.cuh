// The CUDA-core MTTKRP tile routine (FP32 math; FP32 or BF16 storage), shared by the
// single-contraction and work-list kernels (ptg_mttkrp.cu) and the persistent batched
// solver (ptg_batched.cu).  See ptg_mttkrp.cu for the contraction it computes.
#pragma once
#include <cuda_bf16.h>

#include "ptg_internal.h"
#include "ptg_sync.cuh"

namespace ptg {
namespace {

struct KrDev {  // kernel-parameter copy of a KrSide
  int n;
  uint32_t ext[PTG_MAX_ORDER];
  uint32_t valid[PTG_MAX_ORDER];
  const float *fac[PTG_MAX_ORDER];
};

struct SimtParams {
  const void *X;
  int64_t P, Q, S;
  int64_t ktiles_total, ktiles_per_split, pblocks;
  KrDev before, after;
  int R, col0;       // factor row stride and first column handled by this launch
  float *partial;    // [nsplit][Q][ldp] (ldp = BN)
  float *out;        // used when nsplit == 1: row-major [q_write][ldo]
  int64_t q_write;
  int ldo;
  int nsplit;
  const int *skip;   // nonzero: return at once (Contraction::skip; single launches only)
};

template <typename T>
struct Vec;  // 16-byte global load unit
template <>
struct Vec<float> {
  static constexpr int kElems = 4;
};
template <>
struct Vec<__nv_bfloat16> {
  static constexpr int kElems = 8;
};

__device__ __forceinline__ void unpack16(const uint4 &u, float *f, const float *) {
  f[0] = __uint_as_float(u.x);
  f[1] = __uint_as_float(u.y);
  f[2] = __uint_as_float(u.z);
  f[3] = __uint_as_float(u.w);
}
__device__ __forceinline__ void unpack16(const uint4 &u, float *f, const __nv_bfloat16 *) {
  const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    f[2 * i] = __uint_as_float(w[i] << 16);
    f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}

// Khatri-Rao value of one side for linear index `lin` and NV consecutive columns.
template <int NV>
__device__ __forceinline__ void kr_side(const KrDev &s, uint32_t lin, int R, int c, float *v) {
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = 1.0f;
  for (int f = 0; f < s.n; ++f) {
    const uint32_t e = s.ext[f];
    const uint32_t d = lin % e;
    lin /= e;
    if (d >= s.valid[f]) {
#pragma unroll
      for (int j = 0; j < NV; ++j) v[j] = 0.0f;
      return;
    }
    const float *row = s.fac[f] + (size_t)d * R;
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] *= (c + j < R) ? __ldg(row + c + j) : 0.0f;
  }
}

// Tile configuration: BN columns per launch, BM rows of Q, BK contraction elements.
template <int BN>
struct Cfg;
template <>
struct Cfg<16> {
  static constexpr int TN = 4, BM = 128;
};
template <>
struct Cfg<32> {
  static constexpr int TN = 4, BM = 128;
};
template <>
struct Cfg<64> {
  static constexpr int TN = 8, BM = 128;
};
template <>
struct Cfg<128> {
  static constexpr int TN = 8, BM = 64;
};

constexpr int kThreads = 128;
constexpr int BK = 32;

// MMAJOR: mode-0 style (P == 1): q contiguous; tile [BK s][BM q]  -> Xs[k][m]
// KMAJOR: P > 1: p contiguous within (q, s); tile [BM q][BK p]   -> Xs[m][k]
// BMO: M-tile height (0: the configuration's default); TM follows from the 128 threads.
template <typename T, int BN, bool MMAJOR, int BMO = 0, typename Sync = SyncCta>
__device__ __forceinline__ void mttkrp_simt_body(const SimtParams &prm, int mtile, int split, float *smem_dyn,
                                                 int tid, Sync sync = Sync()) {
  using C = Cfg<BN>;
  constexpr int TN = C::TN;
  constexpr int NG = BN / TN;  // column groups
  constexpr int BM = BMO ? BMO : C::BM;
  constexpr int TM = BM * NG / kThreads;
  static_assert(TM == 2 || TM % 4 == 0, "row tiling");
  static_assert(NG * (BM / TM) == kThreads, "thread tiling");
  constexpr int EV = Vec<T>::kElems;                   // elements per 16-byte load
  constexpr int XLD = MMAJOR ? (BM + 4) : (BK + 4);    // smem row stride (floats)
  constexpr int XROWS = MMAJOR ? BK : BM;
  constexpr int LOADS = (BM * BK) / (EV * kThreads);   // 16-byte loads per thread per tile
  static_assert(LOADS * EV * kThreads == BM * BK, "load tiling");

  // shared memory (smem_dyn, 16-byte aligned): two X tiles then two Khatri-Rao tiles
  constexpr int XS = XROWS * XLD, KS = BK * BN;

  const int ng = tid % NG, mg = tid / NG;
  const int64_t q0 = (int64_t)mtile * BM;
  const int64_t t_begin = (int64_t)split * prm.ktiles_per_split;
  const int64_t t_end = min(prm.ktiles_total, t_begin + prm.ktiles_per_split);
  const T *X = reinterpret_cast<const T *>(prm.X);

  float acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0f;

  uint4 regs[LOADS];

  // ---- global -> registers for tile t ----
  auto load_tile = [&](int64_t t) {
    if (MMAJOR) {
      const int64_t s0 = t * BK;
#pragma unroll
      for (int i = 0; i < LOADS; ++i) {
        const int f = tid + i * kThreads;
        const int k = f / (BM / EV), mv = (f % (BM / EV)) * EV;
        const int64_t s = s0 + k, q = q0 + mv;
        if (s < prm.S && q < prm.Q)
          regs[i] = __ldg(reinterpret_cast<const uint4 *>(X + q + prm.Q * s));
        else
          regs[i] = make_uint4(0, 0, 0, 0);
      }
    } else {
      const int64_t s = t / prm.pblocks;
      const int64_t p0 = (t % prm.pblocks) * BK;
#pragma unroll
      for (int i = 0; i < LOADS; ++i) {
        const int f = tid + i * kThreads;
        const int m = f / (BK / EV), kv = (f % (BK / EV)) * EV;
        const int64_t p = p0 + kv, q = q0 + m;
        if (p < prm.P && q < prm.Q)
          regs[i] = __ldg(reinterpret_cast<const uint4 *>(X + p + prm.P * (q + prm.Q * s)));
        else
          regs[i] = make_uint4(0, 0, 0, 0);
      }
    }
  };

  // ---- registers -> shared, and the Khatri-Rao tile ----
  auto store_tile = [&](int64_t t, int buf) {
#pragma unroll
    for (int i = 0; i < LOADS; ++i) {
      const int f = tid + i * kThreads;
      float v[EV];
      unpack16(regs[i], v, (const T *)nullptr);
      float *dst;
      if (MMAJOR) {
        const int k = f / (BM / EV), mv = (f % (BM / EV)) * EV;
        dst = &smem_dyn[buf * XS + k * XLD + mv];
      } else {
        const int m = f / (BK / EV), kv = (f % (BK / EV)) * EV;
        dst = &smem_dyn[buf * XS + m * XLD + kv];
      }
#pragma unroll
      for (int e = 0; e < EV; e += 4)
        *reinterpret_cast<float4 *>(dst + e) = make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
    }
    // KR tile: thread -> one k row, KPT consecutive columns
    constexpr int KPT = (BK * BN) / kThreads;
    const int k = tid / (BN / KPT), c = (tid % (BN / KPT)) * KPT;
    float va[KPT], vb[KPT];
    if (MMAJOR) {
      const int64_t s = t * BK + k;
      if (s < prm.S) {
        kr_side<KPT>(prm.after, (uint32_t)s, prm.R, prm.col0 + c, va);
      } else {
#pragma unroll
        for (int j = 0; j < KPT; ++j) va[j] = 0.0f;
      }
#pragma unroll
      for (int j = 0; j < KPT; ++j) vb[j] = 1.0f;
    } else {
      const int64_t s = t / prm.pblocks;
      const int64_t p = (t % prm.pblocks) * BK + k;
      kr_side<KPT>(prm.after, (uint32_t)s, prm.R, prm.col0 + c, va);
      if (p < prm.P) {
        kr_side<KPT>(prm.before, (uint32_t)p, prm.R, prm.col0 + c, vb);
      } else {
#pragma unroll
        for (int j = 0; j < KPT; ++j) vb[j] = 0.0f;
      }
    }
#pragma unroll
    for (int j = 0; j < KPT; j += 4)
      *reinterpret_cast<float4 *>(&smem_dyn[2 * XS + buf * KS + k * BN + c + j]) =
          make_float4(va[j] * vb[j], va[j + 1] * vb[j + 1], va[j + 2] * vb[j + 2],
                      va[j + 3] * vb[j + 3]);
  };

  auto compute = [&](int buf) {
    const float *xs = smem_dyn + buf * XS;
    const float *ks = smem_dyn + 2 * XS + buf * KS;
    if (MMAJOR) {
#pragma unroll 4
      for (int k = 0; k < BK; ++k) {
        float a[TM], b[TN];
        if constexpr (TM == 2) {
          const float2 v = *reinterpret_cast<const float2 *>(xs + k * XLD + mg * TM);
          a[0] = v.x; a[1] = v.y;
        } else {
#pragma unroll
          for (int i = 0; i < TM; i += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(xs + k * XLD + mg * TM + i);
            a[i] = v.x; a[i + 1] = v.y; a[i + 2] = v.z; a[i + 3] = v.w;
          }
        }
#pragma unroll
        for (int j = 0; j < TN; j += 4) {
          const float4 v = *reinterpret_cast<const float4 *>(ks + k * BN + ng * TN + j);
          b[j] = v.x; b[j + 1] = v.y; b[j + 2] = v.z; b[j + 3] = v.w;
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
    } else {
#pragma unroll 2
      for (int k = 0; k < BK; k += 4) {
        float a[TM][4], b[4][TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) {
          const float4 v = *reinterpret_cast<const float4 *>(xs + (mg + i * (BM / TM)) * XLD + k);
          a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; a[i][3] = v.w;
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int j = 0; j < TN; j += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(ks + (k + kk) * BN + ng * TN + j);
            b[kk][j] = v.x; b[kk][j + 1] = v.y; b[kk][j + 2] = v.z; b[kk][j + 3] = v.w;
          }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i][kk], b[kk][j], acc[i][j]);
      }
    }
  };

  if (t_begin < t_end) {
    load_tile(t_begin);
    store_tile(t_begin, 0);
    sync();
    int cur = 0;
    for (int64_t t = t_begin; t < t_end; ++t) {
      const bool more = (t + 1 < t_end);
      if (more) load_tile(t + 1);
      compute(cur);
      if (more) store_tile(t + 1, cur ^ 1);
      sync();
      cur ^= 1;
    }
  }

  // ---- epilogue: rows of this thread ----
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = MMAJOR ? (mg * TM + i) : (mg + i * (BM / TM));
    const int64_t q = q0 + m;
    if (q >= prm.Q) continue;
    const int c = ng * TN;
    if (prm.nsplit == 1) {
      if (q < prm.q_write) {
#pragma unroll
        for (int j = 0; j < TN; ++j)
          if (prm.col0 + c + j < prm.R) prm.out[q * prm.ldo + prm.col0 + c + j] = acc[i][j];
      }
    } else {
      float *dst = prm.partial + ((int64_t)split * prm.Q + q) * BN + c;
#pragma unroll
      for (int j = 0; j < TN; j += 4)
        *reinterpret_cast<float4 *>(dst + j) =
            make_float4(acc[i][j], acc[i][j + 1], acc[i][j + 2], acc[i][j + 3]);
    }
  }
}

KrDev to_dev(const KrSide &s) {
  KrDev d{};
  d.n = s.n;
  for (int i = 0; i < s.n; ++i) {
    d.ext[i] = (uint32_t)s.ext[i];
    d.valid[i] = (uint32_t)s.valid[i];
    d.fac[i] = s.fac[i];
  }
  return d;
}

template <int BN>
size_t simt_smem_bytes(bool mmajor, int bm = 0) {
  using Cf = Cfg<BN>;
  const size_t BMv = bm ? bm : Cf::BM;
  const size_t xrows = mmajor ? BK : BMv, xld = mmajor ? (BMv + 4) : (BK + 4);
  return sizeof(float) * (2 * xrows * xld + 2 * BK * BN);
}

}  // namespace
}  // namespace ptg
