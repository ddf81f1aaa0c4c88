// Sparse tensor completion (GTC) on the GPU.
//
// Replaces (paths relative to the reference project's root):
//   sort_ratings_base + SortRows + FillSparseMatricization (include/Gtc.hpp:69-110,
//   include/TensorOperations.hpp:432-487, 622-666): per mode, a stable LSD radix sort of the
//   64-bit key  i_n * J_n + (linear index of the other modes, first other mode fastest),
//   which is exactly SortRows' order, then a gather into a column-compressed layout
//   (row pointers by i_n, the other modes' indices and the value per entry);
//   SparseMTTKRP (include/MTTKRP.hpp:229-309) + local_L::NesterovMNLS
//   (include/NesterovMNLS.hpp:777-976): one CTA per row i_n gathers the Khatri-Rao rows of its
//   entries once, accumulates m_i = sum x kr and H_i = sum kr kr^T, runs PowerMethod on H_i
//   and the max_nesterov_iter projected Nesterov steps with grad = H_i y - m_i + lambda y;
//   dynamic_blocksize::StochasticNesterovMNLS (include/NesterovMNLS.hpp:431-547): the same per
//   row on a contiguous block of floor(c * nnz_i) entries at a counter-hashed pivot; both
//   forms run one warp per row at rank <= 32 (H_i in registers, no CTA barrier), else (and for
//   the ridge solve) one CTA per row;
//   the GTC cost (include/Gtc.hpp:184-214) as per-row FP64 partial sums added in row order.
// No global atomics on the data path; every reduction is in a fixed order.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ptg_internal.h"

namespace ptg {
namespace {

// ----------------------------------------------------------------------------------------
// Stable LSD radix sort of (uint64 key, uint32 value), 8-bit digits.
// ----------------------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

__global__ void rs_hist_kernel(const uint64_t *__restrict__ keys, int64_t n, int shift, int ntiles,
                               uint32_t *__restrict__ counts) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ITEMS; ++r) {
    const int64_t e = base + (int64_t)r * RS_THREADS + threadIdx.x;
    if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m uint32 values in place, three kernels (block sums, scan of sums, apply).
constexpr int SCAN_CHUNK = 4096;

__global__ void scan_block_sums_kernel(const uint32_t *__restrict__ a, int64_t m, uint64_t *__restrict__ sums) {
  __shared__ uint64_t red[32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  uint64_t s = 0;
  for (int i = threadIdx.x; i < SCAN_CHUNK; i += blockDim.x) {
    const int64_t e = base + i;
    if (e < m) s += a[e];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void scan_sums_kernel(uint64_t *sums, int nb) {
  // one block, sequential over chunks of blockDim (nb is small)
  __shared__ uint64_t buf[1024];
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
    const int i = b0 + threadIdx.x;
    buf[threadIdx.x] = (i < nb) ? sums[i] : 0;
    __syncthreads();
    // Hillis-Steele inclusive scan
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      const uint64_t v = threadIdx.x >= (unsigned)o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += v;
      __syncthreads();
    }
    const uint64_t incl = buf[threadIdx.x];
    const uint64_t excl = incl - ((i < nb) ? sums[i] : 0);
    __syncthreads();
    if (i < nb) sums[i] = carry + excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += incl;
    __syncthreads();
  }
}

__global__ void scan_apply_kernel(uint32_t *__restrict__ a, int64_t m, const uint64_t *__restrict__ sums,
                                  uint64_t *__restrict__ out) {
  // sequential within the chunk by one warp-parallel pass: each thread scans 16 entries
  __shared__ uint64_t part[256];
  const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
  const int per = SCAN_CHUNK / 256;
  uint64_t loc[SCAN_CHUNK / 256];
  uint64_t s = 0;
  for (int j = 0; j < per; ++j) {
    const int64_t e = base + (int64_t)threadIdx.x * per + j;
    loc[j] = (e < m) ? a[e] : 0;
    s += loc[j];
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const uint64_t v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint64_t run = sums[blockIdx.x] + part[threadIdx.x] - s;
  for (int j = 0; j < per; ++j) {
    const int64_t e = base + (int64_t)threadIdx.x * per + j;
    if (e < m) out[e] = run;
    run += loc[j];
  }
}

__global__ void rs_scatter_kernel(const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin, int64_t n,
                                  int shift, int ntiles, const uint64_t *__restrict__ offs,
                                  uint64_t *__restrict__ kout, uint32_t *__restrict__ vout) {
  __shared__ uint32_t wcnt[RS_THREADS / 32][256];
  __shared__ uint32_t wpre[RS_THREADS / 32][256];
  __shared__ uint32_t running[256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  running[tid] = 0;
  for (int w = 0; w < RS_THREADS / 32; ++w) wcnt[w][tid] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  const uint64_t my_off = offs[(int64_t)tid * ntiles + blockIdx.x];   // digit tid of this tile
  __shared__ uint64_t goff[256];
  goff[tid] = my_off;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < RS_ITEMS; ++r) {
    const int64_t e = base + (int64_t)r * RS_THREADS + tid;
    const bool valid = e < n;
    uint64_t k = 0;
    uint32_t v = 0;
    uint32_t d = 256;   // sentinel digit for invalid lanes
    if (valid) {
      k = kin[e];
      v = vin[e];
      d = (uint32_t)((k >> shift) & 255u);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lt);
    const bool leader = (peers & lt) == 0;
    if (valid && leader) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    {   // thread tid owns digit tid: prefix over warps in warp order
      uint32_t run = running[tid];
      for (int w = 0; w < RS_THREADS / 32; ++w) {
        wpre[w][tid] = run;
        run += wcnt[w][tid];
        wcnt[w][tid] = 0;
      }
      running[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const uint64_t pos = goff[d] + wpre[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------------------
// Per-mode compressed layout.
// ----------------------------------------------------------------------------------------
struct ModeLayout {
  int mode = 0;
  int64_t rows = 0;
  int64_t *ptr = nullptr;      // [rows + 1]
  int32_t *oidx = nullptr;     // [N-1][nnz] other-mode indices (modes in increasing order)
  float *vals = nullptr;       // [nnz]
  uint32_t *perm = nullptr;    // [nnz] input position of each sorted entry
};

struct KeyArgs {
  const int32_t *idx;  // [N][nnz]
  int64_t nnz;
  int N, mode;
  uint64_t stride[PTG_MAX_ORDER];   // of the other modes (0 for `mode`)
  uint64_t J;
};

__global__ void make_keys_kernel(KeyArgs a, uint64_t *__restrict__ keys, uint32_t *__restrict__ pos) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.nnz; e += (int64_t)gridDim.x * blockDim.x) {
    uint64_t lin = 0;
    for (int k = 0; k < a.N; ++k)
      if (k != a.mode) lin += (uint64_t)a.idx[(int64_t)k * a.nnz + e] * a.stride[k];
    keys[e] = (uint64_t)a.idx[(int64_t)a.mode * a.nnz + e] * a.J + lin;
    pos[e] = (uint32_t)e;
  }
}

struct GatherArgs {
  const int32_t *idx;
  const float *vals;
  int64_t nnz;
  int N, mode;
  const uint32_t *perm;
  int32_t *oidx;
  float *ovals;
};

__global__ void gather_mode_kernel(GatherArgs a) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.nnz; s += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t e = a.perm[s];
    int j = 0;
    for (int k = 0; k < a.N; ++k) {
      if (k == a.mode) continue;
      a.oidx[(int64_t)j * a.nnz + s] = a.idx[(int64_t)k * a.nnz + e];
      ++j;
    }
    a.ovals[s] = a.vals[e];
  }
}

// row pointers: ptr[i] = first sorted position with key >= i * J (binary search)
__global__ void row_ptr_kernel(const uint64_t *__restrict__ keys, int64_t nnz, uint64_t J, int64_t rows,
                               int64_t *__restrict__ ptr) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= rows; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t target = (uint64_t)i * J;
    int64_t lo = 0, hi = nnz;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < target) lo = mid + 1; else hi = mid;
    }
    ptr[i] = lo;
  }
}

__global__ void count_dups_kernel(const uint64_t *__restrict__ keys, int64_t nnz, unsigned long long *dups) {
  unsigned long long c = 0;
  for (int64_t s = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnz; s += (int64_t)gridDim.x * blockDim.x)
    c += keys[s] == keys[s - 1];
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(dups, c);   // count only: not on the data path
}

// ----------------------------------------------------------------------------------------
// Per-row solvers.
// ----------------------------------------------------------------------------------------
constexpr int GT_THREADS = 128;
constexpr int GT_CHUNK = 64;    // entries gathered per chunk
constexpr int GT_MAXR = 64;

struct RowArgs {
  const int64_t *ptr;
  const int32_t *oidx;     // [N-1][nnz]
  const float *vals;
  int64_t nnz;
  int N, mode, R;
  const float *fac[PTG_MAX_ORDER];   // row-major [I_k][R], the other modes in increasing order
  float *A;                // factor being updated, row-major [I_mode][R]
  float lambda;
  int max_iter;
  // stochastic
  int stochastic;
  float c;
  unsigned long long seed;
  int outer;
  // cost
  double *row_cost;        // optional: per-row sum of squared residuals with the new row
  int ridge;               // 1: unconstraint_update, a_i = (H_i + lambda I)^{-1} m_i
  int *err;                // device error word (a non-positive pivot in the ridge solve)
  int tc;                  // warp solver: H_i on the tensor cores (TF32, three-term split)
};

// Hadamard of the other modes' factor rows for entry s, multiplied from the last mode down
// (the order of include/MTTKRP.hpp:248-259).
__device__ __forceinline__ float kr_value(const RowArgs &a, int64_t s, int r) {
  float v = 1.0f;
  for (int j = a.N - 2; j >= 0; --j) {
    const int32_t row = a.oidx[(int64_t)j * a.nnz + s];
    v *= __ldg(a.fac[j] + (size_t)row * a.R + r);
  }
  return v;
}

__device__ unsigned long long splitmix_draw(unsigned long long seed, unsigned long long outer, unsigned long long mode,
                                            unsigned long long inner, unsigned long long row) {
  unsigned long long z = seed * 0x9E3779B97F4A7C15ull + outer * 0xBF58476D1CE4E5B9ull +
                         mode * 0x94D049BB133111EBull + inner * 0x2545F4914F6CDD1Dull + row * 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct RowShared {
  float kr[GT_CHUNK][GT_MAXR];
  float xv[GT_CHUNK];
  int32_t rows[PTG_MAX_ORDER - 1][GT_CHUNK];   // the chunk's entries' rows in the other modes
  float H[GT_MAXR][GT_MAXR + 1];
  float m[GT_MAXR];
  float x[GT_MAXR], xn[GT_MAXR];
  float a[GT_MAXR], y[GT_MAXR], a0[GT_MAXR];
  float red[GT_THREADS / 32];
};

// Register tiles of 2 x 4 entries of H over Rp x Rp (Rp = R rounded up to 4): per entry a
// thread reads 2 + 4 values of the entry's Khatri-Rao row and does 8 FMAs.
constexpr int GT_MAXTILES = (GT_MAXR / 2) * (GT_MAXR / 4) / GT_THREADS;   // 4 at R = 64

__device__ __forceinline__ void tiles_zero(float (*acc)[8]) {
#pragma unroll
  for (int q = 0; q < GT_MAXTILES; ++q)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[q][j] = 0.0f;
}

// acc += sum over the chunk's entries [0, cnt) of kr kr^T; m += sum x kr (threads < R)
__device__ void accumulate_chunk(RowShared &sh, int cnt, int R, float (*acc)[8], float &macc) {
  const int Rp = (R + 3) & ~3;
  const int tc = Rp / 4, ntile = (Rp / 2) * tc;
#pragma unroll
  for (int q = 0; q < GT_MAXTILES; ++q) {
    const int t = threadIdx.x + q * GT_THREADS;
    if (t < ntile) {
      const int r1 = (t / tc) * 2, r2 = (t % tc) * 4;
      for (int c = 0; c < cnt; ++c) {
        const float2 u = *reinterpret_cast<const float2 *>(&sh.kr[c][r1]);
        const float4 v = *reinterpret_cast<const float4 *>(&sh.kr[c][r2]);
        acc[q][0] = fmaf(u.x, v.x, acc[q][0]);
        acc[q][1] = fmaf(u.x, v.y, acc[q][1]);
        acc[q][2] = fmaf(u.x, v.z, acc[q][2]);
        acc[q][3] = fmaf(u.x, v.w, acc[q][3]);
        acc[q][4] = fmaf(u.y, v.x, acc[q][4]);
        acc[q][5] = fmaf(u.y, v.y, acc[q][5]);
        acc[q][6] = fmaf(u.y, v.z, acc[q][6]);
        acc[q][7] = fmaf(u.y, v.w, acc[q][7]);
      }
    }
  }
  if ((int)threadIdx.x < R)
    for (int c = 0; c < cnt; ++c) macc = fmaf(sh.xv[c], sh.kr[c][threadIdx.x], macc);
}

__device__ void tiles_store(RowShared &sh, int R, float (*acc)[8], float macc) {
  const int Rp = (R + 3) & ~3;
  const int tc = Rp / 4, ntile = (Rp / 2) * tc;
#pragma unroll
  for (int q = 0; q < GT_MAXTILES; ++q) {
    const int t = threadIdx.x + q * GT_THREADS;
    if (t < ntile) {
      const int r1 = (t / tc) * 2, r2 = (t % tc) * 4;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int a = r1 + j / 4, b = r2 + j % 4;
        if (a < R && b < R) sh.H[a][b] = acc[q][j];
      }
    }
  }
  if ((int)threadIdx.x < R) sh.m[threadIdx.x] = macc;
}

// Stage a chunk of entries: their rows in the other modes and values, then each entry's
// Khatri-Rao row (the product from the last mode down, as kr_value), zero beyond R.  The row
// indices go through shared memory first, so that the factor loads of a chunk are independent
// and in flight together (float4s where R is a multiple of 4).  Ends with a CTA barrier.
__device__ void load_chunk(const RowArgs &a, RowShared &sh, int64_t s0, int cnt) {
  const int R = a.R, Rp = (R + 3) & ~3, nj = a.N - 1;
  for (int idx = threadIdx.x; idx < cnt * nj; idx += GT_THREADS) {
    const int j = idx / cnt, c = idx - j * cnt;
    sh.rows[j][c] = a.oidx[(int64_t)j * a.nnz + s0 + c];
  }
  for (int c = threadIdx.x; c < cnt; c += GT_THREADS) sh.xv[c] = a.vals[s0 + c];
  __syncthreads();
  if ((R & 3) == 0) {
    const int q4 = R >> 2;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < cnt * q4; idx += GT_THREADS) {
      const int c = idx / q4, r4 = (idx - c * q4) * 4;
      float4 v = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
#pragma unroll
      for (int j = PTG_MAX_ORDER - 2; j >= 0; --j) {
        if (j < nj) {
          const float4 f = __ldg(reinterpret_cast<const float4 *>(a.fac[j] + (size_t)sh.rows[j][c] * R + r4));
          v.x *= f.x;
          v.y *= f.y;
          v.z *= f.z;
          v.w *= f.w;
        }
      }
      *reinterpret_cast<float4 *>(&sh.kr[c][r4]) = v;
    }
  } else {
#pragma unroll 4
    for (int idx = threadIdx.x; idx < cnt * Rp; idx += GT_THREADS) {
      const int c = idx / Rp, r = idx - c * Rp;
      float v = 0.0f;
      if (r < R) {
        v = 1.0f;
#pragma unroll
        for (int j = PTG_MAX_ORDER - 2; j >= 0; --j)
          if (j < nj) v *= __ldg(a.fac[j] + (size_t)sh.rows[j][c] * R + r);
      }
      sh.kr[c][r] = v;
    }
  }
  __syncthreads();
}

// Power method of include/NesterovMNLS.hpp:131-160 on sh.H from the all-ones vector, by warp 0.
__device__ float power_method_warp(RowShared &sh, int R, float eps) {
  const int lane = threadIdx.x & 31;
  for (int r = lane; r < R; r += 32) sh.x[r] = 1.0f;
  __syncwarp();
  float lam = 0.0f;
  for (int it = 0;; ++it) {
    float ax[2] = {0.f, 0.f};
    float nrm2 = 0.0f;
    for (int q = 0; q < 2; ++q) {
      const int r = lane + 32 * q;
      if (r < R) {
        float s = 0.f;
        for (int c = 0; c < R; ++c) s = fmaf(sh.H[r][c], sh.x[c], s);
        ax[q] = s;
        nrm2 += s * s;
      }
    }
    for (int o = 16; o > 0; o >>= 1) nrm2 += __shfl_xor_sync(0xffffffffu, nrm2, o);
    const float inv = 1.0f / (sqrtf(nrm2) + 1e-12f);
    float d2 = 0.0f;
    for (int q = 0; q < 2; ++q) {
      const int r = lane + 32 * q;
      if (r < R) {
        const float xn = __fmul_rn(ax[q], inv);   // kept out of an FMA with the difference
        const float df = xn - sh.x[r];
        d2 += df * df;
        sh.xn[r] = xn;
      }
    }
    for (int o = 16; o > 0; o >>= 1) d2 += __shfl_xor_sync(0xffffffffu, d2, o);
    __syncwarp();
    if (sqrtf(d2) <= eps || it >= 10000) {
      float q2 = 0.0f;
      for (int q = 0; q < 2; ++q) {
        const int r = lane + 32 * q;
        if (r < R) {
          float s = 0.f;
          for (int c = 0; c < R; ++c) s = fmaf(sh.H[r][c], sh.xn[c], s);
          q2 += sh.xn[r] * s;
        }
      }
      for (int o = 16; o > 0; o >>= 1) q2 += __shfl_xor_sync(0xffffffffu, q2, o);
      lam = q2;
      break;
    }
    for (int r = lane; r < R; r += 32) sh.x[r] = sh.xn[r];
    __syncwarp();
  }
  return lam;
}

// unconstraint_update (include/Gtc.hpp:275-315) by warp 0: sh.a = (H + lambda I)^{-1} m through
// a Cholesky factorisation in place in the lower triangle of sh.H (FP32; lambda > 0 keeps the
// system positive definite), then the two triangular solves.
__device__ void ridge_solve_warp(RowShared &sh, int R, float lam, int *err) {
  const int lane = threadIdx.x & 31;
  bool bad = false;
  for (int j = 0; j < R; ++j) {
    float s = 0.0f;
    for (int k = lane; k < j; k += 32) s = fmaf(sh.H[j][k], sh.H[j][k], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float d2 = sh.H[j][j] + lam - s;
    bad |= !(d2 > 0.0f);
    const float d = sqrtf(fmaxf(d2, 1e-30f));
    __syncwarp();
    for (int i = j + 1 + lane; i < R; i += 32) {
      float t = sh.H[i][j];
      for (int k = 0; k < j; ++k) t = fmaf(-sh.H[i][k], sh.H[j][k], t);
      sh.H[i][j] = t / d;
    }
    if (lane == 0) sh.H[j][j] = d;
    __syncwarp();
  }
  // L y = m (y in sh.y), then L^T a = y
  for (int i = 0; i < R; ++i) {
    float s = 0.0f;
    for (int k = lane; k < i; k += 32) s = fmaf(sh.H[i][k], sh.y[k], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sh.y[i] = (sh.m[i] - s) / sh.H[i][i];
    __syncwarp();
  }
  for (int i = R - 1; i >= 0; --i) {
    float s = 0.0f;
    for (int k = i + 1 + lane; k < R; k += 32) s = fmaf(sh.H[k][i], sh.a[k], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sh.a[i] = (sh.y[i] - s) / sh.H[i][i];
    __syncwarp();
  }
  if (bad && lane == 0) atomicExch(err, PTG_ERR_NUMERIC);
}

// The scalar parts of one projected Nesterov step (include/NesterovMNLS.hpp:525-539, :855-864), with
// explicit FMAs so that the one-CTA and the one-warp row kernels round them alike.
__device__ __forceinline__ float step_grad0(float m, float lam, float y, float prox, float a) {
  return fmaf(lam, fmaf(prox, a, y), -m);   // -m + lambda (y + prox a)
}
__device__ __forceinline__ float step_project(float y, float invL, float g) { return fmaxf(fmaf(-invL, g, y), 0.0f); }
__device__ __forceinline__ float step_extrapolate(float beta, float na, float a) {
  return fmaf(1.0f + beta, na, -(beta * a));
}
__device__ __forceinline__ void step_constants(float lmax, float lam, float &invL, float &beta) {
  invL = 1.0f / (lmax + lam);
  const float sq = sqrtf(lam * invL);
  beta = (1.0f - sq) / (1.0f + sq);
}

// One projected Nesterov step of warp 0: grad = H y - m + lambda * (y + prox * a_prev)
__device__ void nesterov_step_warp(RowShared &sh, int R, float lam, float invL, float beta, float prox) {
  const int lane = threadIdx.x & 31;
  float na[2];
  for (int q = 0; q < 2; ++q) {
    const int r = lane + 32 * q;
    na[q] = 0.f;
    if (r < R) {
      float g = step_grad0(sh.m[r], lam, sh.y[r], prox, sh.a[r]);
      for (int c = 0; c < R; ++c) g = fmaf(sh.H[r][c], sh.y[c], g);
      na[q] = step_project(sh.y[r], invL, g);
    }
  }
  __syncwarp();
  for (int q = 0; q < 2; ++q) {
    const int r = lane + 32 * q;
    if (r < R) {
      sh.y[r] = step_extrapolate(beta, na[q], sh.a[r]);
      sh.a[r] = na[q];
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(GT_THREADS) gtc_row_kernel(const RowArgs a) {
  extern __shared__ __align__(16) unsigned char gsm[];
  RowShared &sh = *reinterpret_cast<RowShared *>(gsm);
  const int64_t i = blockIdx.x;
  const int64_t p0 = a.ptr[i], p1 = a.ptr[i + 1];
  const int64_t cnt_row = p1 - p0;
  const int R = a.R, tid = threadIdx.x;
  for (int r = tid; r < R; r += GT_THREADS) {
    sh.a[r] = a.A[i * R + r];
    sh.y[r] = sh.a[r];
  }
  if (!a.stochastic) {
    // ---- local_L::NesterovMNLS: H_i, m_i over all entries, then max_iter steps ----
    float acc[GT_MAXTILES][8];
    float macc = 0.0f;
    tiles_zero(acc);
    __syncthreads();
    for (int64_t s0 = p0; s0 < p1; s0 += GT_CHUNK) {
      const int cnt = (int)(p1 - s0 < GT_CHUNK ? p1 - s0 : GT_CHUNK);
      load_chunk(a, sh, s0, cnt);
      accumulate_chunk(sh, cnt, R, acc, macc);
      __syncthreads();
    }
    tiles_store(sh, R, acc, macc);
    __syncthreads();
    if (a.ridge) {
      if (tid < 32) ridge_solve_warp(sh, R, a.lambda, a.err);   // an empty row gives a_i = 0
    } else if (tid < 32 && cnt_row > 0) {
      float invL, beta;
      step_constants(power_method_warp(sh, R, 1e-3f), a.lambda, invL, beta);
      for (int it = 0; it < a.max_iter; ++it) nesterov_step_warp(sh, R, a.lambda, invL, beta, 0.0f);
    } else if (tid < 32) {
      // an empty row: H = 0, m = 0, L = lambda; the steps only shrink the row
      float invL, beta;
      step_constants(0.0f, a.lambda, invL, beta);
      for (int it = 0; it < a.max_iter; ++it) nesterov_step_warp(sh, R, a.lambda, invL, beta, 0.0f);
    }
  } else {
    // ---- dynamic_blocksize::StochasticNesterovMNLS ----
    const int64_t b = (int64_t)(a.c * (float)cnt_row);   // floor(c * nnz_i)
    if (b > 0) {
      for (int it = 0; it < a.max_iter; ++it) {
        const unsigned long long draw = splitmix_draw(a.seed, (unsigned long long)a.outer,
                                                      (unsigned long long)a.mode, (unsigned long long)it,
                                                      (unsigned long long)i);
        const int64_t pivot = (int64_t)(draw % (unsigned long long)(cnt_row - b + 1));
        float acc[GT_MAXTILES][8];
        float macc = 0.0f;
        tiles_zero(acc);
        __syncthreads();
        for (int64_t s0 = p0 + pivot; s0 < p0 + pivot + b; s0 += GT_CHUNK) {
          const int cnt = (int)(p0 + pivot + b - s0 < GT_CHUNK ? p0 + pivot + b - s0 : GT_CHUNK);
          load_chunk(a, sh, s0, cnt);
          accumulate_chunk(sh, cnt, R, acc, macc);
          __syncthreads();
        }
        tiles_store(sh, R, acc, macc);
        __syncthreads();
        if (tid < 32) {
          // grad = sum (kr.y - x) kr + lambda (y + a) = H y - m + lambda (y + a)  (:516, :525)
          float invL, beta;
          step_constants(power_method_warp(sh, R, 1e-3f), a.lambda, invL, beta);
          nesterov_step_warp(sh, R, a.lambda, invL, beta, 1.0f);
        }
        __syncthreads();
      }
    }
  }
  __syncthreads();
  for (int r = tid; r < R; r += GT_THREADS) a.A[i * R + r] = sh.a[r];
  if (a.row_cost) {
    // sum over the row's entries of (x - <kr, a_i>)^2 in FP64, in entry order per thread,
    // then a fixed-order block reduction
    double s = 0.0;
    for (int64_t e = p0 + tid; e < p1; e += GT_THREADS) {
      float pred = 0.0f;
      for (int r = 0; r < R; ++r) pred = fmaf(kr_value(a, e, r), sh.a[r], pred);
      const double d = (double)a.vals[e] - (double)pred;
      s = fma(d, d, s);
    }
    __shared__ double dred[GT_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((tid & 31) == 0) dred[tid >> 5] = s;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < GT_THREADS / 32; ++w) t += dred[w];
      a.row_cost[i] = t;
    }
  }
}

// ---- one warp per row (rank <= 32): both Nesterov forms of the nonnegative modes ----
// The one-CTA kernel keeps three of its four warps waiting at barriers while warp 0 runs the
// power method and the steps.  Here each warp owns a row: lane r holds row r of the sampled H_i
// in registers (H is symmetric, so it is also column r), m_i[r], a_i[r] and the extrapolated
// y[r]; a vector every lane needs (a Khatri-Rao row, the power iterate, y) passes through the
// warp's own shared-memory slots, and only __syncwarp orders them.  The arithmetic and its
// order are those of the one-CTA kernel, so the two give the same bits.  72 registers (7 CTAs,
// 28 warps per SM, a few bytes spilled) measured faster than 64 (8 CTAs, more spilled) and than
// 92 without spills (5 CTAs).
constexpr int GW_WARPS = 4;
constexpr int GW_CHUNK = 32;

constexpr int GW_KRS = 40;   // row stride of the Khatri-Rao staging: 16-byte rows, and the MMA
                             // fragments' reads (rows t, t + 4; columns g) fall in distinct banks

struct WarpRowShared {
  float kr[GW_CHUNK][GW_KRS];   // one entry's Khatri-Rao row per row; after a block, H_i by rows
  float xv[GW_CHUNK];
  float v[32];
  int32_t rows[PTG_MAX_ORDER - 1][GW_CHUNK];
};

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// s + (H v)[lane], the products added in increasing column order
__device__ __forceinline__ float row_dot(const float (&H)[32], const float *v, float s) {
  const float4 *v4 = reinterpret_cast<const float4 *>(v);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 t = v4[q];
    s = fmaf(H[4 * q], t.x, s);
    s = fmaf(H[4 * q + 1], t.y, s);
    s = fmaf(H[4 * q + 2], t.z, s);
    s = fmaf(H[4 * q + 3], t.w, s);
  }
  return s;
}

// power_method_warp with the matrix in the lanes' registers
__device__ __forceinline__ float power_method_lane(const float (&H)[32], float *v, bool own, float eps) {
  const int lane = threadIdx.x & 31;
  float x = own ? 1.0f : 0.0f;
  v[lane] = x;
  __syncwarp();
  for (int it = 0;; ++it) {
    const float s = row_dot(H, v, 0.0f);
    const float nrm2 = warp_sum(s * s);
    const float inv = 1.0f / (sqrtf(nrm2) + 1e-12f);
    const float xn = __fmul_rn(s, inv);
    const float df = xn - x;
    const float d2 = warp_sum(df * df);
    __syncwarp();
    v[lane] = xn;
    __syncwarp();
    if (sqrtf(d2) <= eps || it >= 10000) {
      const float q2 = warp_sum(xn * row_dot(H, v, 0.0f));
      __syncwarp();
      return q2;
    }
    x = xn;
  }
}

// NJ = order - 1 other modes; VEC: R is a multiple of 4, so every factor row starts on a
// 16-byte boundary and 8 lanes gather one entry's Khatri-Rao row as float4s (4 entries per
// warp instruction); otherwise lane r gathers rank r of one entry at a time.
// H_i = sum kr kr^T and m_i = sum x kr over the entries [s1, s1 + nb) of a row, by one warp.
// Lane (rg, cg) = (lane / 4, lane % 4) accumulates the 4 x 8 block of H_i at rows 4 rg..,
// columns 8 cg..: 3 float4 reads per entry for 32 FMAs, where a whole row per lane needs 8
// broadcast reads and shared memory, not the FMA pipe, sets the pace.  On return lane r holds
// row r of H_i in H (through the staging buffer) and m_i[r] in m.
template <int NJ, bool VEC>
__device__ __forceinline__ void warp_row_hessian(const RowArgs &a, WarpRowShared &sh, int64_t s1, int64_t nb,
                                                 float (&H)[32], float &m) {
  const int lane = threadIdx.x & 31, R = a.R;
  const bool own = lane < R;
  const int rg = lane >> 2, cg = lane & 3;
  float Hb[4][8];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 8; ++j) Hb[k][j] = 0.0f;
  float m4[4] = {0.0f, 0.0f, 0.0f, 0.0f};   // m_i at rows 4 rg.. (the 4 lanes of a row group alike)
  for (int64_t s0 = s1; s0 < s1 + nb; s0 += GW_CHUNK) {
    const int cnt = (int)(s1 + nb - s0 < GW_CHUNK ? s1 + nb - s0 : GW_CHUNK);
    // lane e reads entry e's rows in the other modes and its value
    if (lane < cnt) {
#pragma unroll
      for (int j = 0; j < NJ; ++j) sh.rows[j][lane] = a.oidx[(int64_t)j * a.nnz + s0 + lane];
      sh.xv[lane] = a.vals[s0 + lane];
    }
    __syncwarp();
    // each entry's Khatri-Rao row, the product taken from the last mode down (kr_value);
    // ranks >= R are zero
    if (VEC) {
      const int sub = lane >> 3, r4 = (lane & 7) * 4;
#pragma unroll 2
      for (int e = sub; e < cnt; e += 4) {
        float4 kv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (r4 < R) {
          kv = __ldg(reinterpret_cast<const float4 *>(a.fac[NJ - 1] + (size_t)sh.rows[NJ - 1][e] * R + r4));
#pragma unroll
          for (int j = NJ - 2; j >= 0; --j) {
            const float4 f = __ldg(reinterpret_cast<const float4 *>(a.fac[j] + (size_t)sh.rows[j][e] * R + r4));
            kv.x *= f.x;
            kv.y *= f.y;
            kv.z *= f.z;
            kv.w *= f.w;
          }
        }
        *reinterpret_cast<float4 *>(&sh.kr[e][r4]) = kv;
      }
    } else {
#pragma unroll 4
      for (int e = 0; e < cnt; ++e) {
        float kv = 0.0f;
        if (own) {
          kv = __ldg(a.fac[NJ - 1] + (size_t)sh.rows[NJ - 1][e] * R + lane);
#pragma unroll
          for (int j = NJ - 2; j >= 0; --j) kv *= __ldg(a.fac[j] + (size_t)sh.rows[j][e] * R + lane);
        }
        sh.kr[e][lane] = kv;
      }
    }
    __syncwarp();
#pragma unroll 2
    for (int e = 0; e < cnt; ++e) {
      const float4 ra = *reinterpret_cast<const float4 *>(&sh.kr[e][4 * rg]);
      const float rk[4] = {ra.x, ra.y, ra.z, ra.w};
      const float xe = sh.xv[e];
#pragma unroll
      for (int k = 0; k < 4; ++k) m4[k] = fmaf(xe, rk[k], m4[k]);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float4 cb = *reinterpret_cast<const float4 *>(&sh.kr[e][8 * cg + 4 * h]);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          Hb[k][4 * h] = fmaf(rk[k], cb.x, Hb[k][4 * h]);
          Hb[k][4 * h + 1] = fmaf(rk[k], cb.y, Hb[k][4 * h + 1]);
          Hb[k][4 * h + 2] = fmaf(rk[k], cb.z, Hb[k][4 * h + 2]);
          Hb[k][4 * h + 3] = fmaf(rk[k], cb.w, Hb[k][4 * h + 3]);
        }
      }
    }
    __syncwarp();
  }
  // H_i to one row per lane (row r in lane r) through the staging buffer
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int h = 0; h < 2; ++h)
      *reinterpret_cast<float4 *>(&sh.kr[4 * rg + k][8 * cg + 4 * h]) =
          make_float4(Hb[k][4 * h], Hb[k][4 * h + 1], Hb[k][4 * h + 2], Hb[k][4 * h + 3]);
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 t = *reinterpret_cast<const float4 *>(&sh.kr[lane][4 * q]);
    H[4 * q] = t.x;
    H[4 * q + 1] = t.y;
    H[4 * q + 2] = t.z;
    H[4 * q + 3] = t.w;
  }
  __syncwarp();   // the staging buffer is gathered into again by the next block
  m = cg == 0 ? m4[0] : cg == 1 ? m4[1] : cg == 2 ? m4[2] : m4[3];   // m_i[lane]
}

// x rounded to TF32 (nearest, ties away), as the bits an mma.sync .tf32 operand takes
__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// d += a b for one m16n8k8 tile (TF32 operands, FP32 accumulator)
__device__ __forceinline__ void mma_tf32_16x8x8(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// warp_row_hessian with H_i = K^T K on the tensor cores (R <= 32, R % 4 == 0): K is the block's
// entries x 32 Khatri-Rao rows staged in shared memory, eight entries per m16n8k8 step.  With
// g = lane / 4 and t = lane % 4, the A fragment of K^T's rows 16 mt.. (K[e0 + t][16 mt + g],
// K[e0 + t][16 mt + g + 8], K[e0 + t + 4][16 mt + g], K[e0 + t + 4][16 mt + g + 8]) also holds
// the B fragments of K's columns 16 mt.. and 16 mt + 8.., so eight shared loads feed the six
// tiles of the lower triangle's blocks (rows 0-15 x columns 0-15, rows 16-31 x columns 0-31);
// the block above the diagonal is their transpose.  Each product is the three-term split
// hi*hi + hi*lo + lo*hi of x = hi + lo (Markidis et al. 2018), so H_i keeps FP32 accuracy.
// m_i[lane] = sum x_e K[e][lane] stays on the FMA pipe.
template <int NJ>
__device__ __forceinline__ void warp_row_hessian_mma(const RowArgs &a, WarpRowShared &sh, int64_t s1, int64_t nb,
                                                     float (&H)[32], float &m) {
  const int lane = threadIdx.x & 31, R = a.R;
  const int g = lane >> 2, t = lane & 3;
  float acc[6][4];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
  float mv = 0.0f;
  for (int64_t s0 = s1; s0 < s1 + nb; s0 += GW_CHUNK) {
    const int cnt = (int)(s1 + nb - s0 < GW_CHUNK ? s1 + nb - s0 : GW_CHUNK);
    const int cnt8 = (cnt + 7) & ~7;
    if (lane < cnt) {
#pragma unroll
      for (int j = 0; j < NJ; ++j) sh.rows[j][lane] = a.oidx[(int64_t)j * a.nnz + s0 + lane];
      sh.xv[lane] = a.vals[s0 + lane];
    }
    __syncwarp();
    {   // each entry's Khatri-Rao row (the product from the last mode down); ranks >= R and the
        // rows that pad the chunk to a multiple of eight entries are zero
      const int sub = lane >> 3, r4 = (lane & 7) * 4;
#pragma unroll 2
      for (int e = sub; e < cnt8; e += 4) {
        float4 kv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (e < cnt && r4 < R) {
          kv = __ldg(reinterpret_cast<const float4 *>(a.fac[NJ - 1] + (size_t)sh.rows[NJ - 1][e] * R + r4));
#pragma unroll
          for (int j = NJ - 2; j >= 0; --j) {
            const float4 f = __ldg(reinterpret_cast<const float4 *>(a.fac[j] + (size_t)sh.rows[j][e] * R + r4));
            kv.x *= f.x;
            kv.y *= f.y;
            kv.z *= f.z;
            kv.w *= f.w;
          }
        }
        *reinterpret_cast<float4 *>(&sh.kr[e][r4]) = kv;
      }
    }
    __syncwarp();
    for (int e = 0; e < cnt; ++e) mv = fmaf(sh.xv[e], sh.kr[e][lane], mv);
    for (int e0 = 0; e0 < cnt8; e0 += 8) {
      uint32_t hi[2][4], lo[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const float x[4] = {sh.kr[e0 + t][16 * mt + g], sh.kr[e0 + t][16 * mt + g + 8], sh.kr[e0 + t + 4][16 * mt + g],
                            sh.kr[e0 + t + 4][16 * mt + g + 8]};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          hi[mt][i] = tf32_rna(x[i]);
          lo[mt][i] = tf32_rna(x[i] - __uint_as_float(hi[mt][i]));
        }
      }
      // tile (mt, nt): rows 16 mt.., columns 8 nt..; B of columns 8 nt.. is A fragment nt / 2's
      // elements (nt & 1, (nt & 1) + 2)
#pragma unroll
      for (int tile = 0; tile < 6; ++tile) {
        const int mt = tile < 2 ? 0 : 1, nt = tile < 2 ? tile : tile - 2;
        const int bm = nt >> 1, bh = nt & 1;
        mma_tf32_16x8x8(acc[tile], hi[mt], hi[bm][bh], hi[bm][bh + 2]);
        mma_tf32_16x8x8(acc[tile], hi[mt], lo[bm][bh], lo[bm][bh + 2]);
        mma_tf32_16x8x8(acc[tile], lo[mt], hi[bm][bh], hi[bm][bh + 2]);
      }
    }
    __syncwarp();   // the staging buffer is gathered into again by the next chunk
  }
  // H_i through the staging buffer: each tile's elements, and the transposes of the tiles
  // below the diagonal blocks; then lane r takes row r
#pragma unroll
  for (int tile = 0; tile < 6; ++tile) {
    const int mt = tile < 2 ? 0 : 1, nt = tile < 2 ? tile : tile - 2;
    const int r0 = 16 * mt + g, c0 = 8 * nt + 2 * t;
    sh.kr[r0][c0] = acc[tile][0];
    sh.kr[r0][c0 + 1] = acc[tile][1];
    sh.kr[r0 + 8][c0] = acc[tile][2];
    sh.kr[r0 + 8][c0 + 1] = acc[tile][3];
    if (mt == 1 && nt < 2) {
      sh.kr[c0][r0] = acc[tile][0];
      sh.kr[c0 + 1][r0] = acc[tile][1];
      sh.kr[c0][r0 + 8] = acc[tile][2];
      sh.kr[c0 + 1][r0 + 8] = acc[tile][3];
    }
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 v = *reinterpret_cast<const float4 *>(&sh.kr[lane][4 * q]);
    H[4 * q] = v.x;
    H[4 * q + 1] = v.y;
    H[4 * q + 2] = v.z;
    H[4 * q + 3] = v.w;
  }
  __syncwarp();
  m = mv;
}

// one projected Nesterov step of this lane's column: grad = H y - m + lambda (y + prox a)
__device__ __forceinline__ void warp_row_step(const float (&H)[32], float *v, float m, bool own, float lam,
                                              float invL, float beta, float prox, float &av, float &yv) {
  const int lane = threadIdx.x & 31;
  v[lane] = yv;
  __syncwarp();
  const float g = row_dot(H, v, step_grad0(m, lam, yv, prox, av));
  const float na = own ? step_project(yv, invL, g) : 0.0f;
  __syncwarp();
  yv = step_extrapolate(beta, na, av);
  av = na;
}

// STOCH: dynamic_blocksize::StochasticNesterovMNLS, a fresh sampled block per inner step;
// else local_L::NesterovMNLS, H_i over all the row's entries, then max_iter steps
// (nonnegative modes; the ridge solve of unconstrained modes stays on the one-CTA kernel).
template <int NJ, bool VEC, bool STOCH, bool MMA = false>
__global__ void __launch_bounds__(GW_WARPS * 32, MMA ? 6 : 7) gtc_warp_kernel(const RowArgs a, int64_t rows) {
  __shared__ __align__(16) WarpRowShared shw[GW_WARPS];
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * GW_WARPS + (threadIdx.x >> 5);
  if (i >= rows) return;   // whole warps leave: the kernel has no CTA-wide barrier
  WarpRowShared &sh = shw[threadIdx.x >> 5];
  const int R = a.R;
  const bool own = lane < R;
  const int64_t p0 = a.ptr[i], cnt_row = a.ptr[i + 1] - p0;
  float av = own ? a.A[i * R + lane] : 0.0f;
  float yv = av;
  float H[32], m;
  if (STOCH) {
    const int64_t b = (int64_t)(a.c * (float)cnt_row);   // floor(c * nnz_i)
    if (b > 0) {
      for (int it = 0; it < a.max_iter; ++it) {
        const unsigned long long draw = splitmix_draw(a.seed, (unsigned long long)a.outer,
                                                      (unsigned long long)a.mode, (unsigned long long)it,
                                                      (unsigned long long)i);
        const int64_t s1 = p0 + (int64_t)(draw % (unsigned long long)(cnt_row - b + 1));
        if constexpr (MMA) warp_row_hessian_mma<NJ>(a, sh, s1, b, H, m);
        else warp_row_hessian<NJ, VEC>(a, sh, s1, b, H, m);
        float invL, beta;
        step_constants(power_method_lane(H, sh.v, own, 1e-3f), a.lambda, invL, beta);
        // grad = sum (kr.y - x) kr + lambda (y + a) = H y - m + lambda (y + a)
        // (include/NesterovMNLS.hpp:516, :525)
        warp_row_step(H, sh.v, m, own, a.lambda, invL, beta, 1.0f, av, yv);
      }
    }
  } else {
    if constexpr (MMA) warp_row_hessian_mma<NJ>(a, sh, p0, cnt_row, H, m);   // an empty row: H = 0, m = 0
    else warp_row_hessian<NJ, VEC>(a, sh, p0, cnt_row, H, m);
    float invL, beta;
    step_constants(cnt_row > 0 ? power_method_lane(H, sh.v, own, 1e-3f) : 0.0f, a.lambda, invL, beta);
    for (int it = 0; it < a.max_iter; ++it) warp_row_step(H, sh.v, m, own, a.lambda, invL, beta, 0.0f, av, yv);
  }
  if (own) a.A[i * R + lane] = av;
}

template <int NJ>
void launch_warp_rows_nj(const RowArgs &a, int64_t rows, cudaStream_t S) {
  const unsigned grid = (unsigned)((rows + GW_WARPS - 1) / GW_WARPS);
  const bool vec = a.R % 4 == 0;
  if (a.stochastic) {
    if (vec && a.tc) gtc_warp_kernel<NJ, true, true, true><<<grid, GW_WARPS * 32, 0, S>>>(a, rows);
    else if (vec) gtc_warp_kernel<NJ, true, true><<<grid, GW_WARPS * 32, 0, S>>>(a, rows);
    else gtc_warp_kernel<NJ, false, true><<<grid, GW_WARPS * 32, 0, S>>>(a, rows);
  } else {
    if (vec && a.tc) gtc_warp_kernel<NJ, true, false, true><<<grid, GW_WARPS * 32, 0, S>>>(a, rows);
    else if (vec) gtc_warp_kernel<NJ, true, false><<<grid, GW_WARPS * 32, 0, S>>>(a, rows);
    else gtc_warp_kernel<NJ, false, false><<<grid, GW_WARPS * 32, 0, S>>>(a, rows);
  }
}

void launch_warp_rows(const RowArgs &a, int64_t rows, cudaStream_t S) {
  switch (a.N - 1) {
    case 1: launch_warp_rows_nj<1>(a, rows, S); break;
    case 2: launch_warp_rows_nj<2>(a, rows, S); break;
    case 3: launch_warp_rows_nj<3>(a, rows, S); break;
    case 4: launch_warp_rows_nj<4>(a, rows, S); break;
    case 5: launch_warp_rows_nj<5>(a, rows, S); break;
    case 6: launch_warp_rows_nj<6>(a, rows, S); break;
    default: launch_warp_rows_nj<7>(a, rows, S); break;
  }
}

// Cost of the current factors over one mode's entries (rows of that mode), per row.
__global__ void gtc_cost_rows_kernel(const RowArgs a) {
  const int64_t i = blockIdx.x;
  const int64_t p0 = a.ptr[i], p1 = a.ptr[i + 1];
  const int R = a.R, tid = threadIdx.x;
  __shared__ float arow[GT_MAXR];
  for (int r = tid; r < R; r += blockDim.x) arow[r] = a.A[i * R + r];
  __syncthreads();
  double s = 0.0;
  for (int64_t e = p0 + tid; e < p1; e += blockDim.x) {
    float pred = 0.0f;
    for (int r = 0; r < R; ++r) pred = fmaf(kr_value(a, e, r), arow[r], pred);
    const double d = (double)a.vals[e] - (double)pred;
    s = fma(d, d, s);
  }
  __shared__ double dred[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((tid & 31) == 0) dred[tid >> 5] = s;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += dred[w];
    a.row_cost[i] = t;
  }
}

__global__ void sum_rows_kernel(const double *__restrict__ v, int64_t n, double *out) {
  // one block; fixed order: thread-strided partials then a serial sum of the partials
  __shared__ double part[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) t += part[k];
    *out = t;
  }
}

__global__ void sumsq_kernel(const float *__restrict__ v, int64_t n, double *out) {
  __shared__ double part[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma((double)v[i], (double)v[i], s);
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) t += part[k];
    *out = t;
  }
}

int key_bits(uint64_t maxkey) {
  int b = 0;
  while (b < 64 && (maxkey >> b) != 0) ++b;
  return b;
}

}  // namespace

// Sort one mode: returns the permutation (sorted position -> input position) in perm and
// the sorted keys in keys_out.  All buffers are caller-provided device memory of nnz entries
// (two key buffers, two value buffers), counts/offsets of 256 * ceil(nnz / 4096) entries.
int gtc_sort_mode(ptg_ctx *ctx, int order, const int64_t *dims, int64_t nnz, const int32_t *idx, int mode,
                  uint64_t *keys_a, uint64_t *keys_b, uint32_t *vals_a, uint32_t *vals_b, uint32_t *counts,
                  uint64_t *offs, uint64_t *sums, uint64_t **keys_sorted, uint32_t **perm_sorted,
                  cudaStream_t stream) {
  KeyArgs ka{};
  ka.idx = idx;
  ka.nnz = nnz;
  ka.N = order;
  ka.mode = mode;
  uint64_t s = 1;
  for (int k = 0; k < order; ++k) {
    if (k == mode) continue;
    ka.stride[k] = s;
    s *= (uint64_t)dims[k];
  }
  ka.J = s;
  const uint64_t maxkey = (uint64_t)dims[mode] * s - 1;
  const int blocks = (int)std::min<int64_t>((nnz + 255) / 256, (int64_t)ctx->sm_count * 32);
  make_keys_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(ka, keys_a, vals_a);
  count_launches(ctx, 1);
  const int bits = key_bits(maxkey);
  const int ntiles = (int)((nnz + RS_TILE - 1) / RS_TILE);
  const int64_t m = (int64_t)256 * ntiles;
  const int nchunks = (int)((m + SCAN_CHUNK - 1) / SCAN_CHUNK);
  uint64_t *kin = keys_a, *kout = keys_b;
  uint32_t *vin = vals_a, *vout = vals_b;
  for (int shift = 0; shift < bits; shift += 8) {
    rs_hist_kernel<<<ntiles, RS_THREADS, 0, stream>>>(kin, nnz, shift, ntiles, counts);
    scan_block_sums_kernel<<<nchunks, 256, 0, stream>>>(counts, m, sums);
    scan_sums_kernel<<<1, 1024, 0, stream>>>(sums, nchunks);
    scan_apply_kernel<<<nchunks, 256, 0, stream>>>(counts, m, sums, offs);
    rs_scatter_kernel<<<ntiles, RS_THREADS, 0, stream>>>(kin, vin, nnz, shift, ntiles, offs, kout, vout);
    count_launches(ctx, 5);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  PTG_CUDA(cudaGetLastError());
  *keys_sorted = kin;
  *perm_sorted = vin;
  return PTG_OK;
}

}  // namespace ptg

using namespace ptg;

namespace {

struct GtcWork {
  std::vector<void *> allocs;
  ~GtcWork() {
    for (void *p : allocs) cudaFree(p);
  }
  template <typename T>
  int alloc(T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc(GTC)", __FILE__, __LINE__);
    allocs.push_back(q);
    *p = static_cast<T *>(q);
    return PTG_OK;
  }
};

}  // namespace

extern "C" {

void ptg_gtc_default_options(int order, ptg_gtc_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  for (int k = 0; k < PTG_MAX_ORDER; ++k) {
    o->constraints[k] = k < order ? PTG_NONNEGATIVITY : 0;
    o->lambdas[k] = 0.01;
  }
  o->threshold_error = 1e-3;
  o->max_nesterov_iter = 20;
  o->max_iter = 20;
  o->c_stochastic_perc = 0.5;
  o->stochastic = 0;
  o->seed = 0;
}

int ptg_gtc_sort_mode(ptg_ctx *ctx, int order, const int64_t *dims, int64_t nnz, const int32_t *idx_dev, int mode,
                      uint32_t *perm_out_dev) {
  if (!ctx || !dims || !idx_dev || !perm_out_dev) return set_error(PTG_ERR_INVALID, "NULL argument");
  if (order < 2 || order > PTG_MAX_ORDER || mode < 0 || mode >= order || nnz < 1 || nnz > 0xffffffffLL)
    return set_error(PTG_ERR_INVALID, "bad order, mode or nnz");
  PTG_CUDA(cudaSetDevice(ctx->device));
  GtcWork w;
  uint64_t *ka, *kb, *offs, *sums, *ks;
  uint32_t *va, *vb, *counts, *ps;
  const int ntiles = (int)((nnz + RS_TILE - 1) / RS_TILE);
  const int64_t m = (int64_t)256 * ntiles;
  PTG_TRY(w.alloc(&ka, nnz));
  PTG_TRY(w.alloc(&kb, nnz));
  PTG_TRY(w.alloc(&va, nnz));
  PTG_TRY(w.alloc(&vb, nnz));
  PTG_TRY(w.alloc(&counts, m));
  PTG_TRY(w.alloc(&offs, m));
  PTG_TRY(w.alloc(&sums, (m + SCAN_CHUNK - 1) / SCAN_CHUNK));
  PTG_TRY(gtc_sort_mode(ctx, order, dims, nnz, idx_dev, mode, ka, kb, va, vb, counts, offs, sums, &ks, &ps,
                        ctx->stream));
  PTG_CUDA(cudaMemcpyAsync(perm_out_dev, ps, sizeof(uint32_t) * nnz, cudaMemcpyDeviceToDevice, ctx->stream));
  PTG_CUDA(cudaStreamSynchronize(ctx->stream));
  return PTG_OK;
}

int ptg_gtc(ptg_ctx *ctx, int order, const int64_t *dims, int64_t nnz, const int32_t *idx, const float *vals,
            int src_on_device, int rank, const ptg_gtc_options *opt, const double *const *init_factors,
            double *const *out_factors, ptg_gtc_result *result, ptg_sweep_trace *trace) {
  if (!ctx || !dims || !idx || !vals || !opt || !init_factors || !out_factors)
    return set_error(PTG_ERR_INVALID, "NULL argument");
  if (order < 3 || order > PTG_MAX_ORDER) return set_error(PTG_ERR_UNSUPPORTED, "GTC order must be in [3, 8]");
  if (rank < 1 || rank > GT_MAXR) return set_error(PTG_ERR_UNSUPPORTED, "GTC rank must be in [1, 64]");
  if (nnz < 1 || nnz > 0xffffffffLL) return set_error(PTG_ERR_INVALID, "nnz must be in [1, 2^32)");
  if (opt->max_iter < 1 || opt->max_nesterov_iter < 0) return set_error(PTG_ERR_INVALID, "bad iteration limits");
  for (int k = 0; k < order; ++k) {
    if (dims[k] < 1 || dims[k] > 0x7fffffffLL) return set_error(PTG_ERR_INVALID, "bad dimension");
    if (opt->constraints[k] < PTG_UNCONSTRAINED || opt->constraints[k] > PTG_CONSTANT)
      return set_error(PTG_ERR_UNSUPPORTED, "GTC: symmetric constraints are not implemented");
  }
  PTG_CUDA(cudaSetDevice(ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t S = ctx->stream;
  GtcWork w;
  const int N = order, R = rank;
  int32_t *d_idx;
  float *d_vals;
  if (src_on_device) {
    d_idx = const_cast<int32_t *>(idx);
    d_vals = const_cast<float *>(vals);
  } else {
    PTG_TRY(w.alloc(&d_idx, (size_t)N * nnz));
    PTG_TRY(w.alloc(&d_vals, nnz));
    PTG_CUDA(cudaMemcpyAsync(d_idx, idx, sizeof(int32_t) * N * nnz, cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaMemcpyAsync(d_vals, vals, sizeof(float) * nnz, cudaMemcpyHostToDevice, S));
  }
  // ---- per-mode sort and compressed layout ----
  const int ntiles = (int)((nnz + RS_TILE - 1) / RS_TILE);
  const int64_t m = (int64_t)256 * ntiles;
  uint64_t *ka, *kb, *offs, *sums;
  uint32_t *va, *vb, *counts;
  PTG_TRY(w.alloc(&ka, nnz));
  PTG_TRY(w.alloc(&kb, nnz));
  PTG_TRY(w.alloc(&va, nnz));
  PTG_TRY(w.alloc(&vb, nnz));
  PTG_TRY(w.alloc(&counts, m));
  PTG_TRY(w.alloc(&offs, m));
  PTG_TRY(w.alloc(&sums, (m + SCAN_CHUNK - 1) / SCAN_CHUNK));
  unsigned long long *d_dups;
  PTG_TRY(w.alloc(&d_dups, 1));
  PTG_CUDA(cudaMemsetAsync(d_dups, 0, sizeof(unsigned long long), S));
  std::vector<ModeLayout> lay(N);
  for (int n = 0; n < N; ++n) {
    uint64_t *ks;
    uint32_t *ps;
    PTG_TRY(gtc_sort_mode(ctx, N, dims, nnz, d_idx, n, ka, kb, va, vb, counts, offs, sums, &ks, &ps, S));
    ModeLayout &L = lay[n];
    L.mode = n;
    L.rows = dims[n];
    PTG_TRY(w.alloc(&L.ptr, dims[n] + 1));
    PTG_TRY(w.alloc(&L.oidx, (size_t)(N - 1) * nnz));
    PTG_TRY(w.alloc(&L.vals, nnz));
    uint64_t J = 1;
    for (int k = 0; k < N; ++k)
      if (k != n) J *= (uint64_t)dims[k];
    const int blocks = (int)std::min<int64_t>((nnz + 255) / 256, (int64_t)ctx->sm_count * 32);
    if (n == 0) {
      count_dups_kernel<<<std::max(blocks, 1), 256, 0, S>>>(ks, nnz, d_dups);
      count_launches(ctx, 1);
    }
    row_ptr_kernel<<<(int)((dims[n] + 1 + 255) / 256), 256, 0, S>>>(ks, nnz, J, dims[n], L.ptr);
    GatherArgs ga{d_idx, d_vals, nnz, N, n, ps, L.oidx, L.vals};
    gather_mode_kernel<<<std::max(blocks, 1), 256, 0, S>>>(ga);
    count_launches(ctx, 2);
    PTG_CUDA(cudaGetLastError());
  }
  unsigned long long h_dups = 0;
  PTG_CUDA(cudaMemcpyAsync(&h_dups, d_dups, sizeof(h_dups), cudaMemcpyDeviceToHost, S));
  PTG_CUDA(cudaStreamSynchronize(S));
  if (h_dups) return set_error(PTG_ERR_INVALID, "duplicate indices in the observed entries");
  const double setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  // ---- factors ----
  std::vector<float *> fac(N);
  std::vector<float> hb;
  for (int k = 0; k < N; ++k) {
    PTG_TRY(w.alloc(&fac[k], (size_t)dims[k] * R));
    hb.resize((size_t)dims[k] * R);
    for (int64_t i = 0; i < dims[k]; ++i)
      for (int r = 0; r < R; ++r) {
        const double v = init_factors[k][i + dims[k] * r];
        if (!std::isfinite(v)) return set_error(PTG_ERR_NUMERIC, "initial factor contains NaN or Inf");
        hb[(size_t)i * R + r] = (float)v;
      }
    PTG_CUDA(cudaMemcpyAsync(fac[k], hb.data(), sizeof(float) * hb.size(), cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaStreamSynchronize(S));
  }
  int64_t maxrows = 0;
  for (int k = 0; k < N; ++k) maxrows = std::max<int64_t>(maxrows, dims[k]);
  double *row_cost, *d_scal;
  PTG_TRY(w.alloc(&row_cost, maxrows));
  PTG_TRY(w.alloc(&d_scal, 2));
  sumsq_kernel<<<1, 256, 0, S>>>(lay[0].vals, nnz, d_scal);
  count_launches(ctx, 1);
  const int last = N - 1;
  auto make_args = [&](int n) {
    RowArgs a{};
    a.ptr = lay[n].ptr;
    a.oidx = lay[n].oidx;
    a.vals = lay[n].vals;
    a.nnz = nnz;
    a.N = N;
    a.mode = n;
    a.R = R;
    int j = 0;
    for (int k = 0; k < N; ++k)
      if (k != n) a.fac[j++] = fac[k];
    a.A = fac[n];
    a.lambda = (float)opt->lambdas[n];
    a.max_iter = opt->max_nesterov_iter;
    a.stochastic = opt->stochastic;
    a.c = (float)opt->c_stochastic_perc;
    a.seed = opt->seed;
    a.ridge = 0;
    a.err = ctx->dev_err;
    return a;
  };
  auto cost = [&](double *f) -> int {
    RowArgs a = make_args(last);
    a.row_cost = row_cost;
    gtc_cost_rows_kernel<<<(unsigned)dims[last], 128, 0, S>>>(a);
    sum_rows_kernel<<<1, 256, 0, S>>>(row_cost, dims[last], d_scal + 1);
    count_launches(ctx, 2);
    double h[2];
    PTG_CUDA(cudaMemcpyAsync(h, d_scal, sizeof(h), cudaMemcpyDeviceToHost, S));
    PTG_TRY(check_device_error(ctx));
    f[0] = h[0];
    f[1] = h[1];
    return PTG_OK;
  };
  const size_t smem = sizeof(RowShared);
  PTG_CUDA(cudaFuncSetAttribute(gtc_row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  double fr[2];
  PTG_TRY(cost(fr));
  const double frob = fr[0];
  double f = fr[1];
  double rel = f / frob;
  // stochastic epoch (include/GtcStochastic.hpp:431, :590)
  int epoch = 1;
  if (opt->stochastic) {
    const long long block0 = (long long)(opt->c_stochastic_perc * (double)nnz / (double)dims[0]) + 1;
    epoch = (int)(nnz / (block0 * dims[0])) + 1;
  }
  int ao_iter = 0, epochs = 0, ntr = 0;
  for (;;) {
    ++ao_iter;
    for (int n = 0; n < N; ++n) {
      // update_factor (include/Gtc.hpp:330-355; include/GtcStochastic.hpp:325-345): the full
      // form updates unconstrained modes by the ridge solve and nonnegative modes by local_L
      // Nesterov, the stochastic form only the nonnegative modes; every other mode is kept
      const int con = opt->constraints[n];
      const bool ridge = !opt->stochastic && con == PTG_UNCONSTRAINED;
      if (!ridge && con != PTG_NONNEGATIVITY) continue;
      RowArgs a = make_args(n);
      a.outer = ao_iter;
      a.ridge = ridge ? 1 : 0;
      // row solvers: 0 auto (one warp per row at R <= 32, H_i on the tensor cores where
      // R % 4 == 0), 1 one CTA per row, 2 one warp per row with H_i on the FMA pipe
      a.tc = ctx->gtc_rows == 0 ? 1 : 0;
      if (R <= 32 && !a.ridge && ctx->gtc_rows != 1)
        launch_warp_rows(a, dims[n], S);
      else
        gtc_row_kernel<<<(unsigned)dims[n], GT_THREADS, smem, S>>>(a);
      count_launches(ctx, 1);
      PTG_CUDA(cudaGetLastError());
    }
    bool evaluated = false;
    if (!opt->stochastic || ao_iter % epoch == 0) {
      ++epochs;
      PTG_TRY(cost(fr));
      f = fr[1];
      rel = f / frob;
      evaluated = true;
      if (!std::isfinite(f)) return set_error(PTG_ERR_NUMERIC, "GTC cost is NaN or Inf");
    }
    if (evaluated && trace && ntr < opt->max_iter) {
      ptg_sweep_trace tr{};
      tr.f_value = f;
      tr.rel_costFunction = rel;
      tr.seconds = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
      trace[ntr++] = tr;
    }
    const int count = opt->stochastic ? epochs : ao_iter;
    if (rel < opt->threshold_error || count >= opt->max_iter) break;
  }
  for (int k = 0; k < N; ++k) {
    hb.resize((size_t)dims[k] * R);
    PTG_CUDA(cudaMemcpyAsync(hb.data(), fac[k], sizeof(float) * hb.size(), cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    for (int64_t i = 0; i < dims[k]; ++i)
      for (int r = 0; r < R; ++r) out_factors[k][i + dims[k] * r] = (double)hb[(size_t)i * R + r];
  }
  if (result) {
    result->frob_tns = frob;
    result->f_value = f;
    result->rel_costFunction = rel;
    result->ao_iter = ao_iter;
    result->epochs = epochs;
    result->seconds_setup = setup_s;
    result->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return PTG_OK;
}

}  // extern "C"
