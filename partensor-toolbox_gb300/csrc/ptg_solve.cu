// Per-mode solver kernels of the CPD-ALS sweep.
//
//   eigen_bounds_kernel  FP64: Z = Hadamard of the Grams (include/PartialCwiseProd.hpp:54-222),
//                        its extreme eigenvalues (= singular values of the SPD Z,
//                        include/NesterovMNLS.hpp:45-52), GLambda (:75-91) and the beta
//                        sequence of UpdateAlpha (:103-113, :224-226).
//   nnls_cluster_kernel  the dense Nesterov MNLS (include/NesterovMNLS.hpp:181-234) over all
//                        rows of a factor on one thread-block cluster, with the global KKT
//                        stop test reduced through distributed shared memory, followed by the
//                        zero-column repair (include/Cpd.hpp:206-207), the Gram A^T A
//                        (include/Cpd.hpp:227) and the FP64 cost term <M, A>.
//   normalize_kernel     include/Normalize.hpp:92-174 (quirks included).
//   accel_combine_kernel A_acc = A_old + s (A - A_old)  (include/Cpd.hpp:257-261).
//   gram / cost-term kernels.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "ptg_internal.h"
#include "ptg_blockops.cuh"

namespace cg = cooperative_groups;

namespace ptg {

namespace {

__global__ void __launch_bounds__(kEigThreads)
eigen_bounds_kernel(GramPtrs gp, int order, int mode, int R, NnlsParams *out) {
  eigen_bounds_body<kEigThreads>(gp, order, mode, R, out, threadIdx.x);
}

// ------------------------------------------------------------------------------------
// Row-batched Nesterov MNLS on one cluster.
// ------------------------------------------------------------------------------------
// Warps per CTA of the NNLS cluster kernel (its template parameter W).  16 warps (512 threads,
// at most 128 registers each, a few spilled at 4+ rows per warp) measured faster than 8 warps
// without spills: 1000^3 BF16 solve 30.4 vs 30.8 ms.
constexpr int kNnlsWarpsLarge = 16;
constexpr int kNnlsWindowMax = 8;
constexpr int kNnlsMaxCluster = 16;   // the largest cluster the launch asks for

struct NnlsArgs {
  const float *M;        // [I][R]
  float *A;              // [I][R] in: prox centre / start, out: solution
  int I, R;
  const NnlsParams *np;
  float delta1, delta2;
  float *gram_out;       // [R][R]
  double *inner_MA;      // <M, A_new> (FP64)
  double *had_ZG;        // sum(Z .* G_new) (FP64)
  int *iters_out;
  int *repaired_out;
  // learned warm start (optional)
  const float *theta;    // MLP parameters: W1 [H][Din], b1, W2 [H][H], b2, W3 [R][H], b3
  int hidden;
  float *log_X;          // [I][R + 8] features of each row (optional)
  float *log_T;          // [I][R] solution scaled by L / ||m_i|| (optional)
  int window;            // iterations per cluster barrier, 1..kNnlsWindowMax (launch sets it)
};

template <int RB, int ROWS, int W>
__global__ void __launch_bounds__(W * 32, 1) nnls_cluster_kernel(const NnlsArgs a) {
  constexpr int kNnlsWarps = W;
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int R = a.R, I = a.I;

  extern __shared__ __align__(16) float sm[];
  float *Zt = sm;                                   // R*R
  const int KW = a.window;
  float *As = Zt + R * R;                           // KW slots of (kNnlsWarps*ROWS) x R: A_it per step
  const int aslot = kNnlsWarps * ROWS * R;
  float *Gp = As + KW * aslot;                      // R*R  (this CTA's partial Gram)
  float *colsum = Gp + R * R;                       // R
  float *slots = colsum + ((R + 1) & ~1);          // [2][2] stop test (max |g.y|, min g)
  float *wred = slots + 4;                          // kNnlsWarps * 2
  double *wredd = reinterpret_cast<double *>(wred + 2 * kNnlsWarps);   // kNnlsWarps
  double *ma = wredd + kNnlsWarps;                  // 1: this CTA's <M, A>
  int *flags = reinterpret_cast<int *>(ma + 2);     // [0]: repaired, [8..32): stop-test words
  float *bt = reinterpret_cast<float *>(flags + 8 + 3 * kNnlsWindowMax);   // kMaxInner: the beta sequence
  float *rsc = bt + kMaxInner;                      // kNnlsWarps*ROWS: row scales of the warm start
  // RB == 1 only: the warps' Y rows, (kNnlsWarps*ROWS) x 32, on a 16-byte boundary
  float *Ys = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(rsc + kNnlsWarps * ROWS) + 15) &
                                        ~(uintptr_t)15);

  const NnlsParams *np = a.np;
  const float L = (float)np->L, lam = (float)np->lambda;
  const float invL = 1.0f / L;
  for (int idx = tid; idx < R * R; idx += blockDim.x) {
    float z = (float)np->Z[idx];
    if (idx / R == idx % R) z += lam;               // Z~ = Z + lambda I   (:205)
    Zt[idx] = z;
  }
  for (int k = tid; k < kMaxInner; k += blockDim.x) bt[k] = np->beta[k];

  // rows of this lane: row(j) = gw + j * (CS * warps)
  const int gw = rank * kNnlsWarps + warp;
  const int stride = CS * kNnlsWarps;
  float Y[ROWS][RB], Ac[ROWS][RB], Wt[ROWS][RB];
  bool colok[RB];
#pragma unroll
  for (int b = 0; b < RB; ++b) colok[b] = (lane + 32 * b) < R;
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int i = gw + j * stride;
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int c = lane + 32 * b;
      float a0 = 0.f, m = 0.f;
      if (i < I && colok[b]) {
        a0 = a.A[(size_t)i * R + c];
        m = a.M[(size_t)i * R + c];
      }
      Ac[j][b] = a0;
      Y[j][b] = a0;
      Wt[j][b] = m + lam * a0;                      // W~ = W + lambda A0   (:206)
    }
  }
  // ---- learned warm start: features of each row, network inference, logging ----
  if (a.theta || a.log_X) {   // uniform over the CTA
    __syncthreads();          // Z~ is complete: the choice of start below reads it
    const int Din = R + 8, H = a.hidden;
    const float Lf = (float)np->L;
    float feat[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) feat[t] = np->feat[t];
#pragma unroll
    for (int j = 0; j < ROWS; ++j) {
      const int i = gw + j * stride;
      float m[RB];
      float s2 = 0.0f;
#pragma unroll
      for (int b = 0; b < RB; ++b) {
        const int c = lane + 32 * b;
        m[b] = (i < I && colok[b]) ? a.M[(size_t)i * R + c] : 0.0f;
        s2 = fmaf(m[b], m[b], s2);
      }
      for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      const float sc = sqrtf(s2) + 1e-30f;
      if (lane == 0) rsc[warp * ROWS + j] = sc;
      float x[RB];
#pragma unroll
      for (int b = 0; b < RB; ++b) x[b] = m[b] / sc;
      if (a.log_X && i < I) {
#pragma unroll
        for (int b = 0; b < RB; ++b)
          if (colok[b]) a.log_X[(size_t)i * Din + lane + 32 * b] = x[b];
        if (lane < 8) a.log_X[(size_t)i * Din + R + lane] = feat[lane];
      }
      if (a.theta && i < I) {   // uniform per warp: i depends on the warp only
        // theta is the transposed copy (mlp_theta_infer): W1^T [Din][H], b1, W2^T [H][H], b2,
        // W3^T [H][R], b3, so every step below reads one contiguous weight row across the lanes
        const float *W1 = a.theta, *b1 = W1 + (size_t)H * Din, *W2 = b1 + H, *b2 = W2 + (size_t)H * H;
        const float *W3 = b2 + H, *b3 = W3 + (size_t)R * H;
        float h1[4], h2[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) h1[q] = (lane + 32 * q < H) ? __ldg(b1 + lane + 32 * q) : 0.0f;
#pragma unroll 8
        for (int jj = 0; jj < R; ++jj) {
          const float xj = __shfl_sync(0xffffffffu, (jj >> 5) == 0 ? x[0] : x[RB - 1], jj & 31);
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (lane + 32 * q < H) h1[q] = fmaf(__ldg(W1 + (size_t)jj * H + lane + 32 * q), xj, h1[q]);
        }
#pragma unroll
        for (int t = 0; t < 8; ++t)
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (lane + 32 * q < H) h1[q] = fmaf(__ldg(W1 + (size_t)(R + t) * H + lane + 32 * q), feat[t], h1[q]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          h1[q] = fmaxf(h1[q], 0.0f);
          h2[q] = (lane + 32 * q < H) ? __ldg(b2 + lane + 32 * q) : 0.0f;
        }
#pragma unroll 8
        for (int v = 0; v < H; ++v) {
          const int qv = v >> 5;
          const float hv = __shfl_sync(0xffffffffu, qv == 0 ? h1[0] : qv == 1 ? h1[1] : qv == 2 ? h1[2] : h1[3], v & 31);
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (lane + 32 * q < H) h2[q] = fmaf(__ldg(W2 + (size_t)v * H + lane + 32 * q), hv, h2[q]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) h2[q] = fmaxf(h2[q], 0.0f);
        float y[RB];
#pragma unroll
        for (int b = 0; b < RB; ++b) y[b] = colok[b] ? __ldg(b3 + lane + 32 * b) : 0.0f;
#pragma unroll 8
        for (int u = 0; u < H; ++u) {
          const int qu = u >> 5;
          const float hu = __shfl_sync(0xffffffffu, qu == 0 ? h2[0] : qu == 1 ? h2[1] : qu == 2 ? h2[2] : h2[3], u & 31);
#pragma unroll
          for (int b = 0; b < RB; ++b)
            if (colok[b]) y[b] = fmaf(__ldg(W3 + (size_t)u * R + lane + 32 * b), hu, y[b]);
        }
        // the row starts from the network's guess only where it has the lower proximal
        // objective phi(y) = y.Z~y / 2 - W~.y than the reference's own start, the previous
        // row (include/NesterovMNLS.hpp:200-205): the learned start can only improve it
        float yn[RB], zn[RB], zp[RB];
#pragma unroll
        for (int b = 0; b < RB; ++b) {
          yn[b] = colok[b] ? fmaxf(y[b] * sc / Lf, 0.0f) : 0.0f;
          zn[b] = 0.0f;
          zp[b] = 0.0f;
        }
        for (int k = 0; k < R; ++k) {
          const float vn = __shfl_sync(0xffffffffu, (k >> 5) == 0 ? yn[0] : yn[RB - 1], k & 31);
          const float vp = __shfl_sync(0xffffffffu, (k >> 5) == 0 ? Ac[j][0] : Ac[j][RB - 1], k & 31);
#pragma unroll
          for (int b = 0; b < RB; ++b)
            if (colok[b]) {
              const float z = Zt[k * R + lane + 32 * b];   // Z~ is symmetric: row k, column c
              zn[b] = fmaf(z, vn, zn[b]);
              zp[b] = fmaf(z, vp, zp[b]);
            }
        }
        float pn = 0.0f, pp = 0.0f;
#pragma unroll
        for (int b = 0; b < RB; ++b) {
          pn = fmaf(yn[b], fmaf(0.5f, zn[b], -Wt[j][b]), pn);
          pp = fmaf(Ac[j][b], fmaf(0.5f, zp[b], -Wt[j][b]), pp);
        }
        for (int o = 16; o > 0; o >>= 1) {
          pn += __shfl_xor_sync(0xffffffffu, pn, o);
          pp += __shfl_xor_sync(0xffffffffu, pp, o);
        }
        if (pn < pp) {
#pragma unroll
          for (int b = 0; b < RB; ++b) {
            Y[j][b] = yn[b];
            Ac[j][b] = yn[b];
          }
        }
      }
    }
  }
  __syncthreads();

  // Global stop test without a reduction: the test of include/NesterovMNLS.hpp:217-218
  // (max |grad .* Y| <= delta1 and min grad >= -delta2) fails iff some element violates it,
  // so each warp that sees a violation at an iteration writes 1 into that iteration's flag
  // word in CTA 0's shared memory.  Rows are independent apart from this test, so the
  // iterations run in windows of KW steps with one split cluster barrier per window: every
  // step keeps its A_it in a slot of As, and after the barrier the first step of the window
  // whose word is still 0 is where the reference stops (its A_it is the result); the steps
  // after it were speculative.  The barrier is split: arrive after the window's last update,
  // wait after the next gradient, so its latency hides behind that product.  The words of
  // three windows are used in rotation.
  int *vflag0 = cluster.map_shared_rank(flags + 8, 0);
  if (tid < 3 * kNnlsWindowMax) flags[8 + tid] = 0;
  cluster.sync();
  float g[ROWS][RB];
  // R <= 32: this lane's column of Z~ stays in registers for the whole solve and the warp's
  // Y rows are read back from shared memory as float4 broadcasts (4 FMAs per load) instead of
  // one shuffle per (row, k); the FMAs and their order are the same.  Columns k >= R of Z~
  // and of Y are zero, so the extra terms add exact zeros.
  float zr[RB == 1 ? 32 : 1];
  if constexpr (RB == 1) {
#pragma unroll
    for (int k = 0; k < 32; ++k) zr[k] = (k < R && colok[0]) ? Zt[k * R + lane] : 0.0f;
  }
  auto stage_y = [&]() {
    if constexpr (RB == 1) {
      __syncwarp();   // every lane has read the previous Y rows
#pragma unroll
      for (int j = 0; j < ROWS; ++j) Ys[(warp * ROWS + j) * 32 + lane] = Y[j][0];
      __syncwarp();
    }
  };
  auto gradient = [&]() {   // grad = Y Z~ - W~
#pragma unroll
    for (int j = 0; j < ROWS; ++j)
#pragma unroll
      for (int b = 0; b < RB; ++b) g[j][b] = -Wt[j][b];
    if constexpr (RB == 1) {
#pragma unroll
      for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int j = 0; j < ROWS; ++j) {
          const float4 y4 = *reinterpret_cast<const float4 *>(&Ys[(warp * ROWS + j) * 32 + 4 * q]);
          g[j][0] = fmaf(y4.x, zr[4 * q], g[j][0]);
          g[j][0] = fmaf(y4.y, zr[4 * q + 1], g[j][0]);
          g[j][0] = fmaf(y4.z, zr[4 * q + 2], g[j][0]);
          g[j][0] = fmaf(y4.w, zr[4 * q + 3], g[j][0]);
        }
    } else {
      for (int k = 0; k < R; ++k) {
        const int kb = k >> 5, kl = k & 31;
        float z[RB];
#pragma unroll
        for (int b = 0; b < RB; ++b) z[b] = colok[b] ? Zt[k * R + lane + 32 * b] : 0.f;
#pragma unroll
        for (int j = 0; j < ROWS; ++j) {
          const float yk = __shfl_sync(0xffffffffu, kb == 0 ? Y[j][0] : Y[j][RB - 1], kl);
#pragma unroll
          for (int b = 0; b < RB; ++b) g[j][b] = fmaf(yk, z[b], g[j][b]);
        }
      }
    }
  };
  stage_y();
  gradient();
  int it = 0;
  for (int w = 0; it < kMaxInner; ++w) {
    const int wslot = (w % 3) * kNnlsWindowMax;
    const int t0 = it;
    int steps = 0;
    for (; steps < KW && it < kMaxInner; ++steps, ++it) {
      bool viol = false;
#pragma unroll
      for (int j = 0; j < ROWS; ++j) {
        const bool rowok = (gw + j * stride) < I;
#pragma unroll
        for (int b = 0; b < RB; ++b)
          if (rowok && colok[b]) viol |= (fabsf(g[j][b] * Y[j][b]) > a.delta1) || (g[j][b] < -a.delta2);
      }
      if (__any_sync(0xffffffffu, viol) && lane == 0) *(volatile int *)&vflag0[wslot + steps] = 1;
      const float beta = bt[it];
      float *slot = As + steps * aslot;
#pragma unroll
      for (int j = 0; j < ROWS; ++j)
#pragma unroll
        for (int b = 0; b < RB; ++b) {
          if (colok[b]) slot[(warp * ROWS + j) * R + lane + 32 * b] = Ac[j][b];   // A_it
          const float na = fmaxf(Y[j][b] - g[j][b] * invL, 0.0f);       // :220
          Y[j][b] = (1.0f + beta) * na - beta * Ac[j][b];                 // :228
          Ac[j][b] = na;
        }
      if (steps + 1 < KW && it + 1 < kMaxInner) {   // the next step of this window
        stage_y();
        gradient();
      }
    }
    // the words of window w+1 (read last in window w-2, before every CTA's arrive of w-1)
    if (rank == 0 && tid < kNnlsWindowMax) flags[8 + ((w + 1) % 3) * kNnlsWindowMax + tid] = 0;
    asm volatile("barrier.cluster.arrive.release;" ::: "memory");
    stage_y();
    gradient();   // of the next window's first step (discarded if the solve stops here)
    asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
    const int wv = lane < steps ? *(volatile int *)&vflag0[wslot + lane] : 1;
    const unsigned clear = __ballot_sync(0xffffffffu, wv == 0);
    if (clear) {   // the first step without a violation: stop there, the result is its A_it
      const int first = __ffs(clear) - 1;
      it = t0 + first;
      const float *slot = As + first * aslot;
#pragma unroll
      for (int j = 0; j < ROWS; ++j)
#pragma unroll
        for (int b = 0; b < RB; ++b)
          if (colok[b]) Ac[j][b] = slot[(warp * ROWS + j) * R + lane + 32 * b];
      break;
    }
  }

  // ---- zero-column test (sum of |A| per column over all rows), include/Cpd.hpp:206 ----
  for (int c = tid; c < R; c += blockDim.x) colsum[c] = 0.0f;
  __syncthreads();
  // per-warp column partials -> As as scratch, then fixed-order sum into colsum
#pragma unroll
  for (int b = 0; b < RB; ++b) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < ROWS; ++j) s += fabsf(Ac[j][b]);
    if (colok[b]) As[warp * R + lane + 32 * b] = s;
  }
  __syncthreads();
  for (int c = tid; c < R; c += blockDim.x) {
    float s = 0.f;
    for (int w = 0; w < kNnlsWarps; ++w) s += As[w * R + c];
    colsum[c] = s;
  }
  cluster.sync();
  if (warp == 0) {   // a lane per column; the CTAs' sums loaded together, added in rank order
    float mincol = INFINITY;
    for (int c = lane; c < R; c += 32) {
      float v[kNnlsMaxCluster];
#pragma unroll
      for (int r2 = 0; r2 < kNnlsMaxCluster; ++r2) v[r2] = r2 < CS ? cluster.map_shared_rank(colsum, r2)[c] : 0.f;
      float s = 0.f;
#pragma unroll
      for (int r2 = 0; r2 < kNnlsMaxCluster; ++r2)
        if (r2 < CS) s += v[r2];
      mincol = fminf(mincol, s);
    }
    for (int o = 16; o > 0; o >>= 1) mincol = fminf(mincol, __shfl_xor_sync(0xffffffffu, mincol, o));
    if (lane == 0) flags[0] = (mincol == 0.0f) ? 1 : 0;
  }
  __syncthreads();
  const bool repair = flags[0] != 0;

  // ---- final rows: repair, write A, stage rows for the Gram, <M, A> in FP64 ----
  double ma_part = 0.0;
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int i = gw + j * stride;
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int c = lane + 32 * b;
      float v = 0.f;
      if (i < I && colok[b]) {
        v = Ac[j][b];
        if (repair) v = 0.9f * v + 0.1f * a.A[(size_t)i * R + c];   // :206-207
      }
      if (colok[b]) As[(warp * ROWS + j) * R + c] = v;
      if (i < I && colok[b]) ma_part = fma((double)a.M[(size_t)i * R + c], (double)v, ma_part);
    }
  }
  __syncthreads();   // every CTA has read its old A rows before anyone writes new ones
  cluster.sync();
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int i = gw + j * stride;
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int c = lane + 32 * b;
      if (i < I && colok[b]) {
        const float v = As[(warp * ROWS + j) * R + c];
        a.A[(size_t)i * R + c] = v;
        if (a.log_T) a.log_T[(size_t)i * R + c] = v * (float)np->L / rsc[warp * ROWS + j];
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) ma_part += __shfl_xor_sync(0xffffffffu, ma_part, o);
  if (lane == 0) wredd[warp] = ma_part;
  // partial Gram of this CTA's rows
  const int nrows = kNnlsWarps * ROWS;
  for (int idx = tid; idx < R * R; idx += blockDim.x) {
    const int r1 = idx / R, r2 = idx % R;
    float s = 0.f;
    for (int i = 0; i < nrows; ++i) s = fmaf(As[i * R + r1], As[i * R + r2], s);
    Gp[idx] = s;
  }
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < kNnlsWarps; ++w) s += wredd[w];
    ma[0] = s;
  }
  cluster.sync();
  if (rank == 0) {
    for (int idx = tid; idx < R * R; idx += blockDim.x) {
      float v[kNnlsMaxCluster];   // the CTAs' partials loaded together, added in rank order
#pragma unroll
      for (int r2 = 0; r2 < kNnlsMaxCluster; ++r2) v[r2] = r2 < CS ? cluster.map_shared_rank(Gp, r2)[idx] : 0.f;
      float s = 0.f;
#pragma unroll
      for (int r2 = 0; r2 < kNnlsMaxCluster; ++r2)
        if (r2 < CS) s += v[r2];
      a.gram_out[idx] = s;
      Zt[idx] = s;   // reuse Zt (no longer needed) for the FP64 Hadamard sum
    }
    __syncthreads();
    if (warp == 0) {
      double h = 0.0;
      for (int idx = lane; idx < R * R; idx += 32) h = fma(np->Z[idx], (double)Zt[idx], h);
      for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
      const double mv = lane < CS ? cluster.map_shared_rank(ma, lane)[0] : 0.0;
      double sma = 0.0;
      for (int r2 = 0; r2 < CS; ++r2) sma += __shfl_sync(0xffffffffu, mv, r2);   // rank order
      if (lane == 0) {
        *a.inner_MA = sma;
        *a.had_ZG = h;
        *a.iters_out = it;
        *a.repaired_out = repair ? 1 : 0;
      }
    }
  }
  cluster.sync();   // keep every CTA's shared memory alive until rank 0 has read it
}

template <int RB, int ROWS, int kNnlsWarps>
size_t nnls_smem_bytes(int R, int window) {
  return sizeof(float) * (2 * R * R + (size_t)window * kNnlsWarps * ROWS * R + ((R + 1) & ~1) + 4 + 2 * kNnlsWarps) +
         sizeof(double) * (kNnlsWarps + 2) + sizeof(int) * (8 + 3 * kNnlsWindowMax) +
         sizeof(float) * (kMaxInner + kNnlsWarps * ROWS) + (RB == 1 ? 16 + sizeof(float) * kNnlsWarps * ROWS * 32 : 0);
}

template <int RB, int ROWS, int kNnlsWarps>
int launch_nnls_t(int cs, const NnlsArgs &args_in, cudaStream_t stream) {
  auto kern = nnls_cluster_kernel<RB, ROWS, kNnlsWarps>;
  // as many iterations per cluster barrier as the A_it slots fit in 96 KB (at most 8)
  NnlsArgs args = args_in;
  const size_t slot = sizeof(float) * kNnlsWarps * ROWS * args.R;
  args.window = (int)std::max<size_t>(1, std::min<size_t>(kNnlsWindowMax, (96u << 10) / slot));
  const size_t smem = nnls_smem_bytes<RB, ROWS, kNnlsWarps>(args.R, args.window);
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (cs > 8) PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if ((int64_t)cs * kNnlsWarps * ROWS < args.I)
    return set_error(PTG_ERR_INVALID, "internal: NNLS row tiling");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(kNnlsWarps * 32, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PTG_CUDA(cudaLaunchKernelEx(&cfg, kern, args));
  return PTG_OK;
}

// Cluster size of the NNLS kernel on this device: 16 (non-portable) when the hardware
// can schedule it, else the portable 8.  Probed once per context.
int nnls_cluster_size(ptg_ctx *ctx) {
  if (ctx->nnls_cluster) return ctx->nnls_cluster;
  int cs = 8;
  auto kern = nnls_cluster_kernel<2, 16, kNnlsWarpsLarge>;
  const size_t smem = nnls_smem_bytes<2, 16, kNnlsWarpsLarge>(kMaxR, 1);   // the largest slot: one step per window
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(kNnlsWarpsLarge * 32, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters > 0) cs = 16;
  }
  cudaGetLastError();
  ctx->nnls_cluster = cs;
  return cs;
}

// ------------------------------------------------------------------------------------
// Gram, normalisation, acceleration, cost terms.
// ------------------------------------------------------------------------------------
constexpr int kGramRowsPerBlock = 256;

__global__ void gram_partial_kernel(const float *__restrict__ A, int I, int R,
                                    float *__restrict__ part) {
  extern __shared__ float rows[];   // kGramRowsPerBlock x R
  const int r0 = blockIdx.x * kGramRowsPerBlock;
  const int nr = min(kGramRowsPerBlock, I - r0);
  // stage the block's rows: eight independent loads in flight per thread, not one
  const float *src = A + (size_t)r0 * R;
  const int n = nr * R, step = blockDim.x;
  int idx0 = threadIdx.x;
  for (; idx0 + 7 * step < n; idx0 += 8 * step) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldg(src + idx0 + u * step);
#pragma unroll
    for (int u = 0; u < 8; ++u) rows[idx0 + u * step] = v[u];
  }
  for (; idx0 < n; idx0 += step) rows[idx0] = __ldg(src + idx0);
  __syncthreads();
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    const int a = idx / R, b = idx % R;
    float s = 0.f;
    for (int i = 0; i < nr; ++i) s = fmaf(rows[i * R + a], rows[i * R + b], s);
    part[(size_t)blockIdx.x * R * R + idx] = s;
  }
}

__global__ void sum_rr_kernel(const float *__restrict__ part, int nb, int RR, float *__restrict__ G) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < RR; idx += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * RR + idx];
    G[idx] = s;
  }
}

}  // namespace

size_t eigen_kernel_smem() {
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, eigen_bounds_kernel) != cudaSuccess) {
    cudaGetLastError();
    return 48 * 1024;
  }
  return fa.sharedSizeBytes;
}

int launch_eigen_bounds(const float *const *grams, int order, int mode, int R, NnlsParams *out,
                        cudaStream_t stream, bool beside_tc) {
  if (R > kMaxR) return set_error(PTG_ERR_UNSUPPORTED, "rank > 64 is not supported by the NNLS path");
  GramPtrs gp{};
  for (int k = 0; k < order; ++k) gp.g[k] = grams[k];
  // CTAs of two kernels share an SM only under the same shared-memory carveout: beside the
  // tensor-core MTTKRP (one CTA per SM, which takes the largest carveout) this kernel asks for
  // the same, else it would wait for an SM to drain and sit on the critical path; beside the
  // CUDA-core MTTKRP the driver's default choice is the one that fits
  PTG_CUDA(cudaFuncSetAttribute(eigen_bounds_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                beside_tc ? (int)cudaSharedmemCarveoutMaxShared
                                          : (int)cudaSharedmemCarveoutDefault));
  eigen_bounds_kernel<<<1, kEigThreads, 0, stream>>>(gp, order, mode, R, out);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

int launch_nnls_full(ptg_ctx *ctx, const float *M, float *A, int I, int R, const NnlsParams *np,
                     float delta1, float delta2, float *gram_out, double *inner_MA, double *had_ZG,
                     int *iters_out, int *repaired_out, cudaStream_t stream, const WarmArgs &warm) {
  if (R > kMaxR) return set_error(PTG_ERR_UNSUPPORTED, "rank > 64 is not supported by the NNLS path");
  NnlsArgs args{M, A, I, R, np, delta1, delta2, gram_out, inner_MA, had_ZG, iters_out, repaired_out,
                warm.theta, warm.hidden, warm.log_X, warm.log_T};
  const int cs = nnls_cluster_size(ctx);
  const bool wide = R > 32;
  const int cap = cs * kNnlsWarpsLarge;   // rows per register slot
  const int rows = (I + cap - 1) / cap;
#define PTG_NNLS_CASE(RWS)                                                                        \
  if (rows <= RWS)                                                                                \
    return wide ? launch_nnls_t<2, RWS, kNnlsWarpsLarge>(cs, args, stream)                        \
                : launch_nnls_t<1, RWS, kNnlsWarpsLarge>(cs, args, stream);
  PTG_NNLS_CASE(1)
  PTG_NNLS_CASE(2)
  PTG_NNLS_CASE(4)
  PTG_NNLS_CASE(8)
  PTG_NNLS_CASE(16)
#undef PTG_NNLS_CASE
  return set_error(PTG_ERR_UNSUPPORTED, "factor has too many rows for the NNLS kernel");
}

int launch_gram(const float *A, int I, int R, float *G, float *part, cudaStream_t stream, bool beside_tc) {
  const int nb = (I + kGramRowsPerBlock - 1) / kGramRowsPerBlock;
  const size_t smem = sizeof(float) * kGramRowsPerBlock * R;
  PTG_CUDA(cudaFuncSetAttribute(gram_partial_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // beside the tensor-core MTTKRP the same carveout, so that the CTAs share SMs with it
  const int carve = beside_tc ? (int)cudaSharedmemCarveoutMaxShared : (int)cudaSharedmemCarveoutDefault;
  PTG_CUDA(cudaFuncSetAttribute(gram_partial_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carve));
  PTG_CUDA(cudaFuncSetAttribute(sum_rr_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carve));
  gram_partial_kernel<<<nb, 256, smem, stream>>>(A, I, R, part);
  sum_rr_kernel<<<(R * R + 255) / 256, 256, 0, stream>>>(part, nb, R * R, G);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

size_t gram_scratch_floats(int I, int R) {
  return (size_t)((I + kGramRowsPerBlock - 1) / kGramRowsPerBlock) * R * R;
}

__global__ void normalize_factors_kernel(NormArgs a) {
  // one thread per (factor row, column) element across all factors, then the Grams
  extern __shared__ float sh[];   // mult[order][R], lf[order][R]
  float *mult = sh, *lfs = sh + a.order * a.R;
  for (int c = threadIdx.x; c < a.R; c += blockDim.x) {
    float m[PTG_MAX_ORDER], l[PTG_MAX_ORDER];
    normalize_column(a, c, m, l);
    for (int k = 0; k < a.order; ++k) {
      mult[k * a.R + c] = m[k];
      lfs[k * a.R + c] = l[k];
    }
  }
  __syncthreads();
  // every block reads the Grams (diagonals) above; writes happen in a second kernel
  for (int k = 0; k < a.order; ++k) {
    const int64_t n = (int64_t)a.rows[k] * a.R;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x)
      a.fac[k][idx] *= mult[k * a.R + (int)(idx % a.R)];
  }
}

__global__ void normalize_grams_kernel(NormArgs a) {
  // single block: Gram scaling G_j ./= lf lf^T, G_w .*= prod_j lf_j lf_j^T  (:159-172)
  extern __shared__ float sh[];
  float *lfs = sh;   // [order][R]
  for (int c = threadIdx.x; c < a.R; c += blockDim.x) {
    float m[PTG_MAX_ORDER], l[PTG_MAX_ORDER];
    normalize_column(a, c, m, l);
    for (int k = 0; k < a.order; ++k) lfs[k * a.R + c] = l[k];
  }
  __syncthreads();
  const int N = a.order, last = N - 1, w = a.weight, R = a.R;
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    const int r1 = idx / R, r2 = idx % R;
    float wm = 1.0f;
    for (int j = 0; j < last; ++j) {
      if (j == w) continue;
      const float nm = lfs[j * R + r1] * lfs[j * R + r2];
      wm *= nm;
      a.gram[j][idx] = a.gram[j][idx] / nm;
    }
    a.gram[w][idx] *= wm;
  }
}

int launch_normalize(float *const *fac, float *const *gram, const int *rows, int order, int weight,
                     int R, cudaStream_t stream) {
  NormArgs a{};
  for (int k = 0; k < order; ++k) {
    a.fac[k] = fac[k];
    a.gram[k] = gram[k];
    a.rows[k] = rows[k];
  }
  a.order = order;
  a.weight = weight;
  a.R = R;
  const size_t smem = sizeof(float) * 2 * order * R;
  int64_t total = 0;
  for (int k = 0; k < order; ++k) total += (int64_t)rows[k] * R;
  const int blocks = (int)std::min<int64_t>(std::max<int64_t>(1, (total + 255) / 256), 1024);
  // factors first (they read the unmodified Gram diagonals), then the Grams
  normalize_factors_kernel<<<blocks, 256, smem, stream>>>(a);
  normalize_grams_kernel<<<1, 256, smem, stream>>>(a);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

// ---- acceleration: acc = old + s (cur - old) for all factors ----
struct AxpyArgs {
  const float *cur[PTG_MAX_ORDER];
  const float *old[PTG_MAX_ORDER];
  float *acc[PTG_MAX_ORDER];
  int64_t n[PTG_MAX_ORDER];
  int order;
  float step;
};

__global__ void accel_combine_kernel(AxpyArgs a) {
  for (int k = 0; k < a.order; ++k)
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < a.n[k];
         idx += (int64_t)gridDim.x * blockDim.x) {
      const float o = a.old[k][idx];
      a.acc[k][idx] = o + a.step * (a.cur[k][idx] - o);
    }
}

int launch_accel_combine(const float *const *cur, const float *const *old, float *const *acc,
                         const int *rows, int order, int R, double step, cudaStream_t stream) {
  AxpyArgs a{};
  int64_t total = 0;
  for (int k = 0; k < order; ++k) {
    a.cur[k] = cur[k];
    a.old[k] = old[k];
    a.acc[k] = acc[k];
    a.n[k] = (int64_t)rows[k] * R;
    total += a.n[k];
  }
  a.order = order;
  a.step = (float)step;
  const int blocks = (int)std::min<int64_t>(std::max<int64_t>(1, (total + 255) / 256), 1024);
  accel_combine_kernel<<<blocks, 256, 0, stream>>>(a);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

// ---- FP64 cost terms for a given point: <M, A_last> and sum(Z .* G_last) ----
// <M, A> over the last factor and sum(Z .* G) over the Grams in FP64 (the cost cancels
// catastrophically).  kCostBlocks CTAs each sum a contiguous range of <M, A> (eight elements of
// a thread in flight, added in order) and a strided share of sum(Z .* G); the CTA that finishes
// last adds the partials in CTA order, so the result does not depend on timing.
constexpr int kCostBlocks = 32, kCostThreads = 256;
static_assert(2 * kCostBlocks <= kCostPartials, "cost-term partials");

__global__ void __launch_bounds__(kCostThreads) cost_terms_kernel(const float *__restrict__ M,
                                                                 const float *__restrict__ A, int64_t n,
                                                                 GramPtrs gp, int order, int R, double *part,
                                                                 unsigned *ticket, double *out2) {
  __shared__ double red[2][kCostThreads / 32];
  __shared__ bool is_last;
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t i0 = blockIdx.x * chunk, i1 = min(n, i0 + chunk);
  double s = 0.0;
  int64_t idx = i0 + threadIdx.x;
  for (; idx + 7 * kCostThreads < i1; idx += 8 * kCostThreads) {
    float m[8], a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      m[u] = __ldg(M + idx + u * kCostThreads);
      a[u] = __ldg(A + idx + u * kCostThreads);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) s = fma((double)m[u], (double)a[u], s);
  }
  for (; idx < i1; idx += kCostThreads) s = fma((double)M[idx], (double)A[idx], s);
  double h = 0.0;
  for (int k = blockIdx.x * kCostThreads + threadIdx.x; k < R * R; k += gridDim.x * kCostThreads) {
    double z = 1.0;
    for (int j = order - 2; j >= 0; --j) z *= (double)gp.g[j][k];
    h = fma(z, (double)gp.g[order - 1][k], h);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    h += __shfl_down_sync(0xffffffffu, h, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = s;
    red[1][w] = h;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < kCostThreads / 32; ++i) {
      a += red[0][i];
      b += red[1][i];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
    __threadfence();
    is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int i = 0; i < (int)gridDim.x; ++i) {
      a += __ldcg(part + 2 * i);
      b += __ldcg(part + 2 * i + 1);
    }
    out2[0] = a;
    out2[1] = b;
    *ticket = 0u;   // ready for the next launch on the stream
  }
}

int launch_cost_terms(const float *M, const float *A_last, int64_t I_last, const float *const *grams,
                      int order, int R, double *out2, CostScratch scratch, cudaStream_t stream) {
  GramPtrs gp{};
  for (int k = 0; k < order; ++k) gp.g[k] = grams[k];
  cost_terms_kernel<<<kCostBlocks, kCostThreads, 0, stream>>>(M, A_last, I_last * R, gp, order, R, scratch.part,
                                                             scratch.ticket, out2);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

namespace {
struct FacPtrs {
  const float *a[PTG_MAX_ORDER];
  int rows[PTG_MAX_ORDER];
};
constexpr int kGramParts = 16;

// Grams accumulated in FP64 from the factors: CTA (r1, k, p) and thread r2 sum
// A_k[i][r1] A_k[i][r2] over the p-th contiguous share of the rows, into
// part[((k * kGramParts + p) * R + r1) * R + r2]
__global__ void gram_fp64_part_kernel(FacPtrs f, int R, double *part) {
  const int r1 = blockIdx.x, k = blockIdx.y, p = blockIdx.z, r2 = threadIdx.x;
  if (r2 >= R) return;
  const int rows = f.rows[k], share = (rows + kGramParts - 1) / kGramParts;
  const int i0 = p * share, i1 = min(rows, i0 + share);
  const float *A = f.a[k];
  double g = 0.0;
  for (int i = i0; i < i1; ++i) g = fma((double)A[(size_t)i * R + r1], (double)A[(size_t)i * R + r2], g);
  part[(((size_t)k * kGramParts + p) * R + r1) * R + r2] = g;
}

// *out = sum over (r1, r2) of prod_k G_k[r1][r2], the parts of each Gram added in order and the
// pairs summed in a fixed order (one CTA of 1024 threads)
__global__ void gram_term_fp64_kernel(const double *part, int order, int R, double *out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    double prod = 1.0;
    for (int k = order - 1; k >= 0; --k) {
      double g = 0.0;
      for (int p = 0; p < kGramParts; ++p) g += part[((size_t)k * kGramParts + p) * R * R + idx];
      prod *= g;
    }
    s += prod;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *out = v;
  }
}
}  // namespace

size_t gram_term_fp64_scratch_doubles(int order, int R) { return (size_t)order * kGramParts * R * R; }

int launch_gram_term_fp64(const float *const *factors, const int *rows, int order, int R, double *part,
                          double *out, cudaStream_t stream) {
  FacPtrs f{};
  for (int k = 0; k < order; ++k) {
    f.a[k] = factors[k];
    f.rows[k] = rows[k];
  }
  gram_fp64_part_kernel<<<dim3(R, order, kGramParts), ((R + 31) / 32) * 32, 0, stream>>>(f, R, part);
  gram_term_fp64_kernel<<<1, 1024, 0, stream>>>(part, order, R, out);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

}  // namespace ptg

// ------------------------------------------------------------------------------------
// Batched forms for many small instances (one CTA per instance; inactive instances
// return at once).  Each reuses the single-instance arithmetic above.
// ------------------------------------------------------------------------------------
namespace ptg {
namespace {

__global__ void __launch_bounds__(kEigThreads) eigen_batched_kernel(const EigDesc *__restrict__ d,
                                                                    const int *__restrict__ active) {
  const EigDesc &e = d[blockIdx.x];
  if (active && !active[e.inst]) return;
  GramPtrs gp{};
  for (int k = 0; k < e.order; ++k) gp.g[k] = e.gram[k];
  eigen_bounds_body<kEigThreads>(gp, e.order, e.mode, e.R, e.out, threadIdx.x);
}

__global__ void gram_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ active, int use_acc) {
  const InstDesc &in = d[blockIdx.x];
  if (active && !active[in.inst]) return;
  gram_block(in, use_acc);
}

__global__ void normalize_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ active) {
  const InstDesc &in = d[blockIdx.x];
  if (active && !active[in.inst]) return;
  normalize_block(in);
}

// acc = old + step (fac - old) for instances with accel[inst] != 0 (step[inst]).
__global__ void accel_combine_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ accel,
                                             const float *__restrict__ step) {
  const InstDesc &in = d[blockIdx.x];
  if (!accel[in.inst]) return;
  accel_combine_block(in, step[in.inst]);
}

// old = fac for instances with flag[inst] != 0
__global__ void copy_old_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ flag) {
  const InstDesc &in = d[blockIdx.x];
  if (!flag[in.inst]) return;
  copy_old_block(in);
}

// fac, gram = acc, gacc for instances with accepted[inst] != 0
__global__ void select_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ accepted) {
  const InstDesc &in = d[blockIdx.x];
  if (!accepted[in.inst]) return;
  select_block(in);
}

__global__ void cost_terms_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ flag,
                                          int use_acc) {
  const InstDesc &in = d[blockIdx.x];
  if (flag && !flag[in.inst]) return;
  cost_terms_block(in, use_acc);
}

}  // namespace

int launch_eigen_batched(ptg_ctx *ctx, const EigDesc *d, int n, const int *active, cudaStream_t s) {
  eigen_batched_kernel<<<n, kEigThreads, 0, s>>>(d, active);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 1);
  return PTG_OK;
}

int launch_batched_op(ptg_ctx *ctx, BatchedOp op, const InstDesc *d, int n, const int *flag, const float *step,
                      cudaStream_t s) {
  switch (op) {
    case BatchedOp::Gram: gram_batched_kernel<<<n, 256, 0, s>>>(d, flag, 0); break;
    case BatchedOp::GramAcc: gram_batched_kernel<<<n, 256, 0, s>>>(d, flag, 1); break;
    case BatchedOp::Normalize: normalize_batched_kernel<<<n, 256, 0, s>>>(d, flag); break;
    case BatchedOp::AccelCombine: accel_combine_batched_kernel<<<n, 256, 0, s>>>(d, flag, step); break;
    case BatchedOp::CopyOld: copy_old_batched_kernel<<<n, 256, 0, s>>>(d, flag); break;
    case BatchedOp::Select: select_batched_kernel<<<n, 256, 0, s>>>(d, flag); break;
    case BatchedOp::CostTerms: cost_terms_batched_kernel<<<n, 256, 0, s>>>(d, flag, 0); break;
    case BatchedOp::CostTermsAcc: cost_terms_batched_kernel<<<n, 256, 0, s>>>(d, flag, 1); break;
  }
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 1);
  return PTG_OK;
}

}  // namespace ptg
