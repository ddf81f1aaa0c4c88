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

namespace cg = cooperative_groups;

namespace ptg {

namespace {

// ------------------------------------------------------------------------------------
// FP64 eigenvalue bounds.  Householder reduction to tridiagonal form (Householder 1958;
// Golub & Van Loan, Matrix Computations, alg. 8.3.1) and Sturm-sequence bisection
// (Givens 1954; Wilkinson, The Algebraic Eigenvalue Problem, ch. 5) run as a 128-way
// multisection per round.
// ------------------------------------------------------------------------------------
constexpr int kEigThreads = 256;
constexpr int kMaxR = 64;

struct GramPtrs {
  const float *g[PTG_MAX_ORDER];
};

// Sturm count (eigenvalues < x) of the symmetric tridiagonal (d, e^2) in FP32, ratio form
// q_i = (d_i - x) - e_{i-1}^2 / q_{i-1}.
__device__ int sturm_count_f32(const float *d, const float *e2, int n, float x) {
  int cnt = 0;
  float q = d[0] - x;
  cnt += q < 0.0f;
  for (int i = 1; i < n; ++i) {
    if (q == 0.0f) q = 1e-30f;
    q = (d[i] - x) - e2[i - 1] / q;
    cnt += q < 0.0f;
  }
  return cnt;
}

// Same count in FP64 without divisions: the sign changes of the characteristic-polynomial
// sequence p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}, rescaled by exact powers of two so
// it neither overflows nor underflows (GB300's FP64 rate is low; a division costs ~10 FMAs).
__device__ int sturm_count_f64(const double *d, const double *e2, int n, double x) {
  double pm2 = 1.0, pm1 = d[0] - x;
  int sprev = 1;                                  // sign of p_{-1} = 1
  int s1 = pm1 < 0.0 ? -1 : (pm1 > 0.0 ? 1 : sprev);
  int cnt = (s1 != sprev);
  sprev = s1;
  for (int i = 1; i < n; ++i) {
    double p = (d[i] - x) * pm1 - e2[i - 1] * pm2;
    const int s = p < 0.0 ? -1 : (p > 0.0 ? 1 : sprev);
    cnt += (s != sprev);
    sprev = s;
    pm2 = pm1;
    pm1 = p;
    const double a = fabs(pm1);
    if (a > 0x1p+256) {
      pm1 *= 0x1p-256;
      pm2 *= 0x1p-256;
    } else if (a < 0x1p-256 && fabs(pm2) < 0x1p-256) {
      pm1 *= 0x1p+256;
      pm2 *= 0x1p+256;
    }
  }
  return cnt;
}

__device__ void eigen_bounds_body(const GramPtrs &gp, int order, int mode, int R, NnlsParams *out) {
  constexpr int lda = kMaxR + 1;              // padded rows: column reads and mirrored writes
  __shared__ double A[kMaxR * lda];           // spread over the banks
  __shared__ double xs[kMaxR], vs[kMaxR], ws[kMaxR];
  __shared__ double ps[kEigThreads / kMaxR][kMaxR];
  __shared__ double d[kMaxR], e[kMaxR], e2[kMaxR];
  __shared__ double redb[2][kEigThreads / 32];
  __shared__ double s_scalar[4];
  __shared__ double lohi[2][2];
  __shared__ float df[kMaxR], e2f[kMaxR];
  const int tid = threadIdx.x;
  const int n = R;

  // Z = prod_{k != mode} G_k (FP64), k from order-1 down to 0 as PartialCwiseProd orders it;
  // the tridiagonalisation works on the lower triangle mirrored, so A is exactly symmetric
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - (idx / n) * n;
    double z = 1.0;
    for (int k = order - 1; k >= 0; --k)
      if (k != mode) z *= (double)gp.g[k][idx];
    out->Z[idx] = z;
    if (j <= i) {
      A[i * lda + j] = z;
      A[j * lda + i] = z;
    }
  }
  __syncthreads();

  // Block sum: warp shuffles, then every thread adds the warps' partials in warp order from one
  // of two alternating buffers, so a sum costs one barrier and no broadcast.  (A buffer is
  // written again two sums later, after a barrier every thread passes once it has read it.)
  int rb = 0;
  auto block_sum = [&](double x) -> double {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((tid & 31) == 0) redb[rb][tid >> 5] = x;
    __syncthreads();
    double sum = 0.0;
    for (int i = 0; i < kEigThreads / 32; ++i) sum += redb[rb][i];
    rb ^= 1;
    return sum;
  };

  // ---- Householder tridiagonalisation (Golub & Van Loan alg. 8.3.1), H = I - beta v v^T,
  // v = x - alpha e_1, A_sub <- A_sub - v w^T - w v^T with p = beta A_sub v, w = p - (beta/2)(p.v) v.
  // A_sub v = A_sub x - alpha A_sub e_1: the product with x runs before alpha is known, beside
  // the square root and the division (one thread: GB300's FP64 pipe is the scarce resource).
  // Thread (q, i) sums a quarter of row i's terms, reading column entries (A is symmetric) so
  // that a warp's threads read consecutive addresses. ----
  const int pi = tid & (kMaxR - 1), pq = tid / kMaxR;
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // length of the column below the diagonal (= row k right of it)
    const double *rowk = A + k * lda + (k + 1);
    const double xi = tid < m ? rowk[tid] : 0.0;
    if (tid < m) xs[tid] = xi;
    const double sigma = block_sum(tid >= 1 && tid < m ? xi * xi : 0.0);   // ||x[1:]||^2
    const double x0 = rowk[0];
    if (sigma == 0.0) {   // uniform: nothing to eliminate, A unchanged
      if (tid == 0) e[k] = x0;
      continue;
    }
    double y = 0.0;       // (A_sub x)_i, partial over j in [16 q, 16 q + 16)
    if (pi < m) {
      const double *col = A + (k + 1) * lda + (k + 1 + pi);
      const int j1 = min(m, (pq + 1) * (kMaxR / (kEigThreads / kMaxR)));
      for (int j = pq * (kMaxR / (kEigThreads / kMaxR)); j < j1; ++j) y = fma(col[j * lda], xs[j], y);
      ps[pq][pi] = y;
    }
    if (tid == kEigThreads - 1) {   // never holds a row of the product (row 63 > m - 1)
      const double al = (x0 >= 0.0 ? -1.0 : 1.0) * sqrt(x0 * x0 + sigma);
      const double dv = x0 - al;
      s_scalar[0] = al;
      s_scalar[3] = 2.0 / (dv * dv + sigma);
    }
    __syncthreads();
    const double alpha = s_scalar[0], beta = s_scalar[3];
    const double v0 = x0 - alpha;
    double pv = 0.0, vi = 0.0, pvi = 0.0;
    if (tid < m) {
      double yi = 0.0;
      for (int q = 0; q < kEigThreads / kMaxR; ++q) yi += ps[q][tid];
      vi = tid == 0 ? v0 : xi;
      pvi = beta * fma(-alpha, A[(k + 1) * lda + (k + 1 + tid)], yi);   // p_i
      pv = pvi * vi;
    }
    const double K = 0.5 * beta * block_sum(pv);
    if (tid < m) {
      vs[tid] = vi;
      ws[tid] = pvi - K * vi;
    }
    __syncthreads();
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      const int i = idx / m, j = idx - (idx / m) * m;
      if (j > i) continue;
      const double a = A[(k + 1 + i) * lda + (k + 1 + j)] - (vs[i] * ws[j] + ws[i] * vs[j]);
      A[(k + 1 + i) * lda + (k + 1 + j)] = a;
      A[(k + 1 + j) * lda + (k + 1 + i)] = a;
    }
    if (tid == 0) e[k] = alpha;
    __syncthreads();
  }
  if (tid == 0) {
    for (int i = 0; i < n; ++i) d[i] = A[i * lda + i];
    if (n >= 2) e[n - 2] = A[(n - 1) * lda + (n - 2)];
    for (int i = 0; i + 1 < n; ++i) e2[i] = e[i] * e[i];
    // Gershgorin interval
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < n; ++i) {
      const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
      lo = fmin(lo, d[i] - r);
      hi = fmax(hi, d[i] + r);
    }
    const double pad = 1e-12 * fmax(fabs(lo), fabs(hi)) + 1e-300;
    lo -= pad;
    hi += pad;
    lohi[0][0] = lo; lohi[0][1] = hi;   // smallest eigenvalue
    lohi[1][0] = lo; lohi[1][1] = hi;   // largest eigenvalue
    s_scalar[1] = fmax(fabs(lo), fabs(hi));   // ||T|| bound
  }
  __syncthreads();   // d and e2 are complete before any thread reads them (n > 32 spans warps)
  for (int i = tid; i < n; i += blockDim.x) {
    df[i] = (float)d[i];
    e2f[i] = (float)e2[i];
  }
  __syncthreads();

  // ---- bisection: warp 0 brackets the smallest eigenvalue, warp 1 the largest, with a
  // 32-way multisection per round: FP32 counts first, then FP64 counts on the widened
  // FP32 bracket ----
  if (tid < 64) {
    const int which = tid >> 5;      // 0: min, 1: max
    const int j = tid & 31;
    const int target = which == 0 ? 1 : n;  // count(x) >= target  <=>  x > lambda
    double lo = lohi[which][0], hi = lohi[which][1];
    for (int round = 0; round < 6; ++round) {
      const double x = lo + (hi - lo) * (double)(j + 1) / 33.0;
      const bool hit = sturm_count_f32(df, e2f, n, (float)x) >= target;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      const int f = m ? (__ffs(m) - 1) : 32;
      const double nlo = (f == 0) ? lo : lo + (hi - lo) * (double)f / 33.0;
      const double nhi = (f == 32) ? hi : lo + (hi - lo) * (double)(f + 1) / 33.0;
      lo = nlo;
      hi = nhi;
    }
    // the FP32 counts are exact for a matrix within a few FP32 ulps of T (entrywise), so
    // the eigenvalue lies within 16 * eps32 * ||T|| of the FP32 bracket
    const double margin = 16.0 * 1.1920929e-7 * s_scalar[1] + 1e-300;
    lo -= margin;
    hi += margin;
    // ... which holds while FP32 represents T well.  Where it does not (entries or their
    // squares out of FP32 range, or counts off by more than the margin) the FP64 counts at
    // the widened ends show it: then the FP64 multisection starts over from the Gershgorin
    // interval, with enough rounds (33^16) to reach FP64 resolution from there.
    int c_end = 0;
    if (j < 2) c_end = sturm_count_f64(d, e2, n, j == 0 ? lo : hi);
    const int c_lo = __shfl_sync(0xffffffffu, c_end, 0), c_hi = __shfl_sync(0xffffffffu, c_end, 1);
    int rounds64 = 8;
    if (!(c_lo < target && c_hi >= target)) {
      lo = lohi[which][0];
      hi = lohi[which][1];
      rounds64 = 16;
    }
    for (int round = 0; round < rounds64; ++round) {
      const double x = lo + (hi - lo) * (double)(j + 1) / 33.0;
      const bool hit = sturm_count_f64(d, e2, n, x) >= target;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      const int f = m ? (__ffs(m) - 1) : 32;
      const double nlo = (f == 0) ? lo : lo + (hi - lo) * (double)f / 33.0;
      const double nhi = (f == 32) ? hi : lo + (hi - lo) * (double)(f + 1) / 33.0;
      lo = nlo;
      hi = nhi;
    }
    if (j == 0) {
      lohi[which][0] = lo;
      lohi[which][1] = hi;
    }
  }
  __syncthreads();
  if (tid == 0) {
    const double lmin = 0.5 * (lohi[0][0] + lohi[0][1]);
    const double lmax = 0.5 * (lohi[1][0] + lohi[1][1]);
    // singular values of a symmetric matrix are |eigenvalues|
    double L = fmax(fabs(lmax), fabs(lmin));
    double mu = fabs(lmin);
    if (n == 1) L = mu = fabs(d[0]);
    {   // scale-free summaries of Z for the warm-start network
      double dsum = 0.0, dmin = 1e300, dmax = -1e300;
      for (int i = 0; i < n; ++i) {
        const double z = out->Z[i * n + i];
        dsum += z;
        dmin = fmin(dmin, z);
        dmax = fmax(dmax, z);
      }
      const double Ls = L > 0.0 ? L : 1.0;
      out->feat[0] = (float)(log10(Ls / fmax(mu, 1e-300)) / 6.0);
      out->feat[1] = (float)(mu / Ls);
      out->feat[2] = (float)(dsum / n / Ls);
      out->feat[3] = (float)(dmin / Ls);
      out->feat[4] = (float)(dmax / Ls);
      out->feat[6] = (float)n / 64.0f;
      out->feat[7] = 1.0f;
    }
    // GLambda, include/NesterovMNLS.hpp:75-91
    double q = mu / L, lam;
    if (1.0 / q > 1e6) lam = 10.0 * mu;
    else if (1.0 / q > 1e3) lam = mu;
    else lam = mu / 10.0;
    L += lam;
    mu += lam;
    q = mu / L;
    out->L = L;
    out->mu = mu;
    out->lambda = lam;
    out->q = q;
    out->feat[5] = (float)(lam / L);
    // UpdateAlpha (:103-113) and beta (:226): the sequence is consumed in FP32 by the
    // solver, so it is generated in FP32 (a serial FP64 chain would dominate the kernel)
    float alpha = 1.0f;
    const float qf = (float)q;
    for (int it = 0; it < kMaxInner; ++it) {
      const float b = alpha * alpha - qf, c = -alpha * alpha;
      const float na = (-b + sqrtf(b * b - 4.0f * c)) * 0.5f;
      out->beta[it] = alpha * (1.0f - alpha) / (alpha * alpha + na);
      alpha = na;
    }
    out->status = (isfinite(L) && isfinite(mu)) ? 0 : PTG_ERR_NUMERIC;
    s_scalar[0] = L;
  }
}

__global__ void __launch_bounds__(kEigThreads)
eigen_bounds_kernel(GramPtrs gp, int order, int mode, int R, NnlsParams *out) {
  eigen_bounds_body(gp, order, mode, R, out);
}

// ------------------------------------------------------------------------------------
// Row-batched Nesterov MNLS on one cluster.
// ------------------------------------------------------------------------------------
constexpr int kNnlsWarps = 16;
constexpr int kNnlsThreads = kNnlsWarps * 32;

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
};

template <int RB, int ROWS>
__global__ void __launch_bounds__(kNnlsThreads, 1) nnls_cluster_kernel(const NnlsArgs a) {
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int R = a.R, I = a.I;

  extern __shared__ __align__(16) float sm[];
  float *Zt = sm;                                   // R*R
  float *As = Zt + R * R;                           // (kNnlsWarps*ROWS) x R
  float *Gp = As + kNnlsWarps * ROWS * R;           // R*R  (this CTA's partial Gram)
  float *colsum = Gp + R * R;                       // R
  float *slots = colsum + ((R + 1) & ~1);          // [2][2] stop test (max |g.y|, min g)
  float *wred = slots + 4;                          // kNnlsWarps * 2
  double *wredd = reinterpret_cast<double *>(wred + 2 * kNnlsWarps);   // kNnlsWarps
  double *ma = wredd + kNnlsWarps;                  // 1: this CTA's <M, A>
  int *flags = reinterpret_cast<int *>(ma + 2);     // [0]: repaired, [1..3]: stop-test words, [4..7]: unused
  float *bt = reinterpret_cast<float *>(flags + 8); // kMaxInner: the beta sequence
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
  // so each warp that sees a violation writes 1 into a flag word of iteration `it` in CTA 0's
  // shared memory (three words used in rotation).  One split cluster barrier per iteration:
  // arrive after the flag write and the speculative update, wait after the next gradient, so
  // the barrier's latency hides behind that product.  The update of iteration `it` keeps A_it
  // in the staging rows (As) in case the flag says stop.  (Copies of the words in every CTA,
  // written by lanes 0..CS-1 of a violating warp and read locally, measured no faster.)
  int *vflag0 = cluster.map_shared_rank(flags + 1, 0);
  if (tid < 3) flags[1 + tid] = 0;
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
  for (;;) {
    if (it >= kMaxInner) break;   // A_it is the result
    bool viol = false;
#pragma unroll
    for (int j = 0; j < ROWS; ++j) {
      const bool rowok = (gw + j * stride) < I;
#pragma unroll
      for (int b = 0; b < RB; ++b)
        if (rowok && colok[b]) viol |= (fabsf(g[j][b] * Y[j][b]) > a.delta1) || (g[j][b] < -a.delta2);
    }
    if (__any_sync(0xffffffffu, viol) && lane == 0) *(volatile int *)&vflag0[it % 3] = 1;
    if (rank == 0 && tid == 0) flags[1 + (it + 1) % 3] = 0;   // the word of it+1 (read last at it-2)
    const float beta = bt[it];
#pragma unroll
    for (int j = 0; j < ROWS; ++j)
#pragma unroll
      for (int b = 0; b < RB; ++b) {
        if (colok[b]) As[(warp * ROWS + j) * R + lane + 32 * b] = Ac[j][b];   // A_it
        const float na = fmaxf(Y[j][b] - g[j][b] * invL, 0.0f);       // :220
        Y[j][b] = (1.0f + beta) * na - beta * Ac[j][b];                 // :228
        Ac[j][b] = na;
      }
    asm volatile("barrier.cluster.arrive.release;" ::: "memory");
    stage_y();
    gradient();   // of it+1 (discarded if it stops at it)
    asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
    if (*(volatile int *)&vflag0[it % 3] == 0) {   // no violation: stop, the result is A_it
#pragma unroll
      for (int j = 0; j < ROWS; ++j)
#pragma unroll
        for (int b = 0; b < RB; ++b)
          if (colok[b]) Ac[j][b] = As[(warp * ROWS + j) * R + lane + 32 * b];
      break;
    }
    ++it;
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
  if (tid == 0) {
    float mincol = INFINITY;
    for (int c = 0; c < R; ++c) {
      float s = 0.f;
      for (int r2 = 0; r2 < CS; ++r2) s += cluster.map_shared_rank(colsum, r2)[c];
      mincol = fminf(mincol, s);
    }
    flags[0] = (mincol == 0.0f) ? 1 : 0;
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
      float s = 0.f;
      for (int r2 = 0; r2 < CS; ++r2) s += cluster.map_shared_rank(Gp, r2)[idx];
      a.gram_out[idx] = s;
      Zt[idx] = s;   // reuse Zt (no longer needed) for the FP64 Hadamard sum
    }
    __syncthreads();
    if (warp == 0) {
      double h = 0.0;
      for (int idx = lane; idx < R * R; idx += 32) h = fma(np->Z[idx], (double)Zt[idx], h);
      for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
      if (lane == 0) {
        double sma = 0.0;
        for (int r2 = 0; r2 < CS; ++r2) sma += cluster.map_shared_rank(ma, r2)[0];
        *a.inner_MA = sma;
        *a.had_ZG = h;
        *a.iters_out = it;
        *a.repaired_out = repair ? 1 : 0;
      }
    }
  }
  cluster.sync();   // keep every CTA's shared memory alive until rank 0 has read it
}

template <int RB, int ROWS>
size_t nnls_smem_bytes(int R) {
  return sizeof(float) * (2 * R * R + kNnlsWarps * ROWS * R + ((R + 1) & ~1) + 4 + 2 * kNnlsWarps) +
         sizeof(double) * (kNnlsWarps + 2) + 32 + sizeof(float) * (kMaxInner + kNnlsWarps * ROWS) +
         (RB == 1 ? 16 + sizeof(float) * kNnlsWarps * ROWS * 32 : 0);
}

template <int RB, int ROWS>
int launch_nnls_t(int cs, const NnlsArgs &args, cudaStream_t stream) {
  auto kern = nnls_cluster_kernel<RB, ROWS>;
  const size_t smem = nnls_smem_bytes<RB, ROWS>(args.R);
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (cs > 8) PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if ((int64_t)cs * kNnlsWarps * ROWS < args.I)
    return set_error(PTG_ERR_INVALID, "internal: NNLS row tiling");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(kNnlsThreads, 1, 1);
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
  auto kern = nnls_cluster_kernel<2, 16>;
  const size_t smem = nnls_smem_bytes<2, 16>(kMaxR);
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(kNnlsThreads, 1, 1);
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
  const int cap = cs * kNnlsWarps;   // rows per register slot
  const int rows = (I + cap - 1) / cap;
  const bool wide = R > 32;
#define PTG_NNLS_CASE(RWS)                                                    \
  if (rows <= RWS)                                                            \
    return wide ? launch_nnls_t<2, RWS>(cs, args, stream)                     \
                : launch_nnls_t<1, RWS>(cs, args, stream);
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

// ---- Normalize ----
struct NormArgs {
  float *fac[PTG_MAX_ORDER];
  float *gram[PTG_MAX_ORDER];
  int rows[PTG_MAX_ORDER];
  int order, weight, R;
};

// Column multipliers of include/Normalize.hpp:92-174 for column c.
__device__ void normalize_column(const NormArgs &a, int c, float *mult /*[order]*/, float *lf /*[order]*/) {
  const int N = a.order, last = N - 1, w = a.weight;
  // the factor behind lambda_fac[last-1] decides nonZeroFlag
  const int flag_fac = (w <= N - 2) ? (N - 1) : (N - 2);
  const bool nonzero = sqrtf(a.gram[flag_fac][c * a.R + c]) != 0.0f;
  float cumul = 1.0f;
  for (int k = 0; k < N; ++k) {
    mult[k] = 1.0f;
    lf[k] = 1.0f;
  }
  for (int j = 0; j < last; ++j) {
    if (j == w) continue;
    const float nf = sqrtf(a.gram[j][c * a.R + c]);
    if (nonzero) {
      mult[j] = 1.0f / nf;
      cumul *= nf;
      lf[j] = nf;
    }
  }
  if (nonzero) mult[w] = cumul;
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
  eigen_bounds_body(gp, e.order, e.mode, e.R, e.out);
}

// G_k = A_k^T A_k for every factor of the instance (fac or acc set).
__global__ void gram_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ active, int use_acc) {
  const InstDesc &in = d[blockIdx.x];
  if (active && !active[in.inst]) return;
  const int R = in.R;
  for (int k = 0; k < in.order; ++k) {
    const float *A = use_acc ? in.acc[k] : in.fac[k];
    float *G = use_acc ? in.gacc[k] : in.gram[k];
    for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
      const int a = idx / R, b = idx % R;
      float s = 0.f;
      for (int i = 0; i < in.rows[k]; ++i) s = fmaf(A[(size_t)i * R + a], A[(size_t)i * R + b], s);
      G[idx] = s;
    }
  }
}

__global__ void normalize_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ active) {
  const InstDesc &in = d[blockIdx.x];
  if (active && !active[in.inst]) return;
  __shared__ float mult[PTG_MAX_ORDER][64], lfs[PTG_MAX_ORDER][64];
  NormArgs a{};
  for (int k = 0; k < in.order; ++k) {
    a.fac[k] = in.fac[k];
    a.gram[k] = in.gram[k];
    a.rows[k] = in.rows[k];
  }
  a.order = in.order;
  a.weight = in.weight;
  a.R = in.R;
  for (int c = threadIdx.x; c < a.R; c += blockDim.x) {
    float m[PTG_MAX_ORDER], l[PTG_MAX_ORDER];
    normalize_column(a, c, m, l);
    for (int k = 0; k < a.order; ++k) {
      mult[k][c] = m[k];
      lfs[k][c] = l[k];
    }
  }
  __syncthreads();   // every Gram diagonal is read before any Gram is written
  for (int k = 0; k < a.order; ++k)
    for (int idx = threadIdx.x; idx < a.rows[k] * a.R; idx += blockDim.x) a.fac[k][idx] *= mult[k][idx % a.R];
  const int N = a.order, last = N - 1, w = a.weight, R = a.R;
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    const int r1 = idx / R, r2 = idx % R;
    float wm = 1.0f;
    for (int j = 0; j < last; ++j) {
      if (j == w) continue;
      const float nm = lfs[j][r1] * lfs[j][r2];
      wm *= nm;
      a.gram[j][idx] = a.gram[j][idx] / nm;
    }
    a.gram[w][idx] *= wm;
  }
}

// acc = old + step (fac - old) for instances with accel[inst] != 0 (step[inst]).
__global__ void accel_combine_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ accel,
                                             const float *__restrict__ step) {
  const InstDesc &in = d[blockIdx.x];
  if (!accel[in.inst]) return;
  const float s = step[in.inst];
  for (int k = 0; k < in.order; ++k)
    for (int idx = threadIdx.x; idx < in.rows[k] * in.R; idx += blockDim.x) {
      const float o = in.old[k][idx];
      in.acc[k][idx] = o + s * (in.fac[k][idx] - o);
    }
}

// old = fac for instances with flag[inst] != 0
__global__ void copy_old_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ flag) {
  const InstDesc &in = d[blockIdx.x];
  if (!flag[in.inst]) return;
  for (int k = 0; k < in.order; ++k)
    for (int idx = threadIdx.x; idx < in.rows[k] * in.R; idx += blockDim.x) in.old[k][idx] = in.fac[k][idx];
}

// fac, gram = acc, gacc for instances with accepted[inst] != 0
__global__ void select_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ accepted) {
  const InstDesc &in = d[blockIdx.x];
  if (!accepted[in.inst]) return;
  for (int k = 0; k < in.order; ++k) {
    for (int idx = threadIdx.x; idx < in.rows[k] * in.R; idx += blockDim.x) in.fac[k][idx] = in.acc[k][idx];
    for (int idx = threadIdx.x; idx < in.R * in.R; idx += blockDim.x) in.gram[k][idx] = in.gacc[k][idx];
  }
}

// FP64 cost terms of a point: out[0] = <M, A_last>, out[1] = sum(Z_last .* G_last)
__global__ void cost_terms_batched_kernel(const InstDesc *__restrict__ d, const int *__restrict__ flag,
                                          int use_acc) {
  const InstDesc &in = d[blockIdx.x];
  if (flag && !flag[in.inst]) return;
  const int last = in.order - 1, R = in.R;
  const float *A = use_acc ? in.acc[last] : in.fac[last];
  float *const *G = use_acc ? in.gacc : in.gram;
  __shared__ double red[2][32];
  double s = 0.0, h = 0.0;
  for (int64_t idx = threadIdx.x; idx < (int64_t)in.rows[last] * R; idx += blockDim.x)
    s = fma((double)in.M[idx], (double)A[idx], s);
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    double z = 1.0;
    for (int k = last - 1; k >= 0; --k) z *= (double)G[k][idx];
    h = fma(z, (double)G[last][idx], h);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    h += __shfl_down_sync(0xffffffffu, h, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s;
    red[1][threadIdx.x >> 5] = h;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    in.cost_out[0] = a;
    in.cost_out[1] = b;
  }
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
