// Block-level bodies shared by the per-mode solver kernels (ptg_solve.cu), the batched
// per-phase kernels and the persistent batched solver (ptg_batched.cu): the FP64 eigenvalue
// bounds of Z, the column normalisation, and the one-instance-per-CTA forms of the Gram,
// normalisation, line-search and cost-term steps.  Each is called by every thread of a CTA.
#pragma once
#include <cmath>

#include "ptg_internal.h"
#include "ptg_sync.cuh"

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

// Sign of p for a Sturm count (0 positive, 1 negative); a zero takes the previous sign.  Read
// from the high and low words with integer instructions.
__device__ __forceinline__ int sturm_sign(double p, int prev) {
  const int hi = __double2hiint(p), lo = __double2loint(p);
  return (((hi & 0x7fffffff) | lo) == 0) ? prev : (int)((unsigned)hi >> 31);
}

// The same count in FP64 for a tridiagonal scaled so that its Gershgorin interval lies in
// [-1, 1]: the sign changes of the characteristic-polynomial sequence
// p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2} (p_{-1} = 1), a zero taking the previous sign.
// With |d_i - x| <= 2 and e^2 <= 1, |p| grows by less than a factor 3 per step, so 64 steps
// cannot overflow; when both of the last two values fall below 2^-600 they are scaled up by
// 2^600 (exact).  On GB300 a warp's FP64 instruction holds its SM sub-partition for about 64
// cycles, so a step is three FP64 instructions (subtract, multiply, fused multiply-add) and
// the sign and range tests run on the integer pipe.
__device__ int sturm_count_f64s(const double *d, const double *e2, int n, double x) {
  double pm2 = 1.0, pm1 = d[0] - x;
  int sprev = sturm_sign(pm1, 0);
  int cnt = sprev;   // p_{-1} = 1 > 0
  for (int i = 1; i < n; ++i) {
    const double p = fma(d[i] - x, pm1, -(e2[i - 1] * pm2));
    const int s = sturm_sign(p, sprev);
    cnt += s ^ sprev;
    sprev = s;
    pm2 = pm1;
    pm1 = p;
    if (((__double2hiint(pm1) >> 20) & 0x7ff) < 423 && ((__double2hiint(pm2) >> 20) & 0x7ff) < 423) {
      pm1 *= 0x1p+600;
      pm2 *= 0x1p+600;
    }
  }
  return cnt;
}

// NT threads (a multiple of 64, at least 128) take part, with indices tid in [0, NT) and the
// barrier `sync` among them (the whole CTA, or a 128-thread group beside other work); every
// one of them must call it.
template <int NT = kEigThreads, typename Sync = SyncCta>
__device__ void eigen_bounds_body(const GramPtrs &gp, int order, int mode, int R, NnlsParams *out, int tid,
                                  Sync sync = Sync()) {
  static_assert(NT % kMaxR == 0 && NT >= 128, "eigenvalue-bound thread count");
  constexpr int lda = kMaxR + 1;              // padded rows: column reads and mirrored writes
  __shared__ double A[kMaxR * lda];           // spread over the banks
  __shared__ double xs[kMaxR], vs[kMaxR], ws[kMaxR];
  __shared__ double ps[4][kMaxR];
  __shared__ double d[kMaxR], e[kMaxR], e2[kMaxR];
  __shared__ double redb[2][NT / 32];
  __shared__ double s_scalar[4];
  __shared__ double lohi[2][2];
  __shared__ float df[kMaxR], e2f[kMaxR];
  const int n = R;

  // Z = prod_{k != mode} G_k (FP64), k from order-1 down to 0 as PartialCwiseProd orders it;
  // the tridiagonalisation works on the lower triangle mirrored, so A is exactly symmetric
  for (int idx = tid; idx < n * n; idx += NT) {
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
  sync();

  // Block sum: warp shuffles, then every thread adds the warps' partials in warp order from one
  // of two alternating buffers, so a sum costs one barrier and no broadcast.  (A buffer is
  // written again two sums later, after a barrier every thread passes once it has read it.)
  int rb = 0;
  auto block_sum = [&](double x) -> double {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((tid & 31) == 0) redb[rb][tid >> 5] = x;
    sync();
    // every warp sums the partials by a butterfly: the same bits in every lane (each step
    // adds the same two values), five FP64 additions instead of one per warp
    double v = (tid & 31) < NT / 32 ? redb[rb][tid & 31] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    rb ^= 1;
    return v;
  };

  // ---- Householder tridiagonalisation (Golub & Van Loan alg. 8.3.1), H = I - beta v v^T,
  // v = x - alpha e_1, A_sub <- A_sub - v w^T - w v^T with p = beta A_sub v, w = p - (beta/2)(p.v) v.
  // A_sub v = A_sub x - alpha A_sub e_1: the product with x runs before alpha is known, beside
  // the square root and the division (one thread: GB300's FP64 pipe is the scarce resource).
  // Thread (q, i) sums a quarter of row i's terms, reading column entries (A is symmetric) so
  // that a warp's threads read consecutive addresses. ----
  // the product A_sub x: thread (pq, pi) sums a part of row pi's terms; rows in 32 or 64
  // slots, at most 4 parts (fewer FP64 instructions on the longest thread, and a short sum)
  const int yrows = n <= 32 ? 32 : kMaxR, yparts = min(NT / yrows, 4);
  const int pi = tid % yrows, pq = tid / yrows;
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
    double y = 0.0;       // (A_sub x)_i, partial over part pq of j
    if (pi < m && pq < yparts) {
      const double *col = A + (k + 1) * lda + (k + 1 + pi);
      const int chunk = (m + yparts - 1) / yparts;
      const int j1 = min(m, (pq + 1) * chunk);
      for (int j = pq * chunk; j < j1; ++j) y = fma(col[j * lda], xs[j], y);
      ps[pq][pi] = y;
    }
    if (tid == NT - 1) {   // holds no row of the product (its row slot is past m - 1)
      const double al = (x0 >= 0.0 ? -1.0 : 1.0) * sqrt(x0 * x0 + sigma);
      const double dv = x0 - al;
      s_scalar[0] = al;
      s_scalar[3] = 2.0 / (dv * dv + sigma);
    }
    sync();
    const double alpha = s_scalar[0], beta = s_scalar[3];
    const double v0 = x0 - alpha;
    double pv = 0.0, vi = 0.0, pvi = 0.0;
    if (tid < m) {
      double yi = 0.0;
      for (int q = 0; q < yparts; ++q) yi += ps[q][tid];
      vi = tid == 0 ? v0 : xi;
      pvi = beta * fma(-alpha, A[(k + 1) * lda + (k + 1 + tid)], yi);   // p_i
      pv = pvi * vi;
    }
    const double K = 0.5 * beta * block_sum(pv);
    if (tid < m) {
      vs[tid] = vi;
      ws[tid] = pvi - K * vi;
    }
    sync();
    for (int idx = tid; idx < m * m; idx += NT) {
      const int i = idx / m, j = idx - (idx / m) * m;
      if (j > i) continue;
      const double a = A[(k + 1 + i) * lda + (k + 1 + j)] - (vs[i] * ws[j] + ws[i] * vs[j]);
      A[(k + 1 + i) * lda + (k + 1 + j)] = a;
      A[(k + 1 + j) * lda + (k + 1 + i)] = a;
    }
    if (tid == 0) e[k] = alpha;
    sync();
  }
  // ---- T = (d, e) scaled by a power of two, sc, so that its Gershgorin interval lies in
  // [-1, 1]; the counts and the bisection run on the scaled T (exact), the result is scaled
  // back at the end ----
  for (int i = tid; i < n; i += NT) d[i] = A[i * lda + i];
  if (tid == 0 && n >= 2) e[n - 2] = A[(n - 1) * lda + (n - 2)];
  sync();
  if (tid < 32) {   // warp 0: the Gershgorin interval
    double glo = 1e300, ghi = -1e300;
    for (int i = tid; i < n; i += 32) {
      const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
      glo = fmin(glo, d[i] - r);
      ghi = fmax(ghi, d[i] + r);
    }
    for (int o = 16; o > 0; o >>= 1) {
      glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, o));
      ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
    }
    if (tid == 0) {
      const double g = fmax(fabs(glo), fabs(ghi));
      int E = 0;
      if (g > 0.0 && isfinite(g)) frexp(g, &E);
      const double sc = ldexp(1.0, -E);
      const double gs = g * sc;                     // in [0.5, 1)
      const double pad = 1e-12 * gs + 1e-300;
      lohi[0][0] = lohi[1][0] = glo * sc - pad;     // smallest and largest eigenvalue
      lohi[0][1] = lohi[1][1] = ghi * sc + pad;
      s_scalar[1] = gs;                             // ||T|| bound, scaled
      s_scalar[2] = sc;
    }
  }
  sync();
  {
    const double sc = s_scalar[2];
    for (int i = tid; i < n; i += NT) {
      const double di = d[i] * sc;
      d[i] = di;
      df[i] = (float)di;
      if (i + 1 < n) {
        const double ei = e[i] * sc;
        e2[i] = ei * ei;
        e2f[i] = (float)(ei * ei);
      }
    }
  }
  sync();   // d and e2 are complete before any thread reads them (n > 32 spans warps)

  // ---- bisection: warp 0 brackets the smallest eigenvalue, warp 1 the largest, with a
  // 32-way multisection per round: FP32 counts first, then FP64 counts on the widened
  // FP32 bracket.  The points of a round come from fixed fractions (j + 1) / 33 and the new
  // bracket from two of them (shuffles), so no round divides ----
  if (tid < 64) {
    const int which = tid >> 5;      // 0: min, 1: max
    const int j = tid & 31;
    const int target = which == 0 ? 1 : n;  // count(x) >= target  <=>  x > lambda
    float flo = __double2float_rd(lohi[which][0]), fhi = __double2float_ru(lohi[which][1]);
    const float cf = (float)(j + 1) * (1.0f / 33.0f);
    for (int round = 0; round < 6; ++round) {
      const float x = fmaf(fhi - flo, cf, flo);
      const bool hit = sturm_count_f32(df, e2f, n, x) >= target;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      const int f = m ? (__ffs(m) - 1) : 32;
      const float xl = __shfl_sync(0xffffffffu, x, (f + 31) & 31), xh = __shfl_sync(0xffffffffu, x, f & 31);
      flo = (f == 0) ? flo : xl;
      fhi = (f == 32) ? fhi : xh;
    }
    // the FP32 counts are exact for a matrix within a few FP32 ulps of T (entrywise), so
    // the eigenvalue lies within 16 * eps32 * ||T|| of the FP32 bracket
    const double margin = 16.0 * 1.1920929e-7 * s_scalar[1] + 1e-300;
    double lo = (double)flo - margin, hi = (double)fhi + margin;
    // ... which holds while FP32 represents T well.  Where it does not (counts off by more
    // than the margin) the FP64 counts at the widened ends show it: then the FP64
    // multisection starts over from the Gershgorin interval, with enough rounds (33^16) to
    // reach FP64 resolution from there.
    int c_end = 0;
    if (j < 2) c_end = sturm_count_f64s(d, e2, n, j == 0 ? lo : hi);
    const int c_lo = __shfl_sync(0xffffffffu, c_end, 0), c_hi = __shfl_sync(0xffffffffu, c_end, 1);
    int rounds64 = 8;
    if (!(c_lo < target && c_hi >= target)) {
      lo = lohi[which][0];
      hi = lohi[which][1];
      rounds64 = 16;
    }
    const double cd = (double)(j + 1) * (1.0 / 33.0);
    for (int round = 0; round < rounds64; ++round) {
      // lo and hi are the same in every lane: the warp leaves together once the bracket is
      // within 2^-42 of the eigenvalue's magnitude
      if (hi - lo <= 0x1p-42 * fmax(fabs(lo), fabs(hi))) break;
      const double x = fma(hi - lo, cd, lo);
      const bool hit = sturm_count_f64s(d, e2, n, x) >= target;
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      const int f = m ? (__ffs(m) - 1) : 32;
      const double xl = __shfl_sync(0xffffffffu, x, (f + 31) & 31), xh = __shfl_sync(0xffffffffu, x, f & 31);
      lo = (f == 0) ? lo : xl;
      hi = (f == 32) ? hi : xh;
    }
    if (j == 0) {
      lohi[which][0] = lo;
      lohi[which][1] = hi;
    }
  }
  sync();
  if (tid < 32) {
    // scale-free summaries of Z for the warm-start network: its diagonal's sum, min and max
    double dsum = 0.0, dmin = 1e300, dmax = -1e300;
    for (int i = tid; i < n; i += 32) {
      const double z = out->Z[i * n + i];
      dsum += z;
      dmin = fmin(dmin, z);
      dmax = fmax(dmax, z);
    }
    for (int o = 16; o > 0; o >>= 1) {
      dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
      dmin = fmin(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
      dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    }
    if (tid == 0) {
      const double unscale = 1.0 / s_scalar[2];   // a power of two: exact
      const double lmin = 0.5 * (lohi[0][0] + lohi[0][1]) * unscale;
      const double lmax = 0.5 * (lohi[1][0] + lohi[1][1]) * unscale;
      // singular values of a symmetric matrix are |eigenvalues|
      double L = fmax(fabs(lmax), fabs(lmin));
      double mu = fabs(lmin);
      if (n == 1) L = mu = fabs(d[0] * unscale);
      {
        const double Ls = L > 0.0 ? L : 1.0;
        const float inv = (float)(1.0 / Ls);
        out->feat[0] = log10f((float)fmin(Ls / fmax(mu, 1e-300), 1e30)) / 6.0f;
        out->feat[1] = (float)mu * inv;
        out->feat[2] = (float)(dsum / n) * inv;
        out->feat[3] = (float)dmin * inv;
        out->feat[4] = (float)dmax * inv;
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

// ---- one instance per CTA (the batched solver) ----

// G_k = A_k^T A_k for every factor of the instance (fac or acc set).
__device__ void gram_block(const InstDesc &in, int use_acc) {
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

// include/Normalize.hpp:92-174 for one instance
__device__ void normalize_block(const InstDesc &in) {
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

// acc = old + s (fac - old)  (include/Cpd.hpp:257-261)
__device__ void accel_combine_block(const InstDesc &in, float s) {
  for (int k = 0; k < in.order; ++k)
    for (int idx = threadIdx.x; idx < in.rows[k] * in.R; idx += blockDim.x) {
      const float o = in.old[k][idx];
      in.acc[k][idx] = o + s * (in.fac[k][idx] - o);
    }
}

// old = fac
__device__ void copy_old_block(const InstDesc &in) {
  for (int k = 0; k < in.order; ++k)
    for (int idx = threadIdx.x; idx < in.rows[k] * in.R; idx += blockDim.x) in.old[k][idx] = in.fac[k][idx];
}

// fac, gram = acc, gacc
__device__ void select_block(const InstDesc &in) {
  for (int k = 0; k < in.order; ++k) {
    for (int idx = threadIdx.x; idx < in.rows[k] * in.R; idx += blockDim.x) in.fac[k][idx] = in.acc[k][idx];
    for (int idx = threadIdx.x; idx < in.R * in.R; idx += blockDim.x) in.gram[k][idx] = in.gacc[k][idx];
  }
}

// FP64 cost terms of a point: out[0] = <M, A_m>, out[1] = sum of the Hadamard product of all
// Grams, with M the MTTKRP of mode m: the last mode for the factors (the sweep's own), mode 0
// for the line-search point (its mode-0 MTTKRP is the next sweep's first one when it is taken)
__device__ void cost_terms_block(const InstDesc &in, int use_acc) {
  const int last = in.order - 1, R = in.R, m = use_acc ? 0 : last;
  const float *A = use_acc ? in.acc[m] : in.fac[m];
  float *const *G = use_acc ? in.gacc : in.gram;
  __shared__ double red[2][32];
  double s = 0.0, h = 0.0;
  for (int64_t idx = threadIdx.x; idx < (int64_t)in.rows[m] * R; idx += blockDim.x)
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

constexpr int BN_THREADS = 512;
constexpr int BN_MAXR = 32;

struct BNnls {
  const float *M;
  float *A;          // in: start and proximal centre; out: solution
  float *Wt;         // scratch [I][R]
  int I, R, inst;
  const NnlsParams *np;
  float d1, d2;
  float *gram_out;
  double *scal;      // [0] <M, A>, [1] sum(Z .* G)
  int *iscal;        // [0] iterations, [1] repaired
};

// Nesterov MNLS of one instance per CTA (include/NesterovMNLS.hpp:181-234 with the zero-column
// repair of include/Cpd.hpp:206-207 and the Gram of :227).  Lane = column; a warp owns
// groups of 4 rows (all columns), so the product Y Z~ of a row needs only its own warp's Y;
// Y is kept transposed in shared memory so the 4 values of a k step are one broadcast 16-byte
// load.  The global stop test (max |grad .* Y| <= delta1 and min grad >= -delta2, :217-218)
// fails iff some element violates it, so a warp that sees a violation sets the iteration's
// flag word (three in rotation) and the block meets once per iteration; the update is done
// speculatively into the other half of a ping-pong A buffer, so A_it survives a stop.
// Shared memory: sm (16-byte aligned) holds nnls_block_smem_floats(I, R) floats; every one
// of the CTA's BN_THREADS threads calls it.
__device__ void nnls_block_body(const BNnls &a, float *sm) {
  const int R = a.R, I = a.I, Ip = (I + 3) & ~3;
  float *Yt = sm;                        // [R][Ip]
  float *Ab[2];
  Ab[0] = Yt + (size_t)R * Ip;           // [I][R]
  Ab[1] = Ab[0] + (size_t)I * R;         // [I][R]
  __shared__ int vflag[3];
  __shared__ double dred[2][BN_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const NnlsParams *np = a.np;
  const float L = (float)np->L, lam = (float)np->lambda, invL = 1.0f / L;
  const int c = lane;
  const bool cok = c < R;
  float z[BN_MAXR];
#pragma unroll
  for (int k = 0; k < BN_MAXR; ++k) {
    float v = 0.0f;
    if (k < R && cok) v = (float)np->Z[k * R + c] + (k == c ? lam : 0.0f);
    z[k] = v;
  }
  for (int idx = tid; idx < I * R; idx += BN_THREADS) {
    const int i = idx / R, cc = idx % R;
    const float a0 = a.A[idx];
    Ab[0][idx] = a0;
    Yt[cc * Ip + i] = a0;
    a.Wt[idx] = a.M[idx] + lam * a0;     // W~ = W + lambda A0 (:206)
  }
  for (int idx = tid; idx < R * (Ip - I); idx += BN_THREADS) Yt[(idx / (Ip - I)) * Ip + I + idx % (Ip - I)] = 0.0f;
  if (tid < 3) vflag[tid] = 0;
  __syncthreads();
  int it = 0;
  for (;; ++it) {
    if (it >= kMaxInner) break;   // A_it is the result
    const float *Acur = Ab[it & 1];
    float *Anext = Ab[(it + 1) & 1];
    const float beta = np->beta[it];
    bool viol = false;
    for (int g = warp; 4 * g < I; g += BN_THREADS / 32) {
      const int i0 = 4 * g;
      float acc[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] = (i0 + r < I && cok) ? -a.Wt[(size_t)(i0 + r) * R + c] : 0.0f;
#pragma unroll
      for (int k = 0; k < BN_MAXR; ++k) {
        if (k < R) {
          const float4 y4 = *reinterpret_cast<const float4 *>(&Yt[k * Ip + i0]);
          acc[0] = fmaf(y4.x, z[k], acc[0]);
          acc[1] = fmaf(y4.y, z[k], acc[1]);
          acc[2] = fmaf(y4.z, z[k], acc[2]);
          acc[3] = fmaf(y4.w, z[k], acc[3]);
        }
      }
      __syncwarp();   // every lane has read this group's Y before any lane writes it
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (i0 + r < I && cok) {
          const int i = i0 + r;
          const float y = Yt[c * Ip + i];
          viol |= (fabsf(acc[r] * y) > a.d1) || (acc[r] < -a.d2);
          const float na = fmaxf(y - acc[r] * invL, 0.0f);                // :220
          Yt[c * Ip + i] = (1.0f + beta) * na - beta * Acur[i * R + c];   // :228
          Anext[i * R + c] = na;
        }
      __syncwarp();
    }
    if (__any_sync(0xffffffffu, viol) && lane == 0) vflag[it % 3] = 1;
    if (tid == 0) vflag[(it + 1) % 3] = 0;   // the word of it+1 (read last at it-2)
    __syncthreads();
    if (vflag[it % 3] == 0) break;           // no violation: stop, the result is A_it
  }
  float *Ac = Ab[it & 1];
  // zero-column repair (:206-207): a column whose |A| sums to zero over all rows
  __shared__ int repair;
  if (tid == 0) repair = 0;
  __syncthreads();
  if (tid < R) {
    float s = 0.0f;
    for (int i = 0; i < I; ++i) s += fabsf(Ac[i * R + tid]);
    if (s == 0.0f) atomicExch(&repair, 1);
  }
  __syncthreads();
  if (repair)
    for (int idx = tid; idx < I * R; idx += BN_THREADS) Ac[idx] = 0.9f * Ac[idx] + 0.1f * a.A[idx];
  __syncthreads();
  double ma = 0.0;
  for (int idx = tid; idx < I * R; idx += BN_THREADS) {
    a.A[idx] = Ac[idx];
    ma = fma((double)a.M[idx], (double)Ac[idx], ma);
  }
  double hz = 0.0;
  for (int idx = tid; idx < R * R; idx += BN_THREADS) {
    const int r1 = idx / R, r2 = idx % R;
    float s = 0.0f;
    for (int i = 0; i < I; ++i) s = fmaf(Ac[i * R + r1], Ac[i * R + r2], s);
    a.gram_out[idx] = s;
    hz = fma(np->Z[idx], (double)s, hz);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ma += __shfl_down_sync(0xffffffffu, ma, o);
    hz += __shfl_down_sync(0xffffffffu, hz, o);
  }
  if (lane == 0) {
    dred[0][warp] = ma;
    dred[1][warp] = hz;
  }
  __syncthreads();
  if (tid == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < BN_THREADS / 32; ++w) {
      s0 += dred[0][w];
      s1 += dred[1][w];
    }
    a.scal[0] = s0;
    a.scal[1] = s1;
    a.iscal[0] = it;
    a.iscal[1] = repair;
  }
}

__host__ __device__ inline size_t nnls_block_smem_floats(int I, int R) {
  return (size_t)R * ((I + 3) & ~3) + 2 * (size_t)I * R;
}

}  // namespace
}  // namespace ptg
