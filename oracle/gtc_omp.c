/*
 * FP64 OpenMP restatement of Partensor's GTC row solvers -- TEST INFRASTRUCTURE ONLY.
 *
 * The CPU baseline that the sparse-completion workload is timed beside, and a second
 * restatement that the numpy oracle (oracle/gtc.py) is cross-checked against.  Never linked
 * into the product library.  It restates (paths relative to the reference project's root):
 *   - local_L::NesterovMNLS, OpenMP form include/NesterovMNLS.hpp:878-976 (rows in parallel):
 *     per row i, m_i = sum x kr and H_i = sum kr kr^T over the row's entries, L_i =
 *     PowerMethod(H_i, 1e-3) + lambda (:131-160), then max_iter steps of
 *     grad = H_i y - m_i + lambda y, a' = max(y - grad / L_i, 0),
 *     beta = (1 - sqrt(lambda / L_i)) / (1 + sqrt(lambda / L_i)), y = (1 + beta) a' - beta a;
 *   - dynamic_blocksize::StochasticNesterovMNLS, OpenMP form (:553-663): per row and inner
 *     iteration a contiguous block of b_i = floor(c nnz_i) entries from pivot
 *     = draw % (nnz_i - b_i + 1), grad = sum (kr.y - x) kr + lambda (y + a), H and L from the
 *     block, the same step;
 * with the two restatement choices of oracle/gtc.py (PowerMethod from the all-ones vector,
 * the pivot drawn from a splitmix64 hash of (seed, outer, mode, inner, row)).
 *
 * Layout: one mode's matricisation in column-compressed form over rows [0, nrows):
 * ptr[nrows + 1], other[e * (N - 1) + j] the index of the j-th other mode (modes in
 * increasing order) of entry e, vals[e]; factors row-major, F_k[i * R + r].
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PTGO_GTC_MAXR 128

static uint64_t pivot_hash(uint64_t seed, uint64_t outer, uint64_t mode, uint64_t inner, uint64_t row) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + outer * 0xBF58476D1CE4E5B9ull + mode * 0x94D049BB133111EBull +
               inner * 0x2545F4914F6CDD1Dull + row * 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Largest eigenvalue of the R x R matrix H by the power method from the all-ones vector. */
static double power_method(const double *H, int R, double eps) {
  double x[PTGO_GTC_MAXR], ax[PTGO_GTC_MAXR], xn[PTGO_GTC_MAXR];
  for (int r = 0; r < R; ++r) x[r] = 1.0;
  for (int it = 0;; ++it) {
    double nrm = 0.0;
    for (int r = 0; r < R; ++r) {
      double s = 0.0;
      for (int c = 0; c < R; ++c) s += H[r * R + c] * x[c];
      ax[r] = s;
      nrm += s * s;
    }
    nrm = sqrt(nrm) + 1e-12;
    double d = 0.0;
    for (int r = 0; r < R; ++r) {
      xn[r] = ax[r] / nrm;
      d += (xn[r] - x[r]) * (xn[r] - x[r]);
    }
    if (sqrt(d) <= eps || it >= 10000) {
      double v = 0.0;
      for (int r = 0; r < R; ++r) {
        double s = 0.0;
        for (int c = 0; c < R; ++c) s += H[r * R + c] * xn[c];
        v += xn[r] * s;
      }
      return v;
    }
    memcpy(x, xn, sizeof(double) * (size_t)R);
  }
}

/* Khatri-Rao row of entry e: the product of the other modes' factor rows, last mode first
 * (include/MTTKRP.hpp:248-259). */
static void kr_row(int N, int mode, int R, const int32_t *other, int64_t e, double *const *F, double *kr) {
  for (int r = 0; r < R; ++r) kr[r] = 1.0;
  for (int j = N - 2; j >= 0; --j) {
    const int k = j < mode ? j : j + 1;
    const double *row = F[k] + (int64_t)other[e * (N - 1) + j] * R;
    for (int r = 0; r < R; ++r) kr[r] *= row[r];
  }
}

/* One GTC update of factor `mode`, rows [0, nrows), nonnegative.  stochastic = 0: local_L;
 * 1: the stochastic block solver of outer iteration `outer`.  Returns 0, or -1 if R is too
 * large or memory runs out. */
int ptgo_gtc_rows(int N, int R, int mode, const int64_t *ptr, int64_t nrows, const int32_t *other,
                  const double *vals, double **F, int stochastic, double c, int max_inner, double lam,
                  uint64_t seed, int outer, int nthreads) {
  if (R > PTGO_GTC_MAXR) return -1;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  int fail = 0;
#pragma omp parallel num_threads(nthreads)
  {
    double *H = (double *)malloc(sizeof(double) * (size_t)R * R);
    double *kr = (double *)malloc(sizeof(double) * (size_t)R);
    double *m = (double *)malloc(sizeof(double) * (size_t)R);
    double *y = (double *)malloc(sizeof(double) * (size_t)R);
    double *g = (double *)malloc(sizeof(double) * (size_t)R);
    double *an = (double *)malloc(sizeof(double) * (size_t)R);
    if (!H || !kr || !m || !y || !g || !an) {
#pragma omp atomic write
      fail = 1;
    } else {
#pragma omp for schedule(dynamic, 4)
      for (int64_t i = 0; i < nrows; ++i) {
        const int64_t p0 = ptr[i], p1 = ptr[i + 1], nz = p1 - p0;
        double *a = F[mode] + i * R;
        memcpy(y, a, sizeof(double) * (size_t)R);
        if (!stochastic) {
          memset(H, 0, sizeof(double) * (size_t)R * R);
          memset(m, 0, sizeof(double) * (size_t)R);
          for (int64_t e = p0; e < p1; ++e) {
            kr_row(N, mode, R, other, e, F, kr);
            for (int r = 0; r < R; ++r) {
              m[r] += vals[e] * kr[r];
              for (int s = 0; s < R; ++s) H[r * R + s] += kr[r] * kr[s];
            }
          }
          const double L = power_method(H, R, 1e-3) + lam;
          const double sq = sqrt(lam / L), beta = (1.0 - sq) / (1.0 + sq);
          for (int it = 0; it < max_inner; ++it) {
            for (int r = 0; r < R; ++r) {
              double s = 0.0;
              for (int t = 0; t < R; ++t) s += H[r * R + t] * y[t];
              g[r] = s - m[r] + lam * y[r];
            }
            for (int r = 0; r < R; ++r) an[r] = fmax(y[r] - g[r] / L, 0.0);
            for (int r = 0; r < R; ++r) {
              y[r] = (1.0 + beta) * an[r] - beta * a[r];
              a[r] = an[r];
            }
          }
        } else {
          const int64_t b = (int64_t)(c * (double)nz);
          if (b <= 0) continue;
          for (int it = 0; it < max_inner; ++it) {
            const int64_t pivot = (int64_t)(pivot_hash(seed, (uint64_t)outer, (uint64_t)mode, (uint64_t)it,
                                                       (uint64_t)i) %
                                            (uint64_t)(nz - b + 1));
            memset(H, 0, sizeof(double) * (size_t)R * R);
            for (int r = 0; r < R; ++r) g[r] = lam * (y[r] + a[r]);
            for (int64_t e = p0 + pivot; e < p0 + pivot + b; ++e) {
              kr_row(N, mode, R, other, e, F, kr);
              double ky = 0.0;
              for (int r = 0; r < R; ++r) ky += kr[r] * y[r];
              const double res = ky - vals[e];
              for (int r = 0; r < R; ++r) {
                g[r] += res * kr[r];
                for (int s = 0; s < R; ++s) H[r * R + s] += kr[r] * kr[s];
              }
            }
            const double L = power_method(H, R, 1e-3) + lam;
            const double sq = sqrt(lam / L), beta = (1.0 - sq) / (1.0 + sq);
            for (int r = 0; r < R; ++r) an[r] = fmax(y[r] - g[r] / L, 0.0);
            for (int r = 0; r < R; ++r) {
              y[r] = (1.0 + beta) * an[r] - beta * a[r];
              a[r] = an[r];
            }
          }
        }
      }
    }
    free(H); free(kr); free(m); free(y); free(g); free(an);
  }
  return fail ? -1 : 0;
}
