/*
 * FP64 OpenMP restatement of Partensor's CpdOpenMP driver -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the CPU baseline the GPU path is timed beside, and a second, independent
 * restatement that the numpy oracle (oracle/cpd.py) is cross-checked against.  It is
 * never linked into the product library.
 *
 * It restates (paths relative to the reference project's root):
 *   - the blocked OpenMP MTTKRP, include/MTTKRP.hpp:102-225: per block of I_first
 *     columns of X_(n), build the partial Khatri-Rao block row by row (198-217) and do
 *     result += X_(n)block * PKR with a per-thread matrix reduction (34-37, 194-220).
 *     Difference: X_(n) is addressed in place instead of being materialised N times
 *     (include/CpdOpenMP.hpp:272-275); the arithmetic per block is the same.
 *   - the OpenMP ALS loop, include/CpdOpenMP.hpp:266-329, with its explicit-residual cost
 *     (121-125), update_factor (165-204), line_search_accel (223-255);
 *   - NesterovMNLS, include/NesterovMNLS.hpp:45-234 (singular values of the SPD Hessian
 *     from a cyclic Jacobi eigenvalue iteration, a published method restated here);
 *   - Normalize, include/Normalize.hpp:92-174, literally (quirks included);
 *   - PartialCwiseProd, include/PartialCwiseProd.hpp:54-222.
 *
 * Layout: X is ColMajor (i0 fastest); factor k is I_k x R ColMajor (A[i + I_k*r]).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PTGO_MAXN 8

typedef struct {
  int constraints[PTGO_MAXN]; /* 0 unconstrained, 1 nonnegativity, 2 orthogonality */
  double threshold_error;
  double nesterov_delta_1;
  double nesterov_delta_2;
  int max_iter;
  int accel_coeff;
  int accel_fail;
  int acceleration;
  int normalization;
  int nthreads;
} ptgo_options;

typedef struct {
  double frob_tns;
  double f_value;
  double rel_costFunction;
  int ao_iter;
  int accel_coeff;
  int accel_fail;
  double seconds_mttkrp;
  double seconds_total;
} ptgo_status;

static int64_t prod_except(int N, const int64_t *dims, int skip) {
  int64_t p = 1;
  for (int k = 0; k < N; ++k)
    if (k != skip) p *= dims[k];
  return p;
}

/* Blocked OpenMP MTTKRP, include/MTTKRP.hpp:102-225.  out: I_mode x R ColMajor. */
void ptgo_mttkrp(int N, const int64_t *dims, const double *X, const double *const *factors, int R,
                 int mode, double *out, int nthreads) {
  const int first = (mode == 0) ? 1 : 0;
  const int64_t In = dims[mode], If = dims[first];
  const int64_t J = prod_except(N, dims, mode);
  const int64_t nblocks = J / If;
  int64_t stride[PTGO_MAXN];
  stride[0] = 1;
  for (int k = 1; k < N; ++k) stride[k] = stride[k - 1] * dims[k - 1];
  /* the modes enumerated by the block index, lowest mode fastest */
  int bm[PTGO_MAXN], nb = 0;
  for (int k = 0; k < N; ++k)
    if (k != mode && k != first) bm[nb++] = k;
  memset(out, 0, sizeof(double) * (size_t)(In * R));
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
  {
    double *acc = (double *)calloc((size_t)(In * R), sizeof(double));
    double *pkr = (double *)malloc(sizeof(double) * (size_t)(If * R));
    double *kr = (double *)malloc(sizeof(double) * (size_t)R);
#pragma omp for schedule(static, 1)
    for (int64_t b = 0; b < nblocks; ++b) {
      /* Kr = Hadamard of the factor rows selected by the block's digits (:198-206) */
      int64_t rem = b, base = 0;
      for (int r = 0; r < R; ++r) kr[r] = 1.0;
      for (int t = 0; t < nb; ++t) {
        const int k = bm[t];
        const int64_t ik = rem % dims[k];
        rem /= dims[k];
        base += ik * stride[k];
        const double *Ak = factors[k];
        for (int r = 0; r < R; ++r) kr[r] *= Ak[ik + dims[k] * r];
      }
      /* PartialKR(row, :) = A_first(row, :) .* Kr  (:209-212), stored row-major */
      const double *Af = factors[first];
      for (int64_t row = 0; row < If; ++row)
        for (int r = 0; r < R; ++r) pkr[row * R + r] = Af[row + If * r] * kr[r];
      /* acc += X_(n)block * PKR  (:214) */
      for (int64_t in = 0; in < In; ++in) {
        const double *xrow = X + base + in * stride[mode];
        double a[256];
        for (int r = 0; r < R; ++r) a[r] = 0.0;
        for (int64_t row = 0; row < If; ++row) {
          const double x = xrow[row * stride[first]];
          const double *p = pkr + row * R;
          for (int r = 0; r < R; ++r) a[r] += x * p[r];
        }
        for (int r = 0; r < R; ++r) acc[in + In * r] += a[r];
      }
    }
    /* matrix reduction, include/MTTKRP.hpp:34-37 */
#pragma omp critical
    for (int64_t i = 0; i < In * R; ++i) out[i] += acc[i];
    free(acc);
    free(pkr);
    free(kr);
  }
}

/* ||X_(N-1) - A_{N-1} * PKR^T||_F^2 without materialising PKR (include/CpdOpenMP.hpp:121-125) */
static double residual_sq(int N, const int64_t *dims, const double *X, const double *const *factors,
                          int R, int nthreads) {
  const int last = N - 1;
  const int64_t J = prod_except(N, dims, last), Il = dims[last];
  const int64_t I0 = dims[0];
  const int64_t nb = J / I0;
  double total = 0.0;
#pragma omp parallel num_threads(nthreads) reduction(+ : total)
  {
    double *kr = (double *)malloc(sizeof(double) * (size_t)R);
    double *row = (double *)malloc(sizeof(double) * (size_t)(I0 * R));
#pragma omp for schedule(static)
    for (int64_t b = 0; b < nb; ++b) {
      int64_t rem = b;
      for (int r = 0; r < R; ++r) kr[r] = 1.0;
      for (int k = 1; k < last; ++k) {
        const int64_t ik = rem % dims[k];
        rem /= dims[k];
        for (int r = 0; r < R; ++r) kr[r] *= factors[k][ik + dims[k] * r];
      }
      for (int64_t i0 = 0; i0 < I0; ++i0)
        for (int r = 0; r < R; ++r) row[i0 * R + r] = factors[0][i0 + I0 * r] * kr[r];
      for (int64_t il = 0; il < Il; ++il) {
        const double *xs = X + b * I0 + il * J;
        for (int64_t i0 = 0; i0 < I0; ++i0) {
          double m = 0.0;
          for (int r = 0; r < R; ++r) m += row[i0 * R + r] * factors[last][il + Il * r];
          const double d = xs[i0] - m;
          total += d * d;
        }
      }
    }
    free(kr);
    free(row);
  }
  return total;
}

/* Eigenvalues of a symmetric R x R matrix by cyclic Jacobi rotations (Jacobi 1846;
 * Golub & Van Loan, "Matrix Computations", sec. 8.5).  a is overwritten. */
static void jacobi_eigvals(int n, double *a, double *w) {
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += a[i * n + j] * a[i * n + j];
        if (i != j) off += a[i * n + j] * a[i * n + j];
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p * n + q];
        if (apq == 0.0) continue;
        const double app = a[p * n + p], aqq = a[q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = a[i * n + i];
}

static double update_alpha(double alpha, double q) { /* include/NesterovMNLS.hpp:103-113 */
  const double b = alpha * alpha - q, c = -alpha * alpha;
  const double D = b * b - 4.0 * c;
  return (-b + sqrt(D)) / 2.0;
}

/* include/NesterovMNLS.hpp:181-234.  Z: R x R (row-major = col-major, symmetric);
 * W, A: I x R ColMajor.  A is the proximal centre on entry and the result on exit. */
int ptgo_nesterov_mnls(int64_t I, int R, const double *Z, const double *W, double d1, double d2,
                       double *A, int nthreads) {
  double *tmp = (double *)malloc(sizeof(double) * (size_t)R * R);
  double *ev = (double *)malloc(sizeof(double) * (size_t)R);
  memcpy(tmp, Z, sizeof(double) * (size_t)R * R);
  jacobi_eigvals(R, tmp, ev);
  double L = 0.0, mu = INFINITY;
  for (int i = 0; i < R; ++i) { /* singular values of a symmetric matrix = |eigenvalues| */
    const double s = fabs(ev[i]);
    if (s > L) L = s;
    if (s < mu) mu = s;
  }
  double q = mu / L, lam; /* GLambda, :75-91 */
  if (1.0 / q > 1e6) lam = 10.0 * mu;
  else if (1.0 / q > 1e3) lam = mu;
  else lam = mu / 10.0;
  L += lam;
  mu += lam;
  q = mu / L;
  double *Zt = tmp;
  for (int i = 0; i < R * R; ++i) Zt[i] = Z[i];
  for (int i = 0; i < R; ++i) Zt[i * R + i] += lam;
  const size_t sz = (size_t)(I * R);
  double *Wt = (double *)malloc(sizeof(double) * sz);
  double *Aold = (double *)malloc(sizeof(double) * sz);
  double *Y = (double *)malloc(sizeof(double) * sz);
  double *G = (double *)malloc(sizeof(double) * sz);
  for (size_t i = 0; i < sz; ++i) {
    Wt[i] = W[i] + lam * A[i];
    Aold[i] = A[i];
    Y[i] = A[i];
  }
  double alpha = 1.0;
  int iter = 0;
  for (;;) {
    double mx = 0.0, mn = INFINITY;
#pragma omp parallel for num_threads(nthreads) reduction(max : mx) reduction(min : mn)
    for (int64_t i = 0; i < I; ++i)
      for (int c = 0; c < R; ++c) {
        double g = -Wt[i + I * c];
        for (int k = 0; k < R; ++k) g += Y[i + I * k] * Zt[k * R + c];
        G[i + I * c] = g;
        const double v = fabs(g * Y[i + I * c]);
        if (v > mx) mx = v;
        if (g < mn) mn = g;
      }
    if ((mx <= d1 && mn >= -d2) || iter >= 50) break;
    const double na = update_alpha(alpha, q);
    const double beta = alpha * (1.0 - alpha) / (alpha * alpha + na);
#pragma omp parallel for num_threads(nthreads)
    for (int64_t i = 0; i < (int64_t)sz; ++i) {
      double v = Y[i] - G[i] / L;
      v = v > 0.0 ? v : 0.0;
      Y[i] = (1.0 + beta) * v - beta * Aold[i];
      Aold[i] = v;
    }
    alpha = na;
    ++iter;
  }
  memcpy(A, Aold, sizeof(double) * sz);
  free(tmp); free(ev); free(Wt); free(Aold); free(Y); free(G);
  return iter;
}

static void gram(int64_t I, int R, const double *A, double *G) {
  for (int a = 0; a < R; ++a)
    for (int b = 0; b < R; ++b) {
      double s = 0.0;
      for (int64_t i = 0; i < I; ++i) s += A[i + I * a] * A[i + I * b];
      G[a * R + b] = s;
    }
}

static void partial_cwise(int N, int R, double *const *grams, int mode, double *Z) {
  for (int i = 0; i < R * R; ++i) Z[i] = 1.0;
  for (int k = N - 1; k >= 0; --k)
    if (k != mode)
      for (int i = 0; i < R * R; ++i) Z[i] *= grams[k][i];
}

/* include/Normalize.hpp:92-174, literally. */
static void normalize(int N, int weight, int R, double *const *grams, double *const *factors,
                      const int64_t *dims) {
  const int last = N - 1;
  int pass = 0;
  double cumul = 1.0;
  int nonzero = 1;
  double *lf[PTGO_MAXN];
  double nf[PTGO_MAXN];
  double *nm[PTGO_MAXN];
  for (int i = 0; i < N; ++i) {
    nm[i] = (double *)malloc(sizeof(double) * (size_t)R * R);
    if (i != weight) {
      nf[i - pass] = 1.0;
      lf[i - pass] = (double *)malloc(sizeof(double) * (size_t)R);
      for (int r = 0; r < R; ++r) lf[i - pass][r] = grams[i][r * R + r];
      for (int t = 0; t < R * R; ++t) nm[i][t] = 0.0;
    } else {
      for (int t = 0; t < R * R; ++t) nm[i][t] = 1.0;
      pass = 1;
    }
  }
  for (int i = 0; i < R; ++i) {
    for (int j = 0; j < last; ++j) {
      nf[j] = sqrt(lf[j][i]);
      nonzero = !(nf[j] == 0.0);
    }
    if (!nonzero) {
      for (int j = 0; j < last; ++j) lf[j][i] = 1.0;
    } else {
      pass = 0;
      for (int j = 0; j < last; ++j) {
        if (j == weight) { pass = 1; continue; }
        const double inv = 1.0 / nf[j - pass];
        for (int64_t t = 0; t < dims[j]; ++t) factors[j][t + dims[j] * i] *= inv;
        cumul *= nf[j - pass];
        lf[j - pass][i] = nf[j - pass];
      }
      for (int64_t t = 0; t < dims[weight]; ++t) factors[weight][t + dims[weight] * i] *= cumul;
      cumul = 1.0;
    }
  }
  pass = 0;
  for (int i = 0; i < last; ++i) {
    if (i == weight) { pass = 1; continue; }
    for (int a = 0; a < R; ++a)
      for (int b = 0; b < R; ++b) nm[i][a * R + b] = lf[i - pass][a] * lf[i - pass][b];
    for (int t = 0; t < R * R; ++t) {
      nm[weight][t] *= nm[i][t];
      grams[i][t] /= nm[i][t];
    }
  }
  for (int t = 0; t < R * R; ++t) grams[weight][t] *= nm[weight][t];
  for (int i = 0; i < last; ++i) free(lf[i]);
  for (int i = 0; i < N; ++i) free(nm[i]);
}

/* include/CpdOpenMP.hpp:266-329 with the factorsInit entry.  factors (in/out) hold the
 * initial factors on entry and the result on exit.  trace (optional, 3 doubles per
 * sweep: f_value, rel, accel accepted 0/1) must hold max_iter entries. */
int ptgo_cpd_als(int N, const int64_t *dims, const double *X, int R, ptgo_options *opt,
                 double **factors, ptgo_status *st, double *trace) {
  const int last = N - 1;
  int nth = opt->nthreads > 0 ? opt->nthreads : omp_get_max_threads();
  double t_start = omp_get_wtime(), t_mttkrp = 0.0;
  double *grams[PTGO_MAXN], *M[PTGO_MAXN], *old[PTGO_MAXN], *acc[PTGO_MAXN], *accg[PTGO_MAXN];
  double *prev[PTGO_MAXN]; /* temp_matrix of update_factor (include/CpdOpenMP.hpp:181) */
  double *Z = (double *)malloc(sizeof(double) * (size_t)R * R);
  for (int k = 0; k < N; ++k) {
    const size_t sz = (size_t)(dims[k] * R);
    grams[k] = (double *)malloc(sizeof(double) * (size_t)R * R);
    accg[k] = (double *)malloc(sizeof(double) * (size_t)R * R);
    M[k] = (double *)malloc(sizeof(double) * sz);
    old[k] = (double *)malloc(sizeof(double) * sz);
    acc[k] = (double *)malloc(sizeof(double) * sz);
    prev[k] = (double *)malloc(sizeof(double) * sz);
    gram(dims[k], R, factors[k], grams[k]);
  }
  int all_orth = 1, weight = 0;
  if (opt->normalization)
    for (int i = 0; i < N; ++i)
      if (opt->constraints[i] != 2) { all_orth = 0; weight = i; break; }
  int64_t total = 1;
  for (int k = 0; k < N; ++k) total *= dims[k];
  double frob = 0.0;
#pragma omp parallel for num_threads(nth) reduction(+ : frob)
  for (int64_t i = 0; i < total; ++i) frob += X[i] * X[i];
  st->frob_tns = frob;
  st->f_value = sqrt(residual_sq(N, dims, X, (const double *const *)factors, R, nth));
  st->rel_costFunction = st->f_value / sqrt(frob);
  st->ao_iter = 0;
  int have_old = 0;
  for (;;) {
    st->ao_iter++;
    for (int i = 0; i < N; ++i) {
      double t0 = omp_get_wtime();
      ptgo_mttkrp(N, dims, X, (const double *const *)factors, R, i, M[i], nth);
      t_mttkrp += omp_get_wtime() - t0;
      partial_cwise(N, R, grams, i, Z);
      const size_t sz = (size_t)(dims[i] * R);
      if (opt->constraints[i] == 1) {
        memcpy(prev[i], factors[i], sizeof(double) * sz);
        ptgo_nesterov_mnls(dims[i], R, Z, M[i], opt->nesterov_delta_1, opt->nesterov_delta_2,
                           factors[i], nth);
        double minsum = INFINITY;
        for (int r = 0; r < R; ++r) {
          double s = 0.0;
          for (int64_t t = 0; t < dims[i]; ++t) s += fabs(factors[i][t + dims[i] * r]);
          if (s < minsum) minsum = s;
        }
        if (minsum == 0.0)
          for (size_t t = 0; t < sz; ++t) factors[i][t] = 0.9 * factors[i][t] + 0.1 * prev[i][t];
      }
      gram(dims[i], R, factors[i], grams[i]);
      if (i == last)
        st->f_value = sqrt(residual_sq(N, dims, X, (const double *const *)factors, R, nth));
    }
    st->rel_costFunction = st->f_value / sqrt(frob);
    if (opt->normalization && !all_orth) normalize(N, weight, R, grams, factors, dims);
    int accepted = 0;
    const double f_sweep = st->f_value;
    const int stop = st->rel_costFunction < opt->threshold_error || st->ao_iter >= opt->max_iter;
    if (!stop && opt->acceleration) {
      if (have_old && st->ao_iter > 1) {
        const double step = pow((double)(st->ao_iter + 1), 1.0 / (double)opt->accel_coeff);
        for (int k = 0; k < N; ++k) {
          for (int64_t t = 0; t < dims[k] * R; ++t)
            acc[k][t] = old[k][t] + step * (factors[k][t] - old[k][t]);
          gram(dims[k], R, acc[k], accg[k]);
        }
        double t0 = omp_get_wtime();
        ptgo_mttkrp(N, dims, X, (const double *const *)acc, R, last, M[last], nth);
        t_mttkrp += omp_get_wtime() - t0;
        partial_cwise(N, R, accg, last, Z);
        double s1 = 0.0, s2 = 0.0;
        for (int t = 0; t < R * R; ++t) s1 += Z[t] * accg[last][t];
        for (int64_t t = 0; t < dims[last] * R; ++t) s2 += M[last][t] * acc[last][t];
        double f2 = frob + s1 - 2.0 * s2;
        const double fa = sqrt(f2 > 0.0 ? f2 : 0.0);
        /* the normalised factors become old_factors whatever the outcome (:348-353) */
        for (int k = 0; k < N; ++k) memcpy(old[k], factors[k], sizeof(double) * (size_t)(dims[k] * R));
        if (st->f_value > fa) {
          for (int k = 0; k < N; ++k) {
            memcpy(factors[k], acc[k], sizeof(double) * (size_t)(dims[k] * R));
            memcpy(grams[k], accg[k], sizeof(double) * (size_t)R * R);
          }
          st->f_value = fa;
          accepted = 1;
        } else {
          opt->accel_fail++;
        }
        if (opt->accel_fail == 5) {
          opt->accel_fail = 0;
          opt->accel_coeff++;
        }
      } else {
        for (int k = 0; k < N; ++k) memcpy(old[k], factors[k], sizeof(double) * (size_t)(dims[k] * R));
        have_old = 1;
      }
    }
    if (trace) {
      trace[3 * (st->ao_iter - 1) + 0] = f_sweep;
      trace[3 * (st->ao_iter - 1) + 1] = st->rel_costFunction;
      trace[3 * (st->ao_iter - 1) + 2] = accepted;
    }
    if (stop) break;
  }
  st->accel_coeff = opt->accel_coeff;
  st->accel_fail = opt->accel_fail;
  st->seconds_mttkrp = t_mttkrp;
  st->seconds_total = omp_get_wtime() - t_start;
  for (int k = 0; k < N; ++k) {
    free(grams[k]); free(accg[k]); free(M[k]); free(old[k]); free(acc[k]); free(prev[k]);
  }
  free(Z);
  return 0;
}
