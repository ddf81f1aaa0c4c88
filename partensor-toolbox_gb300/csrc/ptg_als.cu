// CPD-ALS driver: the outer loop of include/Cpd.hpp:288-356 (and of its CUDA policy,
// include/CUDA/CpdCUDA.hpp:277-383) with every per-iteration step on the GPU.
//
// Per mode n (main stream S, side stream T):
//   T: FP64 eigenbounds of Z_n = Hadamard of the Grams k != n      (runs beside the MTTKRP)
//   S: MTTKRP_n                                                     (reads the tensor once)
//   S: Nesterov MNLS on a cluster, fused zero-column repair, Gram and <M, A> (FP64)
// After the sweep: cost f = sqrt(||X||^2 - 2<M_N, A_N> + sum(Z_N .* G_N)) assembled in FP64
// (include/CUDA/CpdCUDA.hpp:137-142), Normalize, the stop test and the line-search
// acceleration (include/Cpd.hpp:247-278) with one more last-mode MTTKRP.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ptg_internal.h"

namespace ptg {
namespace {

struct AlsBuffers {
  int N = 0, R = 0;
  int rows[PTG_MAX_ORDER] = {0};
  float *fac[PTG_MAX_ORDER] = {nullptr};
  float *old[PTG_MAX_ORDER] = {nullptr};
  float *acc[PTG_MAX_ORDER] = {nullptr};
  float *gram[PTG_MAX_ORDER] = {nullptr};
  float *gacc[PTG_MAX_ORDER] = {nullptr};
  float *M = nullptr;
  float *TL = nullptr, *TR = nullptr;   // dimension-tree node tensors (when used)
  float *gpart = nullptr;
  NnlsParams *np = nullptr;
  double *dsc = nullptr;  // [N][2]: <M, A>, sum(Z .* G); [N][2..3]: cost terms of a point
  int *isc = nullptr;     // [N][2]: iterations, repaired
  double *W = nullptr;    // R x R FP64: Z^{-1} or (M^T M)^{-1/2} (other constraints)
  void *base = nullptr;

  int alloc(const int64_t *dims, int order, int rank, int64_t rows_left = 0, int64_t rows_right = 0) {
    N = order;
    R = rank;
    size_t off = 0;
    auto take = [&](size_t bytes) {
      const size_t o = off;
      off += (bytes + 255) / 256 * 256;
      return o;
    };
    size_t o_fac[PTG_MAX_ORDER], o_old[PTG_MAX_ORDER], o_acc[PTG_MAX_ORDER], o_g[PTG_MAX_ORDER],
        o_ga[PTG_MAX_ORDER];
    int64_t maxrows = 0;
    size_t gp = 0;
    for (int k = 0; k < N; ++k) {
      rows[k] = (int)dims[k];
      maxrows = std::max<int64_t>(maxrows, dims[k]);
      const size_t fb = sizeof(float) * dims[k] * R;
      o_fac[k] = take(fb);
      o_old[k] = take(fb);
      o_acc[k] = take(fb);
      o_g[k] = take(sizeof(float) * R * R);
      o_ga[k] = take(sizeof(float) * R * R);
      gp = std::max(gp, gram_scratch_floats((int)dims[k], R));
    }
    const size_t o_M = take(sizeof(float) * maxrows * R);
    const size_t o_TL = take(sizeof(float) * std::max<int64_t>(rows_left, 1) * R);
    const size_t o_TR = take(sizeof(float) * std::max<int64_t>(rows_right, 1) * R);
    const size_t o_gp = take(sizeof(float) * gp);
    const size_t o_np = take(sizeof(NnlsParams));
    const size_t o_d = take(sizeof(double) * 4 * N);
    const size_t o_i = take(sizeof(int) * 2 * N);
    const size_t o_W = take(sizeof(double) * R * R);
    cudaError_t e = cudaMalloc(&base, off);
    if (e != cudaSuccess) {
      base = nullptr;
      return cuda_error(e, "cudaMalloc(ALS buffers)", __FILE__, __LINE__);
    }
    char *b = (char *)base;
    for (int k = 0; k < N; ++k) {
      fac[k] = (float *)(b + o_fac[k]);
      old[k] = (float *)(b + o_old[k]);
      acc[k] = (float *)(b + o_acc[k]);
      gram[k] = (float *)(b + o_g[k]);
      gacc[k] = (float *)(b + o_ga[k]);
    }
    M = (float *)(b + o_M);
    TL = (float *)(b + o_TL);
    TR = (float *)(b + o_TR);
    gpart = (float *)(b + o_gp);
    np = (NnlsParams *)(b + o_np);
    dsc = (double *)(b + o_d);
    isc = (int *)(b + o_i);
    W = (double *)(b + o_W);
    return PTG_OK;
  }
  ~AlsBuffers() {
    if (base) cudaFree(base);
  }
};

struct Runner {
  ptg_ctx *ctx;
  const ptg_cpd_options *opt;
  AlsBuffers b;
  int weight = 0;
  bool all_orth = true;
  bool dimtree = false;
  WarmArgs warm[PTG_MAX_ORDER];   // per mode, for the sweep being run
  std::chrono::steady_clock::time_point t0;

  // one ALS sweep over all modes on tensor X; fills f (before acceleration) and per-mode
  // iteration counts
  int sweep(const ptg_tensor *X, double frob, double *f_out, int *iters) {
    cudaStream_t S = ctx->stream, T = ctx->side;
    const int N = b.N, R = b.R;
    for (int n = 0; n < N; ++n) {
      const int con = opt->constraints[n];
      if (con != PTG_NONNEGATIVITY) {
        PTG_TRY(other_update(X, n));
        continue;
      }
      PTG_CUDA(cudaEventRecord(ctx->ev_fork, S));
      PTG_CUDA(cudaStreamWaitEvent(T, ctx->ev_fork, 0));
      // beside the tensor-core MTTKRP: a direct contraction, or the node contraction of a tree
      const bool beside_tc = contraction_uses_tc(ctx, X, R) && (!dimtree || n == 0 || n == dimtree_split(N));
      PTG_TRY(launch_eigen_bounds(b.gram, N, n, R, b.np, T, beside_tc));
      count_launches(ctx, 1);
      PTG_CUDA(cudaEventRecord(ctx->ev_join, T));
      if (!dimtree) {
        Contraction c = mttkrp_contraction(X, b.fac, n);
        PTG_TRY(contraction_launch(ctx, X, c, R, b.M, S));
      } else {
        // node tensors: the left node before mode 0 (current right-half factors), the
        // right node before the first right-half mode (updated left-half factors)
        const int h = dimtree_split(N);
        if (n == 0) PTG_TRY(contraction_launch(ctx, X, node_contraction(X, b.fac, true), R, b.TL, S));
        if (n == h) PTG_TRY(contraction_launch(ctx, X, node_contraction(X, b.fac, false), R, b.TR, S));
        PTG_TRY(launch_leaf_mttkrp(ctx, X, n < h ? b.TL : b.TR, b.fac, n, R, b.M, S));
      }
      PTG_CUDA(cudaStreamWaitEvent(S, ctx->ev_join, 0));
      PTG_TRY(launch_nnls_full(ctx, b.M, b.fac[n], b.rows[n], R, b.np, (float)opt->nesterov_delta_1,
                               (float)opt->nesterov_delta_2, b.gram[n], b.dsc + 4 * n,
                               b.dsc + 4 * n + 1, b.isc + 2 * n, b.isc + 2 * n + 1, S, warm[n]));
      count_launches(ctx, 1);
    }
    double hd[4 * PTG_MAX_ORDER];
    int hi[2 * PTG_MAX_ORDER];
    PTG_CUDA(cudaMemcpyAsync(hd, b.dsc, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaMemcpyAsync(hi, b.isc, sizeof(int) * 2 * N, cudaMemcpyDeviceToHost, S));
    PTG_TRY(check_device_error(ctx));
    const int last = N - 1;
    const double f2 = frob - 2.0 * hd[4 * last] + hd[4 * last + 1];
    if (!std::isfinite(f2)) return set_error(PTG_ERR_NUMERIC, "cost is NaN or Inf");
    *f_out = std::sqrt(std::max(f2, 0.0));
    for (int n = 0; n < N; ++n) iters[n] = hi[2 * n];
    return PTG_OK;
  }

  // the MTTKRP of mode n into b.M (direct or through the dimension-tree nodes)
  int mode_mttkrp(const ptg_tensor *X, int n) {
    cudaStream_t S = ctx->stream;
    if (!dimtree) {
      Contraction c = mttkrp_contraction(X, b.fac, n);
      return contraction_launch(ctx, X, c, b.R, b.M, S);
    }
    const int h = dimtree_split(b.N);
    if (n == 0) PTG_TRY(contraction_launch(ctx, X, node_contraction(X, b.fac, true), b.R, b.TL, S));
    if (n == h) PTG_TRY(contraction_launch(ctx, X, node_contraction(X, b.fac, false), b.R, b.TR, S));
    return launch_leaf_mttkrp(ctx, X, n < h ? b.TL : b.TR, b.fac, n, b.R, b.M, S);
  }

  // update_factor for the constraints other than nonnegativity (include/Cpd.hpp:196-222),
  // then the Gram (:227); the cost terms of the last mode are those of the Gram form
  int other_update(const ptg_tensor *X, int n) {
    cudaStream_t S = ctx->stream;
    const int N = b.N, R = b.R, con = opt->constraints[n];
    PTG_TRY(mode_mttkrp(X, n));
    if (con == PTG_UNCONSTRAINED) {
      PTG_TRY(launch_eigen_bounds(b.gram, N, n, R, b.np, S));   // Z = Hadamard of the other Grams
      count_launches(ctx, 1);
      PTG_TRY(launch_update_unconstrained(ctx, b.M, b.fac[n], b.rows[n], R, b.np, b.W, S));
    } else if (con == PTG_ORTHOGONALITY) {
      if (b.rows[n] < R) return set_error(PTG_ERR_INVALID, "orthogonality needs I_n >= R");
      PTG_TRY(launch_update_orthogonal(ctx, b.M, b.fac[n], b.rows[n], R, b.W, S));
    } else if (con != PTG_SPARSITY && con != PTG_CONSTANT) {
      return set_error(PTG_ERR_INVALID, "unknown constraint");
    }
    PTG_TRY(launch_gram(b.fac[n], b.rows[n], R, b.gram[n], b.gpart, S));
    count_launches(ctx, 2);
    PTG_CUDA(cudaMemsetAsync(b.isc + 2 * n, 0, 2 * sizeof(int), S));
    if (n == N - 1) {
      PTG_TRY(launch_cost_terms(b.M, b.fac[n], b.rows[n], b.gram, N, R, b.dsc + 4 * n, S));
      count_launches(ctx, 1);
    }
    return PTG_OK;
  }

  // cost of the point (factors, grams) by one last-mode MTTKRP: sqrt(||X||^2 + sum(Z.*G) - 2<M,A>)
  int point_cost(const ptg_tensor *X, double frob, float *const *factors, float *const *grams,
                 double *f_out) {
    cudaStream_t S = ctx->stream;
    const int last = b.N - 1;
    Contraction c = mttkrp_contraction(X, factors, last);
    PTG_TRY(contraction_launch(ctx, X, c, b.R, b.M, S));
    PTG_TRY(launch_cost_terms(b.M, factors[last], b.rows[last], grams, b.N, b.R, b.dsc + 2, S));
    count_launches(ctx, 1);
    double h[2];
    PTG_CUDA(cudaMemcpyAsync(h, b.dsc + 2, sizeof(h), cudaMemcpyDeviceToHost, S));
    PTG_TRY(check_device_error(ctx));
    const double f2 = frob + h[1] - 2.0 * h[0];
    if (!std::isfinite(f2)) return set_error(PTG_ERR_NUMERIC, "cost is NaN or Inf");
    *f_out = std::sqrt(std::max(f2, 0.0));
    return PTG_OK;
  }

  float elapsed() const {
    return std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
  }
};

}  // namespace
}  // namespace ptg

using namespace ptg;

extern "C" {

void ptg_cpd_default_options(int order, ptg_cpd_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  for (int k = 0; k < PTG_MAX_ORDER; ++k) o->constraints[k] = (k < order) ? PTG_NONNEGATIVITY : 0;
  o->threshold_error = 1e-3;
  o->nesterov_delta_1 = 1e-2;
  o->nesterov_delta_2 = 1e-2;
  o->max_iter = 20;
  o->accel_coeff = 3;
  o->accel_fail = 0;
  o->acceleration = 1;
  o->normalization = 1;
  o->refine_sweeps = 0;
  o->warm_start = 0;
  o->cost_every_sweep = 1;
  o->verify_fp32 = 0;
}

}  // extern "C"

static int cpd_als_impl(ptg_ctx *ctx, const ptg_tensor *X, const ptg_tensor *refine, int rank,
                        const ptg_cpd_options *opts_in, const double *const *init_factors,
                        double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace,
                        bool dimtree) {
  if (!ctx || !X || !opts_in || !init_factors || !out_factors)
    return set_error(PTG_ERR_INVALID, "NULL argument");
  if (rank < 1 || rank > 64) return set_error(PTG_ERR_UNSUPPORTED, "rank must be in [1, 64]");
  const int N = X->order;
  if (N < 3) return set_error(PTG_ERR_UNSUPPORTED, "CPD needs a tensor of order >= 3");
  if (refine) {
    if (refine->order != N) return set_error(PTG_ERR_INVALID, "refine tensor order differs");
    for (int k = 0; k < N; ++k)
      if (refine->dims[k] != X->dims[k]) return set_error(PTG_ERR_INVALID, "refine tensor dims differ");
  }
  if (opts_in->max_iter < 1) return set_error(PTG_ERR_INVALID, "max_iter must be >= 1");
  for (int k = 0; k < N; ++k)
    if (!init_factors[k] || !out_factors[k]) return set_error(PTG_ERR_INVALID, "factor pointer is NULL");
  PTG_CUDA(cudaSetDevice(ctx->device));
  ptg_cpd_options opt = *opts_in;
  Runner run{ctx, &opt};
  run.t0 = std::chrono::steady_clock::now();
  run.dimtree = dimtree;
  PTG_TRY(run.b.alloc(X->dims, N, rank, dimtree ? node_rows(X, true) : 0, dimtree ? node_rows(X, false) : 0));
  AlsBuffers &b = run.b;
  cudaStream_t S = ctx->stream;

  // initial factors: host FP64 ColMajor -> device FP32 row-major
  std::vector<float> hbuf;
  for (int k = 0; k < N; ++k) {
    const int64_t I = X->dims[k];
    hbuf.resize((size_t)I * rank);
    for (int64_t i = 0; i < I; ++i)
      for (int r = 0; r < rank; ++r) {
        const double v = init_factors[k][i + I * r];
        if (!std::isfinite(v)) return set_error(PTG_ERR_NUMERIC, "initial factor contains NaN or Inf");
        hbuf[(size_t)i * rank + r] = (float)v;
      }
    PTG_CUDA(cudaMemcpyAsync(b.fac[k], hbuf.data(), sizeof(float) * I * rank, cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    PTG_TRY(launch_gram(b.fac[k], (int)I, rank, b.gram[k], b.gpart, S));
    count_launches(ctx, 2);
  }
  // choose_normilization_factor, include/Normalize.hpp:53-67
  run.all_orth = true;
  run.weight = 0;
  if (opt.normalization)
    for (int k = 0; k < N; ++k)
      if (opt.constraints[k] != PTG_ORTHOGONALITY) {
        run.all_orth = false;
        run.weight = k;
        break;
      }

  const ptg_tensor *Xa = X;
  double frob = Xa->frob_stored;
  double f = 0.0, rel = 0.0;
  PTG_TRY(run.point_cost(Xa, frob, b.fac, b.gram, &f));
  int ao_iter = 0, ntrace = 0;
  long long inner_total = 0;
  int iters[PTG_MAX_ORDER];
  // learned warm start: log sweeps 1..n, train, then infer (or infer from sweep 1)
  ptg_mlp *model = opt.warm_start ? opt.warm_model : nullptr;
  if (opt.warm_start && !model) return set_error(PTG_ERR_INVALID, "warm_start needs warm_model");
  if (model && mlp_din(model) != rank + 8) return set_error(PTG_ERR_INVALID, "warm_model rank differs");
  const int log_sweeps = model ? std::max(0, opt.warm_log_sweeps) : 0;
  int64_t rows_per_sweep = 0;
  for (int k = 0; k < N; ++k) rows_per_sweep += X->dims[k];
  float *logX = nullptr, *logT = nullptr;
  struct FreeOnExit {
    void *p = nullptr;
    ~FreeOnExit() { if (p) cudaFree(p); }
  } logmem;
  if (log_sweeps > 0) {
    const size_t rows = (size_t)log_sweeps * rows_per_sweep;
    PTG_CUDA(cudaMalloc(&logmem.p, sizeof(float) * rows * (2 * rank + 8)));
    logX = (float *)logmem.p;
    logT = logX + rows * (rank + 8);
  }
  int64_t logged = 0;
  for (;;) {
    ++ao_iter;
    for (int n = 0; n < N; ++n) run.warm[n] = WarmArgs();
    if (model) {
      if (ao_iter <= log_sweeps) {
        int64_t off = logged;
        for (int n = 0; n < N; ++n) {
          run.warm[n].log_X = logX + off * (rank + 8);
          run.warm[n].log_T = logT + off * rank;
          run.warm[n].hidden = mlp_hidden(model);
          off += X->dims[n];
        }
        logged = off;
      } else {
        for (int n = 0; n < N; ++n) {
          run.warm[n].theta = mlp_theta(model);
          run.warm[n].hidden = mlp_hidden(model);
        }
      }
    }
    PTG_TRY(run.sweep(Xa, frob, &f, iters));
    if (model && ao_iter == log_sweeps && opt.warm_train_steps > 0) {
      double loss = 0.0;
      PTG_TRY(ptg_mlp_train(ctx, model, logX, logT, logged, opt.warm_train_steps, 256, 1e-3f, 1234, &loss));
    }
    for (int n = 0; n < N; ++n) inner_total += iters[n];
    rel = f / std::sqrt(frob);
    if (opt.normalization && !run.all_orth) {
      PTG_TRY(launch_normalize(b.fac, b.gram, b.rows, N, run.weight, rank, S));
      count_launches(ctx, 2);
    }
    ptg_sweep_trace tr{};
    tr.f_value = f;
    tr.rel_costFunction = rel;
    for (int n = 0; n < N; ++n) tr.nesterov_iters[n] = iters[n];
    const bool stop = rel < opt.threshold_error || ao_iter >= opt.max_iter;
    if (!stop && opt.acceleration) {
      if (ao_iter > 1) {
        const double step = std::pow((double)(ao_iter + 1), 1.0 / (double)opt.accel_coeff);
        PTG_TRY(launch_accel_combine(b.fac, b.old, b.acc, b.rows, N, rank, step, S));
        for (int k = 0; k < N; ++k) PTG_TRY(launch_gram(b.acc[k], b.rows[k], rank, b.gacc[k], b.gpart, S));
        count_launches(ctx, 1 + 2 * N);
        for (int k = 0; k < N; ++k)
          PTG_CUDA(cudaMemcpyAsync(b.old[k], b.fac[k], sizeof(float) * b.rows[k] * rank,
                                   cudaMemcpyDeviceToDevice, S));
        double fa = 0.0;
        PTG_TRY(run.point_cost(Xa, frob, b.acc, b.gacc, &fa));
        tr.f_accel = fa;
        if (f > fa) {
          for (int k = 0; k < N; ++k) {
            std::swap(b.fac[k], b.acc[k]);
            std::swap(b.gram[k], b.gacc[k]);
          }
          f = fa;
          tr.accel_accepted = 1;
        } else {
          opt.accel_fail++;
        }
        if (opt.accel_fail == 5) {
          opt.accel_fail = 0;
          opt.accel_coeff++;
        }
      } else {
        for (int k = 0; k < N; ++k)
          PTG_CUDA(cudaMemcpyAsync(b.old[k], b.fac[k], sizeof(float) * b.rows[k] * rank,
                                   cudaMemcpyDeviceToDevice, S));
      }
    }
    tr.seconds = run.elapsed();
    if (trace) trace[ntrace] = tr;
    ++ntrace;
    if (stop) break;
  }
  // FP32 refinement sweeps on the FP32 copy (no acceleration)
  int refined = 0;
  if (refine && opt.refine_sweeps > 0) {
    Xa = refine;
    frob = Xa->frob_stored;
    for (int n = 0; n < N; ++n) run.warm[n] = WarmArgs();
    for (; refined < opt.refine_sweeps; ++refined) {
      PTG_TRY(run.sweep(Xa, frob, &f, iters));
      for (int n = 0; n < N; ++n) inner_total += iters[n];
      rel = f / std::sqrt(frob);
      if (opt.normalization && !run.all_orth) {
        PTG_TRY(launch_normalize(b.fac, b.gram, b.rows, N, run.weight, rank, S));
        count_launches(ctx, 2);
      }
      ptg_sweep_trace tr{};
      tr.f_value = f;
      tr.rel_costFunction = rel;
      for (int n = 0; n < N; ++n) tr.nesterov_iters[n] = iters[n];
      tr.seconds = run.elapsed();
      if (trace) trace[ntrace] = tr;
      ++ntrace;
    }
  }
  // the cost of the final factors on the FP32 copy (one MTTKRP in the Gram form)
  if (refine && refined == 0 && opt.verify_fp32) {
    Xa = refine;
    frob = Xa->frob_stored;
    PTG_TRY(run.point_cost(Xa, frob, b.fac, b.gram, &f));
    rel = f / std::sqrt(frob);
  }
  // results: device FP32 row-major -> host FP64 ColMajor
  for (int k = 0; k < N; ++k) {
    const int64_t I = X->dims[k];
    hbuf.resize((size_t)I * rank);
    PTG_CUDA(cudaMemcpyAsync(hbuf.data(), b.fac[k], sizeof(float) * I * rank, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    for (int64_t i = 0; i < I; ++i)
      for (int r = 0; r < rank; ++r) out_factors[k][i + I * r] = (double)hbuf[(size_t)i * rank + r];
  }
  if (result) {
    result->frob_tns = frob;
    result->f_value = f;
    result->rel_costFunction = rel;
    result->ao_iter = ao_iter;
    result->accel_coeff = opt.accel_coeff;
    result->accel_fail = opt.accel_fail;
    result->refine_sweeps_done = refined;
    result->nesterov_iters_total = inner_total;
    result->seconds_total = run.elapsed();
  }
  return PTG_OK;
}

extern "C" {

int ptg_cpd_als(ptg_ctx *ctx, const ptg_tensor *X, const ptg_tensor *refine, int rank,
                const ptg_cpd_options *opts, const double *const *init_factors,
                double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace) {
  return cpd_als_impl(ctx, X, refine, rank, opts, init_factors, out_factors, result, trace, false);
}

int ptg_cpd_dimtree_als(ptg_ctx *ctx, const ptg_tensor *X, const ptg_tensor *refine, int rank,
                        const ptg_cpd_options *opts, const double *const *init_factors,
                        double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace) {
  return cpd_als_impl(ctx, X, refine, rank, opts, init_factors, out_factors, result, trace, true);
}

}  // extern "C"

static int cpd_host_impl(ptg_ctx *ctx, int order, const int64_t *dims, const double *host_tensor,
                         ptg_dtype dtype, int rank, const ptg_cpd_options *opts,
                         const double *const *init_factors, double *const *out_factors,
                         ptg_cpd_result *result, ptg_sweep_trace *trace, bool dimtree) {
  if (!ctx || !dims || !host_tensor || !opts) return set_error(PTG_ERR_INVALID, "NULL argument");
  ptg_tensor *X = nullptr, *Xr = nullptr;
  const bool want_refine = dtype != PTG_F32 && (opts->refine_sweeps > 0 || opts->verify_fp32);
  int rc = PTG_OK;
  // the stored tensors live in context-owned buffers kept for the next call; the host data is
  // streamed through page-locked chunks (copy of chunk k+1 beside the conversion of chunk k),
  // and one pass writes both the BF16 tensor and its FP32 copy
  if (!want_refine)
    rc = tensor_create_impl(ctx, order, dims, dtype, host_tensor, 0, &ctx->cache_x, &X);
  else
    rc = tensor_create_impl(ctx, order, dims, dtype, host_tensor, 0, &ctx->cache_x, &X, &ctx->cache_xr, &Xr);
  if (rc == PTG_OK) rc = cpd_als_impl(ctx, X, Xr, rank, opts, init_factors, out_factors, result, trace, dimtree);
  ptg_tensor_destroy(X);
  ptg_tensor_destroy(Xr);
  return rc;
}

extern "C" {

int ptg_cpd(ptg_ctx *ctx, int order, const int64_t *dims, const double *host_tensor, ptg_dtype dtype,
            int rank, const ptg_cpd_options *opts, const double *const *init_factors,
            double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace) {
  return cpd_host_impl(ctx, order, dims, host_tensor, dtype, rank, opts, init_factors, out_factors, result,
                       trace, false);
}

int ptg_cpd_dimtree(ptg_ctx *ctx, int order, const int64_t *dims, const double *host_tensor, ptg_dtype dtype,
                    int rank, const ptg_cpd_options *opts, const double *const *init_factors,
                    double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace) {
  return cpd_host_impl(ctx, order, dims, host_tensor, dtype, rank, opts, init_factors, out_factors, result,
                       trace, true);
}

}  // extern "C"
