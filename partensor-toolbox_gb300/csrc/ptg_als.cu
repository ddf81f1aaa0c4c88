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
  float *TL = nullptr, *TR = nullptr;   // dimension-tree node tensors of the root's children
  float *TD = nullptr;                  // the deeper node tensors (orders >= 5)
  float *gpart = nullptr;
  NnlsParams *np = nullptr;
  NnlsParams *np_acc = nullptr;   // mode 0's bounds for the line-search point, computed beside it
  double *dsc = nullptr;  // [N][2]: <M, A>, sum(Z .* G); [0][2..3]: cost terms of a point;
                          // [4N], [4N + 1]: the line-search decision (accel_select_kernel)
  int *isc = nullptr;     // [N][2]: iterations, repaired; [2N]: the line search's stop gate;
                          // [2N + 1]: 1 when the line search took its point (its mode-0
                          // MTTKRP in M is then the next sweep's)
  double *W = nullptr;    // R x R FP64: Z^{-1} or (M^T M)^{-1/2} (other constraints)
  double *cpart = nullptr;        // launch_cost_terms partials
  unsigned *cticket = nullptr;    // and its ticket (zero between launches)
  void *base = nullptr;

  int alloc(const ptg_ctx *ctx, const int64_t *dims, int order, int rank, int64_t rows_left = 0,
            int64_t rows_right = 0, size_t deep_floats = 0) {
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
    const size_t o_TD = take(sizeof(float) * std::max<size_t>(deep_floats, 1));
    const size_t o_gp = take(sizeof(float) * gp);
    const size_t o_np = take(sizeof(NnlsParams));
    const size_t o_npa = take(sizeof(NnlsParams));
    const size_t o_d = take(sizeof(double) * (4 * N + 2));
    const size_t o_i = take(sizeof(int) * (2 * N + 2));
    const size_t o_W = take(sizeof(double) * R * R);
    const size_t o_cp = take(sizeof(double) * kCostPartials);
    const size_t o_ct = take(sizeof(unsigned));
    const int rc = ctx_malloc(ctx, &base, off, "ALS buffers");
    if (rc != PTG_OK) {
      base = nullptr;
      return rc;
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
    TD = (float *)(b + o_TD);
    gpart = (float *)(b + o_gp);
    np = (NnlsParams *)(b + o_np);
    np_acc = (NnlsParams *)(b + o_npa);
    dsc = (double *)(b + o_d);
    isc = (int *)(b + o_i);
    W = (double *)(b + o_W);
    cpart = (double *)(b + o_cp);
    cticket = (unsigned *)(b + o_ct);
    const cudaError_t e = cudaMemset(cticket, 0, sizeof(unsigned));
    if (e != cudaSuccess) return cuda_error(e, "cudaMemset(ALS ticket)", __FILE__, __LINE__);
    return PTG_OK;
  }
  ~AlsBuffers() {
    if (base) cudaFree(base);
  }
};

// The line-search decision of include/Cpd.hpp:262-271 on the device, so that the host does not
// wait for it: the sweep's cost and the accelerated point's cost from their terms (the host's
// arithmetic in the host's order: the doublings are exact, so contraction cannot change a
// result), the stop test of the sweep, then acc -> fac and gacc -> gram when the point is
// taken.  Every block decides alike; block 0 records the point's f^2 and the decision, as a
// double for the host and as an int for the next sweep's mode-0 MTTKRP (Contraction::skip).
struct SelectArgs {
  const double *dsc;     // sweep terms at [4 last], [4 last + 1]; the point's at [2], [3]
  int last, N, R;
  double frob, threshold;
  int ao_iter, max_iter;
  int rows[PTG_MAX_ORDER];
  float *fac[PTG_MAX_ORDER];
  float *gram[PTG_MAX_ORDER];
  const float *acc[PTG_MAX_ORDER];
  const float *gacc[PTG_MAX_ORDER];
  double *sel;           // out: [0] the point's f^2, [1] 1.0 when taken
  int *taken;            // out: 1 when taken, else 0
  const NnlsParams *np_acc;   // mode 0's bounds from the point's Grams ...
  NnlsParams *np;             // ... installed for the next sweep when the point is taken
};

__global__ void accel_select_kernel(const SelectArgs a) {
  __shared__ int take;
  if (threadIdx.x == 0) {
    const double f2 = a.frob - 2.0 * a.dsc[4 * a.last] + a.dsc[4 * a.last + 1];
    const double fa2 = a.frob + a.dsc[3] - 2.0 * a.dsc[2];
    const double f = sqrt(fmax(f2, 0.0)), fa = sqrt(fmax(fa2, 0.0));
    const bool stop = f / sqrt(a.frob) < a.threshold || a.ao_iter >= a.max_iter;
    take = (!stop && f > fa) ? 1 : 0;   // a NaN cost compares false: nothing is taken
    if (blockIdx.x == 0) {
      a.sel[0] = fa2;
      a.sel[1] = take ? 1.0 : 0.0;
      *a.taken = take;
    }
  }
  __syncthreads();
  if (!take) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  {
    const int64_t nw = (int64_t)(sizeof(NnlsParams) / sizeof(double));
    const double *src = reinterpret_cast<const double *>(a.np_acc);
    double *dst = reinterpret_cast<double *>(a.np);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nw; i += stride) dst[i] = src[i];
  }
  for (int k = 0; k < a.N; ++k) {
    const int64_t n = (int64_t)a.rows[k] * a.R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) a.fac[k][i] = a.acc[k][i];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)a.R * a.R; i += stride)
      a.gram[k][i] = a.gacc[k][i];
  }
}

// The stop test of the sweep just queued, for the line search queued behind it: that line
// search's MTTKRP returns at once when the sweep is the last (Contraction::skip), so a stopping
// sweep does not pay for it.  Same arithmetic as accel_select_kernel and the host.
__global__ void stop_gate_kernel(const double *dsc, int last, double frob, double threshold, int ao_iter,
                                 int max_iter, int *gate) {
  const double f2 = frob - 2.0 * dsc[4 * last] + dsc[4 * last + 1];
  const double f = sqrt(fmax(f2, 0.0));
  *gate = (f / sqrt(frob) < threshold || ao_iter >= max_iter) ? 1 : 0;
}

// page-locked copy of the per-sweep scalars (ptg_ctx::pinned_scalars)
struct HostScalars {
  double dsc[4 * PTG_MAX_ORDER];
  int isc[2 * PTG_MAX_ORDER];
  int err, pad;
  double sel[2];   // the line search: the point's f^2, taken (1.0) or not
};
static_assert(sizeof(HostScalars) <= kPinnedScalarBytes, "pinned scalar block too small");

struct Runner {
  ptg_ctx *ctx;
  const ptg_cpd_options *opt;
  AlsBuffers b;
  int weight = 0;
  bool all_orth = true;
  bool dimtree = false;
  DimTree tree;                   // the dimension tree's nodes and their freshness (dimtree)
  WarmArgs warm[PTG_MAX_ORDER];   // per mode, for the sweep being run
  std::chrono::steady_clock::time_point t0;

  HostScalars *hs() const { return static_cast<HostScalars *>(ctx->pinned_scalars); }

  // one ALS sweep over all modes on tensor X, then sweep_finish: f (before acceleration) and
  // the per-mode iteration counts
  int sweep(const ptg_tensor *X, double frob, double *f_out, int *iters) {
    PTG_TRY(sweep_enqueue(X));
    return sweep_finish(frob, f_out, iters);
  }

  // the sweep's kernels, then its cost terms, iteration counts and the device error word
  // copied to pinned memory behind them (ctx->ev_cost); nothing waits.  reuse_m0: a device
  // word that, when nonzero, cancels mode 0's MTTKRP because M already holds it (the line
  // search before this sweep took its point, whose cost it computed from that product).
  // np0_ready: mode 0's bounds are already in b.np (computed beside the line search).
  int sweep_enqueue(const ptg_tensor *X, const int *reuse_m0 = nullptr, bool np0_ready = false) {
    cudaStream_t S = ctx->stream, T = ctx->side;
    const int N = b.N, R = b.R;
    if (dimtree) tree.new_sweep();   // normalisation and the line search changed every factor
    for (int n = 0; n < N; ++n) {
      const int con = opt->constraints[n];
      if (con != PTG_NONNEGATIVITY) {
        PTG_TRY(other_update(X, n));
        continue;
      }
      const bool bounds = !(n == 0 && np0_ready);
      if (bounds) {
        PTG_CUDA(cudaEventRecord(ctx->ev_fork, S));
        PTG_CUDA(cudaStreamWaitEvent(T, ctx->ev_fork, 0));
        // beside the tensor-core MTTKRP: a direct contraction, or the node contraction of a tree
        const bool beside_tc = contraction_uses_tc(ctx, X, R) && (!dimtree || n == 0 || n == dimtree_split(N));
        PTG_TRY(launch_eigen_bounds(b.gram, N, n, R, b.np, T, beside_tc));
        count_launches(ctx, 1);
        PTG_CUDA(cudaEventRecord(ctx->ev_join, T));
      }
      if (!dimtree) {
        Contraction c = mttkrp_contraction(X, b.fac, n);
        if (n == 0) c.skip = reuse_m0;
        PTG_TRY(contraction_launch(ctx, X, c, R, b.M, S));
      } else {
        // through the tree: the nodes on the path to leaf n that a changed factor made stale
        // are recomputed (the root's children once per sweep, before modes 0 and h)
        PTG_TRY(tree.mttkrp(ctx, X, b.fac, n, R, b.M, S));
      }
      if (bounds) PTG_CUDA(cudaStreamWaitEvent(S, ctx->ev_join, 0));
      PTG_TRY(launch_nnls_full(ctx, b.M, b.fac[n], b.rows[n], R, b.np, (float)opt->nesterov_delta_1,
                               (float)opt->nesterov_delta_2, b.gram[n], b.dsc + 4 * n,
                               b.dsc + 4 * n + 1, b.isc + 2 * n, b.isc + 2 * n + 1, S, warm[n]));
      count_launches(ctx, 1);
      if (dimtree) tree.updated(n);
    }
    HostScalars *h = hs();
    PTG_CUDA(cudaMemcpyAsync(h->dsc, b.dsc, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaMemcpyAsync(h->isc, b.isc, sizeof(int) * 2 * N, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaMemcpyAsync(&h->err, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaEventRecord(ctx->ev_cost, S));
    return PTG_OK;
  }

  // waits for the scalars of the last queued sweep
  int sweep_finish(double frob, double *f_out, int *iters) {
    PTG_CUDA(cudaEventSynchronize(ctx->ev_cost));
    const HostScalars *h = hs();
    PTG_TRY(report_device_error(ctx, h->err));
    const int N = b.N, last = N - 1;
    const double f2 = frob - 2.0 * h->dsc[4 * last] + h->dsc[4 * last + 1];
    if (!std::isfinite(f2)) return set_error(PTG_ERR_NUMERIC, "cost is NaN or Inf");
    *f_out = std::sqrt(std::max(f2, 0.0));
    for (int n = 0; n < N; ++n) iters[n] = h->isc[2 * n];
    return PTG_OK;
  }

  // the line-search point's cost terms into b.dsc[2..3], queued, in the Gram form from one
  // MTTKRP: <X, [[A]]> = <MTTKRP_0(X, A), A_0>, the same cost as the reference's last-mode
  // form (include/Cpd.hpp:262-266).  Mode 0 because, when the point is taken, that product
  // (left in b.M) is the next sweep's first MTTKRP, which the sweep then skips.
  int point_cost_enqueue(const ptg_tensor *X, float *const *factors, float *const *grams,
                         const int *skip = nullptr, cudaEvent_t grams_ready = nullptr, bool exact = false) {
    cudaStream_t S = ctx->stream;
    Contraction c = mttkrp_contraction(X, factors, 0);
    c.skip = skip;
    c.exact_fp32 = exact;
    PTG_TRY(contraction_launch(ctx, X, c, b.R, b.M, S));
    if (grams_ready) PTG_CUDA(cudaStreamWaitEvent(S, grams_ready, 0));
    PTG_TRY(launch_cost_terms(b.M, factors[0], b.rows[0], grams, b.N, b.R, b.dsc + 2,
                              CostScratch{b.cpart, b.cticket}, S));
    // the exact fit: the Gram term from FP64 Grams of the factors (the FP32 Grams' rounding,
    // ~1e-7 of ||X||^2, would move f^2 = ||X||^2 - 2<M, A> + ... by ~1e-7 / rel^2 of itself)
    if (exact) {
      PTG_TRY(ctx->scratch.ensure(sizeof(double) * gram_term_fp64_scratch_doubles(b.N, b.R)));
      PTG_TRY(launch_gram_term_fp64(factors, b.rows, b.N, b.R, reinterpret_cast<double *>(ctx->scratch.ptr),
                                    b.dsc + 3, S));
      count_launches(ctx, 2);
    }
    count_launches(ctx, 1);
    return PTG_OK;
  }

  // accel_select_kernel behind the point's cost, its decision copied to pinned memory
  // (ctx->ev_sel)
  int select_enqueue(double frob, double threshold, int ao_iter, int max_iter) {
    cudaStream_t S = ctx->stream;
    SelectArgs a{};
    a.dsc = b.dsc;
    a.N = b.N;
    a.R = b.R;
    a.last = b.N - 1;
    a.frob = frob;
    a.threshold = threshold;
    a.ao_iter = ao_iter;
    a.max_iter = max_iter;
    int64_t most = 0;
    for (int k = 0; k < b.N; ++k) {
      a.rows[k] = b.rows[k];
      a.fac[k] = b.fac[k];
      a.gram[k] = b.gram[k];
      a.acc[k] = b.acc[k];
      a.gacc[k] = b.gacc[k];
      most = std::max<int64_t>(most, (int64_t)b.rows[k] * b.R);
    }
    a.sel = b.dsc + 4 * b.N;
    a.taken = b.isc + 2 * b.N + 1;
    a.np_acc = b.np_acc;
    a.np = b.np;
    const int blocks = (int)std::min<int64_t>((most + 255) / 256, (int64_t)ctx->sm_count);
    accel_select_kernel<<<std::max(blocks, 1), 256, 0, S>>>(a);
    PTG_CUDA(cudaGetLastError());
    count_launches(ctx, 1);
    PTG_CUDA(cudaMemcpyAsync(hs()->sel, a.sel, sizeof(double) * 2, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaEventRecord(ctx->ev_sel, S));
    return PTG_OK;
  }

  // the MTTKRP of mode n into b.M (direct or through the dimension-tree nodes)
  int mode_mttkrp(const ptg_tensor *X, int n) {
    cudaStream_t S = ctx->stream;
    if (!dimtree) {
      Contraction c = mttkrp_contraction(X, b.fac, n);
      return contraction_launch(ctx, X, c, b.R, b.M, S);
    }
    return tree.mttkrp(ctx, X, b.fac, n, b.R, b.M, S);
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
    if (dimtree) tree.updated(n);
    count_launches(ctx, 2);
    PTG_CUDA(cudaMemsetAsync(b.isc + 2 * n, 0, 2 * sizeof(int), S));
    if (n == N - 1) {
      PTG_TRY(launch_cost_terms(b.M, b.fac[n], b.rows[n], b.gram, N, R, b.dsc + 4 * n,
                                CostScratch{b.cpart, b.cticket}, S));
      count_launches(ctx, 1);
    }
    return PTG_OK;
  }

  // cost of the point (factors, grams) by one MTTKRP: sqrt(||X||^2 + sum(Z.*G) - 2<M,A>)
  int point_cost(const ptg_tensor *X, double frob, float *const *factors, float *const *grams,
                 double *f_out, bool exact = false) {
    cudaStream_t S = ctx->stream;
    PTG_TRY(point_cost_enqueue(X, factors, grams, nullptr, nullptr, exact));
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

// writeFactorsToFile, include/Cpd.hpp:112-122: factor k (I_k x R ColMajor FP64) written as
// its transpose's storage, i.e. row-major, to final_factors_paths[k] ("final_<k>.bin" when
// NULL, the reference's default, include/PARTENSOR_basic.hpp:330-333).
static int write_final_factors(const ptg_cpd_options &opt, const int64_t *dims, int N, int rank,
                               double *const *factors) {
  std::vector<double> row;
  for (int k = 0; k < N; ++k) {
    const std::string path = opt.final_factors_paths[k] ? std::string(opt.final_factors_paths[k])
                                                        : "final_" + std::to_string(k) + ".bin";
    const int64_t I = dims[k];
    row.resize((size_t)I * rank);
    for (int64_t i = 0; i < I; ++i)
      for (int r = 0; r < rank; ++r) row[(size_t)i * rank + r] = factors[k][i + I * r];
    FILE *fp = std::fopen(path.c_str(), "wb");
    const bool ok = fp && std::fwrite(row.data(), sizeof(double), row.size(), fp) == row.size();
    if (fp && std::fclose(fp) != 0) return set_error(PTG_ERR_INVALID, "cannot write " + path);
    if (!ok) return set_error(PTG_ERR_INVALID, "cannot write " + path);
  }
  return PTG_OK;
}

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
  if (dimtree) PTG_TRY(run.tree.build(X));
  PTG_TRY(run.b.alloc(ctx, X->dims, N, rank, dimtree ? node_rows(X, true) : 0, dimtree ? node_rows(X, false) : 0,
                      dimtree ? run.tree.deep_floats(rank) : 0));
  if (dimtree) run.tree.bind(run.b.TL, run.b.TR, run.b.TD, rank);
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
  double frob = cost_norm(Xa);
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
  bool sel_pending = false;   // a line search is queued and its decision not yet read
  int sel_sweep = 0;          // the trace entry of that sweep
  // a queued line search's outcome: its sweep's trace entry and the acceleration bookkeeping
  // (include/Cpd.hpp:270-277)
  auto take_selection = [&](int sweep_index) -> int {
    PTG_CUDA(cudaEventSynchronize(ctx->ev_sel));
    const double fa2 = run.hs()->sel[0];
    if (!std::isfinite(fa2)) return set_error(PTG_ERR_NUMERIC, "cost is NaN or Inf");
    const bool taken = run.hs()->sel[1] != 0.0;
    if (trace) {
      trace[sweep_index].f_accel = std::sqrt(std::max(fa2, 0.0));
      trace[sweep_index].accel_accepted = taken ? 1 : 0;
    }
    if (!taken) opt.accel_fail++;
    if (opt.accel_fail == 5) {
      opt.accel_fail = 0;
      opt.accel_coeff++;
    }
    return PTG_OK;
  };
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
          run.warm[n].theta = mlp_theta_infer(model, S);
          run.warm[n].hidden = mlp_hidden(model);
        }
      }
    }
    // The sweep, its normalisation and its line search are queued before the host waits for
    // the sweep's cost: the line search's accept decision and the stop test gating it run on
    // the device (accel_select_kernel), and the host reads the decision one sweep later, before
    // the next line search needs it.  The stream never idles on a host round trip.  When that
    // line search took its point, its mode-0 MTTKRP is this sweep's first one (direct
    // contractions; a tree's nodes would be stale).
    const bool m0_reusable = sel_pending && !run.dimtree && opt.constraints[0] == PTG_NONNEGATIVITY;
    const bool np0_ready = sel_pending && opt.constraints[0] == PTG_NONNEGATIVITY;
    PTG_TRY(run.sweep_enqueue(Xa, m0_reusable ? b.isc + 2 * N + 1 : nullptr, np0_ready));
    if (model && ao_iter == log_sweeps && opt.warm_train_steps > 0) {
      double loss = 0.0;
      PTG_TRY(ptg_mlp_train(ctx, model, logX, logT, logged, opt.warm_train_steps, 256, 1e-3f, 1234, &loss));
    }
    if (opt.normalization && !run.all_orth) {
      PTG_TRY(launch_normalize(b.fac, b.gram, b.rows, N, run.weight, rank, S));
      count_launches(ctx, 2);
    }
    if (sel_pending) {   // the previous sweep's line search (include/Cpd.hpp:247-278)
      PTG_TRY(take_selection(sel_sweep));
      sel_pending = false;
    }
    if (opt.acceleration && ao_iter < opt.max_iter) {   // at max_iter the sweep stops anyway
      if (ao_iter > 1) {
        const double step = std::pow((double)(ao_iter + 1), 1.0 / (double)opt.accel_coeff);
        PTG_TRY(launch_accel_combine(b.fac, b.old, b.acc, b.rows, N, rank, step, S));
        // the accelerated factors' Grams on the side stream, beside the point's MTTKRP: only the
        // point's cost terms need them
        cudaStream_t T = ctx->side;
        PTG_CUDA(cudaEventRecord(ctx->ev_fork, S));
        PTG_CUDA(cudaStreamWaitEvent(T, ctx->ev_fork, 0));
        const bool beside_tc = contraction_uses_tc(ctx, Xa, rank);
        for (int k = 0; k < N; ++k)
          PTG_TRY(launch_gram(b.acc[k], b.rows[k], rank, b.gacc[k], b.gpart, T, beside_tc));
        // old <- fac there too: nothing writes the factors before accel_select_kernel, which
        // runs after the join
        for (int k = 0; k < N; ++k)
          PTG_CUDA(cudaMemcpyAsync(b.old[k], b.fac[k], sizeof(float) * b.rows[k] * rank,
                                   cudaMemcpyDeviceToDevice, T));
        // the next sweep's mode-0 bounds for both outcomes, beside the point's MTTKRP: from the
        // point's Grams (installed by accel_select_kernel if it is taken) and from the current
        // ones (the sweep's own, normalised); that sweep then launches none for mode 0
        // (ev_join: the point's Grams, for its cost terms; ev_join2/3: the two bounds, for
        // accel_select_kernel, which may install one over the other)
        PTG_CUDA(cudaEventRecord(ctx->ev_join, T));
        const bool np0 = opt.constraints[0] == PTG_NONNEGATIVITY;
        if (np0) {
          PTG_TRY(launch_eigen_bounds(b.gacc, N, 0, rank, b.np_acc, T, beside_tc));
          PTG_CUDA(cudaEventRecord(ctx->ev_join3, T));
          PTG_CUDA(cudaStreamWaitEvent(ctx->side2, ctx->ev_fork, 0));
          PTG_TRY(launch_eigen_bounds(b.gram, N, 0, rank, b.np, ctx->side2, beside_tc));
          PTG_CUDA(cudaEventRecord(ctx->ev_join2, ctx->side2));
          count_launches(ctx, 2);
        }
        count_launches(ctx, 1 + 2 * N);
        int *gate = b.isc + 2 * N;
        stop_gate_kernel<<<1, 1, 0, S>>>(b.dsc, N - 1, frob, opt.threshold_error, ao_iter, opt.max_iter, gate);
        PTG_CUDA(cudaGetLastError());
        count_launches(ctx, 1);
        PTG_TRY(run.point_cost_enqueue(Xa, b.acc, b.gacc, gate, ctx->ev_join));
        if (np0) {
          PTG_CUDA(cudaStreamWaitEvent(S, ctx->ev_join3, 0));
          PTG_CUDA(cudaStreamWaitEvent(S, ctx->ev_join2, 0));
        }
        PTG_TRY(run.select_enqueue(frob, opt.threshold_error, ao_iter, opt.max_iter));
        sel_pending = true;
        sel_sweep = ntrace;
      } else {
        for (int k = 0; k < N; ++k)
          PTG_CUDA(cudaMemcpyAsync(b.old[k], b.fac[k], sizeof(float) * b.rows[k] * rank,
                                   cudaMemcpyDeviceToDevice, S));
      }
    }
    PTG_TRY(run.sweep_finish(frob, &f, iters));
    for (int n = 0; n < N; ++n) inner_total += iters[n];
    rel = f / std::sqrt(frob);
    ptg_sweep_trace tr{};
    tr.f_value = f;
    tr.rel_costFunction = rel;
    for (int n = 0; n < N; ++n) tr.nesterov_iters[n] = iters[n];
    const bool stop = rel < opt.threshold_error || ao_iter >= opt.max_iter;
    tr.seconds = run.elapsed();
    if (trace) trace[ntrace] = tr;
    ++ntrace;
    if (stop) break;
  }
  if (sel_pending) {
    // queued behind the stopping sweep: the device's stop test gated it, nothing was taken
    PTG_CUDA(cudaEventSynchronize(ctx->ev_sel));
    if (run.hs()->sel[1] != 0.0) return set_error(PTG_ERR_CUDA, "internal: line search taken after the stop");
    sel_pending = false;
  }
  // FP32 refinement sweeps on the FP32 copy (no acceleration)
  int refined = 0;
  if (refine && opt.refine_sweeps > 0) {
    Xa = refine;
    frob = cost_norm(Xa);
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
  // the cost of the final factors on the FP32 copy (one MTTKRP in the Gram form, on the CUDA
  // cores: unbiased)
  if (refine && refined == 0 && opt.verify_fp32) {
    Xa = refine;
    frob = cost_norm(Xa);
    PTG_TRY(run.point_cost(Xa, frob, b.fac, b.gram, &f, true));
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
  if (opt.write_to_file) PTG_TRY(write_final_factors(opt, X->dims, N, rank, out_factors));
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
