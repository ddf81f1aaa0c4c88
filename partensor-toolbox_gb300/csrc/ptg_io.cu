// File-based entry points: the tensor (and optionally the initial factors) read from the
// reference's raw files straight into HBM.
//
// Format (include/ReadWrite.hpp:100-130, 293-345): a tensor file holds prod(dims) FP64 values
// in ColMajor order (Eigen::Tensor's data(), i0 fastest), after `skip` values; a factor file
// holds an I x R FP64 matrix written through its transpose, i.e. row-major. These are the
// `cpd(tnsDims, R, path[, options])` and `cpd(tnsDims, R, paths[, options])` overloads of
// include/Cpd.hpp:591-850. The file is streamed through a page-locked double buffer into a
// device FP64 buffer (read of chunk k+1 overlaps the copy of chunk k), converted there to the
// storage type(s), and freed.
#include <cmath>
#include <cstdio>
#include <vector>

#include "ptg_internal.h"

namespace ptg {
namespace {

constexpr size_t kFileChunk = 32u << 20;   // bytes per staging half

struct FileCloser {
  FILE *f = nullptr;
  ~FileCloser() {
    if (f) fclose(f);
  }
};

// Reads `numel` FP64 values after `skip` values of `path` into a new device buffer.
int read_file_to_device(ptg_ctx *ctx, const char *path, int64_t skip, int64_t numel, double **out) {
  *out = nullptr;
  FileCloser fc;
  fc.f = fopen(path, "rb");
  if (!fc.f) return set_error(PTG_ERR_INVALID, std::string("cannot open ") + path);
  if (fseek(fc.f, 0, SEEK_END) != 0) return set_error(PTG_ERR_INVALID, std::string("cannot seek in ") + path);
  const long long fsize = ftell(fc.f);
  const long long need = (long long)(skip + numel) * (long long)sizeof(double);
  if (fsize < need)
    return set_error(PTG_ERR_INVALID, std::string("file too short for the requested tensor: ") + path);
  if (fseek(fc.f, (long)(skip * (int64_t)sizeof(double)), SEEK_SET) != 0)
    return set_error(PTG_ERR_INVALID, std::string("cannot seek in ") + path);
  if (ctx->pinned_bytes < 2 * kFileChunk) {
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    PTG_CUDA(cudaHostAlloc(&ctx->pinned, 2 * kFileChunk, cudaHostAllocDefault));
    ctx->pinned_bytes = 2 * kFileChunk;
  }
  double *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * std::max<int64_t>(numel, 1));
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc(file staging)", __FILE__, __LINE__);
  cudaEvent_t copied[2] = {nullptr, nullptr};
  int rc = PTG_OK;
  for (int b = 0; b < 2 && rc == PTG_OK; ++b)
    if ((e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming)) != cudaSuccess)
      rc = cuda_error(e, "cudaEventCreate", __FILE__, __LINE__);
  const int64_t per = (int64_t)(kFileChunk / sizeof(double));
  int64_t done = 0;
  for (int k = 0; rc == PTG_OK && done < numel; ++k) {
    const int b = k & 1;
    double *host = (double *)ctx->pinned + (size_t)b * per;
    if (k >= 2 && (e = cudaEventSynchronize(copied[b])) != cudaSuccess) {
      rc = cuda_error(e, "cudaEventSynchronize", __FILE__, __LINE__);
      break;
    }
    const int64_t n = std::min(per, numel - done);
    if ((int64_t)fread(host, sizeof(double), (size_t)n, fc.f) != n) {
      rc = set_error(PTG_ERR_INVALID, std::string("short read from ") + path);
      break;
    }
    if ((e = cudaMemcpyAsync(d + done, host, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream)) !=
            cudaSuccess ||
        (e = cudaEventRecord(copied[b], ctx->stream)) != cudaSuccess) {
      rc = cuda_error(e, "cudaMemcpyAsync(file chunk)", __FILE__, __LINE__);
      break;
    }
    done += n;
  }
  cudaStreamSynchronize(ctx->stream);
  for (int b = 0; b < 2; ++b)
    if (copied[b]) cudaEventDestroy(copied[b]);
  if (rc != PTG_OK) {
    cudaFree(d);
    return rc;
  }
  *out = d;
  return PTG_OK;
}

// Reads an I x R row-major FP64 factor file into a ColMajor host matrix.
int read_factor_file(const char *path, int64_t I, int R, std::vector<double> &colmajor) {
  FileCloser fc;
  fc.f = fopen(path, "rb");
  if (!fc.f) return set_error(PTG_ERR_INVALID, std::string("cannot open ") + path);
  std::vector<double> rm((size_t)I * R);
  if (fread(rm.data(), sizeof(double), rm.size(), fc.f) != rm.size())
    return set_error(PTG_ERR_INVALID, std::string("factor file too short: ") + path);
  colmajor.resize(rm.size());
  for (int64_t i = 0; i < I; ++i)
    for (int r = 0; r < R; ++r) colmajor[(size_t)i + (size_t)I * r] = rm[(size_t)i * R + r];
  return PTG_OK;
}

// U[0,1] initial factors (makeFactors, include/DataGeneration.hpp:564-581) from a seeded
// splitmix64 stream instead of the reference's clock-seeded engine.
void seeded_factors(const int64_t *dims, int order, int R, unsigned long long seed,
                    std::vector<std::vector<double>> &f) {
  unsigned long long st = seed;
  auto next = [&st]() {
    unsigned long long z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  f.resize(order);
  for (int k = 0; k < order; ++k) {
    f[k].resize((size_t)dims[k] * R);
    for (double &v : f[k]) v = (double)(next() >> 11) * (1.0 / 9007199254740992.0);
  }
}

int cpd_file_impl(ptg_ctx *ctx, int order, const int64_t *dims, const char *tensor_path, int64_t skip,
                  const char *const *factor_paths, unsigned long long seed, ptg_dtype dtype, int rank,
                  const ptg_cpd_options *opts, double *const *out_factors, ptg_cpd_result *result,
                  ptg_sweep_trace *trace, bool dimtree) {
  if (!ctx || !dims || !tensor_path || !opts || !out_factors) return set_error(PTG_ERR_INVALID, "NULL argument");
  if (order < 3 || order > PTG_MAX_ORDER) return set_error(PTG_ERR_UNSUPPORTED, "order must be in [3, 8]");
  if (skip < 0) return set_error(PTG_ERR_INVALID, "skip must be >= 0");
  int64_t numel = 1;
  for (int k = 0; k < order; ++k) {
    if (dims[k] < 1) return set_error(PTG_ERR_INVALID, "every dimension must be >= 1");
    numel *= dims[k];
  }
  // initial factors: the files, or seeded U[0,1]
  std::vector<std::vector<double>> init;
  if (factor_paths) {
    init.resize(order);
    for (int k = 0; k < order; ++k) {
      if (!factor_paths[k]) return set_error(PTG_ERR_INVALID, "NULL factor path");
      PTG_TRY(read_factor_file(factor_paths[k], dims[k], rank, init[k]));
    }
  } else {
    seeded_factors(dims, order, rank, seed, init);
  }
  std::vector<const double *> ip(order);
  for (int k = 0; k < order; ++k) ip[k] = init[k].data();
  PTG_CUDA(cudaSetDevice(ctx->device));
  double *dsrc = nullptr;
  PTG_TRY(read_file_to_device(ctx, tensor_path, skip, numel, &dsrc));
  ptg_tensor *X = nullptr, *Xr = nullptr;
  int rc = ptg_tensor_create(ctx, order, dims, dtype, dsrc, 1, &X);
  const bool want_fp32 = dtype != PTG_F32 && (opts->refine_sweeps > 0 || opts->verify_fp32);
  if (rc == PTG_OK && want_fp32) rc = ptg_tensor_create(ctx, order, dims, PTG_F32, dsrc, 1, &Xr);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(dsrc);
  if (rc == PTG_OK)
    rc = dimtree ? ptg_cpd_dimtree_als(ctx, X, Xr, rank, opts, ip.data(), out_factors, result, trace)
                 : ptg_cpd_als(ctx, X, Xr, rank, opts, ip.data(), out_factors, result, trace);
  ptg_tensor_destroy(X);
  ptg_tensor_destroy(Xr);
  return rc;
}

}  // namespace
}  // namespace ptg

using namespace ptg;

extern "C" {

int ptg_tensor_create_file(ptg_ctx *ctx, int order, const int64_t *dims, ptg_dtype dtype, const char *path,
                           int64_t skip, ptg_tensor **out) {
  if (!ctx || !dims || !path || !out) return set_error(PTG_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (order < 2 || order > PTG_MAX_ORDER) return set_error(PTG_ERR_UNSUPPORTED, "tensor order must be in [2, 8]");
  if (skip < 0) return set_error(PTG_ERR_INVALID, "skip must be >= 0");
  int64_t numel = 1;
  for (int k = 0; k < order; ++k) {
    if (dims[k] < 1) return set_error(PTG_ERR_INVALID, "every dimension must be >= 1");
    numel *= dims[k];
  }
  PTG_CUDA(cudaSetDevice(ctx->device));
  double *dsrc = nullptr;
  PTG_TRY(read_file_to_device(ctx, path, skip, numel, &dsrc));
  const int rc = ptg_tensor_create(ctx, order, dims, dtype, dsrc, 1, out);
  cudaStreamSynchronize(ctx->stream);
  cudaFree(dsrc);
  return rc;
}

int ptg_cpd_file(ptg_ctx *ctx, int order, const int64_t *dims, const char *tensor_path, int64_t skip,
                 const char *const *factor_paths, unsigned long long seed, ptg_dtype dtype, int rank,
                 const ptg_cpd_options *opts, double *const *out_factors, ptg_cpd_result *result,
                 ptg_sweep_trace *trace) {
  return cpd_file_impl(ctx, order, dims, tensor_path, skip, factor_paths, seed, dtype, rank, opts, out_factors,
                       result, trace, false);
}

int ptg_cpd_dimtree_file(ptg_ctx *ctx, int order, const int64_t *dims, const char *tensor_path, int64_t skip,
                         const char *const *factor_paths, unsigned long long seed, ptg_dtype dtype, int rank,
                         const ptg_cpd_options *opts, double *const *out_factors, ptg_cpd_result *result,
                         ptg_sweep_trace *trace) {
  return cpd_file_impl(ctx, order, dims, tensor_path, skip, factor_paths, seed, dtype, rank, opts, out_factors,
                       result, trace, true);
}

}  // extern "C"
