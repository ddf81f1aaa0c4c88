// C ABI: errors, contexts, resident tensors, MTTKRP.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ptg_internal.h"

namespace ptg {

static thread_local std::string g_last_error;

int set_error(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_error(cudaError_t e, const char *what, const char *file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  return set_error(e == cudaErrorMemoryAllocation ? PTG_ERR_OOM : PTG_ERR_CUDA, buf);
}

int DevBuf::ensure(size_t need) {
  if (need <= bytes) return PTG_OK;
  if (ptr) {
    cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  size_t sz = std::max(need, (size_t)1 << 20);
  if (limit && *limit > 0 && sz > (size_t)*limit) {
    if (need > (size_t)*limit) return set_error(PTG_ERR_OOM, "device allocation above the context's limit");
    sz = need;
  }
  cudaError_t e = cudaMalloc(&ptr, sz);
  if (e != cudaSuccess) {
    ptr = nullptr;
    return cuda_error(e, "cudaMalloc(scratch)", __FILE__, __LINE__);
  }
  bytes = sz;
  return PTG_OK;
}

int ctx_malloc(const ptg_ctx *ctx, void **p, size_t bytes, const char *what) {
  *p = nullptr;
  if (ctx && ctx->alloc_limit > 0 && bytes > (size_t)ctx->alloc_limit)
    return set_error(PTG_ERR_OOM, std::string("cudaMalloc(") + what + "): above the context's allocation limit");
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_error(e, what, __FILE__, __LINE__);
  }
  return PTG_OK;
}

uint32_t spin_limit(const ptg_ctx *ctx) {
  return ctx->spin_limit < 0 ? kDefaultSpinLimit : (uint32_t)ctx->spin_limit;
}

void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

int stats_begin(ptg_ctx *ctx, cudaStream_t s, cudaEvent_t *ev) {
  *ev = nullptr;
  if (!ctx->stats.enabled) return PTG_OK;
  if (ctx->stats.pool.empty()) {
    cudaEvent_t e;
    PTG_CUDA(cudaEventCreate(&e));
    ctx->stats.pool.push_back(e);
  }
  *ev = ctx->stats.pool.back();
  ctx->stats.pool.pop_back();
  PTG_CUDA(cudaEventRecord(*ev, s));
  return PTG_OK;
}

int stats_end(ptg_ctx *ctx, cudaStream_t s, cudaEvent_t ev0, double bytes, double flops, bool tc) {
  if (!ctx->stats.enabled || !ev0) return PTG_OK;
  cudaEvent_t ev1;
  if (ctx->stats.pool.empty()) {
    PTG_CUDA(cudaEventCreate(&ev1));
  } else {
    ev1 = ctx->stats.pool.back();
    ctx->stats.pool.pop_back();
  }
  PTG_CUDA(cudaEventRecord(ev1, s));
  ctx->stats.pending.push_back({ev0, ev1, tc});
  ctx->stats.mttkrp_launches++;
  ctx->stats.mttkrp_bytes += bytes;
  ctx->stats.mttkrp_flops += flops;
  if (tc) {
    ctx->stats.tc_launches++;
    ctx->stats.tc_bytes += bytes;
  }
  return PTG_OK;
}

int stats_resolve(ptg_ctx *ctx) {
  for (auto &pr : ctx->stats.pending) {
    PTG_CUDA(cudaEventSynchronize(pr.b));
    float ms = 0.f;
    PTG_CUDA(cudaEventElapsedTime(&ms, pr.a, pr.b));
    ctx->stats.mttkrp_ms += ms;
    if (pr.tc) ctx->stats.tc_ms += ms;
    ctx->stats.pool.push_back(pr.a);
    ctx->stats.pool.push_back(pr.b);
  }
  ctx->stats.pending.clear();
  return PTG_OK;
}

int check_device_error(ptg_ctx *ctx) {
  int h = 0;
  PTG_CUDA(cudaMemcpyAsync(&h, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PTG_CUDA(cudaStreamSynchronize(ctx->stream));
  return report_device_error(ctx, h);
}

int report_device_error(ptg_ctx *ctx, int h) {
  if (h != 0) {
    PTG_CUDA(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream));
    PTG_CUDA(cudaStreamSynchronize(ctx->stream));
    return set_error(h, h == PTG_ERR_TIMEOUT ? "a device-side bounded wait gave up (kernel returned early)"
                                             : "a kernel reported a singular or non-finite R x R system");
  }
  return PTG_OK;
}

namespace {

// FP64 ColMajor source chunk -> padded storage, with FP64 partial sums of squares of the
// source and of the stored values (one pair per block, summed later in block order).
// the stored value of x (xf = (float)x, computed once): FP32 stores xf, BF16 rounds x directly
template <typename T>
__device__ __forceinline__ T stored(double x, float xf);
template <>
__device__ __forceinline__ float stored<float>(double, float xf) { return xf; }
template <>
__device__ __forceinline__ __nv_bfloat16 stored<__nv_bfloat16>(double x, float) { return __double2bfloat16(x); }
__device__ __forceinline__ double back(float x) { return (double)x; }
__device__ __forceinline__ double back(__nv_bfloat16 x) { return (double)__bfloat162float(x); }

constexpr int kConvBlocks = 1024;
constexpr int kConvThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kConvThreads)
convert_kernel(const double *__restrict__ src, int64_t I0, int64_t pI0, int64_t fiber0,
               int64_t nfibers, T *__restrict__ dst, float *__restrict__ dst32, double *__restrict__ part) {
  // a block per fibre (grid-stride over fibres), threads along i0: no index division.  The
  // squares of four entries of a thread are summed in FP32 and then added in FP64 (the FP64
  // pipe is the scarce one on this part; 4-entry FP32 partials keep ||X||^2 to ~1e-10
  // relative)
  double s64 = 0.0, sst = 0.0;
  for (int64_t f = blockIdx.x; f < nfibers; f += gridDim.x) {
    const double *s = src + f * I0;
    T *d = dst + (fiber0 + f) * pI0;
    float *d32 = dst32 ? dst32 + (fiber0 + f) * pI0 : nullptr;   // optional FP32 copy
    // four entries per thread per pass: their loads are in flight together
    for (int64_t base = threadIdx.x; base < pI0; base += 4 * (int64_t)blockDim.x) {
      double x[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t i0 = base + j * (int64_t)blockDim.x;
        x[j] = i0 < I0 ? __ldcs(s + i0) : 0.0;
      }
      float p64 = 0.0f, pst = 0.0f;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t i0 = base + j * (int64_t)blockDim.x;
        if (i0 < pI0) {
          // one FP64 -> FP32 conversion per entry (it runs on the slow FP64 pipe)
          const float xf = (float)x[j];
          const T v = stored<T>(x[j], xf);   // pads (i0 >= I0) store zero
          const float bf = (float)back(v);
          p64 = fmaf(xf, xf, p64);
          pst = fmaf(bf, bf, pst);
          d[i0] = v;
          if (d32) d32[i0] = xf;
        }
      }
      s64 += (double)p64;
      sst += (double)pst;
    }
  }
  __shared__ double r64[kConvThreads / 32], rst[kConvThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s64 += __shfl_down_sync(0xffffffffu, s64, o);
    sst += __shfl_down_sync(0xffffffffu, sst, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r64[threadIdx.x >> 5] = s64;
    rst[threadIdx.x >> 5] = sst;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kConvThreads / 32; ++w) {
      a += r64[w];
      b += rst[w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

__global__ void sum_partials_kernel(const double *part, int nblocks, double *acc) {
  // single thread, fixed order: deterministic
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = acc[0], b = acc[1];
    for (int i = 0; i < nblocks; ++i) {
      a += part[2 * i];
      b += part[2 * i + 1];
    }
    acc[0] = a;
    acc[1] = b;
  }
}

}  // namespace
}  // namespace ptg

using namespace ptg;

extern "C" {

const char *ptg_last_error(void) { return g_last_error.c_str(); }

const char *ptg_version(void) { return "ptg 0.1 (sm_103a)"; }

int ptg_ctx_create(int device, ptg_ctx **out) {
  if (!out) return set_error(PTG_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  PTG_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return set_error(PTG_ERR_INVALID, "no such device");
  PTG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  PTG_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10)
    return set_error(PTG_ERR_UNSUPPORTED, "libptg is built for sm_103a (GB300) only");
  ptg_ctx *c = new ptg_ctx();
  c->device = device;
  c->sm_count = prop.multiProcessorCount;
  c->cc_major = prop.major;
  c->cc_minor = prop.minor;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  {
    const size_t eig = eigen_kernel_smem() + prop.reservedSharedMemPerBlock;
    const size_t avail = prop.sharedMemPerMultiprocessor - prop.reservedSharedMemPerBlock;
    c->smem_beside_eigen = std::min(c->smem_optin, avail > eig ? avail - eig : (size_t)0);
  }
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) {
    pageable = host_tables = 0;
    cudaGetLastError();
  }
  c->pageable_ats = pageable == 1 && host_tables == 1;
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join3, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_cost, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_sel, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaHostAlloc(&c->pinned_scalars, kPinnedScalarBytes, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMalloc(&c->dev_err, 256);
  if (e == cudaSuccess) e = cudaMemset(c->dev_err, 0, 256);
  if (e != cudaSuccess) {
    ptg_ctx_destroy(c);
    return cuda_error(e, "ptg_ctx_create", __FILE__, __LINE__);
  }
  c->stream = c->own_stream;
  c->scratch.limit = c->cache_x.limit = c->cache_xr.limit = &c->alloc_limit;
  *out = c;
  return PTG_OK;
}

int ptg_ctx_destroy(ptg_ctx *c) {
  if (!c) return PTG_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->scratch.release();
  stats_resolve(c);
  for (cudaEvent_t e : c->stats.pool) cudaEventDestroy(e);
  if (c->dev_err) cudaFree(c->dev_err);
  if (c->f8_work) cudaFree(c->f8_work);
  if (c->pinned) cudaFreeHost(c->pinned);
  c->cache_x.release();
  c->cache_xr.release();
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_join2) cudaEventDestroy(c->ev_join2);
  if (c->ev_join3) cudaEventDestroy(c->ev_join3);
  if (c->ev_cost) cudaEventDestroy(c->ev_cost);
  if (c->ev_sel) cudaEventDestroy(c->ev_sel);
  if (c->pinned_scalars) cudaFreeHost(c->pinned_scalars);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->side2) cudaStreamDestroy(c->side2);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return PTG_OK;
}

int ptg_ctx_set_stream(ptg_ctx *c, void *s) {
  if (!c) return set_error(PTG_ERR_INVALID, "ctx is NULL");
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return PTG_OK;
}

int ptg_ctx_synchronize(ptg_ctx *c) {
  if (!c) return set_error(PTG_ERR_INVALID, "ctx is NULL");
  PTG_CUDA(cudaSetDevice(c->device));
  PTG_CUDA(cudaStreamSynchronize(c->stream));
  return check_device_error(c);
}

int ptg_ctx_set_option(ptg_ctx *c, int option, long long value) {
  if (!c) return set_error(PTG_ERR_INVALID, "ctx is NULL");
  switch (option) {
    case PTG_OPT_MTTKRP_IMPL:
      if (value < 0 || value > 2) return set_error(PTG_ERR_INVALID, "MTTKRP impl must be 0, 1 or 2");
      c->mttkrp_impl = (int)value;
      return PTG_OK;
    case PTG_OPT_NNLS_CLUSTER:
      if (value != 0 && value != 2 && value != 4 && value != 8 && value != 16)
        return set_error(PTG_ERR_INVALID, "NNLS cluster size must be 0 (auto), 2, 4, 8 or 16");
      c->nnls_cluster = (int)value;   // 0: probe again on the next solve
      return PTG_OK;
    case PTG_OPT_GTC_ROWS:
      if (value < 0 || value > 2) return set_error(PTG_ERR_INVALID, "GTC row solver must be 0 (auto), 1 or 2");
      c->gtc_rows = (int)value;
      return PTG_OK;
    case PTG_OPT_SPIN_LIMIT:
      if (value < -1 || value > 0xffffffffLL) return set_error(PTG_ERR_INVALID, "spin limit must be -1 or in [0, 2^32)");
      c->spin_limit = value;
      return PTG_OK;
    case PTG_OPT_ALLOC_LIMIT:
      if (value < 0) return set_error(PTG_ERR_INVALID, "allocation limit must be >= 0");
      c->alloc_limit = value;
      return PTG_OK;
    case PTG_OPT_HOST_READ:
      if (value < 0 || value > 2)
        return set_error(PTG_ERR_INVALID, "host read must be 0 (auto), 1 (staged) or 2 (in place)");
      c->host_read = (int)value;
      return PTG_OK;
    case PTG_OPT_BATCHED_IMPL:
      if (value != 0 && value != 1)
        return set_error(PTG_ERR_INVALID, "batched impl must be 0 (persistent) or 1 (per-phase graphs)");
      c->batched_impl = (int)value;
      return PTG_OK;
    default:
      return set_error(PTG_ERR_INVALID, "unknown option");
  }
}

int ptg_ctx_enable_stats(ptg_ctx *c, int enable) {
  if (!c) return set_error(PTG_ERR_INVALID, "ctx is NULL");
  c->stats.enabled = enable != 0;
  return PTG_OK;
}

int ptg_ctx_get_stats(ptg_ctx *c, ptg_stats *out) {
  if (!c || !out) return set_error(PTG_ERR_INVALID, "NULL argument");
  PTG_CUDA(cudaSetDevice(c->device));
  PTG_CUDA(cudaStreamSynchronize(c->stream));
  PTG_TRY(stats_resolve(c));
  out->launches = c->stats.launches;
  out->mttkrp_launches = c->stats.mttkrp_launches;
  out->mttkrp_ms = c->stats.mttkrp_ms;
  out->mttkrp_bytes = c->stats.mttkrp_bytes;
  out->mttkrp_flops = c->stats.mttkrp_flops;
  out->tc_launches = c->stats.tc_launches;
  out->tc_ms = c->stats.tc_ms;
  out->tc_bytes = c->stats.tc_bytes;
  out->batch_pass_launches = c->stats.batch_pass_launches;
  out->batch_pass_ms = c->stats.batch_pass_ms;
  out->batch_pass_bytes = c->stats.batch_pass_bytes;
  return PTG_OK;
}

int ptg_ctx_reset_stats(ptg_ctx *c) {
  if (!c) return set_error(PTG_ERR_INVALID, "ctx is NULL");
  PTG_CUDA(cudaSetDevice(c->device));
  PTG_CUDA(cudaStreamSynchronize(c->stream));
  PTG_TRY(stats_resolve(c));
  const bool en = c->stats.enabled;
  c->stats.launches = c->stats.mttkrp_launches = 0;
  c->stats.mttkrp_ms = c->stats.mttkrp_bytes = c->stats.mttkrp_flops = 0.0;
  c->stats.tc_launches = 0;
  c->stats.tc_ms = c->stats.tc_bytes = 0.0;
  c->stats.batch_pass_launches = 0;
  c->stats.batch_pass_ms = c->stats.batch_pass_bytes = 0.0;
  c->stats.enabled = en;
  return PTG_OK;
}

int ptg_tensor_create(ptg_ctx *c, int order, const int64_t *dims, ptg_dtype dtype,
                      const double *src, int src_on_device, ptg_tensor **out) {
  return ptg::tensor_create_impl(c, order, dims, dtype, src, src_on_device, nullptr, out, nullptr, nullptr);
}

}  // extern "C"

namespace ptg {

// A device address through which the conversion kernels of context c read the host buffer
// src in place, or nullptr to stage it through device chunks by copies.  The device can
// address page-locked (or registered) memory by its mapped pointer, and pageable memory where
// it reads through the host's page tables.  Measured on GB300 (Grace host, 8 GB FP64 source):
// the copy engine moves 200-210 GB/s from either kind of memory; the BF16/FP32 conversion
// reading page-locked memory in place reaches 203 GB/s and needs no staging buffers, reading
// pageable memory in place only 175 GB/s, and the FP8 encoder, which reads every slab twice
// (its maximum, then the codes), 75 GB/s in place against 200 staged.  So auto (0) reads in
// place only page-locked memory into BF16/FP32 storage; 2 reads in place wherever the device
// can address the buffer.  Nothing here pins, registers or migrates memory.
static const double *host_device_view(ptg_ctx *c, const double *src, bool fp8) {
  if (c->host_read == 1 || (c->host_read == 0 && fp8)) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, src) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost) return static_cast<const double *>(a.devicePointer);
  if (a.type == cudaMemoryTypeUnregistered && c->pageable_ats && c->host_read == 2) return src;
  return nullptr;
}

int tensor_create_impl(ptg_ctx *c, int order, const int64_t *dims, ptg_dtype dtype, const double *src,
                       int src_on_device, DevBuf *storage, ptg_tensor **out, DevBuf *storage32,
                       ptg_tensor **out32) {
  if (!c || !dims || !src || !out) return set_error(PTG_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (out32) {
    *out32 = nullptr;
    if (dtype == PTG_F32) return set_error(PTG_ERR_INVALID, "internal: an FP32 copy beside an FP32 tensor");
  }
  if (order < 2 || order > PTG_MAX_ORDER)
    return set_error(PTG_ERR_UNSUPPORTED, "tensor order must be in [2, 8]");
  if (dtype != PTG_F32 && dtype != PTG_BF16 && dtype != PTG_FP8E4M3) return set_error(PTG_ERR_UNSUPPORTED, "dtype");
  const bool fp8 = dtype == PTG_FP8E4M3;
  int64_t numel = 1;
  for (int k = 0; k < order; ++k) {
    if (dims[k] < 1 || dims[k] > 0x7fffffffLL)
      return set_error(PTG_ERR_INVALID, "every dimension must be in [1, 2^31)");
    numel *= dims[k];
  }
  PTG_CUDA(cudaSetDevice(c->device));
  if (!src_on_device) {   // a host source the kernels can address is read in one pass, in place
    if (const double *view = host_device_view(c, src, dtype == PTG_FP8E4M3)) {
      src = view;
      src_on_device = 1;
    }
  }
  ptg_tensor *t = new ptg_tensor();
  t->order = order;
  for (int k = 0; k < order; ++k) t->dims[k] = dims[k];
  // rows of 16 bytes: TMA copies start on 16-byte boundaries
  const int64_t pad = fp8 ? 16 : 8;
  t->pdim0 = (dims[0] + pad - 1) / pad * pad;
  t->numel_padded = numel / dims[0] * t->pdim0;
  t->dtype = dtype;
  t->device = c->device;
  const size_t esz = dtype == PTG_F32 ? 4 : dtype == PTG_BF16 ? 2 : 1;
  // FP8: the codes, then the slab scales and the slab maxima in the same allocation
  const int64_t nslab = dims[order - 1];
  const size_t code_bytes = ((size_t)t->numel_padded * esz + 255) / 256 * 256;
  const size_t scale_bytes = fp8 ? ((size_t)nslab * sizeof(float) + 255) / 256 * 256 : 0;
  const size_t total_bytes = code_bytes + scale_bytes + (fp8 ? (size_t)nslab * sizeof(unsigned long long) : 0);
  if (storage) {   // a context-owned buffer, kept for the next call
    const int rs = storage->ensure(total_bytes);
    if (rs != PTG_OK) {
      delete t;
      return rs;
    }
    t->data = storage->ptr;
    t->owns = false;
  } else {
    const int rs = ctx_malloc(c, &t->data, total_bytes, "tensor");
    if (rs != PTG_OK) {
      delete t;
      return rs;
    }
  }
  cudaError_t e = cudaSuccess;
  unsigned long long *slab_bits = nullptr;
  if (fp8) {
    t->f8_scales = (float *)((char *)t->data + code_bytes);
    slab_bits = (unsigned long long *)((char *)t->data + code_bytes + scale_bytes);
  }
  // the optional FP32 copy, written by the same pass
  ptg_tensor *t32 = nullptr;
  if (out32) {
    t32 = new ptg_tensor(*t);
    t32->dtype = PTG_F32;
    t32->owns = true;
    t32->f8_scales = nullptr;
    int rs = PTG_OK;
    if (storage32) {
      rs = storage32->ensure((size_t)t->numel_padded * 4);
      t32->data = storage32->ptr;
      t32->owns = false;
    } else {
      rs = ctx_malloc(c, &t32->data, (size_t)t->numel_padded * 4, "tensor");
    }
    if (rs != PTG_OK) {
      if (t->owns) cudaFree(t->data);
      delete t;
      delete t32;
      return rs;
    }
  }
  float *d32 = t32 ? (float *)t32->data : nullptr;
  const int64_t I0 = dims[0], pI0 = t->pdim0;
  const int64_t nfib = numel / I0;
  // staging for host sources: two chunk buffers, copies on `side`, conversion on `stream`
  // (a device source is converted in one launch; a host source streams through 64 MB chunks)
  // (FP8: a chunk holds whole slabs, whose maxima set the scales before they are encoded)
  const int64_t fps = nfib / nslab;   // mode-0 fibres per slab
  int64_t chunk_fib =
      src_on_device ? nfib : std::max<int64_t>(1, std::min<int64_t>(nfib, (64ll << 20) / I0));
  if (fp8 && !src_on_device) chunk_fib = std::min<int64_t>(nfib, std::max<int64_t>(1, chunk_fib / fps) * fps);
  double *stage[2] = {nullptr, nullptr};
  double *part = nullptr, *acc = nullptr;
  cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
  int rc = PTG_OK;
  auto fail = [&](int code) {
    rc = code;
    return code;
  };
  do {
    if ((e = cudaMalloc(&part, sizeof(double) * 2 * kConvBlocks)) != cudaSuccess) {
      fail(cuda_error(e, "cudaMalloc", __FILE__, __LINE__));
      break;
    }
    if ((e = cudaMalloc(&acc, sizeof(double) * 2)) != cudaSuccess) {
      fail(cuda_error(e, "cudaMalloc", __FILE__, __LINE__));
      break;
    }
    cudaMemsetAsync(acc, 0, sizeof(double) * 2, c->stream);
    if (fp8) cudaMemsetAsync(slab_bits, 0, sizeof(unsigned long long) * nslab, c->stream);
    if (!src_on_device) {
      for (int b = 0; b < 2 && rc == PTG_OK; ++b) {
        if ((e = cudaMalloc(&stage[b], sizeof(double) * chunk_fib * I0)) != cudaSuccess)
          fail(cuda_error(e, "cudaMalloc(stage)", __FILE__, __LINE__));
        else if ((e = cudaEventCreateWithFlags(&copied[b], cudaEventDisableTiming)) != cudaSuccess ||
                 (e = cudaEventCreateWithFlags(&consumed[b], cudaEventDisableTiming)) != cudaSuccess)
          fail(cuda_error(e, "cudaEventCreate", __FILE__, __LINE__));
      }
      if (rc != PTG_OK) break;
    }
    int chunk_idx = 0;
    for (int64_t f0 = 0; f0 < nfib; f0 += chunk_fib, ++chunk_idx) {
      const int64_t nf = std::min(chunk_fib, nfib - f0);
      const double *csrc;
      if (src_on_device) {
        csrc = src + f0 * I0;
      } else {
        const int b = chunk_idx & 1;
        if (chunk_idx >= 2) cudaStreamWaitEvent(c->side, consumed[b], 0);
        e = cudaMemcpyAsync(stage[b], src + f0 * I0, sizeof(double) * nf * I0,
                            cudaMemcpyHostToDevice, c->side);
        if (e != cudaSuccess) {
          fail(cuda_error(e, "cudaMemcpyAsync(H2D)", __FILE__, __LINE__));
          break;
        }
        cudaEventRecord(copied[b], c->side);
        cudaStreamWaitEvent(c->stream, copied[b], 0);
        csrc = stage[b];
      }
      const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(kConvBlocks, nf));
      if (fp8) {
        int r8 = f8_slab_max_launch(csrc, I0, f0, nf, fps, slab_bits, c->sm_count, c->stream);
        if (r8 == PTG_OK)
          r8 = f8_encode_launch(csrc, I0, pI0, f0, nf, fps, slab_bits, (uint8_t *)t->data, d32, t->f8_scales, part,
                                blocks, c->stream);
        if (r8 != PTG_OK) {
          fail(r8);
          break;
        }
        count_launches(c, 1);
      } else if (dtype == PTG_F32)
        convert_kernel<float><<<blocks, kConvThreads, 0, c->stream>>>(
            csrc, I0, pI0, f0, nf, (float *)t->data, nullptr, part);
      else
        convert_kernel<__nv_bfloat16><<<blocks, kConvThreads, 0, c->stream>>>(
            csrc, I0, pI0, f0, nf, (__nv_bfloat16 *)t->data, d32, part);
      sum_partials_kernel<<<1, 32, 0, c->stream>>>(part, blocks, acc);
      count_launches(c, 2);
      if (!src_on_device) cudaEventRecord(consumed[chunk_idx & 1], c->stream);
      if ((e = cudaGetLastError()) != cudaSuccess) {
        fail(cuda_error(e, "convert_kernel", __FILE__, __LINE__));
        break;
      }
    }
    if (rc != PTG_OK) break;
    double h[2];
    e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
      fail(cuda_error(e, "ptg_tensor_create", __FILE__, __LINE__));
      break;
    }
    t->frob64 = h[0];
    t->frob_stored = h[1];
    if (t32) t32->frob64 = t32->frob_stored = h[0];   // the FP32 copy stores exactly the squared values summed
    if (fp8) {   // the largest slab scale bounds the scaled Khatri-Rao values of the MTTKRP
      std::vector<float> sc((size_t)nslab);
      e = cudaMemcpy(sc.data(), t->f8_scales, sizeof(float) * nslab, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        fail(cuda_error(e, "cudaMemcpy(slab scales)", __FILE__, __LINE__));
        break;
      }
      t->f8_scale_max = *std::max_element(sc.begin(), sc.end());
    }
    if (!std::isfinite(h[0]) || !std::isfinite(h[1]))
      fail(set_error(PTG_ERR_NUMERIC, "tensor contains NaN or Inf"));
  } while (0);
  if (src_on_device == 0) cudaStreamSynchronize(c->side);
  for (int b = 0; b < 2; ++b) {
    if (stage[b]) cudaFree(stage[b]);
    if (copied[b]) cudaEventDestroy(copied[b]);
    if (consumed[b]) cudaEventDestroy(consumed[b]);
  }
  if (part) cudaFree(part);
  if (acc) cudaFree(acc);
  if (rc != PTG_OK) {
    if (t32) {
      if (t32->owns) cudaFree(t32->data);
      delete t32;
    }
    if (t->owns) cudaFree(t->data);
    delete t;
    return rc;
  }
  *out = t;
  if (out32) *out32 = t32;
  return PTG_OK;
}

}  // namespace ptg

extern "C" {

int ptg_tensor_destroy(ptg_tensor *t) {
  if (!t) return PTG_OK;
  cudaSetDevice(t->device);
  if (t->data && t->owns) cudaFree(t->data);
  delete t;
  return PTG_OK;
}

int ptg_tensor_norms(const ptg_tensor *t, double *frob64, double *frob_stored) {
  if (!t) return set_error(PTG_ERR_INVALID, "tensor is NULL");
  if (frob64) *frob64 = t->frob64;
  if (frob_stored) *frob_stored = t->frob_stored;
  return PTG_OK;
}

int ptg_tensor_storage(const ptg_tensor *t, const void **data, int64_t *padded_dim0, const float **slab_scales) {
  if (!t) return set_error(PTG_ERR_INVALID, "tensor is NULL");
  if (data) *data = t->data;
  if (padded_dim0) *padded_dim0 = t->pdim0;
  if (slab_scales) *slab_scales = t->f8_scales;
  return PTG_OK;
}

int ptg_mttkrp(ptg_ctx *c, const ptg_tensor *X, const float *const *factors, int rank, int mode,
               float *out) {
  if (!c || !X || !factors || !out) return set_error(PTG_ERR_INVALID, "NULL argument");
  if (mode < 0 || mode >= X->order) return set_error(PTG_ERR_INVALID, "mode out of range");
  if (rank < 1) return set_error(PTG_ERR_INVALID, "rank must be >= 1");
  for (int k = 0; k < X->order; ++k)
    if (k != mode && !factors[k]) return set_error(PTG_ERR_INVALID, "factor pointer is NULL");
  PTG_CUDA(cudaSetDevice(c->device));
  Contraction con = mttkrp_contraction(X, factors, mode);
  return contraction_launch(c, X, con, rank, out, c->stream);
}

}  // extern "C"
