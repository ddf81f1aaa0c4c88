// MTTKRP entry point that allocates no device memory.
//
// Who needs it: callers that are not allowed to call cudaMalloc at the moment they need an
// MTTKRP.  Examples are a host framework that owns all of HBM through its own arena and
// forbids third-party allocations, a solver step issued from inside a region that must not
// synchronise the device (cudaMalloc/cudaFree can synchronise), and latency-bound loops that
// cannot afford an allocation on their first call.  The regular entry point (ptg_mttkrp)
// grows a per-context scratch buffer with cudaMalloc when a larger problem comes along;
// this one uses a fixed block of device memory that is part of the library image instead.
//
// The block is a file-scope __device__ array of kScratchFloats floats (8 MiB).  Every GPU
// that loads the library holds it until the process exits.  Host code cannot use the
// array's name as a device address, so the address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on that device.
// Make that first call before any stream capture begins: the look-up may load the module.
//
// All calls share the block, and it keeps the contents of the last call.  Nothing in it
// needs to start at zero: each call writes every partial it later reads.  Two calls whose
// kernels overlap on the GPU (different streams, or the same stream from different host
// threads without ordering) race on the block.
//
// The looked-up address is kept for the life of the process.  A cudaDeviceReset (or any
// teardown of the device's primary context) reloads the module at a new address, so the
// entry point must not be used across one.  X, out, the factors and the stream must belong
// to the current device; X and out are checked.
#include <mutex>

#include "ptg_internal.h"

namespace ptg {
namespace {

constexpr size_t kScratchFloats = size_t(2) << 20;   // 2,097,152 floats = 8 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

std::mutex g_mu;
float *g_addr[kMaxDevices] = {nullptr};

// Device address of the block on the current device (looked up once per device).
int scratch_address(int device, float **out) {
  if (device < 0 || device >= kMaxDevices) return set_error(PTG_ERR_UNSUPPORTED, "device ordinal >= 64");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    g_addr[device] = static_cast<float *>(p);
  }
  *out = g_addr[device];
  return PTG_OK;
}

}  // namespace
}  // namespace ptg

using namespace ptg;

extern "C" int ptg_mttkrp_noalloc(const float *X, int order, const int64_t *dims, int64_t ld0,
                                  const float *const *factors, int rank, int mode, float *out,
                                  void *stream) {
  if (!X || !dims || !factors || !out) return set_error(PTG_ERR_INVALID, "NULL argument");
  if (order < 2 || order > PTG_MAX_ORDER) return set_error(PTG_ERR_UNSUPPORTED, "order must be in [2, 8]");
  if (mode < 0 || mode >= order) return set_error(PTG_ERR_INVALID, "mode out of range");
  if (rank < 1) return set_error(PTG_ERR_INVALID, "rank must be >= 1");
  for (int k = 0; k < order; ++k) {
    if (dims[k] < 1 || dims[k] > 0x7fffffffLL) return set_error(PTG_ERR_INVALID, "every dimension must be in [1, 2^31)");
    if (k != mode && !factors[k]) return set_error(PTG_ERR_INVALID, "factor pointer is NULL");
  }
  if (ld0 < dims[0] || (ld0 % 8) != 0)
    return set_error(PTG_ERR_INVALID, "ld0 must be >= dims[0] and a multiple of 8");
  if ((reinterpret_cast<uintptr_t>(X) & 15) != 0) return set_error(PTG_ERR_INVALID, "X must be 16-byte aligned");
  int device = 0;
  PTG_CUDA(cudaGetDevice(&device));
  // the buffers must live on the current device, whose copy of the block the kernel uses
  for (const void *p : {static_cast<const void *>(X), static_cast<const void *>(out)}) {
    cudaPointerAttributes a;
    PTG_CUDA(cudaPointerGetAttributes(&a, p));
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
      return set_error(PTG_ERR_INVALID, "X and out must be device memory");
    if (a.device != device) return set_error(PTG_ERR_INVALID, "X and out must belong to the current device");
  }
  int sms = 0;
  PTG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  // a stack description of the caller's tensor (no allocation)
  ptg_tensor t;
  t.order = order;
  for (int k = 0; k < order; ++k) t.dims[k] = dims[k];
  t.pdim0 = ld0;
  t.dtype = PTG_F32;
  t.data = const_cast<float *>(X);
  t.device = device;
  Contraction c = mttkrp_contraction(&t, factors, mode);
  if (simt_fixed_scratch_floats_needed(c, rank) > kScratchFloats) {
    return set_error(PTG_ERR_UNSUPPORTED,
                     "ptg_mttkrp_noalloc: I_mode (ld0 for mode 0) x R rounded up to 16/32/64/128 columns "
                     "must be <= 2097152 floats (the fixed 8 MiB scratch block)");
  }
  float *scratch = nullptr;
  PTG_TRY(scratch_address(device, &scratch));
  return simt_mttkrp_fixed_scratch(&t, c, rank, out, static_cast<cudaStream_t>(stream), sms, scratch,
                                   kScratchFloats);
}
