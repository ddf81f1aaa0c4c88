// Many small, uneven CPDs solved together (the fMRI-style batch): every phase of an ALS
// sweep is one launch for all instances, and the sweep's launch sequence is captured once
// as a CUDA graph and replayed.
//
//   eigenbounds      eigen_batched_kernel             one CTA per instance
//   MTTKRP           mttkrp_simt_batched_kernel       work list of (instance, q-tile, K-split)
//                    + batched_reduce_kernel          (one list per rank class of 16/32/64)
//   Nesterov MNLS    nnls_block_kernel                one CTA per instance, block-wide global
//                                                     stop test, fused repair/Gram/cost terms
//   normalise / acceleration / selection              one CTA per instance
// Per-instance state that the reference keeps on the host (accel_coeff, accel_fail, the stop
// test, include/Cpd.hpp:333-354) stays on the host; the device reads per-instance flags
// (active, accelerate, accepted) instead of swapped pointers, so the graphs never change.
// The split-K planning of the batched MTTKRP is tuned once per batch by timing candidate
// CTA targets (the autotuner), and the choice is cached in the context.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <map>
#include <thread>
#include <tuple>
#include <string>
#include <vector>

#include "ptg_internal.h"
#include "ptg_blockops.cuh"
#include "ptg_simt.cuh"

namespace ptg {
namespace {

__global__ void __launch_bounds__(BN_THREADS) nnls_block_kernel(const BNnls *__restrict__ tab,
                                                                const int *__restrict__ active) {
  const BNnls a = tab[blockIdx.x];
  if (active && !active[a.inst]) return;
  extern __shared__ __align__(16) float sm[];
  nnls_block_body(a, sm);
}

constexpr int kUpBlocks = 128, kUpThreads = 256;
constexpr size_t kStageBytes = 64u << 20;

// Bump allocation inside one device block (256-byte aligned); with base == nullptr it only
// measures the block.
struct Carve {
  char *base = nullptr;
  size_t off = 0, last = 0;
  template <typename T>
  T *take(size_t n) {
    off = (off + 255) & ~(size_t)255;
    last = off;
    T *p = base ? (T *)(base + off) : nullptr;
    off += std::max<size_t>(n, 1) * sizeof(T);
    return p;
  }
};

// FP64 fibres [f0, f0 + nf) of one tensor (ColMajor, mode-0 extent I0) -> FP32 storage
// padded to pI0, adding the FP64 sums of squares of the source and of the stored values into
// acc[0..1].  The last block to finish sums the per-block partials in block order
// (deterministic) and re-arms the ticket for the next launch.
__global__ void __launch_bounds__(kUpThreads)
upload_convert_kernel(const double *__restrict__ src, int64_t I0, int64_t pI0, int64_t f0, int64_t nf,
                      float *__restrict__ dst, double *__restrict__ part, unsigned *ticket, double *acc) {
  // a piece holds at most one staging chunk (64 MB), so 32-bit index arithmetic suffices; the
  // squares are summed in FP32 per thread-step and added in FP64 (the FP64 pipe is the scarce
  // one); the stored FP32 value's square is the source's square rounded the same way
  const uint32_t n = (uint32_t)(nf * pI0), upI0 = (uint32_t)pI0, uI0 = (uint32_t)I0;
  double s64 = 0.0;
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const uint32_t f = e / upI0, i0 = e - f * upI0;
    float v = 0.0f;
    if (i0 < uI0) {
      v = (float)__ldcs(src + (size_t)f * uI0 + i0);
      s64 += (double)(v * v);
    }
    dst[(f0 + f) * pI0 + i0] = v;
  }
  double sst = s64;
  __shared__ double r64[kUpThreads / 32], rst[kUpThreads / 32];
  __shared__ bool last;
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
    for (int w = 0; w < kUpThreads / 32; ++w) {
      a += r64[w];
      b += rst[w];
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double a = acc[0], b = acc[1];
    for (unsigned i = 0; i < gridDim.x; ++i) {
      a += ((volatile double *)part)[2 * i];
      b += ((volatile double *)part)[2 * i + 1];
    }
    acc[0] = a;
    acc[1] = b;
    *ticket = 0;
  }
}

// ------------------------------------------------------------------------------------
// Persistent solver: one launch for the whole batch.  Each CTA takes the next instance from
// an atomic queue (the host orders the queue largest first) and runs that instance's whole
// ALS loop -- Grams, eigenvalue bounds, MTTKRP, Nesterov MNLS, normalisation, the stop test
// and the line search, with the same bodies and in the same order as the per-phase graphs --
// then takes the next.  No CTA ever waits for another: the queue is a fetch-and-add.  The
// MTTKRP of a mode is split into (m-tile, K-split) items that the CTA's four 128-thread
// groups run independently (named barriers); K-split partials are summed in split order
// (deterministic).
// ------------------------------------------------------------------------------------
constexpr int kPGroups = BN_THREADS / 128;

struct PResult {
  double f, rel;
  long long inner;
  unsigned long long done_ns;
  int ao, acoef, afail, err;
};

struct PMeta {            // one contraction of an instance: its tile shape and K-split count
  int bn, bm, mmajor, nsplit;
};

struct PersistArgs {
  const InstDesc *desc;
  const EigDesc *eig;      // [mode * n_inst + instance]
  const BNnls *nn;         // [mode * n_inst + instance]
  const SimtParams *pm;    // [instance * (N + 1) + set]: set n < N mode n on the factors,
  const PMeta *meta;       //   set N mode 0 on the line-search point
  const int *order;        // the queue: instance indices, largest first
  const double *thr, *frob;
  PResult *res;
  int *queue;
  unsigned long long *t0;  // earliest CTA start (globaltimer, ns)
  float *scratch;          // per CTA: K-split partials
  size_t scratch_floats;
  int group_floats;        // shared memory of one MTTKRP group
  int n_inst, N, max_iter, acceleration, normalization, accel_coeff, accel_fail;
  int mttkrp_only;         // 1: every mode's MTTKRP of every instance once, nothing else
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// The items of one MTTKRP on the CTA's 128-thread groups g0..kPGroups-1 (the calling
// thread's group is threadIdx.x / 128; groups below g0 are busy with other work).
template <int BN, bool MM, int BM>
__device__ void cta_mttkrp_cfg(const SimtParams &prm, int nsplit, float *sm, int group_floats, int g0) {
  const int g = (threadIdx.x >> 7) - g0, gt = threadIdx.x & 127, ng = kPGroups - g0;
  const int mtiles = (int)((prm.Q + BM - 1) / BM);
  const int items = mtiles * nsplit;
  float *gs = sm + (size_t)g * group_floats;
  for (int it = g; it < items; it += ng)
    mttkrp_simt_body<float, BN, MM, BM, SyncGroup128>(prm, it / nsplit, it % nsplit, gs, gt,
                                                      SyncGroup128{1 + g0 + g});
}

// MTTKRP of contraction `set` of instance i into its M buffer, in three steps: the setup and
// the split sum are CTA-wide (every thread calls them); the items run on groups g0.. only.
__device__ PMeta cta_mttkrp_setup(const PersistArgs &a, int i, int set, float *scr, SimtParams *s_prm) {
  const int k = i * (a.N + 1) + set;
  const PMeta m = a.meta[k];
  if (threadIdx.x == 0) {
    *s_prm = a.pm[k];
    s_prm->partial = scr;
    s_prm->nsplit = m.nsplit;
  }
  __syncthreads();
  return m;
}

__device__ void cta_mttkrp_items(const PMeta &m, const SimtParams &p, float *sm, int group_floats, int g0) {
  if (m.bn == 16) {
    if (m.mmajor) {
      if (m.bm == 64) cta_mttkrp_cfg<16, true, 64>(p, m.nsplit, sm, group_floats, g0);
      else cta_mttkrp_cfg<16, true, 128>(p, m.nsplit, sm, group_floats, g0);
    } else {
      if (m.bm == 64) cta_mttkrp_cfg<16, false, 64>(p, m.nsplit, sm, group_floats, g0);
      else cta_mttkrp_cfg<16, false, 128>(p, m.nsplit, sm, group_floats, g0);
    }
  } else {
    if (m.mmajor) {
      if (m.bm == 64) cta_mttkrp_cfg<32, true, 64>(p, m.nsplit, sm, group_floats, g0);
      else cta_mttkrp_cfg<32, true, 128>(p, m.nsplit, sm, group_floats, g0);
    } else {
      if (m.bm == 64) cta_mttkrp_cfg<32, false, 64>(p, m.nsplit, sm, group_floats, g0);
      else cta_mttkrp_cfg<32, false, 128>(p, m.nsplit, sm, group_floats, g0);
    }
  }
}

__device__ void cta_mttkrp_finish(const PMeta &m, const SimtParams &p, const float *scr) {
  __syncthreads();
  if (m.nsplit > 1) {   // the partials of every split, summed in split order
    const int R = p.R, bn = m.bn;
    for (int idx = threadIdx.x; idx < (int)p.q_write * R; idx += blockDim.x) {
      const int q = idx / R, c = idx - q * R;
      float sum = 0.0f;
      for (int sp = 0; sp < m.nsplit; ++sp) sum += scr[((size_t)sp * p.Q + q) * bn + c];
      p.out[(size_t)q * R + c] = sum;
    }
    __syncthreads();
  }
}

__device__ void cta_mttkrp(const PersistArgs &a, int i, int set, float *sm, float *scr, SimtParams *s_prm) {
  const PMeta m = cta_mttkrp_setup(a, i, set, scr, s_prm);
  cta_mttkrp_items(m, *s_prm, sm, a.group_floats, 0);
  cta_mttkrp_finish(m, *s_prm, scr);
}

// The ALS loop of one instance (include/Cpd.hpp:288-356 with the batched path's per-instance
// bookkeeping of the stop test and the line search, :333-354).
__device__ void persist_instance(const PersistArgs &a, int i, float *sm, float *scr, SimtParams *s_prm,
                                 volatile int *s_flag, volatile float *s_step) {
  const InstDesc &in = a.desc[i];
  const int N = a.N, last = N - 1;
  gram_block(in, 0);
  __syncthreads();
  cta_mttkrp(a, i, last, sm, scr, s_prm);
  cost_terms_block(in, 0);
  __syncthreads();
  // scalars: kept by thread 0
  double f = 0.0, rel = 0.0;
  const double frob = a.frob[i];
  int ao = 0, acoef = a.accel_coeff, afail = a.accel_fail, err = 0;
  long long inner = 0;
  int reuse_m0 = 0;   // the last line search took its point: M holds this sweep's mode-0 MTTKRP
  if (threadIdx.x == 0) {
    f = sqrt(fmax(frob + in.cost_out[1] - 2.0 * in.cost_out[0], 0.0));
    rel = f / sqrt(frob);
  }
  for (;;) {
    for (int n = 0; n < N; ++n) {
      const EigDesc &e = a.eig[(size_t)n * a.n_inst + i];
      GramPtrs gp{};
      for (int k = 0; k < N; ++k) gp.g[k] = e.gram[k];
      if (n == 0 && reuse_m0) {   // M already holds mode 0's MTTKRP: the bounds alone
        if (threadIdx.x < 128) eigen_bounds_body<128, SyncGroup128>(gp, N, n, e.R, e.out, threadIdx.x, SyncGroup128{5});
        __syncthreads();
      } else {
        // the FP64 bounds on warps 0-3 (their own barrier) beside the MTTKRP's items on the
        // other three groups: the bounds mostly wait on the FP64 pipe, the MTTKRP on the FP32 one
        const PMeta m = cta_mttkrp_setup(a, i, n, scr, s_prm);
        if (threadIdx.x < 128) eigen_bounds_body<128, SyncGroup128>(gp, N, n, e.R, e.out, threadIdx.x, SyncGroup128{5});
        else cta_mttkrp_items(m, *s_prm, sm, a.group_floats, 1);
        cta_mttkrp_finish(m, *s_prm, scr);
      }
      nnls_block_body(a.nn[(size_t)n * a.n_inst + i], sm);
      __syncthreads();
    }
    if (a.normalization) {
      normalize_block(in);
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      ++ao;
      const BNnls &bl = a.nn[(size_t)last * a.n_inst + i];
      const double f2 = frob - 2.0 * bl.scal[0] + bl.scal[1];
      int stop = 0;
      if (!isfinite(f2)) {
        err = PTG_ERR_NUMERIC;
        stop = 1;
      } else {
        f = sqrt(fmax(f2, 0.0));
        rel = f / sqrt(frob);
        for (int n = 0; n < N; ++n) inner += a.nn[(size_t)n * a.n_inst + i].iscal[0];
        stop = (rel < a.thr[i] || ao >= a.max_iter) ? 1 : 0;
      }
      s_flag[0] = stop;
      s_flag[1] = (!stop && a.acceleration && ao > 1) ? 1 : 0;   // line search this sweep
      s_flag[2] = (!stop && a.acceleration) ? 1 : 0;             // keep this sweep's factors
      *s_step = (float)pow((double)(ao + 1), 1.0 / (double)acoef);
    }
    __syncthreads();
    if (s_flag[0]) break;
    const int accel = s_flag[1], copy = s_flag[2];
    reuse_m0 = 0;
    if (accel) {
      accel_combine_block(in, *s_step);
      __syncthreads();
      gram_block(in, 1);
      __syncthreads();
    }
    if (copy) {
      copy_old_block(in);
      __syncthreads();
    }
    if (accel) {
      cta_mttkrp(a, i, N, sm, scr, s_prm);
      cost_terms_block(in, 1);
      __syncthreads();
      if (threadIdx.x == 0) {
        const double fa = sqrt(fmax(frob + in.cost_out[1] - 2.0 * in.cost_out[0], 0.0));
        int accept = 0;
        if (f > fa) {
          accept = 1;
          f = fa;
        } else {
          ++afail;
        }
        if (afail == 5) {
          afail = 0;
          ++acoef;
        }
        s_flag[3] = accept;
      }
      __syncthreads();
      reuse_m0 = s_flag[3];
      if (reuse_m0) {
        select_block(in);
        __syncthreads();
      }
    }
  }
  if (threadIdx.x == 0) {
    PResult r;
    r.f = f;
    r.rel = rel;
    r.inner = inner;
    r.ao = ao;
    r.acoef = acoef;
    r.afail = afail;
    r.err = err;
    r.done_ns = globaltimer_ns();
    a.res[i] = r;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(BN_THREADS, 1) cpd_persistent_kernel(const PersistArgs a) {
  extern __shared__ __align__(16) float sm[];
  __shared__ SimtParams s_prm;
  __shared__ int s_inst;
  __shared__ int s_flag[4];
  __shared__ float s_step;
  if (threadIdx.x == 0) atomicMin(a.t0, globaltimer_ns());
  float *scr = a.scratch + (size_t)blockIdx.x * a.scratch_floats;
  for (;;) {
    if (threadIdx.x == 0) {
      const int k = atomicAdd(a.queue, 1);
      s_inst = k < a.n_inst ? a.order[k] : -1;
    }
    __syncthreads();
    const int i = s_inst;
    if (i < 0) break;
    if (a.mttkrp_only) {
      for (int n = 0; n < a.N; ++n) cta_mttkrp(a, i, n, sm, scr, &s_prm);   // ends with a barrier
      continue;
    }
    persist_instance(a, i, sm, scr, &s_prm, s_flag, &s_step);   // ends with a barrier
  }
}

struct DevArena {
  std::vector<void *> ptrs;
  ~DevArena() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <typename T>
  int alloc(T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc(batched CPD)", __FILE__, __LINE__);
    ptrs.push_back(q);
    *p = (T *)q;
    return PTG_OK;
  }
};

struct PinnedHost {
  void *p = nullptr;
  ~PinnedHost() {
    if (p) cudaFreeHost(p);
  }
};

struct GraphHolder {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
  ~GraphHolder() {
    if (e) cudaGraphExecDestroy(e);
    if (g) cudaGraphDestroy(g);
  }
};

int bn_class(int R) { return R <= 16 ? 16 : R <= 32 ? 32 : 64; }

}  // namespace
}  // namespace ptg

using namespace ptg;

extern "C" int ptg_cpd_batched(ptg_ctx *ctx, int n_inst, const ptg_cpd_instance *inst, const ptg_cpd_options *opts_in,
                               ptg_cpd_result *results, double *converge_seconds) {
  if (!ctx || !inst || !opts_in || n_inst < 1) return set_error(PTG_ERR_INVALID, "bad argument");
  const int N = inst[0].order;
  if (N < 3 || N > PTG_MAX_ORDER) return set_error(PTG_ERR_UNSUPPORTED, "order must be in [3, 8]");
  for (int i = 0; i < n_inst; ++i) {
    if (inst[i].order != N) return set_error(PTG_ERR_INVALID, "every instance of a batch has the same order");
    if (inst[i].rank < 1 || inst[i].rank > BN_MAXR)
      return set_error(PTG_ERR_UNSUPPORTED, "batched CPD: rank must be in [1, 32]");
    if (!inst[i].tensor || !inst[i].init_factors || !inst[i].out_factors)
      return set_error(PTG_ERR_INVALID, "NULL instance buffer");
    for (int k = 0; k < N; ++k) {
      if (inst[i].dims[k] < 1 || inst[i].dims[k] > 4096) return set_error(PTG_ERR_UNSUPPORTED, "batched CPD: dims in [1, 4096]");
      if (opts_in->constraints[k] != PTG_NONNEGATIVITY)
        return set_error(PTG_ERR_UNSUPPORTED, "batched CPD: nonnegativity constraints only");
    }
  }
  if (opts_in->max_iter < 1) return set_error(PTG_ERR_INVALID, "max_iter must be >= 1");
  PTG_CUDA(cudaSetDevice(ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  auto elapsed = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
  const ptg_cpd_options opt = *opts_in;
  // a private stream (capturable even when the context runs on the legacy stream), ordered
  // after the work already queued on the context's stream
  struct StreamHolder {
    cudaStream_t s = nullptr;
    ~StreamHolder() {
      if (s) cudaStreamDestroy(s);
    }
  } sh;
  PTG_CUDA(cudaStreamCreateWithFlags(&sh.s, cudaStreamNonBlocking));
  PTG_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaStream_t S = sh.s;
  // a second private stream: the eigenvalue bounds of a mode run beside its MTTKRP
  struct SideHolder {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~SideHolder() {
      if (fork) cudaEventDestroy(fork);
      if (join) cudaEventDestroy(join);
      if (s) cudaStreamDestroy(s);
    }
  } side;
  PTG_CUDA(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
  PTG_CUDA(cudaEventCreateWithFlags(&side.fork, cudaEventDisableTiming));
  PTG_CUDA(cudaEventCreateWithFlags(&side.join, cudaEventDisableTiming));

  // ---- one device block for every tensor and per-instance buffer ----
  std::vector<InstDesc> desc(n_inst);
  std::vector<NnlsParams *> np(n_inst);
  std::vector<float *> Wt(n_inst), Xdata(n_inst);
  std::vector<ptg_tensor> Tst(n_inst);
  std::vector<ptg_tensor *> T(n_inst);
  double *d_cost = nullptr, *d_scal = nullptr, *d_up = nullptr, *d_part = nullptr;
  int *d_iscal = nullptr, *d_flags = nullptr;
  unsigned *d_ticket = nullptr;
  float *d_step = nullptr;
  InstDesc *d_desc = nullptr;
  double *d_stage[2] = {nullptr, nullptr};
  size_t fac_begin = 0, fac_end = 0;
  const size_t stage_elems = (size_t)kStageBytes / sizeof(double);
  auto layout = [&](Carve &c) {
    for (int i = 0; i < n_inst; ++i)   // the factors first, contiguous: one copy in, one out
      for (int k = 0; k < N; ++k) {
        desc[i].fac[k] = c.take<float>((size_t)inst[i].dims[k] * inst[i].rank);
        if (i == 0 && k == 0) fac_begin = c.last;
      }
    fac_end = c.off;
    d_cost = c.take<double>(2 * (size_t)n_inst);
    d_scal = c.take<double>(2 * (size_t)n_inst * N);
    d_iscal = c.take<int>(2 * (size_t)n_inst * N);
    d_flags = c.take<int>(5 * (size_t)n_inst);
    d_step = c.take<float>(n_inst);
    d_desc = c.take<InstDesc>(n_inst);
    d_up = c.take<double>(2 * (size_t)n_inst);
    d_part = c.take<double>(2 * (size_t)kUpBlocks);
    d_ticket = c.take<unsigned>(1);
    for (int b = 0; b < 2; ++b) d_stage[b] = c.take<double>(stage_elems);
    for (int i = 0; i < n_inst; ++i) {
      const int R = inst[i].rank;
      int64_t rmax = 1, fibres = 1;
      for (int k = 0; k < N; ++k) {
        const int64_t I = inst[i].dims[k];
        rmax = std::max<int64_t>(rmax, I);
        if (k) fibres *= I;
        desc[i].old[k] = c.take<float>((size_t)I * R);
        desc[i].acc[k] = c.take<float>((size_t)I * R);
        desc[i].gram[k] = c.take<float>((size_t)R * R);
        desc[i].gacc[k] = c.take<float>((size_t)R * R);
      }
      desc[i].M = c.take<float>((size_t)rmax * R);
      Wt[i] = c.take<float>((size_t)rmax * R);
      np[i] = c.take<NnlsParams>(1);
      Xdata[i] = c.take<float>((size_t)((inst[i].dims[0] + 7) / 8 * 8) * fibres);
    }
  };
  Carve sizing;
  layout(sizing);
  DevArena ar;
  char *block = nullptr;
  PTG_TRY(ar.alloc(&block, sizing.off));
  Carve carve{block};
  layout(carve);
  for (int i = 0; i < n_inst; ++i) {
    InstDesc &d = desc[i];
    d.order = N;
    d.R = inst[i].rank;
    d.inst = i;
    d.weight = 0;   // choose_normilization_factor with no orthogonal mode (include/Normalize.hpp:53-67)
    for (int k = 0; k < N; ++k) d.rows[k] = (int)inst[i].dims[k];
    d.cost_out = d_cost + 2 * i;
    ptg_tensor &t = Tst[i];
    t.order = N;
    int64_t fibres = 1;
    for (int k = 0; k < N; ++k) {
      t.dims[k] = inst[i].dims[k];
      if (k) fibres *= inst[i].dims[k];
    }
    t.pdim0 = (t.dims[0] + 7) / 8 * 8;
    t.numel_padded = t.pdim0 * fibres;
    t.dtype = PTG_F32;
    t.data = Xdata[i];
    t.device = ctx->device;
    T[i] = &t;
  }
  PTG_CUDA(cudaMemsetAsync(d_up, 0, sizeof(double) * 2 * n_inst, S));
  PTG_CUDA(cudaMemsetAsync(d_ticket, 0, sizeof(unsigned), S));

  // ---- initial factors: host FP64 ColMajor -> FP32 row-major, one copy ----
  std::vector<float> init_img((fac_end - fac_begin) / sizeof(float), 0.0f);
  {
    std::vector<float> &hf = init_img;
    for (int i = 0; i < n_inst; ++i)
      for (int k = 0; k < N; ++k) {
        const int64_t I = inst[i].dims[k];
        const int R = inst[i].rank;
        float *dst = hf.data() + ((char *)desc[i].fac[k] - block - fac_begin) / sizeof(float);
        for (int64_t r0 = 0; r0 < I; ++r0)
          for (int r = 0; r < R; ++r) {
            const double v = inst[i].init_factors[k][r0 + I * r];
            if (!std::isfinite(v)) return set_error(PTG_ERR_NUMERIC, "initial factor contains NaN or Inf");
            dst[(size_t)r0 * R + r] = (float)v;
          }
      }
    PTG_CUDA(cudaMemcpyAsync(block + fac_begin, hf.data(), fac_end - fac_begin, cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaStreamSynchronize(S));
  }

  // ---- tensors: copied chunk by chunk into a device double buffer on the side stream, FP32
  // conversion with FP64 ||X||^2 on the main stream (the copy of chunk k beside the conversion
  // of chunk k-1) ----
  {
    struct Piece {
      int inst;
      int64_t f0, nf;
      size_t off;   // in doubles, within the chunk
    };
    std::vector<std::vector<Piece>> chunks(1);
    size_t used = 0;
    for (int i = 0; i < n_inst; ++i) {
      const int64_t I0 = inst[i].dims[0], nfib = Tst[i].numel_padded / Tst[i].pdim0;
      const int64_t per = std::max<int64_t>(1, (int64_t)(stage_elems / (size_t)I0));
      if ((size_t)I0 > stage_elems) return set_error(PTG_ERR_UNSUPPORTED, "batched CPD: mode-0 fibre too long");
      for (int64_t f0 = 0; f0 < nfib;) {
        int64_t room = (int64_t)((stage_elems - used) / (size_t)I0);
        if (room == 0) {
          chunks.emplace_back();
          used = 0;
          room = per;
        }
        const int64_t nf = std::min(room, nfib - f0);
        chunks.back().push_back(Piece{i, f0, nf, used});
        used += (size_t)(nf * I0);
        f0 += nf;
      }
    }
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};   // freed[2], copied[2]
    struct EvGuard {
      cudaEvent_t *e;
      ~EvGuard() {
        for (int b = 0; b < 4; ++b)
          if (e[b]) cudaEventDestroy(e[b]);
      }
    } evg{ev};
    for (int b = 0; b < 4; ++b) PTG_CUDA(cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming));
    cudaEvent_t *freed = ev, *copied = ev + 2;
    for (size_t ck = 0; ck < chunks.size(); ++ck) {
      const int b = (int)(ck & 1);
      if (ck >= 2) PTG_CUDA(cudaStreamWaitEvent(side.s, freed[b], 0));
      // the pieces are copied straight from the caller's buffers: on this host a pageable copy
      // runs near the link's rate, so no page-locked bounce is needed
      for (const Piece &p : chunks[ck]) {
        const int64_t I0 = inst[p.inst].dims[0];
        PTG_CUDA(cudaMemcpyAsync(d_stage[b] + p.off, inst[p.inst].tensor + p.f0 * I0,
                                 sizeof(double) * (size_t)(p.nf * I0), cudaMemcpyHostToDevice, side.s));
      }
      PTG_CUDA(cudaEventRecord(copied[b], side.s));
      PTG_CUDA(cudaStreamWaitEvent(S, copied[b], 0));
      for (const Piece &p : chunks[ck]) {
        const int64_t I0 = inst[p.inst].dims[0], pI0 = Tst[p.inst].pdim0;
        upload_convert_kernel<<<kUpBlocks, kUpThreads, 0, S>>>(d_stage[b] + p.off, I0, pI0, p.f0, p.nf, Xdata[p.inst],
                                                               d_part, d_ticket, d_up + 2 * p.inst);
        count_launches(ctx, 1);
      }
      PTG_CUDA(cudaEventRecord(freed[b], S));
      PTG_CUDA(cudaGetLastError());
    }
    PTG_CUDA(cudaStreamSynchronize(side.s));
    std::vector<double> up(2 * (size_t)n_inst);
    PTG_CUDA(cudaMemcpyAsync(up.data(), d_up, sizeof(double) * up.size(), cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    for (int i = 0; i < n_inst; ++i) {
      Tst[i].frob64 = up[2 * i];
      Tst[i].frob_stored = up[2 * i + 1];
      if (!std::isfinite(up[2 * i]) || !std::isfinite(up[2 * i + 1]))
        return set_error(PTG_ERR_NUMERIC, "tensor contains NaN or Inf");
    }
  }
  PTG_CUDA(cudaMemcpyAsync(d_desc, desc.data(), sizeof(InstDesc) * n_inst, cudaMemcpyHostToDevice, S));
  // flags: active, accelerate, accepted, copy-old; steps
  int *d_active = d_flags, *d_accel = d_flags + n_inst, *d_accept = d_flags + 2 * n_inst, *d_copy = d_flags + 3 * n_inst;
  // mode 0's MTTKRP runs for active instances whose last line search did not take its point
  // (a taken point left that product in M)
  int *d_m0 = d_flags + 4 * n_inst;
  PinnedHost hp;
  const size_t host_bytes = sizeof(int) * 5 * n_inst + sizeof(float) * n_inst + sizeof(double) * (2 * n_inst * N + 2 * n_inst) +
                            sizeof(int) * 2 * n_inst * N + 16;   // + alignment of the FP64 block
  PTG_CUDA(cudaHostAlloc(&hp.p, host_bytes, cudaHostAllocDefault));
  int *h_flags = (int *)hp.p;
  float *h_step = (float *)(h_flags + 5 * n_inst);
  double *h_scal = (double *)(((uintptr_t)(h_step + n_inst) + 7) & ~(uintptr_t)7);
  double *h_cost = h_scal + 2 * n_inst * N;
  int *h_iscal = (int *)(h_cost + 2 * n_inst);
  for (int i = 0; i < 5 * n_inst; ++i) h_flags[i] = 0;
  for (int i = 0; i < n_inst; ++i) h_flags[i] = h_flags[4 * n_inst + i] = 1;   // all active

  // ---- eigen / NNLS descriptors per mode ----
  std::vector<EigDesc> eig((size_t)N * n_inst);
  std::vector<BNnls> nn((size_t)N * n_inst);
  for (int n = 0; n < N; ++n)
    for (int i = 0; i < n_inst; ++i) {
      EigDesc &e = eig[(size_t)n * n_inst + i];
      std::memset(&e, 0, sizeof(e));
      for (int k = 0; k < N; ++k) e.gram[k] = desc[i].gram[k];
      e.order = N;
      e.mode = n;
      e.R = desc[i].R;
      e.inst = i;
      e.out = np[i];
      BNnls &b = nn[(size_t)n * n_inst + i];
      b.M = desc[i].M;
      b.A = desc[i].fac[n];
      b.Wt = Wt[i];
      b.I = desc[i].rows[n];
      b.R = desc[i].R;
      b.inst = i;
      b.np = np[i];
      b.d1 = (float)opt.nesterov_delta_1;
      b.d2 = (float)opt.nesterov_delta_2;
      b.gram_out = desc[i].gram[n];
      b.scal = d_scal + ((size_t)n * n_inst + i) * 2;
      b.iscal = d_iscal + ((size_t)n * n_inst + i) * 2;
    }
  EigDesc *d_eig;
  BNnls *d_nn;
  PTG_TRY(ar.alloc(&d_eig, eig.size()));
  PTG_TRY(ar.alloc(&d_nn, nn.size()));
  PTG_CUDA(cudaMemcpy(d_eig, eig.data(), sizeof(EigDesc) * eig.size(), cudaMemcpyHostToDevice));
  PTG_CUDA(cudaMemcpy(d_nn, nn.data(), sizeof(BNnls) * nn.size(), cudaMemcpyHostToDevice));
  // shared memory of the NNLS block: Y^T [R][I rounded to 4], A and the gradient [I][R]
  size_t nnls_smem = 0;
  for (const BNnls &b : nn)
    nnls_smem = std::max(nnls_smem, sizeof(float) * ((size_t)b.R * ((b.I + 3) & ~3) + 2 * (size_t)b.I * b.R));
  if (nnls_smem > ctx->smem_optin)
    return set_error(PTG_ERR_UNSUPPORTED,
                     "batched CPD: a factor (rows x rank) is too large for the one-CTA NNLS (shared memory)");
  PTG_CUDA(cudaFuncSetAttribute(nnls_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nnls_smem));

  // ---- results: one copy of every factor, FP32 row-major -> host FP64 ColMajor ----
  auto write_results = [&](const std::vector<double> &frob, const std::vector<double> &f,
                           const std::vector<double> &rel, const std::vector<int> &ao, const std::vector<int> &acoef,
                           const std::vector<int> &afail, const std::vector<long long> &inner,
                           const std::vector<double> &done_t, double t_solve) -> int {
    std::vector<float> hf((fac_end - fac_begin) / sizeof(float));
    PTG_CUDA(cudaMemcpyAsync(hf.data(), block + fac_begin, fac_end - fac_begin, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    for (int i = 0; i < n_inst; ++i) {
      for (int k = 0; k < N; ++k) {
        const int64_t I = inst[i].dims[k];
        const int R = desc[i].R;
        const float *src = hf.data() + ((char *)desc[i].fac[k] - block - fac_begin) / sizeof(float);
        for (int64_t r0 = 0; r0 < I; ++r0)
          for (int r = 0; r < R; ++r) inst[i].out_factors[k][r0 + I * r] = (double)src[(size_t)r0 * R + r];
      }
      if (results) {
        results[i].frob_tns = frob[i];
        results[i].f_value = f[i];
        results[i].rel_costFunction = rel[i];
        results[i].ao_iter = ao[i];
        results[i].accel_coeff = acoef[i];
        results[i].accel_fail = afail[i];
        results[i].refine_sweeps_done = 0;
        results[i].nesterov_iters_total = inner[i];
        results[i].seconds_total = done_t[i];
      }
      if (converge_seconds) converge_seconds[i] = done_t[i] - t_solve;
    }
    return PTG_OK;
  };

  if (ctx->batched_impl == 0) {
    // ---- the persistent solver: plan every contraction, order the queue, one launch ----
    const int NS = N + 1;
    std::vector<SimtParams> pm((size_t)n_inst * NS);
    std::vector<PMeta> meta((size_t)n_inst * NS);
    size_t scratch_floats = 0;
    int group_floats = 0;
    auto bm_of = [](int64_t Q) {
      const int64_t w64 = (Q + 63) / 64 * 64 - Q, w128 = (Q + 127) / 128 * 128 - Q;
      return w64 < w128 ? 64 : 128;
    };
    // items_per_group: the (m-tile, K-split) items each of the CTA's groups gets per MTTKRP
    auto plan = [&](int items_per_group) {
      scratch_floats = 0;
      group_floats = 0;
      for (int i = 0; i < n_inst; ++i)
        for (int set = 0; set < NS; ++set) {
          const int mode = set < N ? set : 0;
          const Contraction c = mttkrp_contraction(T[i], set < N ? desc[i].fac : desc[i].acc, mode);
          const int bn = bn_class(desc[i].R), bm = bm_of(c.Q);
          const bool mm = c.P == 1;
          SimtParams p{};
          p.X = T[i]->data;
          p.P = c.P;
          p.Q = c.Q;
          p.S = c.S;
          p.before = to_dev(c.before);
          p.after = to_dev(c.after);
          p.R = desc[i].R;
          p.col0 = 0;
          p.out = desc[i].M;
          p.q_write = c.q_write;
          p.ldo = desc[i].R;
          if (mm) {
            p.pblocks = 1;
            p.ktiles_total = (c.S + BK - 1) / BK;
          } else {
            p.pblocks = (c.P + BK - 1) / BK;
            p.ktiles_total = c.S * p.pblocks;
          }
          const int64_t mtiles = (c.Q + bm - 1) / bm;
          const int64_t target = (int64_t)kPGroups * items_per_group;
          int64_t ns = std::max<int64_t>(1, (target + mtiles - 1) / mtiles);
          ns = std::min<int64_t>(ns, p.ktiles_total);
          p.ktiles_per_split = (p.ktiles_total + ns - 1) / ns;
          ns = (p.ktiles_total + p.ktiles_per_split - 1) / p.ktiles_per_split;
          p.nsplit = (int)ns;
          pm[(size_t)i * NS + set] = p;
          meta[(size_t)i * NS + set] = PMeta{bn, bm, mm ? 1 : 0, (int)ns};
          if (ns > 1) scratch_floats = std::max(scratch_floats, (size_t)ns * c.Q * bn);
          const size_t gb = bn == 16 ? simt_smem_bytes<16>(mm, bm) : simt_smem_bytes<32>(mm, bm);
          group_floats = std::max(group_floats, (int)((gb / sizeof(float) + 31) / 32 * 32));
        }
    };
    // the queue, largest instance first (longest-processing-time order)
    std::vector<int> order(n_inst);
    for (int i = 0; i < n_inst; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      return (double)Tst[x].numel_padded * desc[x].R > (double)Tst[y].numel_padded * desc[y].R;
    });
    std::vector<double> thr(n_inst), frobv(n_inst);
    for (int i = 0; i < n_inst; ++i) {
      thr[i] = inst[i].threshold_error > 0.0 ? inst[i].threshold_error : opt.threshold_error;
      frobv[i] = T[i]->frob_stored;
    }
    const int grid = std::min(n_inst, ctx->sm_count);
    cudaFuncAttributes fa;
    PTG_CUDA(cudaFuncGetAttributes(&fa, cpd_persistent_kernel));
    SimtParams *d_pm;
    PMeta *d_meta;
    int *d_order, *d_queue;
    double *d_thr, *d_frob;
    PResult *d_res;
    unsigned long long *d_t0;
    PTG_TRY(ar.alloc(&d_pm, pm.size()));
    PTG_TRY(ar.alloc(&d_meta, meta.size()));
    PTG_TRY(ar.alloc(&d_order, n_inst));
    PTG_TRY(ar.alloc(&d_thr, n_inst));
    PTG_TRY(ar.alloc(&d_frob, n_inst));
    PTG_TRY(ar.alloc(&d_res, n_inst));
    PTG_TRY(ar.alloc(&d_queue, 1));
    PTG_TRY(ar.alloc(&d_t0, 1));
    PTG_CUDA(cudaMemcpyAsync(d_order, order.data(), sizeof(int) * n_inst, cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaMemcpyAsync(d_frob, frobv.data(), sizeof(double) * n_inst, cudaMemcpyHostToDevice, S));
    float *d_scr = nullptr;
    size_t scr_cap = 0;
    PersistArgs pa{};
    pa.desc = d_desc;
    pa.eig = d_eig;
    pa.nn = d_nn;
    pa.pm = d_pm;
    pa.meta = d_meta;
    pa.order = d_order;
    pa.thr = d_thr;
    pa.frob = d_frob;
    pa.res = d_res;
    pa.queue = d_queue;
    pa.t0 = d_t0;
    pa.n_inst = n_inst;
    pa.N = N;
    pa.acceleration = opt.acceleration;
    pa.normalization = opt.normalization;
    pa.accel_coeff = opt.accel_coeff;
    pa.accel_fail = opt.accel_fail;
    // one launch with the plan of `items_per_group` (max_iter sweeps, thresholds `th`)
    auto launch = [&](int items_per_group, int max_iter, const std::vector<double> &th) -> int {
      plan(items_per_group);
      const size_t dyn = std::max((size_t)kPGroups * group_floats * sizeof(float), nnls_smem);
      if (dyn + fa.sharedSizeBytes > ctx->smem_optin)
        return set_error(PTG_ERR_UNSUPPORTED, "batched CPD: persistent solver exceeds shared memory");
      if (scratch_floats * grid > scr_cap) {
        PTG_TRY(ar.alloc(&d_scr, scratch_floats * grid));
        scr_cap = scratch_floats * grid;
      }
      PTG_CUDA(cudaMemcpyAsync(d_pm, pm.data(), sizeof(SimtParams) * pm.size(), cudaMemcpyHostToDevice, S));
      PTG_CUDA(cudaMemcpyAsync(d_meta, meta.data(), sizeof(PMeta) * meta.size(), cudaMemcpyHostToDevice, S));
      PTG_CUDA(cudaMemcpyAsync(d_thr, th.data(), sizeof(double) * n_inst, cudaMemcpyHostToDevice, S));
      PTG_CUDA(cudaMemsetAsync(d_queue, 0, sizeof(int), S));
      PTG_CUDA(cudaMemsetAsync(d_t0, 0xff, sizeof(unsigned long long), S));
      pa.scratch = d_scr;
      pa.scratch_floats = scratch_floats;
      pa.group_floats = group_floats;
      pa.max_iter = max_iter;
      PTG_CUDA(cudaFuncSetAttribute(cpd_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
      cpd_persistent_kernel<<<grid, BN_THREADS, dyn, S>>>(pa);
      PTG_CUDA(cudaGetLastError());
      count_launches(ctx, 1);
      return PTG_OK;
    };
    // autotuner: two sweeps of the whole batch per candidate split target, then the
    // initial factors again (cached per batch shape in the context)
    long long shape_sum = 0;
    for (int i = 0; i < n_inst; ++i) {
      shape_sum = shape_sum * 31 + desc[i].R;
      for (int k = 0; k < N; ++k) shape_sum = shape_sum * 131 + desc[i].rows[k];
    }
    const std::string key = "persist:" + std::to_string(n_inst) + ":" + std::to_string(shape_sum);
    int best = ctx->tuned.count(key) ? ctx->tuned[key] : 0;
    if (!best) {
      cudaEvent_t e0, e1;
      PTG_CUDA(cudaEventCreate(&e0));
      PTG_CUDA(cudaEventCreate(&e1));
      const std::vector<double> never(n_inst, 0.0);
      float best_ms = 1e30f;
      for (int cand : {1, 2, 4}) {
        PTG_CUDA(cudaEventRecord(e0, S));
        PTG_TRY(launch(cand, 2, never));
        PTG_CUDA(cudaEventRecord(e1, S));
        PTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        PTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
          best_ms = ms;
          best = cand;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      ctx->tuned[key] = best;
      PTG_CUDA(cudaMemcpyAsync(block + fac_begin, init_img.data(), fac_end - fac_begin, cudaMemcpyHostToDevice, S));
    }
    if (ctx->stats.enabled) {   // one timed pass of every mode's MTTKRP of every instance
      double bytes = 0.0;
      for (int i = 0; i < n_inst; ++i)
        for (int n = 0; n < N; ++n) {
          bytes += 4.0 * (double)Tst[i].numel_padded;
          for (int k = 0; k < N; ++k) bytes += 4.0 * (double)inst[i].dims[k] * inst[i].rank;
        }
      cudaEvent_t e0, e1;
      PTG_CUDA(cudaEventCreate(&e0));
      PTG_CUDA(cudaEventCreate(&e1));
      const long long l0 = ctx->stats.launches;
      pa.mttkrp_only = 1;
      PTG_CUDA(cudaEventRecord(e0, S));
      PTG_TRY(launch(best, 1, std::vector<double>(n_inst, 0.0)));
      PTG_CUDA(cudaEventRecord(e1, S));
      PTG_CUDA(cudaEventSynchronize(e1));
      pa.mttkrp_only = 0;
      float ms = 0.f;
      PTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      ctx->stats.batch_pass_launches = ctx->stats.launches - l0;
      ctx->stats.batch_pass_ms = ms;
      ctx->stats.batch_pass_bytes = bytes;
    }
    PTG_CUDA(cudaStreamSynchronize(S));
    const double t_solve = elapsed();   // every tensor resident from here on
    PTG_TRY(launch(best, opt.max_iter, thr));
    std::vector<PResult> res(n_inst);
    unsigned long long t0_ns = 0;
    PTG_CUDA(cudaMemcpyAsync(res.data(), d_res, sizeof(PResult) * n_inst, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaMemcpyAsync(&t0_ns, d_t0, sizeof(t0_ns), cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    PTG_TRY(check_device_error(ctx));
    std::vector<double> f(n_inst), rel(n_inst), done_t(n_inst);
    std::vector<int> ao(n_inst), acoef(n_inst), afail(n_inst);
    std::vector<long long> inner(n_inst);
    for (int i = 0; i < n_inst; ++i) {
      const PResult &r = res[i];
      if (r.err) return set_error(r.err, "batched CPD: cost is NaN or Inf");
      f[i] = r.f;
      rel[i] = r.rel;
      ao[i] = r.ao;
      acoef[i] = r.acoef;
      afail[i] = r.afail;
      inner[i] = r.inner;
      done_t[i] = t_solve + 1e-9 * (double)(r.done_ns - t0_ns);
    }
    return write_results(frobv, f, rel, ao, acoef, afail, inner, done_t, t_solve);
  }


  // ---- batched MTTKRP plans: per mode, rank class and M-tile height, plus the accelerated
  // last mode.  The M-tile (64 or 128 output rows) is the one that wastes fewer rows. ----
  using PlanKey = std::tuple<int, int, int>;   // (mode, or N for the accelerated point; BN; BM)
  std::map<PlanKey, BatchedContraction> plans;
  struct PlansGuard {
    std::map<PlanKey, BatchedContraction> *m;
    ~PlansGuard() {
      for (auto &kv : *m) kv.second.release();
    }
  } pguard{&plans};
  auto bm_choice = [](int64_t Q) {
    const int64_t w64 = (Q + 63) / 64 * 64 - Q, w128 = (Q + 127) / 128 * 128 - Q;
    return w64 < w128 ? 64 : 128;
  };
  auto build_plans = [&](int target) -> int {
    for (int n = 0; n <= N; ++n) {
      const int mode = n < N ? n : 0;   // the line-search point: mode 0 (the next sweep's first)
      std::map<std::pair<int, int>, std::vector<int>> cls;
      for (int i = 0; i < n_inst; ++i) {
        const Contraction c = mttkrp_contraction(T[i], desc[i].fac, mode);
        cls[{bn_class(desc[i].R), bm_choice(c.Q)}].push_back(i);
      }
      for (auto &kv : cls) {
        std::vector<const ptg_tensor *> ts;
        std::vector<Contraction> cs;
        std::vector<int> ranks, ids;
        std::vector<float *> outs;
        for (int i : kv.second) {
          float *const *f = n < N ? desc[i].fac : desc[i].acc;
          ts.push_back(T[i]);
          cs.push_back(mttkrp_contraction(T[i], f, mode));
          ranks.push_back(desc[i].R);
          outs.push_back(desc[i].M);
          ids.push_back(i);
        }
        PTG_TRY(batched_plan(ctx, ts, cs, ranks, outs, ids, kv.first.first, kv.first.second, target,
                             &plans[PlanKey{n, kv.first.first, kv.first.second}]));
      }
    }
    return PTG_OK;
  };
  auto mttkrp_all = [&](int n, const int *flags) -> int {
    for (auto &kv : plans)
      if (std::get<0>(kv.first) == n) PTG_TRY(batched_launch(ctx, kv.second, flags, S));
    return PTG_OK;
  };
  // autotuner: time the mode-0..N-1 MTTKRP lists for each candidate CTA target, keep the best
  {
    long long shape_sum = 0;
    for (int i = 0; i < n_inst; ++i) {
      shape_sum = shape_sum * 31 + desc[i].R;
      for (int k = 0; k < N; ++k) shape_sum = shape_sum * 131 + desc[i].rows[k];
    }
    const std::string key = "batch:" + std::to_string(n_inst) + ":" + std::to_string(shape_sum);
    int best = ctx->tuned.count(key) ? ctx->tuned[key] : 0;
    if (!best) {
      cudaEvent_t e0, e1;
      PTG_CUDA(cudaEventCreate(&e0));
      PTG_CUDA(cudaEventCreate(&e1));
      float best_ms = 1e30f;
      for (int cand : {2, 4, 8, 16}) {
        PTG_TRY(build_plans(cand));
        for (int n = 0; n < N; ++n) PTG_TRY(mttkrp_all(n, nullptr));   // warm-up
        PTG_CUDA(cudaEventRecord(e0, S));
        for (int n = 0; n < N; ++n) PTG_TRY(mttkrp_all(n, nullptr));
        PTG_CUDA(cudaEventRecord(e1, S));
        PTG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        PTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
          best_ms = ms;
          best = cand;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      ctx->tuned[key] = best;
    }
    PTG_TRY(build_plans(best));
  }
  if (ctx->stats.enabled) {   // one timed pass of the tuned lists (every mode of every instance)
    double bytes = 0.0;
    for (int i = 0; i < n_inst; ++i)
      for (int n = 0; n < N; ++n) {
        bytes += 4.0 * (double)Tst[i].numel_padded;
        for (int k = 0; k < N; ++k) bytes += 4.0 * (double)inst[i].dims[k] * inst[i].rank;
      }
    cudaEvent_t e0, e1;
    PTG_CUDA(cudaEventCreate(&e0));
    PTG_CUDA(cudaEventCreate(&e1));
    const long long l0 = ctx->stats.launches;
    PTG_CUDA(cudaEventRecord(e0, S));
    for (int n = 0; n < N; ++n) PTG_TRY(mttkrp_all(n, nullptr));
    PTG_CUDA(cudaEventRecord(e1, S));
    PTG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    PTG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->stats.batch_pass_launches = ctx->stats.launches - l0;
    ctx->stats.batch_pass_ms = ms;
    ctx->stats.batch_pass_bytes = bytes;
  }

  // ---- initial Grams and cost ----
  PTG_TRY(launch_batched_op(ctx, BatchedOp::Gram, d_desc, n_inst, nullptr, nullptr, S));
  PTG_TRY(mttkrp_all(N - 1, nullptr));
  PTG_TRY(launch_batched_op(ctx, BatchedOp::CostTerms, d_desc, n_inst, nullptr, nullptr, S));
  PTG_CUDA(cudaMemcpyAsync(h_cost, d_cost, sizeof(double) * 2 * n_inst, cudaMemcpyDeviceToHost, S));
  PTG_CUDA(cudaStreamSynchronize(S));
  std::vector<double> frob(n_inst), f(n_inst), rel(n_inst);
  std::vector<int> ao(n_inst, 0), acoef(n_inst, opt.accel_coeff), afail(n_inst, opt.accel_fail);
  std::vector<long long> inner(n_inst, 0);
  std::vector<double> done_t(n_inst, 0.0);
  for (int i = 0; i < n_inst; ++i) {
    frob[i] = T[i]->frob_stored;
    f[i] = std::sqrt(std::max(frob[i] + h_cost[2 * i + 1] - 2.0 * h_cost[2 * i], 0.0));
    rel[i] = f[i] / std::sqrt(frob[i]);
  }

  // ---- the sweep as a CUDA graph: for each mode, eigenbounds, MTTKRP, NNLS ----
  GraphHolder sweep_graph, accel_graph;
  PTG_CUDA(cudaMemcpyAsync(d_flags, h_flags, sizeof(int) * 5 * n_inst, cudaMemcpyHostToDevice, S));
  // kernels inside a graph are counted once per replay, not at capture
  long long cap0 = ctx->stats.launches;
  PTG_CUDA(cudaStreamBeginCapture(S, cudaStreamCaptureModeThreadLocal));
  int cap_rc = PTG_OK;
  for (int n = 0; n < N && cap_rc == PTG_OK; ++n) {
    // fork: eigenvalue bounds on the side stream, MTTKRP on the main one; join before the NNLS
    cudaError_t fe = cudaEventRecord(side.fork, S);
    if (fe == cudaSuccess) fe = cudaStreamWaitEvent(side.s, side.fork, 0);
    if (fe != cudaSuccess) {
      cap_rc = cuda_error(fe, "graph fork", __FILE__, __LINE__);
      break;
    }
    cap_rc = launch_eigen_batched(ctx, d_eig + (size_t)n * n_inst, n_inst, d_active, side.s);
    if (cap_rc == PTG_OK) {
      fe = cudaEventRecord(side.join, side.s);
      if (fe != cudaSuccess) cap_rc = cuda_error(fe, "graph join", __FILE__, __LINE__);
    }
    if (cap_rc == PTG_OK) cap_rc = mttkrp_all(n, n == 0 ? d_m0 : d_active);
    if (cap_rc == PTG_OK) {
      fe = cudaStreamWaitEvent(S, side.join, 0);
      if (fe != cudaSuccess) cap_rc = cuda_error(fe, "graph join", __FILE__, __LINE__);
    }
    if (cap_rc == PTG_OK) {
      nnls_block_kernel<<<n_inst, BN_THREADS, nnls_smem, S>>>(d_nn + (size_t)n * n_inst, d_active);
      count_launches(ctx, 1);
    }
  }
  cudaError_t ce = cudaStreamEndCapture(S, &sweep_graph.g);
  if (cap_rc != PTG_OK) return cap_rc;
  if (ce != cudaSuccess) return cuda_error(ce, "cudaStreamEndCapture(sweep)", __FILE__, __LINE__);
  PTG_CUDA(cudaGraphInstantiate(&sweep_graph.e, sweep_graph.g, 0));
  const long long sweep_kernels = ctx->stats.launches - cap0;
  ctx->stats.launches = cap0;
  // acceleration evaluation: combine, Grams, last-mode MTTKRP, cost terms (for flagged instances)
  cap0 = ctx->stats.launches;
  PTG_CUDA(cudaStreamBeginCapture(S, cudaStreamCaptureModeThreadLocal));
  cap_rc = launch_batched_op(ctx, BatchedOp::AccelCombine, d_desc, n_inst, d_accel, d_step, S);
  if (cap_rc == PTG_OK) cap_rc = launch_batched_op(ctx, BatchedOp::GramAcc, d_desc, n_inst, d_accel, nullptr, S);
  if (cap_rc == PTG_OK) cap_rc = launch_batched_op(ctx, BatchedOp::CopyOld, d_desc, n_inst, d_copy, nullptr, S);
  if (cap_rc == PTG_OK) cap_rc = mttkrp_all(N, d_accel);
  if (cap_rc == PTG_OK) cap_rc = launch_batched_op(ctx, BatchedOp::CostTermsAcc, d_desc, n_inst, d_accel, nullptr, S);
  ce = cudaStreamEndCapture(S, &accel_graph.g);
  if (cap_rc != PTG_OK) return cap_rc;
  if (ce != cudaSuccess) return cuda_error(ce, "cudaStreamEndCapture(accel)", __FILE__, __LINE__);
  PTG_CUDA(cudaGraphInstantiate(&accel_graph.e, accel_graph.g, 0));
  const long long accel_kernels = ctx->stats.launches - cap0;
  ctx->stats.launches = cap0;

  const int last = N - 1;
  int n_active = n_inst;
  const double t_solve = elapsed();   // every tensor resident from here on
  for (int sweep = 1; n_active > 0; ++sweep) {
    for (int i = 0; i < n_inst; ++i) h_flags[4 * n_inst + i] = h_flags[i] && !h_flags[2 * n_inst + i];
    PTG_CUDA(cudaMemcpyAsync(d_flags, h_flags, sizeof(int) * n_inst, cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaMemcpyAsync(d_m0, h_flags + 4 * n_inst, sizeof(int) * n_inst, cudaMemcpyHostToDevice, S));
    PTG_CUDA(cudaGraphLaunch(sweep_graph.e, S));
    count_launches(ctx, (int)sweep_kernels);
    PTG_CUDA(cudaMemcpyAsync(h_scal, d_scal, sizeof(double) * 2 * n_inst * N, cudaMemcpyDeviceToHost, S));
    PTG_CUDA(cudaMemcpyAsync(h_iscal, d_iscal, sizeof(int) * 2 * n_inst * N, cudaMemcpyDeviceToHost, S));
    if (opt.normalization) PTG_TRY(launch_batched_op(ctx, BatchedOp::Normalize, d_desc, n_inst, d_active, nullptr, S));
    PTG_CUDA(cudaStreamSynchronize(S));
    const double now = elapsed();
    // stop test and the acceleration set (include/Cpd.hpp:333-354)
    for (int i = 0; i < n_inst; ++i) {
      int *act = h_flags, *accel = h_flags + n_inst, *copy = h_flags + 3 * n_inst;
      accel[i] = 0;
      copy[i] = 0;
      if (!act[i]) continue;
      ++ao[i];
      const double *sc = h_scal + ((size_t)last * n_inst + i) * 2;
      const double f2 = frob[i] - 2.0 * sc[0] + sc[1];
      if (!std::isfinite(f2)) return set_error(PTG_ERR_NUMERIC, "batched CPD: cost is NaN or Inf");
      f[i] = std::sqrt(std::max(f2, 0.0));
      rel[i] = f[i] / std::sqrt(frob[i]);
      for (int n = 0; n < N; ++n) inner[i] += h_iscal[((size_t)n * n_inst + i) * 2];
      const double thr = inst[i].threshold_error > 0.0 ? inst[i].threshold_error : opt.threshold_error;
      if (rel[i] < thr || ao[i] >= opt.max_iter) {
        act[i] = 0;
        --n_active;
        done_t[i] = now;
        continue;
      }
      if (opt.acceleration) {
        copy[i] = 1;
        if (ao[i] > 1) {
          accel[i] = 1;
          h_step[i] = (float)std::pow((double)(ao[i] + 1), 1.0 / (double)acoef[i]);
        }
      }
    }
    bool any_accel = false, any_copy = false;
    for (int i = 0; i < n_inst; ++i) {
      any_accel |= h_flags[n_inst + i] != 0;
      any_copy |= h_flags[3 * n_inst + i] != 0;
    }
    if (any_accel || any_copy) {
      PTG_CUDA(cudaMemcpyAsync(d_flags, h_flags, sizeof(int) * 4 * n_inst, cudaMemcpyHostToDevice, S));
      PTG_CUDA(cudaMemcpyAsync(d_step, h_step, sizeof(float) * n_inst, cudaMemcpyHostToDevice, S));
      PTG_CUDA(cudaGraphLaunch(accel_graph.e, S));
      count_launches(ctx, (int)accel_kernels);
      PTG_CUDA(cudaMemcpyAsync(h_cost, d_cost, sizeof(double) * 2 * n_inst, cudaMemcpyDeviceToHost, S));
      PTG_CUDA(cudaStreamSynchronize(S));
      for (int i = 0; i < n_inst; ++i) {
        int *accept = h_flags + 2 * n_inst;
        accept[i] = 0;
        if (!h_flags[n_inst + i]) continue;
        const double fa = std::sqrt(std::max(frob[i] + h_cost[2 * i + 1] - 2.0 * h_cost[2 * i], 0.0));
        if (f[i] > fa) {
          accept[i] = 1;
          f[i] = fa;
        } else {
          afail[i]++;
        }
        if (afail[i] == 5) {
          afail[i] = 0;
          acoef[i]++;
        }
      }
      PTG_CUDA(cudaMemcpyAsync(d_accept, h_flags + 2 * n_inst, sizeof(int) * n_inst, cudaMemcpyHostToDevice, S));
      PTG_TRY(launch_batched_op(ctx, BatchedOp::Select, d_desc, n_inst, d_accept, nullptr, S));
    }
  }
  return write_results(frob, f, rel, ao, acoef, afail, inner, done_t, t_solve);
}
