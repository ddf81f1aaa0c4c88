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

namespace ptg {
namespace {

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
__global__ void __launch_bounds__(BN_THREADS) nnls_block_kernel(const BNnls *__restrict__ tab,
                                                                const int *__restrict__ active) {
  const BNnls a = tab[blockIdx.x];
  if (active && !active[a.inst]) return;
  extern __shared__ __align__(16) float sm[];
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
    d_flags = c.take<int>(4 * (size_t)n_inst);
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
  {
    std::vector<float> hf((fac_end - fac_begin) / sizeof(float), 0.0f);
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
  PinnedHost hp;
  const size_t host_bytes = sizeof(int) * 4 * n_inst + sizeof(float) * n_inst + sizeof(double) * (2 * n_inst * N + 2 * n_inst) +
                            sizeof(int) * 2 * n_inst * N + 16;   // + alignment of the FP64 block
  PTG_CUDA(cudaHostAlloc(&hp.p, host_bytes, cudaHostAllocDefault));
  int *h_flags = (int *)hp.p;
  float *h_step = (float *)(h_flags + 4 * n_inst);
  double *h_scal = (double *)(((uintptr_t)(h_step + n_inst) + 7) & ~(uintptr_t)7);
  double *h_cost = h_scal + 2 * n_inst * N;
  int *h_iscal = (int *)(h_cost + 2 * n_inst);
  for (int i = 0; i < 4 * n_inst; ++i) h_flags[i] = 0;
  for (int i = 0; i < n_inst; ++i) h_flags[i] = 1;   // all active

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
      const int mode = n < N ? n : N - 1;
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
  PTG_CUDA(cudaMemcpyAsync(d_flags, h_flags, sizeof(int) * 4 * n_inst, cudaMemcpyHostToDevice, S));
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
    if (cap_rc == PTG_OK) cap_rc = mttkrp_all(n, d_active);
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
    PTG_CUDA(cudaMemcpyAsync(d_flags, h_flags, sizeof(int) * n_inst, cudaMemcpyHostToDevice, S));
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
  // ---- results: one copy of every factor, FP32 row-major -> host FP64 ColMajor ----
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
}
