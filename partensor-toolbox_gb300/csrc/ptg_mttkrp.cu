// Dense MTTKRP on CUDA cores (FP32 math; FP32 or BF16 tensor storage).
//
// Replaces the reference's MTTKRP family: the sequential X_(n) * PartialKhatriRao
// (include/MTTKRP.hpp:60-69), the blocked OpenMP version (include/MTTKRP.hpp:102-225)
// and the cuBLAS-DGEMM-per-block hybrid (include/CUDA/CUDAMTTKRP.hpp:67-200).
//
// The tensor is read once, in its natural ColMajor order, viewed as [P, Q, S] with
// Q the mode being solved.  No matricisation and no Khatri-Rao matrix are materialised:
// each CTA forms the BK x R Khatri-Rao tile of its K-slice in shared memory from factor
// rows.  The contraction is split over K across CTAs; every split writes its partial
// Q x R block to scratch and a second kernel sums the splits in a fixed order, so the
// result is bit-identical from run to run.
#include <algorithm>
#include <cstdio>

#include "ptg_internal.h"
#include "ptg_simt.cuh"

namespace ptg {

namespace {

template <typename T, int BN, bool MMAJOR>
__global__ void __launch_bounds__(kThreads) mttkrp_simt_kernel(const SimtParams prm) {
  if (prm.skip && *prm.skip) return;
  extern __shared__ __align__(16) float smem_dyn[];
  mttkrp_simt_body<T, BN, MMAJOR>(prm, blockIdx.x, blockIdx.y, smem_dyn, threadIdx.x);
}

// out[q, col0 + c] = sum over splits of partial[split][q][c], in split order.
__global__ void splitk_reduce_kernel(const float *__restrict__ partial, int nsplit, int64_t Q,
                                     int BN, int64_t q_write, int R, int col0, int ldo,
                                     float *__restrict__ out, const int *skip) {
  if (skip && *skip) return;
  const int64_t n = q_write * BN;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = idx / BN;
    const int c = (int)(idx % BN);
    if (col0 + c >= R) continue;
    out[q * ldo + col0 + c] = sum_splits(partial + q * BN + c, Q * BN, nsplit);
  }
}

template <typename T, int BN>
int launch_cfg(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, int col0,
               float *out, cudaStream_t stream) {
  using Cf = Cfg<BN>;
  const bool mmajor = (c.P == 1);
  SimtParams prm{};
  prm.skip = c.skip;
  prm.X = t->data;
  prm.P = c.P;
  prm.Q = c.Q;
  prm.S = c.S;
  prm.before = to_dev(c.before);
  prm.after = to_dev(c.after);
  prm.R = R;
  prm.col0 = col0;
  prm.out = out;
  prm.q_write = c.q_write;
  prm.ldo = R;
  if (mmajor) {
    prm.pblocks = 1;
    prm.ktiles_total = (c.S + BK - 1) / BK;
  } else {
    prm.pblocks = (c.P + BK - 1) / BK;
    prm.ktiles_total = c.S * prm.pblocks;
  }
  const int64_t mtiles = (c.Q + Cf::BM - 1) / Cf::BM;
  const int64_t target = (int64_t)ctx->sm_count * 4;
  int64_t nsplit = std::max<int64_t>(1, (target + mtiles - 1) / mtiles);
  nsplit = std::min<int64_t>(nsplit, prm.ktiles_total);
  nsplit = std::max<int64_t>(nsplit, 1);
  prm.ktiles_per_split = (prm.ktiles_total + nsplit - 1) / nsplit;
  nsplit = (prm.ktiles_total + prm.ktiles_per_split - 1) / prm.ktiles_per_split;
  prm.nsplit = (int)nsplit;
  if (nsplit > 1) {
    PTG_TRY(ctx->scratch.ensure((size_t)nsplit * c.Q * BN * sizeof(float)));
    prm.partial = reinterpret_cast<float *>(ctx->scratch.ptr);
  }
  dim3 grid((unsigned)mtiles, (unsigned)nsplit);
  const size_t smem = simt_smem_bytes<BN>(mmajor);
  if (mmajor) {
    PTG_CUDA(cudaFuncSetAttribute(mttkrp_simt_kernel<T, BN, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mttkrp_simt_kernel<T, BN, true><<<grid, kThreads, smem, stream>>>(prm);
  } else {
    PTG_CUDA(cudaFuncSetAttribute(mttkrp_simt_kernel<T, BN, false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mttkrp_simt_kernel<T, BN, false><<<grid, kThreads, smem, stream>>>(prm);
  }
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, nsplit > 1 ? 2 : 1);
  if (nsplit > 1) {
    const int64_t n = c.q_write * BN;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
    splitk_reduce_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(
        prm.partial, (int)nsplit, c.Q, BN, c.q_write, R, col0, R, out, c.skip);
    PTG_CUDA(cudaGetLastError());
  }
  return PTG_OK;
}

template <typename T>
int launch_typed(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                 cudaStream_t stream) {
  if (R <= 16) return launch_cfg<T, 16>(ctx, t, c, R, 0, out, stream);
  if (R <= 32) return launch_cfg<T, 32>(ctx, t, c, R, 0, out, stream);
  if (R <= 64) return launch_cfg<T, 64>(ctx, t, c, R, 0, out, stream);
  // wider ranks: 128-column chunks (each chunk re-reads the tensor)
  for (int c0 = 0; c0 < R; c0 += 128) PTG_TRY(launch_cfg<T, 128>(ctx, t, c, R, c0, out, stream));
  return PTG_OK;
}

}  // namespace

namespace {

// Launch planning for a caller-owned scratch block of cap_floats floats: the same kernels as
// launch_cfg, with the K-split count capped so the partials fit, and the partials always
// used (even with one split) so the block is the only device memory touched besides the
// inputs and the output.
template <int BN>
int launch_cfg_fixed(const ptg_tensor *t, const Contraction &c, int R, int col0, float *out,
                     cudaStream_t stream, int sm_count, float *scratch, size_t cap_floats) {
  using Cf = Cfg<BN>;
  const bool mmajor = (c.P == 1);
  SimtParams prm{};
  prm.skip = c.skip;
  prm.X = t->data;
  prm.P = c.P;
  prm.Q = c.Q;
  prm.S = c.S;
  prm.before = to_dev(c.before);
  prm.after = to_dev(c.after);
  prm.R = R;
  prm.col0 = col0;
  prm.out = out;
  prm.q_write = c.q_write;
  prm.ldo = R;
  if (mmajor) {
    prm.pblocks = 1;
    prm.ktiles_total = (c.S + BK - 1) / BK;
  } else {
    prm.pblocks = (c.P + BK - 1) / BK;
    prm.ktiles_total = c.S * prm.pblocks;
  }
  const int64_t slab = c.Q * BN;   // floats of one split's partial block
  const int64_t cap_splits = (int64_t)(cap_floats / (size_t)slab);
  if (cap_splits < 1) return set_error(PTG_ERR_UNSUPPORTED, "internal: scratch block too small");
  const int64_t mtiles = (c.Q + Cf::BM - 1) / Cf::BM;
  const int64_t target = (int64_t)sm_count * 4;
  int64_t nsplit = std::max<int64_t>(1, (target + mtiles - 1) / mtiles);
  nsplit = std::min<int64_t>(nsplit, cap_splits);
  nsplit = std::min<int64_t>(nsplit, prm.ktiles_total);
  nsplit = std::max<int64_t>(nsplit, 1);
  prm.ktiles_per_split = (prm.ktiles_total + nsplit - 1) / nsplit;
  nsplit = (prm.ktiles_total + prm.ktiles_per_split - 1) / prm.ktiles_per_split;
  // nsplit >= 2 makes the kernel write partials; a single split is forced through them too
  prm.nsplit = (int)std::max<int64_t>(nsplit, 2);
  prm.partial = scratch;
  dim3 grid((unsigned)mtiles, (unsigned)nsplit);
  const size_t smem = simt_smem_bytes<BN>(mmajor);
  if (mmajor) {
    PTG_CUDA(cudaFuncSetAttribute(mttkrp_simt_kernel<float, BN, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mttkrp_simt_kernel<float, BN, true><<<grid, kThreads, smem, stream>>>(prm);
  } else {
    PTG_CUDA(cudaFuncSetAttribute(mttkrp_simt_kernel<float, BN, false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    mttkrp_simt_kernel<float, BN, false><<<grid, kThreads, smem, stream>>>(prm);
  }
  PTG_CUDA(cudaGetLastError());
  const int64_t n = c.q_write * BN;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count * 8);
  splitk_reduce_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(scratch, (int)nsplit, c.Q, BN, c.q_write, R,
                                                                col0, R, out, c.skip);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

}  // namespace

size_t simt_fixed_scratch_floats_needed(const Contraction &c, int R) {
  const int bn = R <= 16 ? 16 : R <= 32 ? 32 : R <= 64 ? 64 : 128;
  return (size_t)c.Q * bn;
}

int simt_mttkrp_fixed_scratch(const ptg_tensor *t, const Contraction &c, int R, float *out, cudaStream_t stream,
                              int sm_count, float *scratch, size_t cap_floats) {
  if (t->dtype != PTG_F32) return set_error(PTG_ERR_UNSUPPORTED, "internal: FP32 storage expected");
  if (c.P > 0xffffffffLL || c.S > 0xffffffffLL)
    return set_error(PTG_ERR_UNSUPPORTED, "contraction extent exceeds 2^32");
  if (R <= 16) return launch_cfg_fixed<16>(t, c, R, 0, out, stream, sm_count, scratch, cap_floats);
  if (R <= 32) return launch_cfg_fixed<32>(t, c, R, 0, out, stream, sm_count, scratch, cap_floats);
  if (R <= 64) return launch_cfg_fixed<64>(t, c, R, 0, out, stream, sm_count, scratch, cap_floats);
  for (int c0 = 0; c0 < R; c0 += 128)
    PTG_TRY(launch_cfg_fixed<128>(t, c, R, c0, out, stream, sm_count, scratch, cap_floats));
  return PTG_OK;
}

namespace {

struct ReduceDesc {
  const float *partial;   // [nsplit][Q][BN]
  float *out;             // row-major [q_write][R]
  unsigned *tickets;      // one per m-tile, zero between launches
  int64_t Q, q_write;
  int nsplit, BN, R, inst;
};

// Work-list MTTKRP: item = (member, m-tile, K-split, instance).  Every split writes its
// partial tile; the last split of an m-tile to finish (ticket) sums the partials in split
// order (deterministic) into the member's output and re-arms the ticket.
template <int BN, bool MMAJOR, int BMV>
__global__ void __launch_bounds__(kThreads)
mttkrp_simt_batched_kernel(const SimtParams *__restrict__ prms, const int4 *__restrict__ items,
                           const ReduceDesc *__restrict__ red, const int *__restrict__ active) {
  const int4 it = items[blockIdx.x];   // (member, m-tile, split, instance)
  if (active && !active[it.w]) return;
  extern __shared__ __align__(16) float smem_dyn[];
  mttkrp_simt_body<float, BN, MMAJOR, BMV>(prms[it.x], it.y, it.z, smem_dyn, threadIdx.x);
  __shared__ bool last;
  const ReduceDesc &r = red[it.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&r.tickets[it.y], 1u) == (unsigned)(r.nsplit - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int64_t q0 = (int64_t)it.y * BMV;
  const int64_t q1 = min(q0 + (int64_t)BMV, r.q_write);
  const int R = r.R;
  for (int64_t idx = threadIdx.x; idx < (q1 - q0) * R; idx += kThreads) {
    const int64_t q = q0 + idx / R;
    const int c = (int)(idx % R);
    float s = 0.0f;
    for (int sp = 0; sp < r.nsplit; ++sp) s += __ldcg(&r.partial[((int64_t)sp * r.Q + q) * BN + c]);
    r.out[q * R + c] = s;
  }
  if (threadIdx.x == 0) r.tickets[it.y] = 0u;
}

template <int BN>
int batched_plan_bn(ptg_ctx *ctx, const std::vector<const ptg_tensor *> &ts, const std::vector<Contraction> &cs,
                    const std::vector<int> &ranks, const std::vector<float *> &outs, const std::vector<int> &insts,
                    int bm, int target_per_sm, BatchedContraction *bc) {
  const size_t m = cs.size();
  std::vector<SimtParams> prms(m);
  std::vector<int4> items;
  std::vector<ReduceDesc> red(m);
  std::vector<size_t> part_off(m), tick_off(m);
  size_t part_total = 0, tick_total = 0;
  // total work, to size every member's split count in proportion to its share
  double work_total = 0.0;
  for (size_t i = 0; i < m; ++i) work_total += (double)cs[i].P * cs[i].Q * cs[i].S;
  const double target_ctas = (double)ctx->sm_count * target_per_sm;
  bool mmajor = false;
  for (size_t i = 0; i < m; ++i) {
    const Contraction &c = cs[i];
    mmajor = (c.P == 1);
    SimtParams &prm = prms[i];
    prm = SimtParams{};
    prm.X = ts[i]->data;
    prm.P = c.P;
    prm.Q = c.Q;
    prm.S = c.S;
    prm.before = to_dev(c.before);
    prm.after = to_dev(c.after);
    prm.R = ranks[i];
    prm.col0 = 0;
    prm.out = outs[i];
    prm.q_write = c.q_write;
    prm.ldo = ranks[i];
    if (mmajor) {
      prm.pblocks = 1;
      prm.ktiles_total = (c.S + BK - 1) / BK;
    } else {
      prm.pblocks = (c.P + BK - 1) / BK;
      prm.ktiles_total = c.S * prm.pblocks;
    }
    const int64_t mtiles = (c.Q + bm - 1) / bm;
    const double share = ((double)c.P * c.Q * c.S) / work_total * target_ctas;
    int64_t nsplit = std::max<int64_t>(1, (int64_t)(share / (double)mtiles + 0.5));
    nsplit = std::min<int64_t>(nsplit, prm.ktiles_total);
    prm.ktiles_per_split = (prm.ktiles_total + nsplit - 1) / nsplit;
    nsplit = (prm.ktiles_total + prm.ktiles_per_split - 1) / prm.ktiles_per_split;
    prm.nsplit = (int)std::max<int64_t>(nsplit, 2);   // always through the partials
    part_off[i] = part_total;
    part_total += (size_t)nsplit * c.Q * BN;
    tick_off[i] = tick_total;
    tick_total += (size_t)mtiles;
    for (int64_t mt = 0; mt < mtiles; ++mt)
      for (int64_t sp = 0; sp < nsplit; ++sp) items.push_back(make_int4((int)i, (int)mt, (int)sp, insts[i]));
    red[i] = ReduceDesc{nullptr, outs[i], nullptr, c.Q, c.q_write, (int)nsplit, BN, ranks[i], insts[i]};
  }
  bc->release();
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t a1 = up(sizeof(SimtParams) * m), a2 = up(sizeof(int4) * items.size()),
               a3 = up(sizeof(ReduceDesc) * m), a4 = up(sizeof(unsigned) * tick_total);
  cudaError_t e = cudaMalloc(&bc->mem, a1 + a2 + a3 + a4 + sizeof(float) * part_total + 256);
  if (e != cudaSuccess) {
    bc->mem = nullptr;
    return cuda_error(e, "cudaMalloc(batched plan)", __FILE__, __LINE__);
  }
  char *b = (char *)bc->mem;
  SimtParams *d_prm = (SimtParams *)b;
  int4 *d_items = (int4 *)(b + a1);
  ReduceDesc *d_red = (ReduceDesc *)(b + a1 + a2);
  unsigned *d_tick = (unsigned *)(b + a1 + a2 + a3);
  float *d_part = (float *)(b + a1 + a2 + a3 + a4);
  for (size_t i = 0; i < m; ++i) {
    prms[i].partial = d_part + part_off[i];
    red[i].partial = d_part + part_off[i];
    red[i].tickets = d_tick + tick_off[i];
  }
  PTG_CUDA(cudaMemcpy(d_prm, prms.data(), sizeof(SimtParams) * m, cudaMemcpyHostToDevice));
  PTG_CUDA(cudaMemcpy(d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
  PTG_CUDA(cudaMemcpy(d_red, red.data(), sizeof(ReduceDesc) * m, cudaMemcpyHostToDevice));
  PTG_CUDA(cudaMemset(d_tick, 0, sizeof(unsigned) * std::max<size_t>(tick_total, 1)));
  bc->params = d_prm;
  bc->items = d_items;
  bc->reduce = d_red;
  bc->nitems = (int)items.size();
  bc->nmembers = (int)m;
  bc->BN = BN;
  bc->BM = bm;
  bc->mmajor = mmajor;
  return PTG_OK;
}

}  // namespace

void BatchedContraction::release() {
  if (mem) cudaFree(mem);
  mem = params = items = reduce = nullptr;
  nitems = nmembers = 0;
}

int batched_plan(ptg_ctx *ctx, const std::vector<const ptg_tensor *> &ts, const std::vector<Contraction> &cs,
                 const std::vector<int> &ranks, const std::vector<float *> &outs, const std::vector<int> &insts,
                 int bn, int bm, int target_per_sm, BatchedContraction *bc) {
  if (cs.empty()) return PTG_OK;
  for (const ptg_tensor *t : ts)
    if (t->dtype != PTG_F32) return set_error(PTG_ERR_UNSUPPORTED, "batched MTTKRP: FP32 storage only");
  const bool mm = cs[0].P == 1;
  for (const Contraction &c : cs)
    if ((c.P == 1) != mm) return set_error(PTG_ERR_INVALID, "internal: mixed layouts in one batch");
  if (bm != 64 && bm != 128) return set_error(PTG_ERR_INVALID, "internal: batched M-tile must be 64 or 128");
  if (bn == 16) return batched_plan_bn<16>(ctx, ts, cs, ranks, outs, insts, bm, target_per_sm, bc);
  if (bn == 32) return batched_plan_bn<32>(ctx, ts, cs, ranks, outs, insts, bm, target_per_sm, bc);
  if (bn == 64) return batched_plan_bn<64>(ctx, ts, cs, ranks, outs, insts, bm, target_per_sm, bc);
  return set_error(PTG_ERR_UNSUPPORTED, "batched MTTKRP: rank > 64");
}

template <int BNV, bool MM, int BMV>
static int batched_launch_t(const BatchedContraction &bc, const int *active, cudaStream_t stream) {
  auto kern = mttkrp_simt_batched_kernel<BNV, MM, BMV>;
  const size_t smem = simt_smem_bytes<BNV>(MM, BMV);
  PTG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<bc.nitems, kThreads, smem, stream>>>((const SimtParams *)bc.params, (const int4 *)bc.items,
                                              (const ReduceDesc *)bc.reduce, active);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

template <int BNV>
static int batched_launch_bn(const BatchedContraction &bc, const int *active, cudaStream_t stream) {
  if (bc.mmajor) return bc.BM == 64 ? batched_launch_t<BNV, true, 64>(bc, active, stream)
                                    : batched_launch_t<BNV, true, 128>(bc, active, stream);
  return bc.BM == 64 ? batched_launch_t<BNV, false, 64>(bc, active, stream)
                     : batched_launch_t<BNV, false, 128>(bc, active, stream);
}

int batched_launch(ptg_ctx *ctx, const BatchedContraction &bc, const int *active, cudaStream_t stream) {
  if (!bc.nitems) return PTG_OK;
  if (bc.BN == 16) PTG_TRY(batched_launch_bn<16>(bc, active, stream));
  else if (bc.BN == 32) PTG_TRY(batched_launch_bn<32>(bc, active, stream));
  else PTG_TRY(batched_launch_bn<64>(bc, active, stream));
  count_launches(ctx, 1);
  return PTG_OK;
}

Contraction mttkrp_contraction(const ptg_tensor *t, const float *const *factors, int mode) {
  Contraction c;
  const int N = t->order;
  auto ext = [&](int k) { return k == 0 ? t->pdim0 : t->dims[k]; };
  for (int k = 0; k < mode; ++k) {
    c.P *= ext(k);
    c.before.ext[c.before.n] = ext(k);
    c.before.valid[c.before.n] = t->dims[k];
    c.before.fac[c.before.n] = factors[k];
    c.before.n++;
  }
  c.Q = ext(mode);
  for (int k = mode + 1; k < N; ++k) {
    c.S *= ext(k);
    c.after.ext[c.after.n] = ext(k);
    c.after.valid[c.after.n] = t->dims[k];
    c.after.fac[c.after.n] = factors[k];
    c.after.n++;
  }
  c.q_write = t->dims[mode];
  // the last mode's index: the slowest digit of s, or q itself for the last mode
  c.slab_div = 1;
  c.slab_in_q = (mode == N - 1);
  if (!c.slab_in_q)
    for (int k = mode + 1; k < N - 1; ++k) c.slab_div *= ext(k);
  return c;
}

// Algorithmic bytes of one contraction: the tensor entries (unpadded) in their storage
// type, every factor row the Khatri-Rao tiles read, the FP32 result.
static double contraction_bytes(const ptg_tensor *t, const Contraction &c, int R) {
  double numel = 1.0;
  for (int k = 0; k < t->order; ++k) numel *= (double)t->dims[k];
  const double esz = t->dtype == PTG_F32 ? 4.0 : t->dtype == PTG_BF16 ? 2.0 : 1.0;
  double fac = t->dtype == PTG_FP8E4M3 ? (double)t->dims[t->order - 1] * 4.0 : 0.0;   // slab scales
  for (int i = 0; i < c.before.n; ++i) fac += (double)c.before.valid[i] * R * 4.0;
  for (int i = 0; i < c.after.n; ++i) fac += (double)c.after.valid[i] * R * 4.0;
  return numel * esz + fac + (double)c.q_write * R * 4.0;
}

// FP32 storage reaches the tensor cores through the three-term TF32 split (R <= 64); its TMEM
// accumulators are drained into FP32 registers every two K-blocks, which keeps the drift of
// the tensor cores' accumulation (~2^-25 of the running sum per step) below 5e-7 relative.
bool contraction_uses_tc(const ptg_ctx *ctx, const ptg_tensor *t, int R) {
  return t->dtype == PTG_FP8E4M3 || (t->dtype == PTG_BF16 && ctx->mttkrp_impl != 1 && R <= 128) ||
         (t->dtype == PTG_F32 && R <= 64 && ctx->mttkrp_impl != 1);
}

int contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                       cudaStream_t stream) {
  if (R < 1) return set_error(PTG_ERR_INVALID, "rank must be >= 1");
  if (c.P > 0xffffffffLL || c.S > 0xffffffffLL)
    return set_error(PTG_ERR_UNSUPPORTED, "contraction extent exceeds 2^32");
  if (c.P > 1 && (c.P % 8) != 0)
    return set_error(PTG_ERR_INVALID, "internal: P must be a multiple of 8");
  // A launch that a device word may cancel (Contraction::skip) stays out of the MTTKRP
  // statistics: the host cannot tell whether it did the work its bytes stand for.
  const bool timed = c.skip == nullptr;
  cudaEvent_t ev = nullptr;
  if (timed) PTG_TRY(stats_begin(ctx, stream, &ev));
  int rc;
  const bool tc = contraction_uses_tc(ctx, t, R) && !(c.exact_fp32 && t->dtype == PTG_F32);
  if (t->dtype == PTG_FP8E4M3)
    rc = f8_contraction_launch(ctx, t, c, R, out, stream);
  else if (t->dtype == PTG_F32 && tc)
    rc = tc32_contraction_launch(ctx, t, c, R, out, stream);
  else if (t->dtype == PTG_F32)
    rc = launch_typed<float>(ctx, t, c, R, out, stream);
  else if (tc)
    rc = tc_contraction_launch(ctx, t, c, R, out, stream);
  else if (t->dtype == PTG_BF16)
    rc = launch_typed<__nv_bfloat16>(ctx, t, c, R, out, stream);
  else
    return set_error(PTG_ERR_UNSUPPORTED, "tensor dtype");
  if (rc != PTG_OK) return rc;
  if (!timed) return PTG_OK;
  double numel = 1.0;
  for (int k = 0; k < t->order; ++k) numel *= (double)t->dims[k];
  return stats_end(ctx, stream, ev, contraction_bytes(t, c, R), 2.0 * numel * R, tc);
}

}  // namespace ptg
