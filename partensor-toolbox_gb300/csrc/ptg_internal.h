// Internal declarations shared by the translation units of libptg.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "ptg.h"

namespace ptg {

// ---------------------------------------------------------------------------------
// Errors: every C entry point returns a ptg_status; the message is kept per thread.
// ---------------------------------------------------------------------------------
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *what, const char *file, int line);

#define PTG_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t _e = (call);                                                    \
    if (_e != cudaSuccess) return ::ptg::cuda_error(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define PTG_TRY(...)                   \
  do {                                 \
    int _s = (__VA_ARGS__);            \
    if (_s != PTG_OK) return _s;       \
  } while (0)

// Device buffer that grows on demand (never shrinks until the context dies).
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  const long long *limit = nullptr;   // the owning context's allocation limit (0: none)
  int ensure(size_t need);
  void release();
};

}  // namespace ptg

struct ptg_ctx_stats {
  bool enabled = false;
  long long launches = 0;
  long long mttkrp_launches = 0;
  double mttkrp_ms = 0.0, mttkrp_bytes = 0.0, mttkrp_flops = 0.0;
  long long tc_launches = 0;
  double tc_ms = 0.0, tc_bytes = 0.0;
  long long batch_pass_launches = 0;
  double batch_pass_ms = 0.0, batch_pass_bytes = 0.0;
  struct Pending {
    cudaEvent_t a, b;
    bool tc;
  };
  std::vector<Pending> pending;   // unresolved event pairs
  std::vector<cudaEvent_t> pool;
};

struct ptg_ctx {
  int device = 0;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  // dynamic shared memory a one-CTA-per-SM contraction kernel may take so that the FP64
  // eigenvalue-bound kernel, launched beside it on a side stream, still fits on its SM
  size_t smem_beside_eigen = 0;
  cudaStream_t stream = nullptr;      // main stream (own or caller's)
  cudaStream_t own_stream = nullptr;
  cudaStream_t side = nullptr;        // concurrent small kernels (FP64 eigenbounds)
  cudaStream_t side2 = nullptr;       // a second one (the line search's speculative bounds)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr, ev_join3 = nullptr;
  ptg::DevBuf scratch;                // split-K partials and other temporaries
  int nnls_cluster = 0;               // cluster size the NNLS kernel launched with (0 = unknown)
  ptg_ctx_stats stats;
  int mttkrp_impl = 0;                // PTG_OPT_MTTKRP_IMPL
  int gtc_rows = 0;                   // PTG_OPT_GTC_ROWS
  int *dev_err = nullptr;             // device error word written by bounded waits
  long long spin_limit = -1;          // PTG_OPT_SPIN_LIMIT (-1: the kernels' default)
  long long alloc_limit = 0;          // PTG_OPT_ALLOC_LIMIT (0: none)
  int host_read = 0;                  // PTG_OPT_HOST_READ
  int batched_impl = 0;               // PTG_OPT_BATCHED_IMPL
  // the device reads pageable host memory through the host's page tables (address translation
  // over NVLink-C2C on Grace; no page migration)
  bool pageable_ats = false;
  void *f8_work = nullptr;            // FP8 MTTKRP: column-maxima work words + column scales
  std::map<std::string, int> tuned;   // autotuner choices (batched CPD split-K target)
  // buffers of the one-call entry points (ptg_cpd, ptg_cpd_dimtree), kept between calls:
  // the stored tensor and its FP32 copy
  ptg::DevBuf cache_x, cache_xr;
  void *pinned = nullptr;             // page-locked host staging, kept between calls
  size_t pinned_bytes = 0;
  // the ALS loop's per-sweep scalars, read back without stalling the stream
  void *pinned_scalars = nullptr;     // kPinnedScalarBytes, page-locked
  cudaEvent_t ev_cost = nullptr;      // a sweep's cost terms have landed in pinned_scalars
  cudaEvent_t ev_sel = nullptr;       // a line-search decision has landed in pinned_scalars
};

struct ptg_tensor {
  int order = 0;
  int64_t dims[PTG_MAX_ORDER] = {0};
  int64_t pdim0 = 0;   // mode-0 extent padded to a multiple of 8 (pads are zero)
  int64_t numel_padded = 0;
  ptg_dtype dtype = PTG_F32;
  void *data = nullptr;
  double frob64 = 0.0;      // ||X||^2 of the FP64 source
  double frob_stored = 0.0; // ||X||^2 of the stored copy
  bool owns = true;         // false: data lives in a context-owned buffer
  int device = 0;
  // FP8 storage: the scale of each index of the last mode (inside the data allocation) and
  // the largest of them
  float *f8_scales = nullptr;
  float f8_scale_max = 1.0f;
};

namespace ptg {

// Sum of nsplit split-K partials p[0], p[step], p[2 step], ... in split order.  Loads go out
// eight at a time so that their latencies overlap; the additions keep the split order, so
// the result does not depend on the batching.
__device__ __forceinline__ float sum_splits(const float *__restrict__ p, int64_t step, int nsplit) {
  float s = 0.0f;
  int sp = 0;
  for (; sp + 8 <= nsplit; sp += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldg(p + (int64_t)(sp + u) * step);
#pragma unroll
    for (int u = 0; u < 8; ++u) s += v[u];
  }
  for (; sp < nsplit; ++sp) s += __ldg(p + (int64_t)sp * step);
  return s;
}

// Description of one MTTKRP-shaped contraction over the tensor viewed as [P, Q, S]:
//   out[q, r] = sum_{p, s} X[p + P*q + P*Q*s] * KRb[p, r] * KRa[s, r]
// KRb is the Khatri-Rao row of the factors of the modes before q (digits of p, fastest
// first); KRa that of the modes after q (digits of s, fastest first).
struct KrSide {
  int n = 0;                            // number of factors
  int64_t ext[PTG_MAX_ORDER] = {0};     // extent of each digit (padded extent for mode 0)
  int64_t valid[PTG_MAX_ORDER] = {0};   // rows that exist (digit >= valid -> KR value 0)
  const float *fac[PTG_MAX_ORDER] = {nullptr};  // row-major [valid][R]
};

struct Contraction {
  int64_t P = 1, Q = 1, S = 1;
  KrSide before, after;
  int64_t q_write = 0;  // rows of `out` written (q < q_write)
  const int *skip = nullptr;   // device word: when nonzero at launch time the kernels do nothing
  // where the index of the tensor's last mode (the FP8 slab) sits: slab = s / slab_div, or
  // q / slab_div when slab_in_q (0: not set)
  int64_t slab_div = 0;
  bool slab_in_q = false;
  // FP32 storage on the CUDA cores even where the TF32 tensor cores are the automatic choice:
  // their accumulation keeps a ~4e-7 relative bias, which a fit's cancellation (f^2 = ||X||^2
  // - 2<M, A> + ...) amplifies by ~1/rel^2; the fit that verify_fp32 reports has none
  bool exact_fp32 = false;
};

// Whether the factor rows of a contraction can be read as float4: R % 4 == 0 and every
// factor 16-byte aligned.
inline bool kr_vec4_ok(const Contraction &c, int R) {
  if (R % 4 != 0) return false;
  for (int i = 0; i < c.before.n; ++i)
    if (reinterpret_cast<uintptr_t>(c.before.fac[i]) % 16 != 0) return false;
  for (int i = 0; i < c.after.n; ++i)
    if (reinterpret_cast<uintptr_t>(c.after.fac[i]) % 16 != 0) return false;
  return true;
}

// Build the contraction of a mode-n MTTKRP of tensor t.
Contraction mttkrp_contraction(const ptg_tensor *t, const float *const *factors, int mode);

constexpr size_t kPinnedScalarBytes = 4096;

// whether contraction_launch runs this tensor's contractions on the tensor cores
bool contraction_uses_tc(const ptg_ctx *ctx, const ptg_tensor *t, int R);
// Launch an MTTKRP-shaped contraction (FP32 or BF16 storage) on `stream`; out is
// row-major [q_write][R].
int contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                       cudaStream_t stream);

// CUDA-core MTTKRP on FP32 storage with a caller-owned split-K scratch block of cap_floats
// floats (ptg_noalloc.cu); needs at least simt_fixed_scratch_floats_needed() floats.
size_t simt_fixed_scratch_floats_needed(const Contraction &c, int R);
int simt_mttkrp_fixed_scratch(const ptg_tensor *t, const Contraction &c, int R, float *out, cudaStream_t stream,
                              int sm_count, float *scratch, size_t cap_floats);

// Warm-start network accessors (ptg_mlp.cu).
const float *mlp_theta(const ptg_mlp *m);
// the weights transposed for the inference fused into the NNLS kernel, refreshed on `s` when
// training or ptg_mlp_set_params changed them
const float *mlp_theta_infer(ptg_mlp *m, cudaStream_t s);
int mlp_din(const ptg_mlp *m);
int mlp_hidden(const ptg_mlp *m);

// Dimension tree (ptg_dimtree.cu): split point, the root children's contractions and sizes,
// and the tree of node tensors with its lazy updates.
int dimtree_split(int order);
Contraction node_contraction(const ptg_tensor *t, const float *const *factors, bool left_node);
int64_t node_rows(const ptg_tensor *t, bool left_node);
class DimTree {
 public:
  struct Node {
    int a, b;          // modes [a, b)
    int parent;
    int child[2];
    int64_t rows;      // prod of the node's mode extents (mode 0 padded)
    float *T;          // [rows][R], resident (null for leaves)
    long long at;      // step at which it was computed (-1: never)
  };
  int build(const ptg_tensor *t);                  // the structure; deep_floats() after it
  size_t deep_floats(int R) const { return deep * (size_t)R; }   // nodes below the root's children
  void bind(float *left, float *right, float *deep_base, int R);
  void new_sweep();                                // every factor changed since the last sweep
  void updated(int mode);                          // factor `mode` changed
  // M_n into out: the stale nodes on the path to the leaf recomputed first
  int mttkrp(ptg_ctx *ctx, const ptg_tensor *X, const float *const *factors, int mode, int R, float *out,
             cudaStream_t s);
  const std::vector<Node> &all() const { return nodes; }

 private:
  bool fresh(const Node &nd) const;
  std::vector<Node> nodes;
  int N = 0;
  size_t deep = 0;
  long long last[PTG_MAX_ORDER] = {0};
  long long step = 0;
};

// tcgen05 (tensor-core) form of contraction_launch; BF16 storage only.
int tc_contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                          cudaStream_t stream);
// FP8 (e4m3, per-slab scales) storage on the tensor cores (tcgen05 kind::f8f6f4), R <= 128.
int f8_contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                          cudaStream_t stream);
// FP8 upload (ptg_fp8.cu): the max |x| of the slabs met by a run of mode-0 fibres, then the
// codes, the slab scales, an optional FP32 copy and the FP64 partial sums of squares.
int f8_slab_max_launch(const double *src, int64_t I0, int64_t fiber0, int64_t nfib, int64_t fps,
                       unsigned long long *slab_bits, int sm_count, cudaStream_t s);
int f8_encode_launch(const double *src, int64_t I0, int64_t pI0, int64_t fiber0, int64_t nfib, int64_t fps,
                     const unsigned long long *slab_bits, uint8_t *dst, float *dst32, float *scales, double *part,
                     int blocks, cudaStream_t s);
// poll limit of the tensor-core kernels' bounded waits under this context
constexpr uint32_t kDefaultSpinLimit = 1u << 26;
uint32_t spin_limit(const ptg_ctx *ctx);
// cudaMalloc under the context's allocation limit (PTG_OPT_ALLOC_LIMIT)
int ctx_malloc(const ptg_ctx *ctx, void **p, size_t bytes, const char *what);
// ||X||^2 in the ALS cost f^2 = ||X||^2 - 2 <M, A> + 1^T (Z .* G) 1: that of the stored copy,
// except on FP8 storage, whose dithered copy is unbiased but carries the rounding noise's
// energy in its own norm: there the FP64 source norm makes f^2 estimate the data's cost
inline double cost_norm(const ptg_tensor *t) {
  return t->dtype == PTG_FP8E4M3 ? t->frob64 : t->frob_stored;
}
// FP32 storage on the tensor cores (tcgen05 kind::tf32, three-term split), R <= 64.
int tc32_contraction_launch(ptg_ctx *ctx, const ptg_tensor *t, const Contraction &c, int R, float *out,
                            cudaStream_t stream);
// Reads and clears the device error word (synchronises the stream first).
int check_device_error(ptg_ctx *ctx);
// the error word's value h, read back by the caller after the stream reached it: resets the
// word and reports h (PTG_OK when 0)
int report_device_error(ptg_ctx *ctx, int h);

// A batch of MTTKRP-shaped contractions (one per instance, same layout class, FP32
// storage) planned once into a device work list of (member, m-tile, K-split) items; all
// members run in one launch, whose last split per output tile sums the partials.  Pointers
// are fixed at planning time, so a launch can be captured in a CUDA graph.
struct BatchedContraction {
  void *mem = nullptr;                 // one allocation: params, items, reduce descriptors, partials
  void *params = nullptr, *items = nullptr, *reduce = nullptr;
  int nitems = 0, nmembers = 0, BN = 0, BM = 128;
  bool mmajor = false;
  void release();
};
int batched_plan(ptg_ctx *ctx, const std::vector<const ptg_tensor *> &ts, const std::vector<Contraction> &cs,
                 const std::vector<int> &ranks, const std::vector<float *> &outs, const std::vector<int> &insts,
                 int bn, int bm, int target_per_sm, BatchedContraction *bc);
// active[inst] == 0 skips that instance's items (nullptr: all run).
int batched_launch(ptg_ctx *ctx, const BatchedContraction &bc, const int *active, cudaStream_t stream);

// ptg_tensor_create with the storage taken from `storage` (a context-owned buffer that
// outlives the tensor) when it is not null; with out32, the same pass over the source also
// writes an FP32 copy (storage from storage32 when not null) beside a BF16 tensor.
int tensor_create_impl(ptg_ctx *c, int order, const int64_t *dims, ptg_dtype dtype, const double *src,
                       int src_on_device, DevBuf *storage, ptg_tensor **out, DevBuf *storage32 = nullptr,
                       ptg_tensor **out32 = nullptr);

// Statistics helpers: count kernel launches; bracket a contraction with events.
inline void count_launches(ptg_ctx *ctx, int n) { ctx->stats.launches += n; }
int stats_begin(ptg_ctx *ctx, cudaStream_t s, cudaEvent_t *ev);
int stats_end(ptg_ctx *ctx, cudaStream_t s, cudaEvent_t ev, double bytes, double flops, bool tc = false);
int stats_resolve(ptg_ctx *ctx);   // fold completed event pairs into the sums

// ----------------------------------------------------------------------------------
// Solver kernels (ptg_solve.cu)
// ----------------------------------------------------------------------------------
constexpr int kMaxInner = 50;  // include/NesterovMNLS.hpp:187

// Device-side scalars of one NNLS solve, written by the FP64 eigen kernel.
struct NnlsParams {
  double Z[64 * 64];   // Hadamard of the Grams (FP64), R x R row-major
  double L, mu, lambda, q;
  float beta[kMaxInner];
  float feat[8];       // scale-free summaries of Z for the warm-start network
  int status;
};

// Warm start of the NNLS rows (ptg_mlp.cu): network parameters and the training log.
struct WarmArgs {
  const float *theta = nullptr;   // MLP parameters (nullptr: no inference)
  int hidden = 0;
  float *log_X = nullptr;         // [rows][R + 8] features  (nullptr: no logging)
  float *log_T = nullptr;         // [rows][R] targets
};

// beside_tc: the launch runs beside a tensor-core MTTKRP and takes its shared-memory carveout
int launch_eigen_bounds(const float *const *grams, int order, int mode, int R, NnlsParams *out,
                        cudaStream_t stream, bool beside_tc = false);
// Nesterov MNLS of one factor on a thread-block cluster; also writes the new Gram
// (FP32 R x R), <M, A_new> and sum(Z .* G_new) in FP64, the iteration count and whether
// the zero-column repair ran.
int launch_nnls_full(ptg_ctx *ctx, const float *M, float *A, int I, int R, const NnlsParams *np,
                     float delta1, float delta2, float *gram_out, double *inner_MA, double *had_ZG,
                     int *iters_out, int *repaired_out, cudaStream_t stream,
                     const WarmArgs &warm = WarmArgs());
size_t gram_scratch_floats(int I, int R);
// beside_tc: the launch runs beside a tensor-core MTTKRP and takes its shared-memory carveout
int launch_gram(const float *A, int I, int R, float *G, float *part, cudaStream_t stream, bool beside_tc = false);
int launch_normalize(float *const *fac, float *const *gram, const int *rows, int order, int weight,
                     int R, cudaStream_t stream);
int launch_accel_combine(const float *const *cur, const float *const *old, float *const *acc,
                         const int *rows, int order, int R, double step, cudaStream_t stream);
// out2[0] = <M, A_last> (FP64), out2[1] = sum(Z_last .* G_last) with Z_last the Hadamard
// of grams[0..order-2].
// update_factor for unconstrained (A = M Z^{-1}, Z in np->Z) and orthogonal (A = M (M^T M)^{-1/2},
// with the Gram of M in FP64) modes; W is an R x R FP64 scratch.  ptg_constraints.cu.
int launch_update_unconstrained(ptg_ctx *ctx, const float *M, float *A, int I, int R, const NnlsParams *np,
                                double *W, cudaStream_t s);
int launch_update_orthogonal(ptg_ctx *ctx, const float *M, float *A, int I, int R, double *W, cudaStream_t s);
// scratch of launch_cost_terms: 2 doubles per CTA and a ticket word that starts at zero (the
// kernel leaves it at zero)
struct CostScratch {
  double *part;       // kCostPartials doubles
  unsigned *ticket;
};
constexpr int kCostPartials = 64;
int launch_cost_terms(const float *M, const float *A_last, int64_t I_last, const float *const *grams,
                      int order, int R, double *out2, CostScratch scratch, cudaStream_t stream);
// static shared memory of the FP64 eigenvalue-bound kernel (one CTA)
size_t eigen_kernel_smem();
// *out = sum over (r1, r2) of prod_k (A_k^T A_k)[r1][r2], the Grams accumulated in FP64 from the
// factors (part: gram_term_fp64_scratch_doubles(order, R) doubles of scratch)
size_t gram_term_fp64_scratch_doubles(int order, int R);
int launch_gram_term_fp64(const float *const *factors, const int *rows, int order, int R, double *part,
                          double *out, cudaStream_t stream);

// Batched many-instance CPD (ptg_batched.cu, ptg_solve.cu).
struct EigDesc {            // eigenbounds of one instance and mode
  const float *gram[PTG_MAX_ORDER];
  int order, mode, R, inst;
  NnlsParams *out;
};
struct InstDesc {           // device buffers of one instance
  float *fac[PTG_MAX_ORDER], *old[PTG_MAX_ORDER], *acc[PTG_MAX_ORDER];
  float *gram[PTG_MAX_ORDER], *gacc[PTG_MAX_ORDER];
  int rows[PTG_MAX_ORDER];
  int order, R, weight, inst;
  float *M;                 // last MTTKRP result of the instance [max rows][R]
  double *cost_out;         // [2]
};
enum class BatchedOp { Gram, GramAcc, Normalize, AccelCombine, CopyOld, Select, CostTerms, CostTermsAcc };
int launch_eigen_batched(ptg_ctx *ctx, const EigDesc *d, int n, const int *active, cudaStream_t s);
int launch_batched_op(ptg_ctx *ctx, BatchedOp op, const InstDesc *d, int n, const int *flag, const float *step,
                      cudaStream_t s);

}  // namespace ptg
