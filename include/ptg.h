/*
 * ptg.h -- C ABI of the GB300-native CPD-ALS path (libptg.so).
 *
 * The reference (Partensor) exposes this path only through header-only C++ templates;
 * its one extern "C" symbol is cuda_vecAdd (include/CUDA/add_vectors.cu:16-24).  The
 * entry points below are what a binding for those templates needs: plain pointers,
 * sizes and POD structs, no C++ or torch types.  Every function returns a ptg_status
 * code; ptg_last_error() gives the message of the last failure on the calling thread.
 *
 * Data conventions (those of the reference):
 *   - a dense tensor is ColMajor, i0 fastest (include/Tensor.hpp:64, Eigen::Tensor);
 *   - a host factor matrix is I_k x R ColMajor FP64 (Eigen::MatrixXd, include/Tensor.hpp:42);
 *   - device factor matrices used by the lower-level entry points are ROW-major FP32
 *     [I_k][R] (element (i, r) at i*R + r), the layout the kernels read.
 * Paths in the citations are relative to the reference project's root.
 */
#ifndef PTG_H
#define PTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTG_MAX_ORDER 8

typedef enum {
  PTG_OK = 0,
  PTG_ERR_INVALID = 1,     /* bad argument */
  PTG_ERR_CUDA = 2,        /* a CUDA runtime/driver call failed */
  PTG_ERR_OOM = 3,         /* device allocation failed */
  PTG_ERR_UNSUPPORTED = 4, /* shape/rank outside what the kernels handle */
  PTG_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  PTG_ERR_NUMERIC = 6      /* NaN/Inf detected in an input or a result */
} ptg_status;

/* Storage of a dense tensor in HBM.  PTG_FP8E4M3: one byte per entry, the e4m3 code of
 * x / scale_s, where s is the entry's index in the last mode (its slab) and scale_s = 2^k the
 * smallest power of two with max_slab |x| <= 448 * 2^k; rounding is stochastic (up with
 * probability equal to the distance from the lower e4m3 neighbour, from a hash of the
 * entry's position), so the stored copy is unbiased.  The ALS cost on FP8 storage uses the
 * FP64 source norm, which makes it an unbiased estimate of the cost on the data. */
typedef enum { PTG_F32 = 0, PTG_BF16 = 1, PTG_FP8E4M3 = 2 } ptg_dtype;

/* Constraint values of include/Constants.hpp:49-57. */
typedef enum {
  PTG_UNCONSTRAINED = 0,
  PTG_NONNEGATIVITY = 1,
  PTG_ORTHOGONALITY = 2,
  PTG_SPARSITY = 3,
  PTG_CONSTANT = 4
} ptg_constraint;

typedef struct ptg_ctx ptg_ctx;
typedef struct ptg_tensor ptg_tensor;
typedef struct ptg_mlp ptg_mlp;

/* Text of the last error raised on this thread ("" if none). */
const char *ptg_last_error(void);

/* Library version string. */
const char *ptg_version(void);

/* One context per device and caller thread: owns streams, events and workspace.
 * Replaces the per-call cublasCreate/cudaStreamCreate/cudaMallocManaged set-up of
 * include/CUDA/CpdCUDA.hpp:282-300. */
int ptg_ctx_create(int device, ptg_ctx **out);
int ptg_ctx_destroy(ptg_ctx *ctx);
/* Run all work of this context on a caller-provided cudaStream_t (NULL: own stream). */
int ptg_ctx_set_stream(ptg_ctx *ctx, void *cuda_stream);
/* Waits for the context's stream; also reports a device-side error (PTG_ERR_TIMEOUT from a
 * bounded wait inside a kernel) raised since the last check, and clears it. */
int ptg_ctx_synchronize(ptg_ctx *ctx);

/* Context options (GB300 knobs, no reference counterpart). */
typedef enum {
  PTG_OPT_MTTKRP_IMPL = 1 /* 0: auto (tensor cores for BF16, FP8 and, at R <= 64, FP32 storage),
                             1: CUDA cores (BF16, FP32), 2: tensor cores (BF16: kind::f16; FP32,
                             R <= 64: kind::tf32 with a three-term split, each accumulator
                             drained into FP32 registers every 64 terms: -4e-7 relative bias at
                             10^6-term contractions) */,
  PTG_OPT_NNLS_CLUSTER = 2 /* CTAs of the NNLS thread-block cluster: 0 auto (16 where the device
                             schedules it, else 8), or 2, 4, 8, 16 */,
  PTG_OPT_GTC_ROWS = 3 /* sparse row solver of the nonnegative GTC modes: 0 auto (one warp per
                          row for rank <= 32, the row Hessian on the tensor cores when rank % 4
                          == 0 (TF32, three-term split); else one CTA per row), 1 one CTA per
                          row, 2 one warp per row with the Hessian on the FMA pipe (the same
                          bits as 1) */,
  PTG_OPT_SPIN_LIMIT = 4 /* polls of every bounded wait in the tensor-core MTTKRP kernels before
                            they give up with PTG_ERR_TIMEOUT: -1 the default (2^26), 0 give up
                            at once, before any copy or MMA is issued (a test of the failure
                            path) */,
  PTG_OPT_ALLOC_LIMIT = 5 /* largest single device allocation (bytes) this context may make; a
                             larger request fails with PTG_ERR_OOM as cudaMalloc would and
                             leaves the context usable (0: no limit) */,
  PTG_OPT_HOST_READ = 6 /* how a host FP64 source reaches the conversion kernels: 0 auto (the
                           BF16/FP32 conversion reads page-locked or registered memory in place;
                           everything else is staged), 1 always staged through 64 MB device
                           chunks by copies, 2 in place wherever the device can address the
                           buffer (also pageable memory where the device walks the host's page
                           tables, as over NVLink-C2C).  All store the same bits. */,
  PTG_OPT_BATCHED_IMPL = 7 /* ptg_cpd_batched: 0 the persistent solver (one launch for the whole
                              batch: each CTA takes instances from an atomic queue, largest
                              first, and runs each one's ALS loop to its stop test), 1 one launch
                              per ALS phase for all instances, each sweep a replayed CUDA graph.
                              Both run the same per-instance arithmetic. */
} ptg_option;
int ptg_ctx_set_option(ptg_ctx *ctx, int option, long long value);

/* Kernel statistics of a context (no counterpart in the reference, which only has a
 * host stopwatch, include/Timers.hpp:39-142).  When enabled, every MTTKRP launch is
 * bracketed by CUDA events on the stream it runs on. */
typedef struct {
  long long launches;         /* all kernels this context launched */
  long long mttkrp_launches;  /* MTTKRP contractions (main kernel + split-K reduction) */
  double mttkrp_ms;           /* summed event time of those contractions */
  double mttkrp_bytes;        /* algorithmic bytes: tensor + factors read, result written */
  double mttkrp_flops;        /* 2 * prod(I) * R per contraction */
  long long tc_launches;      /* the subset that ran on the tensor cores (tcgen05) */
  double tc_ms;
  double tc_bytes;
  /* ptg_cpd_batched: one MTTKRP pass (every mode of every instance, the tuned work lists)
   * timed with CUDA events right after tuning, and its algorithmic bytes */
  long long batch_pass_launches;
  double batch_pass_ms;
  double batch_pass_bytes;
} ptg_stats;
int ptg_ctx_enable_stats(ptg_ctx *ctx, int enable);
int ptg_ctx_get_stats(ptg_ctx *ctx, ptg_stats *out); /* synchronises the context's stream */
int ptg_ctx_reset_stats(ptg_ctx *ctx);

/* Dense tensor resident in HBM in the requested storage type.  src is an FP64 ColMajor
 * buffer with prod(dims) entries, on the host (src_on_device = 0) or on the device.
 * Replaces the host Matricization copies of include/CUDA/CpdCUDA.hpp:302-306: the
 * tensor is stored once, in its natural order, with mode 0 padded to a multiple of 8
 * entries (16 for FP8 storage; pads are zero).  ||X||^2 (include/TensorOperations.hpp:144-149) is computed in FP64
 * from the FP64 source during the upload. */
int ptg_tensor_create(ptg_ctx *ctx, int order, const int64_t *dims, ptg_dtype dtype,
                      const double *src, int src_on_device, ptg_tensor **out);
int ptg_tensor_destroy(ptg_tensor *t);
/* frob64: ||X||^2 of the FP64 source; frob_stored: ||X||^2 of the stored (rounded) copy. */
int ptg_tensor_norms(const ptg_tensor *t, double *frob64, double *frob_stored);
/* The stored copy, for inspection (no counterpart in the reference, which keeps the FP64
 * tensor itself): device address of the entries (ColMajor, mode 0 padded to *padded_dim0),
 * and for FP8 storage the device address of the slab scales (one float per index of the
 * last mode; NULL for the other types).  Any output pointer may be NULL. */
int ptg_tensor_storage(const ptg_tensor *t, const void **data, int64_t *padded_dim0, const float **slab_scales);

/* Mode-n MTTKRP, M = X_(n) * KhatriRao_{k != n}(A_k).  Replaces mttkrp
 * (include/MTTKRP.hpp:60-69, 102-225) and hybrid_batched_mttkrp
 * (include/CUDA/CUDAMTTKRP.hpp:67-200).  factors[k]: device, row-major FP32 [I_k][R]
 * (factors[mode] is not read).  out: device, row-major FP32 [I_mode][R].
 * Asynchronous on the context's stream. */
int ptg_mttkrp(ptg_ctx *ctx, const ptg_tensor *X, const float *const *factors, int rank, int mode,
               float *out);

/* MTTKRP that allocates no device memory.  This entry point has no counterpart in the
 * reference.  It is for callers that may not call cudaMalloc when they need the product:
 * applications whose allocator owns all of HBM, code that must not synchronise the device
 * (cudaMalloc and cudaFree can), latency-bound loops.  It computes what ptg_mttkrp computes,
 * on CUDA cores, from caller-owned buffers only, with its split-K partials in a fixed 8 MiB
 * block of device memory that the library image carries (held on every GPU that loads the
 * library until the process exits).
 *   X        device FP32 tensor, ColMajor with mode-0 stride ld0: element (i0, i1, ...) at
 *            i0 + ld0*(i1 + I1*(i2 + ...)); ld0 >= dims[0], ld0 % 8 == 0, X 16-byte aligned;
 *            the ld0 - dims[0] padding entries of each fibre must be finite (zeros are best)
 *   factors  device row-major FP32 [I_k][rank] (factors[mode] is not read)
 *   out      device row-major FP32 [I_mode][rank]
 *   stream   cudaStream_t (NULL: the legacy default stream)
 * Limit: I_mode x R_pad <= 2,097,152 floats (ld0 for mode 0; R_pad = rank rounded up to 16,
 * 32, 64 or 128); larger calls return PTG_ERR_UNSUPPORTED.  The first call on a device looks
 * up the block's address on that device: make it before any stream capture.  Calls share the
 * block, so two calls that overlap on the GPU race; the block keeps the last call's data and
 * nothing in it needs clearing.  X, out, the factors and the stream must belong to the
 * current device (X and out are checked: PTG_ERR_INVALID); the looked-up address is kept
 * for the process, so the entry point must not be used across a cudaDeviceReset. */
int ptg_mttkrp_noalloc(const float *X, int order, const int64_t *dims, int64_t ld0,
                       const float *const *factors, int rank, int mode, float *out, void *stream);

/* Options of one CPD-ALS run: the fields of partensor::Options
 * (include/PARTENSOR_basic.hpp:283-336) that the ALS loop reads, plus GB300 knobs. */
typedef struct {
  int constraints[PTG_MAX_ORDER];
  double threshold_error;
  double nesterov_delta_1;
  double nesterov_delta_2;
  int max_iter;
  int accel_coeff;
  int accel_fail;
  int acceleration;
  int normalization;
  /* GB300 extensions (Gb300Options): */
  int refine_sweeps; /* FP32 sweeps run on `refine` after the main loop stops (0: none) */
  int warm_start;    /* 1: learned warm start of the NNLS rows with warm_model */
  int cost_every_sweep; /* reserved, must be 1 */
  ptg_mlp *warm_model;  /* the network (ptg_mlp_create); shared across runs and instances */
  int warm_log_sweeps;  /* sweeps 1..n log (features, solution) pairs, then the network is
                           trained warm_train_steps Adam steps and used from sweep n+1;
                           0: use the network as it is from sweep 1 */
  int warm_train_steps;
  int verify_fp32;      /* 1: after a main loop on BF16 or FP8 storage with no refinement
                           sweeps, the reported cost is that of the final factors on an FP32
                           copy of the tensor (one more MTTKRP); ptg_cpd_als needs `refine`,
                           ptg_cpd and ptg_cpd_dimtree make the copy from the same upload */
  /* partensor::Options::writeToFile / final_factors_paths (include/PARTENSOR_basic.hpp:
   * 326-333, include/Cpd.hpp:112-122,340-342): when write_to_file is 1, the final factors
   * are written when the loop stops, factor k as I_k x R FP64 in row-major order (the
   * reference writes the transpose of the ColMajor matrix, include/ReadWrite.hpp:100-130)
   * to final_factors_paths[k], or to "final_<k>.bin" where that entry is NULL.  A file
   * that cannot be written makes the call return PTG_ERR_INVALID after the factors have
   * been returned (the reference prints to stderr and continues). */
  int write_to_file;
  const char *final_factors_paths[PTG_MAX_ORDER];
} ptg_cpd_options;

/* Fill *o with the reference defaults (include/PARTENSOR_basic.hpp:176-218). */
void ptg_cpd_default_options(int order, ptg_cpd_options *o);

/* Scalars of partensor::Status (include/PARTENSOR_basic.hpp:556-595) plus timing. */
typedef struct {
  double frob_tns;
  double f_value;
  double rel_costFunction;
  int ao_iter;
  int accel_coeff;
  int accel_fail;
  int refine_sweeps_done;
  long long nesterov_iters_total;
  double seconds_total;
} ptg_cpd_result;

/* Per-sweep trace record (optional output). */
typedef struct {
  double f_value;          /* cost after the sweep, before acceleration */
  double rel_costFunction;
  double f_accel;          /* cost of the accelerated point (0 when not tried) */
  int accel_accepted;
  int nesterov_iters[PTG_MAX_ORDER];
  float seconds;           /* wall time since the start of the run */
} ptg_sweep_trace;

/* CPD-ALS on a resident tensor: the loop of include/Cpd.hpp:288-356 /
 * include/CUDA/CpdCUDA.hpp:277-383 with all per-iteration work on the GPU.
 *   X       the tensor the main loop uses (FP32 or BF16 storage);
 *   refine  optional FP32 copy for the refinement sweeps (may be NULL);
 *   init_factors[k]: host FP64 ColMajor I_k x R (the factorsInit overloads,
 *           include/Cpd.hpp:534-577);
 *   out_factors[k]:  host FP64 ColMajor I_k x R (may alias init_factors);
 *   trace (optional) holds max_iter + refine_sweeps records. */
int ptg_cpd_als(ptg_ctx *ctx, const ptg_tensor *X, const ptg_tensor *refine, int rank,
                const ptg_cpd_options *opts, const double *const *init_factors,
                double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace);

/* One-call form with a HOST FP64 tensor: upload (with conversion to `dtype`), solve,
 * download.  This is what partensor::cpd(execution::cuda, tnsX, R, options, factorsInit)
 * (include/Cpd.hpp:1116-1144) binds to.  The host data streams through page-locked chunks
 * (the copy of one chunk beside the conversion of the previous one) into the stored
 * tensor(s), which stay allocated in the context for the next call of the same or a smaller
 * size (ptg_ctx_destroy frees them). */
int ptg_cpd(ptg_ctx *ctx, int order, const int64_t *dims, const double *host_tensor,
            ptg_dtype dtype, int rank, const ptg_cpd_options *opts,
            const double *const *init_factors, double *const *out_factors,
            ptg_cpd_result *result, ptg_sweep_trace *trace);

/* Dimension-tree CPD-ALS: partensor::cpdDimTree (include/CpdDimTree.hpp:809-1362, loop
 * :317-401).  The modes are split at h = (1 + N)/2 (include/DimTrees.hpp:274-276); the two
 * node tensors T_left [prod_{k<h} I_k x R] and T_right [prod_{k>=h} I_k x R] stay resident in
 * HBM, so a sweep reads the tensor twice instead of N times.  Same arguments as
 * ptg_cpd_als / ptg_cpd. */
int ptg_cpd_dimtree_als(ptg_ctx *ctx, const ptg_tensor *X, const ptg_tensor *refine, int rank,
                        const ptg_cpd_options *opts, const double *const *init_factors,
                        double *const *out_factors, ptg_cpd_result *result, ptg_sweep_trace *trace);
int ptg_cpd_dimtree(ptg_ctx *ctx, int order, const int64_t *dims, const double *host_tensor,
                    ptg_dtype dtype, int rank, const ptg_cpd_options *opts,
                    const double *const *init_factors, double *const *out_factors,
                    ptg_cpd_result *result, ptg_sweep_trace *trace);

/* ---- File-based entry points ---------------------------------------------------------
 * The reference's raw files (include/ReadWrite.hpp:100-130, 293-345): a tensor file holds
 * prod(dims) FP64 values in ColMajor order after `skip` values; a factor file holds an I x R
 * FP64 matrix in row-major order (the reference writes the transpose of the ColMajor
 * MatrixXd).  The tensor is streamed through page-locked memory into HBM and converted there.
 * ptg_tensor_create_file replaces read(path, size, skip, tnsX) + the upload;
 * ptg_cpd_file / ptg_cpd_dimtree_file replace cpd(tnsDims, R, path[, options]) and
 * cpd(tnsDims, R, paths[, options]) (include/Cpd.hpp:591-850) and the cpdDimTree overloads:
 * factor_paths = NULL draws the initial factors U[0,1] from `seed` (the reference's
 * makeFactors draws them from the clock). */
int ptg_tensor_create_file(ptg_ctx *ctx, int order, const int64_t *dims, ptg_dtype dtype, const char *path,
                           int64_t skip, ptg_tensor **out);
int ptg_cpd_file(ptg_ctx *ctx, int order, const int64_t *dims, const char *tensor_path, int64_t skip,
                 const char *const *factor_paths, unsigned long long seed, ptg_dtype dtype, int rank,
                 const ptg_cpd_options *opts, double *const *out_factors, ptg_cpd_result *result,
                 ptg_sweep_trace *trace);
int ptg_cpd_dimtree_file(ptg_ctx *ctx, int order, const int64_t *dims, const char *tensor_path, int64_t skip,
                         const char *const *factor_paths, unsigned long long seed, ptg_dtype dtype, int rank,
                         const ptg_cpd_options *opts, double *const *out_factors, ptg_cpd_result *result,
                         ptg_sweep_trace *trace);

/* ---- Many small CPDs in one call ------------------------------------------------------
 * Solves n independent nonnegative CPD-ALS problems of the same order (ranks and dims may
 * differ per instance) with the semantics of ptg_cpd on an FP32 tensor, each instance
 * stopping on its own test.  The reference has no batched entry point: a caller loops over
 * partensor::cpd(tnsX, R, options, factorsInit) (include/Cpd.hpp:534-577), one problem at a
 * time; this call replaces that loop.  By default one persistent launch solves the whole
 * batch (PTG_OPT_BATCHED_IMPL).  Limits: order in [3, 8], every
 * mode PTG_NONNEGATIVITY, rank <= 32, dims <= 4096, and 3 * rows * rank FP32 values of each
 * factor within one CTA's shared memory.  results[i].seconds_total is the wall time from the
 * call's start until instance i's stop test passed; converge_seconds (optional, n entries)
 * the same time counted from the start of the ALS loop, once every tensor is resident. */
typedef struct ptg_cpd_instance {
  int order;
  int64_t dims[PTG_MAX_ORDER];
  const double *tensor;                 /* host FP64, ColMajor (mode 0 fastest) */
  int rank;
  const double *const *init_factors;    /* host FP64 ColMajor I_k x R */
  double *const *out_factors;           /* host FP64 ColMajor I_k x R */
  double threshold_error;               /* this instance's stop target (<= 0: opts->threshold_error) */
} ptg_cpd_instance;
int ptg_cpd_batched(ptg_ctx *ctx, int n, const ptg_cpd_instance *instances, const ptg_cpd_options *opts,
                    ptg_cpd_result *results, double *converge_seconds);

/* ---- Learned warm start (no counterpart in the reference) ------------------------------
 * A two-hidden-layer ReLU network (128 units) maps the features of an NNLS row -- the
 * MTTKRP row divided by its norm and eight scale-free summaries of the Hadamard-of-Grams
 * (Din = R + 8) -- to the solution row scaled by L / ||m_i|| (R outputs).  The Nesterov
 * solver starts from max(output * ||m_i|| / L, 0) and runs to the reference's own stopping
 * rule (include/NesterovMNLS.hpp:217-218).  Training and inference run in libptg's kernels. */
int ptg_mlp_create(ptg_ctx *ctx, int rank, unsigned long long seed, ptg_mlp **out);
int ptg_mlp_destroy(ptg_mlp *m);
long long ptg_mlp_num_params(const ptg_mlp *m);
int ptg_mlp_get_params(ptg_ctx *ctx, const ptg_mlp *m, float *host_out);
int ptg_mlp_set_params(ptg_ctx *ctx, ptg_mlp *m, const float *host_in);
/* Y[rows][R] = network(X[rows][R + 8]); device buffers. */
int ptg_mlp_forward(ptg_ctx *ctx, const ptg_mlp *m, const float *X_dev, long long rows, float *Y_dev);
/* loss = sum 0.5 ||y - t||^2 / (rows * R) over the data set and its gradient (device, laid out
 * W1 [H][Din], b1, W2 [H][H], b2, W3 [R][H], b3); rows <= 65536. */
int ptg_mlp_loss_grad(ptg_ctx *ctx, const ptg_mlp *m, const float *X_dev, const float *T_dev, int rows,
                      double *loss, float *grad_dev);
/* `steps` minibatch Adam steps (lr, betas 0.9/0.999) on device data X [rows][R+8], T [rows][R]. */
int ptg_mlp_train(ptg_ctx *ctx, ptg_mlp *m, const float *X_dev, const float *T_dev, long long rows, int steps,
                  int batch, float lr, unsigned long long seed, double *final_loss);

/* ---- Sparse tensor completion (GTC) ---------------------------------------------------
 * partensor::gtc / gtc_stochastic (include/Gtc.hpp:655-757, include/GtcStochastic.hpp:640-742)
 * with nonnegativity on every mode.  The reference takes an (N+1) x nnz FP64 matrix
 * Ratings_Base_T (indices stored as doubles, then the value); this ABI takes the same data
 * as int32 indices idx[k * nnz + e] (mode k of entry e) and FP32 values. */
typedef struct {
  int constraints[PTG_MAX_ORDER];   /* PTG_NONNEGATIVITY on every mode */
  double threshold_error;           /* stop when f / ||x||^2 < threshold (include/Gtc.hpp:449) */
  int max_nesterov_iter;            /* 20 (include/PARTENSOR_basic.hpp:234) */
  int max_iter;                     /* outer iterations (full) or epochs (stochastic) */
  double c_stochastic_perc;         /* sampled fraction per row and inner step */
  double lambdas[PTG_MAX_ORDER];    /* Tikhonov weights, default 0.01 */
  int stochastic;                   /* 0: aogtc (include/Gtc.hpp:430-490); 1: aogtc_stochastic */
  unsigned long long seed;          /* seed of the counter-based pivot sampler */
} ptg_gtc_options;

void ptg_gtc_default_options(int order, ptg_gtc_options *o);

typedef struct {
  double frob_tns;          /* sum of squared observed values */
  double f_value;           /* sum of squared residuals over the observed entries */
  double rel_costFunction;  /* f_value / frob_tns (not square-rooted, include/Gtc.hpp:449) */
  int ao_iter;
  int epochs;
  double seconds_setup;     /* sorting and layout */
  double seconds_total;
} ptg_gtc_result;

/* idx/vals on the host (src_on_device = 0) or the device; init/out factors host FP64
 * ColMajor I_k x R; trace (optional) receives one record per cost evaluation (max_iter). */
int ptg_gtc(ptg_ctx *ctx, int order, const int64_t *dims, int64_t nnz, const int32_t *idx, const float *vals,
            int src_on_device, int rank, const ptg_gtc_options *opts, const double *const *init_factors,
            double *const *out_factors, ptg_gtc_result *result, ptg_sweep_trace *trace);

/* The mode-n order of the entries (SortRows, include/TensorOperations.hpp:622-666): perm[s]
 * is the input position of the s-th entry of the mode-n matricisation.  idx and perm on the
 * device. */
int ptg_gtc_sort_mode(ptg_ctx *ctx, int order, const int64_t *dims, int64_t nnz, const int32_t *idx_dev,
                      int mode, uint32_t *perm_out_dev);

#ifdef __cplusplus
}
#endif
#endif /* PTG_H */
