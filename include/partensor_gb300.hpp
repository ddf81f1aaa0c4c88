/*
 * partensor_gb300.hpp -- Partensor's cpd / cpdDimTree / gtc / gtc_stochastic on libptg.
 *
 * The reference-side binding of the C ABI in ptg.h.  It is included by the reference in
 * place of include/CUDA/CpdCUDA.hpp (the USE_CUDA include of include/Cpd.hpp:867-870),
 * after the reference's own headers, and it uses only their public types:
 * partensor::Tensor<N> and partensor::Matrix (ColMajor FP64 Eigen storage,
 * include/Tensor.hpp:36-101), Options / Status / SparseOptions / SparseStatus
 * (include/PARTENSOR_basic.hpp:283-640), makeFactors (include/DataGeneration.hpp:564-581)
 * and read (include/ReadWrite.hpp:293-345).  Link with -lptg.
 *
 *  - internal::CPD<Tensor_, execution::cuda_policy> replaces the specialisation of
 *    include/CUDA/CpdCUDA.hpp:44, so cpd(execution::cuda, ...) (include/Cpd.hpp:893-1171)
 *    runs on the GPU with every overload of the reference (rank only, options,
 *    factorsInit, both).
 *  - gb300::cpd_dimtree, gb300::gtc and gb300::gtc_stochastic are the cuda branches that
 *    the reference's policy dispatchers lack (include/CpdDimTree.hpp:813-830,
 *    include/Gtc.hpp:658-671,713-734, include/GtcStochastic.hpp:640-742): each dispatcher
 *    gets one more `else if constexpr (std::is_same_v<ExPolicy, execution::cuda_policy>)`
 *    that returns the matching call below.
 * Errors: every ptg call that fails throws std::runtime_error(ptg_last_error()), as the
 * reference's data generation does (include/DataGeneration.hpp:98,124).
 */
#ifndef PARTENSOR_GB300_HPP
#define PARTENSOR_GB300_HPP

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ptg.h"

namespace partensor {
namespace gb300 {

/* One libptg context per host thread (device 0), created on first use. */
inline ptg_ctx *context() {
  thread_local ptg_ctx *ctx = nullptr;
  if (!ctx && ptg_ctx_create(0, &ctx) != PTG_OK) throw std::runtime_error(ptg_last_error());
  return ctx;
}

inline void check(int rc) {
  if (rc != PTG_OK) throw std::runtime_error(ptg_last_error());
}

/* Storage type of the dense tensor in HBM for the calls below (PTG_F32 is the reference's
 * arithmetic; PTG_BF16 and PTG_FP8E4M3 are the faster forms, with verify_fp32). */
inline ptg_dtype &storage() {
  thread_local ptg_dtype d = PTG_F32;
  return d;
}

/* partensor::Options -> ptg_cpd_options.  `paths` keeps the C strings alive. */
template <typename Options_>
ptg_cpd_options cpd_options(Options_ const &opt, std::size_t N, std::vector<std::string> &paths) {
  ptg_cpd_options o;
  ptg_cpd_default_options((int)N, &o);
  for (std::size_t k = 0; k < N; ++k) o.constraints[k] = (int)opt.constraints[k];
  o.threshold_error = opt.threshold_error;
  o.nesterov_delta_1 = opt.nesterov_delta_1;
  o.nesterov_delta_2 = opt.nesterov_delta_2;
  o.max_iter = (int)opt.max_iter;
  o.accel_coeff = opt.accel_coeff;
  o.accel_fail = opt.accel_fail;
  o.acceleration = opt.acceleration ? 1 : 0;
  o.normalization = opt.normalization ? 1 : 0;
  o.write_to_file = opt.writeToFile ? 1 : 0;
  paths.assign(opt.final_factors_paths.begin(), opt.final_factors_paths.end());
  for (std::size_t k = 0; k < N && k < PTG_MAX_ORDER; ++k) o.final_factors_paths[k] = paths[k].c_str();
  o.verify_fp32 = storage() != PTG_F32 ? 1 : 0;
  return o;
}

/* The dense solve shared by cpd and cpdDimTree: ColMajor FP64 tensor and factors in,
 * partensor::Status out (factors updated in place from factorsInit). */
template <typename Status_, typename Options_, typename Tensor_, typename MatrixArray_>
Status_ solve(Tensor_ const &tnsX, std::size_t R, Options_ const &opt, MatrixArray_ const &init, bool dimtree) {
  constexpr std::size_t N = std::tuple_size<MatrixArray_>::value;
  Status_ st(opt);
  std::vector<std::string> paths;
  ptg_cpd_options o = cpd_options(opt, N, paths);
  int64_t dims[N];
  const double *in[N];
  double *out[N];
  for (std::size_t k = 0; k < N; ++k) {
    dims[k] = (int64_t)tnsX.dimension((int)k);
    st.factors[k] = init[k];                      // I_k x R ColMajor, updated in place
    in[k] = st.factors[k].data();
    out[k] = st.factors[k].data();
  }
  ptg_cpd_result r;
  const auto fn = dimtree ? ptg_cpd_dimtree : ptg_cpd;
  check(fn(context(), (int)N, dims, tnsX.data(), storage(), (int)R, &o, in, out, &r, nullptr));
  st.frob_tns = r.frob_tns;
  st.f_value = r.f_value;
  st.rel_costFunction = r.rel_costFunction;
  st.ao_iter = (unsigned)r.ao_iter;
  st.options.accel_coeff = r.accel_coeff;
  st.options.accel_fail = r.accel_fail;
  return st;
}

/* Random initial factors as the reference draws them (include/DataGeneration.hpp:564-581). */
template <typename MatrixArray_, typename Tensor_, typename Options_>
MatrixArray_ random_factors(Tensor_ const &tnsX, std::size_t R, Options_ const &opt) {
  MatrixArray_ f;
  makeFactors(tnsX.dimensions(), opt.constraints, (int)R, f);
  return f;
}

}  // namespace gb300

inline namespace v1 {
namespace internal {

template <typename Tensor_>
struct CPD<Tensor_, execution::cuda_policy> : public CPD_Base<Tensor_> {
  using typename CPD_Base<Tensor_>::MatrixArray;
  using Options = partensor::Options<Tensor_, execution::cuda_policy, DefaultValues>;
  using Status = partensor::Status<Tensor_, execution::cuda_policy, DefaultValues>;

  Status operator()(Tensor_ const &tnsX, std::size_t const R) {
    Options o;
    return gb300::solve<Status>(tnsX, R, o, gb300::random_factors<MatrixArray>(tnsX, R, o), false);
  }
  Status operator()(Tensor_ const &tnsX, std::size_t const R, Options const &o) {
    return gb300::solve<Status>(tnsX, R, o, gb300::random_factors<MatrixArray>(tnsX, R, o), false);
  }
  Status operator()(Tensor_ const &tnsX, std::size_t const R, MatrixArray const &factorsInit) {
    Options o;
    return gb300::solve<Status>(tnsX, R, o, factorsInit, false);
  }
  Status operator()(Tensor_ const &tnsX, std::size_t const R, Options const &o, MatrixArray const &factorsInit) {
    return gb300::solve<Status>(tnsX, R, o, factorsInit, false);
  }
};

}  // namespace internal
}  // namespace v1

namespace gb300 {

/* cpdDimTree(execution::cuda, tnsX, R[, options][, factorsInit]). */
template <typename Tensor_>
Status<Tensor_, execution::cuda_policy, DefaultValues> cpd_dimtree(Tensor_ const &tnsX, std::size_t R) {
  using S = Status<Tensor_, execution::cuda_policy, DefaultValues>;
  Options<Tensor_, execution::cuda_policy, DefaultValues> o;
  return solve<S>(tnsX, R, o, random_factors<typename TensorTraits<Tensor_>::MatrixArray>(tnsX, R, o), true);
}
template <typename Tensor_>
Status<Tensor_, execution::cuda_policy, DefaultValues> cpd_dimtree(
    Tensor_ const &tnsX, std::size_t R, Options<Tensor_, execution::cuda_policy, DefaultValues> const &o) {
  using S = Status<Tensor_, execution::cuda_policy, DefaultValues>;
  return solve<S>(tnsX, R, o, random_factors<typename TensorTraits<Tensor_>::MatrixArray>(tnsX, R, o), true);
}
template <typename Tensor_>
Status<Tensor_, execution::cuda_policy, DefaultValues> cpd_dimtree(
    Tensor_ const &tnsX, std::size_t R, Options<Tensor_, execution::cuda_policy, DefaultValues> const &o,
    typename TensorTraits<Tensor_>::MatrixArray const &factorsInit) {
  using S = Status<Tensor_, execution::cuda_policy, DefaultValues>;
  return solve<S>(tnsX, R, o, factorsInit, true);
}

/* gtc / gtc_stochastic with the cuda policy.  The reference's input is Ratings_Base_T, an
 * (N+1) x nnz ColMajor FP64 matrix: rows 0..N-1 the 0-based indices of each observed entry
 * (stored as doubles), row N its value (include/Gtc.hpp:655-757).  It becomes int32 indices
 * idx[k * nnz + e] and FP32 values; the initial factors are options.factorsInit when
 * options.initialized_factors is set, else U[0,1] draws of makeFactors. */
template <std::size_t N, typename SparseStatus_, typename SparseOptions_>
SparseStatus_ gtc_impl(Matrix const &Ratings_Base_T, SparseOptions_ const &opt, bool stochastic) {
  SparseStatus_ st(opt);
  const int64_t nnz = (int64_t)Ratings_Base_T.cols();
  if ((std::size_t)Ratings_Base_T.rows() != N + 1)
    throw std::runtime_error("gtc: Ratings_Base_T must have N + 1 rows");
  std::vector<int32_t> idx((size_t)(N * nnz));
  std::vector<float> vals((size_t)nnz);
  const double *rb = Ratings_Base_T.data();
  for (int64_t e = 0; e < nnz; ++e) {
    for (std::size_t k = 0; k < N; ++k) idx[k * nnz + e] = (int32_t)rb[k + (N + 1) * e];
    vals[e] = (float)rb[N + (N + 1) * e];
  }
  ptg_gtc_options o;
  ptg_gtc_default_options((int)N, &o);
  for (std::size_t k = 0; k < N; ++k) {
    o.constraints[k] = (int)opt.constraints[k];
    o.lambdas[k] = opt.lambdas[k];
  }
  o.threshold_error = opt.threshold_error;
  o.max_nesterov_iter = opt.max_nesterov_iter;
  o.max_iter = (int)opt.max_iter;
  o.c_stochastic_perc = opt.c_stochastic_perc;
  o.stochastic = stochastic ? 1 : 0;
  int64_t dims[N];
  const double *in[N];
  double *out[N];
  for (std::size_t k = 0; k < N; ++k) dims[k] = opt.tnsDims[k];
  if (opt.initialized_factors) {
    st.factors = opt.factorsInit;
  } else {
    std::array<Constraint, N> c;
    for (std::size_t k = 0; k < N; ++k) c[k] = opt.constraints[k];
    makeFactors(opt.tnsDims, c, opt.rank, st.factors);
  }
  for (std::size_t k = 0; k < N; ++k) {
    in[k] = st.factors[k].data();
    out[k] = st.factors[k].data();
  }
  ptg_gtc_result r;
  check(ptg_gtc(context(), (int)N, dims, nnz, idx.data(), vals.data(), 0, opt.rank, &o, in, out, &r, nullptr));
  st.frob_tns = r.frob_tns;
  st.f_value = r.f_value;
  st.rel_costFunction = r.rel_costFunction;
  st.ao_iter = (unsigned)r.ao_iter;
  return st;
}

template <std::size_t N>
SparseStatus<N, execution::cuda_policy, SparseDefaultValues> gtc(
    Matrix const &Ratings_Base_T, SparseOptions<N, execution::cuda_policy, SparseDefaultValues> const &options) {
  return gtc_impl<N, SparseStatus<N, execution::cuda_policy, SparseDefaultValues>>(Ratings_Base_T, options, false);
}
template <std::size_t N>
SparseStatus<N, execution::cuda_policy, SparseDefaultValues> gtc_stochastic(
    Matrix const &Ratings_Base_T, SparseOptions<N, execution::cuda_policy, SparseDefaultValues> const &options) {
  return gtc_impl<N, SparseStatus<N, execution::cuda_policy, SparseDefaultValues>>(Ratings_Base_T, options, true);
}

/* The file forms: options.ratings_path holds (N+1) x nonZeros FP64 values, read as the
 * reference reads it (include/Gtc.hpp:533-544). */
template <std::size_t N>
Matrix read_ratings(SparseOptions<N, execution::cuda_policy, SparseDefaultValues> const &options) {
  Matrix rb((int)(N + 1), options.nonZeros);
  read(options.ratings_path, (std::size_t)((N + 1) * (std::size_t)options.nonZeros), 0, rb);
  return rb;
}
template <std::size_t N>
SparseStatus<N, execution::cuda_policy, SparseDefaultValues> gtc(
    SparseOptions<N, execution::cuda_policy, SparseDefaultValues> const &options) {
  return gtc<N>(read_ratings<N>(options), options);
}
template <std::size_t N>
SparseStatus<N, execution::cuda_policy, SparseDefaultValues> gtc_stochastic(
    SparseOptions<N, execution::cuda_policy, SparseDefaultValues> const &options) {
  return gtc_stochastic<N>(read_ratings<N>(options), options);
}

}  // namespace gb300
}  // namespace partensor

#endif  // PARTENSOR_GB300_HPP
