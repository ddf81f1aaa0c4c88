/*
 * A stand-in for the reference's public types -- TEST INFRASTRUCTURE ONLY.
 *
 * include/partensor_gb300.hpp is written against Partensor's Eigen-typed interface, which
 * cannot be compiled here (no Eigen).  This header declares the same names with the same
 * template parameters and the members the binding touches, over plain ColMajor FP64
 * storage, so the binding can be compiled, linked against libptg.so and run:
 *   partensor::Tensor<N> / Matrix (include/Tensor.hpp:36-101), Constraint
 *   (include/Constants.hpp:49-57), execution::cuda_policy (include/execution.hpp:170,279),
 *   Options / Status / SparseOptions / SparseStatus (include/PARTENSOR_basic.hpp:283-640),
 *   makeFactors (include/DataGeneration.hpp:564-581), read (include/ReadWrite.hpp:293-345),
 *   internal::CPD_Base / CPD (include/Cpd.hpp:52-75).
 */
#ifndef PARTENSOR_STANDIN_HPP
#define PARTENSOR_STANDIN_HPP

#include <array>
#include <cstdint>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

namespace partensor {

enum class Constraint : uint8_t {
  unconstrained = 0, nonnegativity = 1, orthogonality = 2, sparsity = 3, constant = 4,
  symmetric_nonnegativity = 5, symmetric = 6
};

namespace execution {
inline namespace v1 {
struct sequenced_policy {};
struct cuda_policy {};
inline constexpr cuda_policy cuda{};
}  // namespace v1
}  // namespace execution

/* ColMajor FP64 matrix: element (i, j) at data()[i + rows * j]. */
class Matrix {
 public:
  Matrix() = default;
  Matrix(long r, long c) : r_(r), c_(c), v_((size_t)(r * c)) {}
  long rows() const { return r_; }
  long cols() const { return c_; }
  double *data() { return v_.data(); }
  const double *data() const { return v_.data(); }
  double &operator()(long i, long j) { return v_[(size_t)(i + r_ * j)]; }
  double operator()(long i, long j) const { return v_[(size_t)(i + r_ * j)]; }

 private:
  long r_ = 0, c_ = 0;
  std::vector<double> v_;
};

/* ColMajor FP64 N-way tensor (i0 fastest). */
template <int N>
class Tensor {
 public:
  using Dimensions = std::array<long, N>;
  explicit Tensor(Dimensions d) : d_(d) {
    size_t n = 1;
    for (long x : d) n *= (size_t)x;
    v_.resize(n);
  }
  long dimension(int k) const { return d_[k]; }
  const Dimensions &dimensions() const { return d_; }
  double *data() { return v_.data(); }
  const double *data() const { return v_.data(); }
  size_t size() const { return v_.size(); }

 private:
  Dimensions d_;
  std::vector<double> v_;
};

template <typename T>
struct TensorTraits;
template <int N>
struct TensorTraits<Tensor<N>> {
  using DataType = double;
  using MatrixType = Matrix;
  using Dimensions = typename Tensor<N>::Dimensions;
  using Constraints = std::array<Constraint, N>;
  using MatrixArray = std::array<Matrix, N>;
  using DoubleArray = std::array<double, N>;
  static constexpr std::size_t TnsSize = N;
};

template <typename T>
struct DefaultValues {};
template <typename T>
struct SparseDefaultValues {};

template <typename Tensor_, typename ExecutionPolicy_ = execution::sequenced_policy,
          template <typename T> class DefaultValues_ = DefaultValues>
struct Options {
  static constexpr std::size_t TnsSize = TensorTraits<Tensor_>::TnsSize;
  typename TensorTraits<Tensor_>::Constraints constraints;
  double threshold_error = 1e-3;
  double nesterov_delta_1 = 1e-2;
  double nesterov_delta_2 = 1e-2;
  unsigned max_iter = 20;
  int accel_coeff = 3;
  int accel_fail = 0;
  bool acceleration = true;
  bool normalization = true;
  bool writeToFile = false;
  std::array<std::string, TnsSize> final_factors_paths;
  Options() {
    constraints.fill(Constraint::nonnegativity);
    for (std::size_t i = 0; i < TnsSize; ++i) final_factors_paths[i] = "final_" + std::to_string(i) + ".bin";
  }
};

template <typename Tensor_, typename ExecutionPolicy_ = execution::sequenced_policy,
          template <typename T> class DefaultValues_ = DefaultValues>
struct Status {
  Options<Tensor_, ExecutionPolicy_, DefaultValues_> options;
  double frob_tns = 0.0, f_value = 0.0, rel_costFunction = 0.0;
  unsigned ao_iter = 0;
  typename TensorTraits<Tensor_>::MatrixArray factors;
  Status() = default;
  Status(Options<Tensor_, ExecutionPolicy_, DefaultValues_> const &opt) : options(opt) {}
};

template <std::size_t N, typename ExecutionPolicy_ = execution::sequenced_policy,
          template <typename T> class DefaultValues_ = SparseDefaultValues>
struct SparseOptions {
  using MatrixArray = std::array<Matrix, N>;
  int rank = 1;
  std::array<int, N> tnsDims{};
  int nonZeros = 0;
  bool initialized_factors = false;
  MatrixArray factorsInit;
  std::array<Constraint, N> constraints;
  double threshold_error = 1e-3;
  int max_nesterov_iter = 20;
  double c_stochastic_perc = 0.5;
  std::array<double, N> lambdas;
  unsigned max_iter = 20;
  std::string ratings_path;
  SparseOptions() {
    constraints.fill(Constraint::nonnegativity);
    lambdas.fill(0.01);
  }
};

template <std::size_t N, typename ExecutionPolicy_ = execution::sequenced_policy,
          template <typename T> class DefaultValues_ = SparseDefaultValues>
struct SparseStatus {
  SparseOptions<N, ExecutionPolicy_, DefaultValues_> options;
  double frob_tns = 0.0, f_value = 0.0, rel_costFunction = 0.0;
  unsigned ao_iter = 0;
  std::array<Matrix, N> factors;
  SparseStatus() = default;
  SparseStatus(SparseOptions<N, ExecutionPolicy_, DefaultValues_> const &opt) : options(opt) {}
};

/* U[0,1] factors (the stand-in's own generator). */
template <std::size_t N, typename Dimensions, typename FactorType>
void makeFactors(Dimensions const &tnsDims, std::array<Constraint, N> const &, int R,
                 std::array<FactorType, N> &factorArray) {
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (std::size_t k = 0; k < N; ++k) {
    factorArray[k] = FactorType((long)tnsDims[k], R);
    for (long i = 0; i < (long)tnsDims[k] * R; ++i) factorArray[k].data()[i] = u(g);
  }
}

/* `size` FP64 values after `skip` from a raw file, in storage order. */
template <typename Data, typename FileName>
void read(FileName const &fileName, std::size_t size, std::size_t skip, Data &dat) {
  FILE *f = std::fopen(std::string(fileName).c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open " + std::string(fileName));
  std::fseek(f, (long)(skip * sizeof(double)), SEEK_SET);
  const size_t got = std::fread(dat.data(), sizeof(double), size, f);
  std::fclose(f);
  if (got != size) throw std::runtime_error("short read");
}

inline namespace v1 {
namespace internal {
template <typename Tensor_>
struct CPD_Base {
  static constexpr std::size_t TnsSize = TensorTraits<Tensor_>::TnsSize;
  using MatrixType = Matrix;
  using MatrixArray = std::array<Matrix, TnsSize>;
};
template <typename Tensor_, typename ExecutionPolicy = execution::sequenced_policy>
struct CPD : public CPD_Base<Tensor_> {};
}  // namespace internal
}  // namespace v1

}  // namespace partensor

#endif  // PARTENSOR_STANDIN_HPP
