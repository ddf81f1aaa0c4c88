/*
 * Drives include/partensor_gb300.hpp the way a Partensor user calls the reference --
 * TEST INFRASTRUCTURE ONLY (built against tests/cpp/partensor_standin.hpp).
 *
 *   binding_driver cpd|dimtree I0 I1 I2 R tensor.bin init_prefix out_prefix [bf16]
 *       tensor.bin: ColMajor FP64; init_prefix<k>.bin: factor k, ColMajor FP64 I_k x R.
 *       Runs partensor's cpd(execution::cuda, ...) dispatch target
 *       internal::CPD<Tensor<3>, execution::cuda_policy> (or gb300::cpd_dimtree) with
 *       writeToFile set, writes out_prefix<k>.bin (ColMajor) and prints
 *       "rel <rel_costFunction> iters <ao_iter>".
 *   binding_driver gtc|gtc_stochastic I0 I1 I2 R nnz ratings.bin init_prefix
 *       ratings.bin: (N+1) x nnz ColMajor FP64 (Ratings_Base_T); prints "rel ... iters ...".
 */
#include <cstdio>
#include <cstdlib>
#include <string>

#include "partensor_standin.hpp"
#include "partensor_gb300.hpp"

using namespace partensor;

static Matrix load(const std::string &path, long rows, long cols) {
  Matrix m(rows, cols);
  read(path, (std::size_t)(rows * cols), 0, m);
  return m;
}

static void save(const std::string &path, const Matrix &m) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fwrite(m.data(), sizeof(double), (size_t)(m.rows() * m.cols()), f);
  std::fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 9) {
    std::fprintf(stderr, "usage: see the header comment\n");
    return 2;
  }
  const std::string mode = argv[1];
  const long I[3] = {std::atol(argv[2]), std::atol(argv[3]), std::atol(argv[4])};
  const int R = std::atoi(argv[5]);
  try {
    if (mode == "cpd" || mode == "dimtree") {
      Tensor<3> X({I[0], I[1], I[2]});
      read(std::string(argv[6]), X.size(), 0, X);
      std::array<Matrix, 3> init;
      for (int k = 0; k < 3; ++k) init[k] = load(std::string(argv[7]) + std::to_string(k) + ".bin", I[k], R);
      if (argc > 9 && std::string(argv[9]) == "bf16") gb300::storage() = PTG_BF16;
      Options<Tensor<3>, execution::cuda_policy, DefaultValues> o;
      o.max_iter = 15;
      o.writeToFile = true;
      for (int k = 0; k < 3; ++k) o.final_factors_paths[k] = std::string(argv[8]) + "final_" + std::to_string(k) + ".bin";
      Status<Tensor<3>, execution::cuda_policy, DefaultValues> st =
          mode == "cpd" ? internal::CPD<Tensor<3>, execution::cuda_policy>()(X, (std::size_t)R, o, init)
                        : gb300::cpd_dimtree(X, (std::size_t)R, o, init);
      for (int k = 0; k < 3; ++k) save(std::string(argv[8]) + std::to_string(k) + ".bin", st.factors[k]);
      std::printf("rel %.17g iters %u\n", st.rel_costFunction, st.ao_iter);
      // the other overloads of the dispatch target compile too (not run: random factors)
      if (argc > 100) {
        internal::CPD<Tensor<3>, execution::cuda_policy>()(X, (std::size_t)R);
        internal::CPD<Tensor<3>, execution::cuda_policy>()(X, (std::size_t)R, o);
        internal::CPD<Tensor<3>, execution::cuda_policy>()(X, (std::size_t)R, init);
        gb300::cpd_dimtree(X, (std::size_t)R);
        gb300::cpd_dimtree(X, (std::size_t)R, o);
      }
    } else {
      const int nnz = std::atoi(argv[6]);
      SparseOptions<3, execution::cuda_policy, SparseDefaultValues> so;
      so.rank = R;
      so.tnsDims = {(int)I[0], (int)I[1], (int)I[2]};
      so.nonZeros = nnz;
      so.max_iter = 3;
      so.threshold_error = 0.0;
      so.lambdas.fill(1e-3);
      so.c_stochastic_perc = 0.1;
      so.initialized_factors = true;
      for (int k = 0; k < 3; ++k) so.factorsInit[k] = load(std::string(argv[8]) + std::to_string(k) + ".bin", I[k], R);
      so.ratings_path = argv[7];
      SparseStatus<3, execution::cuda_policy, SparseDefaultValues> st =
          mode == "gtc" ? gb300::gtc<3>(so) : gb300::gtc_stochastic<3>(so);
      std::printf("rel %.17g iters %u\n", st.rel_costFunction, st.ao_iter);
    }
  } catch (std::exception const &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
