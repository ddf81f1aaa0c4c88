// Factor updates for the constraints other than nonnegativity (include/Cpd.hpp:189-228):
//   unconstrained   A = M Z^{-1}                        (:196-199)
//   orthogonality   A = M (M^T M)^{-1/2}, (M^T M)^{-1/2} = V diag(lambda^{-1/2}) V^T  (:210-217),
//                   with M^T M accumulated in FP64
//   sparsity, constant: the factor is kept (:219-222).
// The R x R algebra runs in FP64 in one CTA (R <= 64): Gauss-Jordan elimination with partial
// pivoting for Z^{-1} (the reference calls Eigen's inverse(), an LU with partial pivoting),
// and the cyclic Jacobi method with a round-robin ordering of disjoint rotations (Jacobi
// 1846; Golub & Van Loan, Matrix Computations, sec. 8.5; Brent & Luk 1985 for the parallel
// ordering) for the symmetric eigendecomposition.  The row products A = M W run over a grid
// with FP64 accumulation.
#include <cmath>

#include "ptg_internal.h"

namespace ptg {
namespace {

constexpr int kAlgThreads = 256;
constexpr int kMaxR = 64;

// W = Z^{-1} (Z: np->Z, FP64 R x R).  Augmented [Z | I] in shared memory.
__global__ void __launch_bounds__(kAlgThreads) inverse_kernel(const NnlsParams *__restrict__ np, int R,
                                                              double *__restrict__ W, int *__restrict__ status) {
  extern __shared__ double aug[];   // R x 2R, row-major
  __shared__ int piv;
  const int tid = threadIdx.x, C = 2 * R;
  for (int idx = tid; idx < R * C; idx += blockDim.x) {
    const int i = idx / C, j = idx % C;
    aug[idx] = j < R ? np->Z[i * R + j] : (j - R == i ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int k = 0; k < R; ++k) {
    if (tid < 32) {   // pivot: the row i >= k with the largest |a_ik| (lowest index on ties)
      double best = -1.0;
      int bi = k;
      for (int i = k + tid; i < R; i += 32) {
        const double v = fabs(aug[i * C + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (tid == 0) {
        piv = bi;
        if (!(best > 0.0)) *status = PTG_ERR_NUMERIC;   // singular
      }
    }
    __syncthreads();
    const int p = piv;
    if (p != k)
      for (int j = tid; j < C; j += blockDim.x) {
        const double t = aug[k * C + j];
        aug[k * C + j] = aug[p * C + j];
        aug[p * C + j] = t;
      }
    __syncthreads();
    const double d = aug[k * C + k];
    __syncthreads();
    for (int j = tid; j < C; j += blockDim.x) aug[k * C + j] /= d;
    __syncthreads();
    for (int idx = tid; idx < R * C; idx += blockDim.x) {
      const int i = idx / C, j = idx % C;
      if (i == k || j == k) continue;
      aug[idx] -= aug[i * C + k] * aug[k * C + j];
    }
    __syncthreads();
    for (int i = tid; i < R; i += blockDim.x)
      if (i != k) aug[i * C + k] = 0.0;
    __syncthreads();
  }
  for (int idx = tid; idx < R * R; idx += blockDim.x) W[idx] = aug[(idx / R) * C + R + idx % R];
}

constexpr int kGramRows = 256;

// FP64 partial Grams of M (rows of one block each): part[b][i][j] = sum_rows M[r][i] M[r][j].
__global__ void gram64_partial_kernel(const float *__restrict__ M, int I, int R, double *__restrict__ part) {
  const int r0 = blockIdx.x * kGramRows;
  const int nr = min(kGramRows, I - r0);
  for (int idx = threadIdx.x; idx < R * R; idx += blockDim.x) {
    const int a = idx / R, b = idx % R;
    double s = 0.0;
    for (int i = 0; i < nr; ++i) s = fma((double)M[(size_t)(r0 + i) * R + a], (double)M[(size_t)(r0 + i) * R + b], s);
    part[(size_t)blockIdx.x * R * R + idx] = s;
  }
}

// W = (C)^{-1/2} for the symmetric positive definite C = M^T M (the FP64 sum of the nb partial
// Grams, in block order), through the cyclic Jacobi eigendecomposition C = V diag(lambda) V^T.
__global__ void __launch_bounds__(kAlgThreads) inv_sqrt_kernel(const double *__restrict__ part, int nb, int R,
                                                               double *__restrict__ W, int *__restrict__ status) {
  extern __shared__ double sh[];
  const int n = R + (R & 1);   // even; an odd R gets an uncoupled padding index
  double *A = sh;              // n x n
  double *V = A + n * n;       // n x n
  double *cs = V + n * n;      // [n/2][2] rotation (c, s)
  int *pp = (int *)(cs + n);   // [n/2][2] pair indices
  __shared__ double red[kAlgThreads / 32];
  __shared__ double s_off, s_nrm;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx % n;
    double c = i == j ? 1.0 : 0.0;
    if (i < R && j < R) {
      c = 0.0;
      for (int b = 0; b < nb; ++b) c += part[(size_t)b * R * R + i * R + j];
    }
    A[idx] = c;
    V[idx] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  auto block_sum = [&](double x) -> double {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((tid & 31) == 0) red[tid >> 5] = x;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      s_off = s;
    }
    __syncthreads();
    return s_off;
  };
  double sq = 0.0;
  for (int idx = tid; idx < n * n; idx += blockDim.x) sq += A[idx] * A[idx];
  const double nrm2 = block_sum(sq);
  if (tid == 0) s_nrm = nrm2;
  __syncthreads();
  const int half = n / 2;
  for (int sweep = 0; sweep < 40; ++sweep) {
    sq = 0.0;
    for (int idx = tid; idx < n * n; idx += blockDim.x)
      if (idx / n != idx % n) sq += A[idx] * A[idx];
    const double off = block_sum(sq);
    if (off <= 1e-30 * s_nrm) break;
    for (int step = 0; step < n - 1; ++step) {
      // round-robin pairing: index 0 fixed, the others rotate
      for (int k = tid; k < half; k += blockDim.x) {
        auto pos = [&](int slot) { return slot == 0 ? 0 : 1 + (slot - 1 + step) % (n - 1); };
        int p = pos(k), q = pos(n - 1 - k);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        pp[2 * k] = p;
        pp[2 * k + 1] = q;
        const double apq = A[p * n + q];
        double c = 1.0, s = 0.0;
        if (apq != 0.0) {   // the symmetric Schur 2x2 (Golub & Van Loan alg. 8.5.1)
          const double tau = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
          const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          c = 1.0 / sqrt(1.0 + t * t);
          s = t * c;
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int idx = tid; idx < half * n; idx += blockDim.x) {
        const int k = idx / n, j = idx % n;
        const int p = pp[2 * k], q = pp[2 * k + 1];
        const double c = cs[2 * k], s = cs[2 * k + 1];
        const double ap = A[p * n + j], aq = A[q * n + j];
        A[p * n + j] = c * ap - s * aq;
        A[q * n + j] = s * ap + c * aq;
      }
      __syncthreads();
      // columns: A <- A J, V <- V J
      for (int idx = tid; idx < half * n; idx += blockDim.x) {
        const int k = idx / n, i = idx % n;
        const int p = pp[2 * k], q = pp[2 * k + 1];
        const double c = cs[2 * k], s = cs[2 * k + 1];
        const double ap = A[i * n + p], aq = A[i * n + q];
        A[i * n + p] = c * ap - s * aq;
        A[i * n + q] = s * ap + c * aq;
        const double vp = V[i * n + p], vq = V[i * n + q];
        V[i * n + p] = c * vp - s * vq;
        V[i * n + q] = s * vp + c * vq;
      }
      __syncthreads();
    }
  }
  // W = V diag(lambda^{-1/2}) V^T over the first R indices (the padding index, if any, is
  // uncoupled and keeps eigenvector e_R)
  for (int i = tid; i < n; i += blockDim.x) {
    const double lam = A[i * n + i];
    if (i < R && !(lam > 0.0)) *status = PTG_ERR_NUMERIC;
    cs[i] = lam > 0.0 ? 1.0 / sqrt(lam) : 0.0;   // reuse cs as the scale vector (n entries)
  }
  __syncthreads();
  for (int idx = tid; idx < R * R; idx += blockDim.x) {
    const int i = idx / R, j = idx % R;
    double s = 0.0;
    for (int k = 0; k < n; ++k) s = fma(V[i * n + k] * cs[k], V[j * n + k], s);
    W[idx] = s;
  }
}

// A[i][:] = M[i][:] W, FP64 accumulation; one warp per row, lane = column block.
__global__ void rows_times_kernel(const float *__restrict__ M, const double *__restrict__ W, int I, int R,
                                  float *__restrict__ A) {
  const int warps = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int i = blockIdx.x * warps + (threadIdx.x >> 5); i < I; i += gridDim.x * warps)
    for (int c = lane; c < R; c += 32) {
      double s = 0.0;
      for (int k = 0; k < R; ++k) s = fma((double)M[(size_t)i * R + k], W[k * R + c], s);
      A[(size_t)i * R + c] = (float)s;
    }
}

}  // namespace

int launch_update_unconstrained(ptg_ctx *ctx, const float *M, float *A, int I, int R, const NnlsParams *np,
                                double *W, cudaStream_t s) {
  if (R > kMaxR) return set_error(PTG_ERR_UNSUPPORTED, "rank > 64 is not supported by the unconstrained update");
  const size_t smem = sizeof(double) * R * 2 * R;
  PTG_CUDA(cudaFuncSetAttribute(inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  inverse_kernel<<<1, kAlgThreads, smem, s>>>(np, R, W, ctx->dev_err);
  rows_times_kernel<<<(I + 7) / 8, 256, 0, s>>>(M, W, I, R, A);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 2);
  return PTG_OK;
}

int launch_update_orthogonal(ptg_ctx *ctx, const float *M, float *A, int I, int R, double *W, cudaStream_t s) {
  if (R > kMaxR) return set_error(PTG_ERR_UNSUPPORTED, "rank > 64 is not supported by the orthogonal update");
  const int nb = (I + kGramRows - 1) / kGramRows;
  PTG_TRY(ctx->scratch.ensure(sizeof(double) * nb * R * R));   // MTTKRP partials are consumed by now
  double *part = reinterpret_cast<double *>(ctx->scratch.ptr);
  gram64_partial_kernel<<<nb, 256, 0, s>>>(M, I, R, part);
  const int n = R + (R & 1);
  const size_t smem = sizeof(double) * (2 * n * n + n) + sizeof(int) * n + 16;
  PTG_CUDA(cudaFuncSetAttribute(inv_sqrt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  inv_sqrt_kernel<<<1, kAlgThreads, smem, s>>>(part, nb, R, W, ctx->dev_err);
  rows_times_kernel<<<(I + 7) / 8, 256, 0, s>>>(M, W, I, R, A);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 3);
  return PTG_OK;
}

}  // namespace ptg
