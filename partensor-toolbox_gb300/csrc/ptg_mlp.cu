// Learned warm start for the NNLS rows: a two-hidden-layer ReLU MLP trained and run by
// the library's own kernels (no counterpart in the reference, whose Nesterov solver always
// starts from the previous factor, include/NesterovMNLS.hpp:207-209).
//
// Input of row i (Din = R + 8): the MTTKRP row m_i / ||m_i|| and eight scale-free summaries
// of the Hadamard-of-Grams Z (NnlsParams::feat).  Output (R): the NNLS solution row scaled
// by L / ||m_i||.  The Nesterov solver then starts from max(output * ||m_i|| / L, 0) and
// still runs to the reference's own stopping rule, so the plain solver is the fallback.
//
// Training: full-batch-free minibatch Adam on (features, converged row) pairs the solver
// logs; each step is one kernel computing per-CTA partial gradients of 32 rows and one
// kernel that sums them in CTA order and applies Adam (deterministic).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ptg_internal.h"

namespace ptg {
namespace {

constexpr int MLP_ROWS = 32;       // rows per CTA in a training step
constexpr int MLP_THREADS = 256;

__device__ __forceinline__ float hash_uniform(unsigned long long seed, unsigned long long i) {
  unsigned long long z = seed * 0x9E3779B97F4A7C15ull + (i + 1) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);
}

__global__ void mlp_init_kernel(float *theta, int din, int h, int dout, unsigned long long seed) {
  const int64_t o1 = 0, o2 = (int64_t)h * din + h, o3 = o2 + (int64_t)h * h + h;
  const int64_t n = o3 + (int64_t)dout * h + dout;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float v = 0.0f;
    int fan = 0;
    if (i < o1 + (int64_t)h * din) fan = din;
    else if (i >= o2 && i < o2 + (int64_t)h * h) fan = h;
    else if (i >= o3 && i < o3 + (int64_t)dout * h) fan = h;
    if (fan) v = (2.0f * hash_uniform(seed, (unsigned long long)i) - 1.0f) * sqrtf(6.0f / (float)fan);
    theta[i] = v;
  }
}

struct MlpDims {
  int din, h, dout;
  int64_t oW1, ob1, oW2, ob2, oW3, ob3, n;
};

MlpDims mlp_dims(int din, int h, int dout) {
  MlpDims d{din, h, dout, 0, 0, 0, 0, 0, 0, 0};
  d.oW1 = 0;
  d.ob1 = d.oW1 + (int64_t)h * din;
  d.oW2 = d.ob1 + h;
  d.ob2 = d.oW2 + (int64_t)h * h;
  d.oW3 = d.ob2 + h;
  d.ob3 = d.oW3 + (int64_t)dout * h;
  d.n = d.ob3 + dout;
  return d;
}

// One training step, part 1: CTA c takes rows [c*32, c*32+32) of the batch (batch rows are
// `idx[b]` of the data set), runs forward and backward and writes its partial gradient.
// Also used with rows = batch for the loss/gradient check (idx = identity).
struct StepArgs {
  const float *theta;
  const float *X;      // [rows][din]
  const float *T;      // [rows][dout]
  const int *idx;      // batch -> data row
  int B;               // batch size
  MlpDims d;
  float *partial;      // [nctas][n]
  double *loss_part;   // [nctas]
};

__global__ void __launch_bounds__(MLP_THREADS) mlp_grad_kernel(const StepArgs a) {
  extern __shared__ float sm[];
  const MlpDims d = a.d;
  const int H = d.h, Din = d.din, Dout = d.dout;
  float *x = sm;                          // [32][Din]
  float *z1 = x + MLP_ROWS * Din;         // [32][H]
  float *z2 = z1 + MLP_ROWS * H;          // [32][H]
  float *y = z2 + MLP_ROWS * H;           // [32][Dout]  (becomes dY)
  float *d2 = y + MLP_ROWS * Dout;        // [32][H]
  float *d1 = d2 + MLP_ROWS * H;          // [32][H]
  __shared__ double lred[MLP_THREADS / 32];
  const int tid = threadIdx.x;
  const int r0 = blockIdx.x * MLP_ROWS;
  const int nr = min(MLP_ROWS, a.B - r0);
  const float *W1 = a.theta + d.oW1, *b1 = a.theta + d.ob1, *W2 = a.theta + d.oW2, *b2 = a.theta + d.ob2;
  const float *W3 = a.theta + d.oW3, *b3 = a.theta + d.ob3;
  for (int p = tid; p < MLP_ROWS * Din; p += MLP_THREADS) {
    const int r = p / Din, j = p % Din;
    x[p] = r < nr ? a.X[(int64_t)a.idx[r0 + r] * Din + j] : 0.0f;
  }
  __syncthreads();
  for (int p = tid; p < MLP_ROWS * H; p += MLP_THREADS) {
    const int r = p / H, u = p % H;
    float s = b1[u];
    for (int j = 0; j < Din; ++j) s = fmaf(W1[(int64_t)u * Din + j], x[r * Din + j], s);
    z1[p] = s;
  }
  __syncthreads();
  for (int p = tid; p < MLP_ROWS * H; p += MLP_THREADS) {
    const int r = p / H, u = p % H;
    float s = b2[u];
    for (int j = 0; j < H; ++j) s = fmaf(W2[(int64_t)u * H + j], fmaxf(z1[r * H + j], 0.0f), s);
    z2[p] = s;
  }
  __syncthreads();
  double lsum = 0.0;
  const float scale = 1.0f / ((float)a.B * (float)Dout);
  for (int p = tid; p < MLP_ROWS * Dout; p += MLP_THREADS) {
    const int r = p / Dout, o = p % Dout;
    float s = b3[o];
    for (int j = 0; j < H; ++j) s = fmaf(W3[(int64_t)o * H + j], fmaxf(z2[r * H + j], 0.0f), s);
    float dy = 0.0f;
    if (r < nr) {
      const float e = s - a.T[(int64_t)a.idx[r0 + r] * Dout + o];
      lsum += 0.5 * (double)e * (double)e;
      dy = e * scale;
    }
    y[p] = dy;
  }
  __syncthreads();
  // dA2 = dY W3, masked by z2 > 0
  for (int p = tid; p < MLP_ROWS * H; p += MLP_THREADS) {
    const int r = p / H, u = p % H;
    float s = 0.0f;
    for (int o = 0; o < Dout; ++o) s = fmaf(y[r * Dout + o], W3[(int64_t)o * H + u], s);
    d2[p] = z2[p] > 0.0f ? s : 0.0f;
  }
  __syncthreads();
  for (int p = tid; p < MLP_ROWS * H; p += MLP_THREADS) {
    const int r = p / H, u = p % H;
    float s = 0.0f;
    for (int v = 0; v < H; ++v) s = fmaf(d2[r * H + v], W2[(int64_t)v * H + u], s);
    d1[p] = z1[p] > 0.0f ? s : 0.0f;
  }
  __syncthreads();
  float *g = a.partial + (int64_t)blockIdx.x * d.n;
  // gradients summed over this CTA's rows, in row order
  for (int64_t p = tid; p < (int64_t)H * Din; p += MLP_THREADS) {
    const int u = (int)(p / Din), j = (int)(p % Din);
    float s = 0.0f;
    for (int r = 0; r < MLP_ROWS; ++r) s = fmaf(d1[r * H + u], x[r * Din + j], s);
    g[d.oW1 + p] = s;
  }
  for (int u = tid; u < H; u += MLP_THREADS) {
    float s1 = 0.0f, s2 = 0.0f;
    for (int r = 0; r < MLP_ROWS; ++r) {
      s1 += d1[r * H + u];
      s2 += d2[r * H + u];
    }
    g[d.ob1 + u] = s1;
    g[d.ob2 + u] = s2;
  }
  for (int64_t p = tid; p < (int64_t)H * H; p += MLP_THREADS) {
    const int u = (int)(p / H), v = (int)(p % H);
    float s = 0.0f;
    for (int r = 0; r < MLP_ROWS; ++r) s = fmaf(d2[r * H + u], fmaxf(z1[r * H + v], 0.0f), s);
    g[d.oW2 + p] = s;
  }
  for (int64_t p = tid; p < (int64_t)Dout * H; p += MLP_THREADS) {
    const int o = (int)(p / H), v = (int)(p % H);
    float s = 0.0f;
    for (int r = 0; r < MLP_ROWS; ++r) s = fmaf(y[r * Dout + o], fmaxf(z2[r * H + v], 0.0f), s);
    g[d.oW3 + p] = s;
  }
  for (int o = tid; o < Dout; o += MLP_THREADS) {
    float s = 0.0f;
    for (int r = 0; r < MLP_ROWS; ++r) s += y[r * Dout + o];
    g[d.ob3 + o] = s;
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if ((tid & 31) == 0) lred[tid >> 5] = lsum;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < MLP_THREADS / 32; ++w) t += lred[w];
    a.loss_part[blockIdx.x] = t;
  }
}

// Part 2: sum the CTA partials in CTA order; optionally Adam-update theta.
struct AdamArgs {
  float *theta, *m, *v, *grad_out;
  const float *partial;
  int nctas;
  int64_t n;
  float lr, b1, b2, eps, c1, c2;   // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)
  int update;
};

__global__ void mlp_adam_kernel(const AdamArgs a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    float g = 0.0f;
    for (int c = 0; c < a.nctas; ++c) g += a.partial[(int64_t)c * a.n + i];
    if (a.grad_out) a.grad_out[i] = g;
    if (a.update) {
      const float m = a.b1 * a.m[i] + (1.0f - a.b1) * g;
      const float v = a.b2 * a.v[i] + (1.0f - a.b2) * g * g;
      a.m[i] = m;
      a.v[i] = v;
      a.theta[i] -= a.lr * (m * a.c1) / (sqrtf(v * a.c2) + a.eps);
    }
  }
}

__global__ void mlp_forward_kernel(const float *theta, MlpDims d, const float *X, int64_t rows, float *Y) {
  // one warp per row; lane-strided hidden units
  extern __shared__ float hs[];   // per warp: 2 * H
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float *h1 = hs + w * 2 * d.h, *h2 = h1 + d.h;
  for (int64_t r = (int64_t)blockIdx.x * nw + w; r < rows; r += (int64_t)gridDim.x * nw) {
    const float *x = X + r * d.din;
    for (int u = lane; u < d.h; u += 32) {
      float s = theta[d.ob1 + u];
      for (int j = 0; j < d.din; ++j) s = fmaf(theta[d.oW1 + (int64_t)u * d.din + j], x[j], s);
      h1[u] = fmaxf(s, 0.0f);
    }
    __syncwarp();
    for (int u = lane; u < d.h; u += 32) {
      float s = theta[d.ob2 + u];
      for (int j = 0; j < d.h; ++j) s = fmaf(theta[d.oW2 + (int64_t)u * d.h + j], h1[j], s);
      h2[u] = fmaxf(s, 0.0f);
    }
    __syncwarp();
    for (int o = lane; o < d.dout; o += 32) {
      float s = theta[d.ob3 + o];
      for (int j = 0; j < d.h; ++j) s = fmaf(theta[d.oW3 + (int64_t)o * d.h + j], h2[j], s);
      Y[r * d.dout + o] = s;
    }
    __syncwarp();
  }
}

__global__ void batch_index_kernel(int *idx, int B, int64_t rows, unsigned long long seed, int step) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    const float u = hash_uniform(seed ^ 0x5851F42D4C957F2Dull, (unsigned long long)step * 1048576ull + b);
    int64_t r = (int64_t)(u * (float)rows);
    if (r >= rows) r = rows - 1;
    idx[b] = (int)r;
  }
}

__global__ void iota_kernel(int *idx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) idx[i] = i;
}

size_t grad_smem(const MlpDims &d) {
  return sizeof(float) * (size_t)MLP_ROWS * (d.din + 4 * d.h + d.dout);
}

}  // namespace
}  // namespace ptg

struct ptg_mlp {
  int rank = 0, din = 0, hidden = 0, dout = 0;
  ptg::MlpDims d{};
  float *theta = nullptr, *m = nullptr, *v = nullptr;
  float *theta_t = nullptr;   // the weights transposed for the fused inference
  bool t_dirty = true;        // theta changed since theta_t was made
  int adam_t = 0;
  int device = 0;
};

using namespace ptg;

namespace ptg {
namespace {
// theta_t: W1^T [Din][H], b1, W2^T [H][H], b2, W3^T [H][Dout], b3 (same offsets as theta), so
// that the inference fused into the NNLS kernel, with one hidden unit or output per lane,
// reads each weight row of a step as one coalesced line.
__global__ void mlp_transpose_kernel(const float *__restrict__ th, float *__restrict__ tt, MlpDims d, int din, int h,
                                     int dout) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t dst = i;
    if (i >= d.oW1 && i < d.ob1) {          // W1 [h][din] -> [din][h]
      const int64_t u = (i - d.oW1) / din, j = (i - d.oW1) % din;
      dst = d.oW1 + j * h + u;
    } else if (i >= d.oW2 && i < d.ob2) {   // W2 [h][h] -> transposed
      const int64_t u = (i - d.oW2) / h, j = (i - d.oW2) % h;
      dst = d.oW2 + j * h + u;
    } else if (i >= d.oW3 && i < d.ob3) {   // W3 [dout][h] -> [h][dout]
      const int64_t o = (i - d.oW3) / h, j = (i - d.oW3) % h;
      dst = d.oW3 + j * dout + o;
    }
    tt[dst] = th[i];
  }
}
}  // namespace

const float *mlp_theta(const ptg_mlp *m) { return m->theta; }

const float *mlp_theta_infer(ptg_mlp *m, cudaStream_t s) {
  if (m->t_dirty) {
    mlp_transpose_kernel<<<64, 256, 0, s>>>(m->theta, m->theta_t, m->d, m->din, m->hidden, m->dout);
    m->t_dirty = false;
  }
  return m->theta_t;
}
int mlp_din(const ptg_mlp *m) { return m->din; }
int mlp_hidden(const ptg_mlp *m) { return m->hidden; }
}  // namespace ptg

extern "C" {

int ptg_mlp_create(ptg_ctx *ctx, int rank, unsigned long long seed, ptg_mlp **out) {
  if (!ctx || !out) return set_error(PTG_ERR_INVALID, "NULL argument");
  if (rank < 1 || rank > 64) return set_error(PTG_ERR_UNSUPPORTED, "MLP warm start needs rank in [1, 64]");
  *out = nullptr;
  PTG_CUDA(cudaSetDevice(ctx->device));
  ptg_mlp *m = new ptg_mlp();
  m->rank = rank;
  m->din = rank + 8;
  m->hidden = 128;
  m->dout = rank;
  m->d = mlp_dims(m->din, m->hidden, m->dout);
  m->device = ctx->device;
  cudaError_t e = cudaMalloc(&m->theta, sizeof(float) * 4 * m->d.n);
  if (e != cudaSuccess) {
    delete m;
    return cuda_error(e, "cudaMalloc(MLP)", __FILE__, __LINE__);
  }
  m->m = m->theta + m->d.n;
  m->v = m->m + m->d.n;
  m->theta_t = m->v + m->d.n;
  cudaMemsetAsync(m->m, 0, sizeof(float) * 2 * m->d.n, ctx->stream);
  mlp_init_kernel<<<64, 256, 0, ctx->stream>>>(m->theta, m->din, m->hidden, m->dout, seed);
  count_launches(ctx, 1);
  PTG_CUDA(cudaGetLastError());
  PTG_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = m;
  return PTG_OK;
}

int ptg_mlp_destroy(ptg_mlp *m) {
  if (!m) return PTG_OK;
  cudaSetDevice(m->device);
  if (m->theta) cudaFree(m->theta);
  delete m;
  return PTG_OK;
}

long long ptg_mlp_num_params(const ptg_mlp *m) { return m ? (long long)m->d.n : 0; }

int ptg_mlp_get_params(ptg_ctx *ctx, const ptg_mlp *m, float *host_out) {
  if (!ctx || !m || !host_out) return set_error(PTG_ERR_INVALID, "NULL argument");
  PTG_CUDA(cudaMemcpyAsync(host_out, m->theta, sizeof(float) * m->d.n, cudaMemcpyDeviceToHost, ctx->stream));
  PTG_CUDA(cudaStreamSynchronize(ctx->stream));
  return PTG_OK;
}

int ptg_mlp_set_params(ptg_ctx *ctx, ptg_mlp *m, const float *host_in) {
  if (!ctx || !m || !host_in) return set_error(PTG_ERR_INVALID, "NULL argument");
  PTG_CUDA(cudaMemcpyAsync(m->theta, host_in, sizeof(float) * m->d.n, cudaMemcpyHostToDevice, ctx->stream));
  m->t_dirty = true;
  PTG_CUDA(cudaMemsetAsync(m->m, 0, sizeof(float) * 2 * m->d.n, ctx->stream));
  m->adam_t = 0;
  PTG_CUDA(cudaStreamSynchronize(ctx->stream));
  return PTG_OK;
}

int ptg_mlp_forward(ptg_ctx *ctx, const ptg_mlp *m, const float *X_dev, long long rows, float *Y_dev) {
  if (!ctx || !m || !X_dev || !Y_dev || rows < 0) return set_error(PTG_ERR_INVALID, "bad argument");
  if (rows == 0) return PTG_OK;
  const int threads = 256;
  const size_t smem = sizeof(float) * 2 * m->hidden * (threads / 32);
  const int blocks = (int)std::min<long long>((rows + 7) / 8, (long long)ctx->sm_count * 8);
  mlp_forward_kernel<<<blocks, threads, smem, ctx->stream>>>(m->theta, m->d, X_dev, rows, Y_dev);
  count_launches(ctx, 1);
  PTG_CUDA(cudaGetLastError());
  return PTG_OK;
}

// Loss and gradient of the whole data set (rows <= 65536) at the current parameters, for
// gradient checks: loss = sum 0.5 ||y - t||^2 / (rows * R).
int ptg_mlp_loss_grad(ptg_ctx *ctx, const ptg_mlp *m, const float *X_dev, const float *T_dev, int rows,
                      double *loss, float *grad_dev) {
  if (!ctx || !m || !X_dev || !T_dev || rows < 1 || rows > 65536) return set_error(PTG_ERR_INVALID, "bad argument");
  const int nctas = (rows + MLP_ROWS - 1) / MLP_ROWS;
  float *partial = nullptr;
  double *lp = nullptr;
  int *idx = nullptr;
  PTG_CUDA(cudaMalloc(&partial, sizeof(float) * (size_t)nctas * m->d.n));
  cudaMalloc(&lp, sizeof(double) * nctas);
  cudaMalloc(&idx, sizeof(int) * rows);
  iota_kernel<<<(rows + 255) / 256, 256, 0, ctx->stream>>>(idx, rows);
  StepArgs sa{m->theta, X_dev, T_dev, idx, rows, m->d, partial, lp};
  const size_t smem = grad_smem(m->d);
  cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  mlp_grad_kernel<<<nctas, MLP_THREADS, smem, ctx->stream>>>(sa);
  AdamArgs aa{};
  aa.partial = partial;
  aa.nctas = nctas;
  aa.n = m->d.n;
  aa.grad_out = grad_dev;
  aa.update = 0;
  mlp_adam_kernel<<<(int)((m->d.n + 255) / 256), 256, 0, ctx->stream>>>(aa);
  count_launches(ctx, 3);
  std::vector<double> h(nctas);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), lp, sizeof(double) * nctas, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(partial);
  cudaFree(lp);
  cudaFree(idx);
  if (e != cudaSuccess) return cuda_error(e, "ptg_mlp_loss_grad", __FILE__, __LINE__);
  double t = 0.0;
  for (double x : h) t += x;
  if (loss) *loss = t / ((double)rows * m->dout);
  return PTG_OK;
}

// Minibatch Adam on a data set of `rows` (features X [rows][R+8], targets T [rows][R]).
int ptg_mlp_train(ptg_ctx *ctx, ptg_mlp *m, const float *X_dev, const float *T_dev, long long rows, int steps,
                  int batch, float lr, unsigned long long seed, double *final_loss) {
  if (!ctx || !m || !X_dev || !T_dev || rows < 1 || steps < 0 || batch < 1)
    return set_error(PTG_ERR_INVALID, "bad argument");
  PTG_CUDA(cudaSetDevice(ctx->device));
  const int B = (int)std::min<long long>(batch, rows);
  const int nctas = (B + MLP_ROWS - 1) / MLP_ROWS;
  float *partial = nullptr;
  double *lp = nullptr;
  int *idx = nullptr;
  PTG_CUDA(cudaMalloc(&partial, sizeof(float) * (size_t)nctas * m->d.n));
  cudaError_t e = cudaMalloc(&lp, sizeof(double) * nctas);
  if (e == cudaSuccess) e = cudaMalloc(&idx, sizeof(int) * B);
  if (e != cudaSuccess) {
    cudaFree(partial);
    cudaFree(lp);
    return cuda_error(e, "cudaMalloc(MLP train)", __FILE__, __LINE__);
  }
  const size_t smem = grad_smem(m->d);
  cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const float b1 = 0.9f, b2 = 0.999f;
  for (int s = 0; s < steps; ++s) {
    batch_index_kernel<<<(B + 255) / 256, 256, 0, ctx->stream>>>(idx, B, rows, seed, m->adam_t);
    StepArgs sa{m->theta, X_dev, T_dev, idx, B, m->d, partial, lp};
    mlp_grad_kernel<<<nctas, MLP_THREADS, smem, ctx->stream>>>(sa);
    m->adam_t++;
    AdamArgs aa{};
    aa.theta = m->theta;
    aa.m = m->m;
    aa.v = m->v;
    aa.partial = partial;
    aa.nctas = nctas;
    aa.n = m->d.n;
    aa.lr = lr;
    aa.b1 = b1;
    aa.b2 = b2;
    aa.eps = 1e-8f;
    aa.c1 = (float)(1.0 / (1.0 - std::pow((double)b1, m->adam_t)));
    aa.c2 = (float)(1.0 / (1.0 - std::pow((double)b2, m->adam_t)));
    aa.update = 1;
    mlp_adam_kernel<<<(int)((m->d.n + 255) / 256), 256, 0, ctx->stream>>>(aa);
    count_launches(ctx, 3);
  }
  if (steps > 0) m->t_dirty = true;
  std::vector<double> h(nctas, 0.0);
  e = cudaGetLastError();
  if (e == cudaSuccess && steps > 0)
    e = cudaMemcpyAsync(h.data(), lp, sizeof(double) * nctas, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(partial);
  cudaFree(lp);
  cudaFree(idx);
  if (e != cudaSuccess) return cuda_error(e, "ptg_mlp_train", __FILE__, __LINE__);
  if (final_loss) {
    double t = 0.0;
    for (double x : h) t += x;
    *final_loss = t / ((double)B * m->dout);
  }
  return PTG_OK;
}

}  // extern "C"
