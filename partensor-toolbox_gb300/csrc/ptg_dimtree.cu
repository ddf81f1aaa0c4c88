// Dimension-tree MTTKRP: the two node tensors of a binary split of the modes kept
// resident in HBM (replaces ExprTree / TreeMode_N_Product / TTVs of
// include/DimTrees.hpp:541-928 as used by CPD_DIMTREE::als, include/CpdDimTree.hpp:317-401).
//
// The root is split at h = (1 + N) / 2 (DIM_HALF_SIZE, include/DimTrees.hpp:274-276).
//   left node   T_L[(i_0..i_{h-1}), r] = sum over the right modes of X * prod A_k   (one tensor read)
//   right node  T_R[(i_h..i_{N-1}), r] = sum over the left modes of X * prod A_k    (one tensor read)
// Both are MTTKRP-shaped contractions of the same [P, Q, S] view, so they run on the
// tensor-core or CUDA-core MTTKRP kernels.  A leaf MTTKRP is then a small contraction of
// a node tensor with the node's other factors (leaf_mttkrp_kernel).
#include <algorithm>

#include "ptg_internal.h"

namespace ptg {
namespace {

struct LeafArgs {
  const float *T;            // node tensor, row-major [rows][R]
  int nm;                    // modes in the node
  uint32_t ext[PTG_MAX_ORDER];     // digit extents of the node's row index (padded for mode 0)
  uint32_t valid[PTG_MAX_ORDER];
  const float *fac[PTG_MAX_ORDER];
  int pos;                   // position of the solved mode inside the node
  int R;
  float *out;                // [valid[pos]][R]
};

// out[i, r] = sum over the other digits j of T[row(i, j), r] * prod_{k != pos} A_k[d_k(j), r]
__global__ void leaf_mttkrp_kernel(const LeafArgs a) {
  const int64_t n = (int64_t)a.valid[a.pos] * a.R;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / a.R), r = (int)(idx % a.R);
    // the other digits enumerate in row order; stride of the solved digit
    uint32_t stride_pos = 1, others = 1;
    for (int k = 0; k < a.nm; ++k) {
      if (k < a.pos) stride_pos *= a.ext[k];
      if (k != a.pos) others *= a.valid[k];
    }
    float s = 0.0f;
    for (uint32_t j = 0; j < others; ++j) {
      uint32_t rem = j, row = 0, mul = 1;
      float w = 1.0f;
      for (int k = 0; k < a.nm; ++k) {
        uint32_t d;
        if (k == a.pos) {
          d = (uint32_t)i;
        } else {
          d = rem % a.valid[k];
          rem /= a.valid[k];
          w *= __ldg(a.fac[k] + (size_t)d * a.R + r);
        }
        row += d * mul;
        mul *= a.ext[k];
      }
      s = fmaf(__ldg(a.T + (size_t)row * a.R + r), w, s);
    }
    (void)stride_pos;
    a.out[idx] = s;
  }
}

}  // namespace

int dimtree_split(int order) { return (1 + order) / 2; }

Contraction node_contraction(const ptg_tensor *t, const float *const *factors, bool left_node) {
  const int N = t->order, h = dimtree_split(N);
  Contraction c;
  auto ext = [&](int k) { return k == 0 ? t->pdim0 : t->dims[k]; };
  if (left_node) {
    // [P = 1, Q = prod_{k<h} ext, S = prod_{k>=h} I_k]; the right modes are contracted
    for (int k = 0; k < h; ++k) c.Q *= ext(k);
    for (int k = h; k < N; ++k) {
      c.S *= ext(k);
      c.after.ext[c.after.n] = ext(k);
      c.after.valid[c.after.n] = t->dims[k];
      c.after.fac[c.after.n] = factors[k];
      c.after.n++;
    }
  } else {
    for (int k = 0; k < h; ++k) {
      c.P *= ext(k);
      c.before.ext[c.before.n] = ext(k);
      c.before.valid[c.before.n] = t->dims[k];
      c.before.fac[c.before.n] = factors[k];
      c.before.n++;
    }
    for (int k = h; k < N; ++k) c.Q *= ext(k);
  }
  c.q_write = c.Q;
  // the last mode's index: the slowest digit of s (left node) or of q (right node)
  c.slab_div = 1;
  for (int k = h; k < N - 1; ++k) c.slab_div *= ext(k);
  c.slab_in_q = !left_node;
  return c;
}

int64_t node_rows(const ptg_tensor *t, bool left_node) {
  const int N = t->order, h = dimtree_split(N);
  int64_t q = 1;
  for (int k = left_node ? 0 : h; k < (left_node ? h : N); ++k) q *= (k == 0 ? t->pdim0 : t->dims[k]);
  return q;
}

int launch_leaf_mttkrp(ptg_ctx *ctx, const ptg_tensor *t, const float *T, const float *const *factors, int mode,
                       int R, float *out, cudaStream_t stream) {
  const int N = t->order, h = dimtree_split(N);
  const bool left = mode < h;
  LeafArgs a{};
  a.T = T;
  a.R = R;
  a.out = out;
  const int k0 = left ? 0 : h, k1 = left ? h : N;
  for (int k = k0; k < k1; ++k) {
    a.ext[a.nm] = (uint32_t)(k == 0 ? t->pdim0 : t->dims[k]);
    a.valid[a.nm] = (uint32_t)t->dims[k];
    a.fac[a.nm] = factors[k];
    if (k == mode) a.pos = a.nm;
    a.nm++;
  }
  const int64_t n = (int64_t)t->dims[mode] * R;
  const int blocks = (int)std::min<int64_t>((n + 127) / 128, (int64_t)ctx->sm_count * 16);
  leaf_mttkrp_kernel<<<std::max(blocks, 1), 128, 0, stream>>>(a);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 1);
  return PTG_OK;
}

}  // namespace ptg
