// Dimension-tree MTTKRP: a binary tree over the modes whose node tensors stay resident in
// HBM (replaces ExprTree / TreeMode_N_Product / TTVs / UpdateTree of
// include/DimTrees.hpp:541-928 as used by CPD_DIMTREE::als, include/CpdDimTree.hpp:317-401).
//
// Node [a, b) holds T[(i_a..i_{b-1}), r], the contraction of X with the factors of every mode
// outside [a, b); a node splits at a + (1 + (b - a)) / 2 (DIM_HALF_SIZE,
// include/DimTrees.hpp:274-276), down to single-mode leaves, where T is M_n.
//   root's children  T_L = [0, h) and T_R = [h, N): MTTKRP-shaped contractions of the
//                    tensor itself (one tensor read each), on the tensor-core or CUDA-core
//                    MTTKRP kernels
//   deeper nodes     contractions of the parent's tensor with the sibling's factors
//                    (node_mttkrp_kernel), kept for reuse
// A node is recomputed when a factor outside it has changed since it was made, so a sweep
// reads the tensor twice and each intermediate node once.
#include <algorithm>

#include "ptg_internal.h"

namespace ptg {
namespace {

struct NodeArgs {
  const float *T;            // parent node tensor, row-major [rows][R]
  int nm;                    // modes in the parent
  uint32_t ext[PTG_MAX_ORDER];     // digit extents of the parent's row index (padded for mode 0)
  uint32_t valid[PTG_MAX_ORDER];
  const float *fac[PTG_MAX_ORDER];
  int k0, k1;                // the child's modes: parent positions [k0, k1)
  int compact;               // 1: a leaf (k1 = k0 + 1) written with its valid rows only (M_n)
  int R;
  float *out;                // child tensor [crows][R]
  int64_t crows;
};

// out[c, r] = sum over the other digits j of T[row(c, j), r] * prod_{k outside [k0, k1)} A_k[d_k(j), r]:
// the child node (or leaf) of a dimension-tree node, the partial contraction of TTVs
// (include/DimTrees.hpp:732-848).  The other digits enumerate in row order (first fastest)
// and each term's weight is the product over them in mode order.
__global__ void node_mttkrp_kernel(const NodeArgs a) {
  const int64_t n = a.crows * a.R;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx / a.R;
    const int r = (int)(idx % a.R);
    // the child's digits (padded layout, or valid rows of a compact leaf)
    uint32_t cd[PTG_MAX_ORDER];
    bool pad = false;
    {
      int64_t rem = c;
      for (int k = a.k0; k < a.k1; ++k) {
        const uint32_t e = a.compact ? a.valid[k] : a.ext[k];
        cd[k] = (uint32_t)(rem % e);
        rem /= e;
        pad = pad || cd[k] >= a.valid[k];
      }
    }
    uint32_t others = 1;
    for (int k = 0; k < a.nm; ++k)
      if (k < a.k0 || k >= a.k1) others *= a.valid[k];
    float s = 0.0f;
    for (uint32_t j = 0; !pad && j < others; ++j) {
      uint32_t rem = j, row = 0, mul = 1;
      float w = 1.0f;
      for (int k = 0; k < a.nm; ++k) {
        uint32_t d;
        if (k >= a.k0 && k < a.k1) {
          d = cd[k];
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

static uint32_t mode_ext(const ptg_tensor *t, int k) { return (uint32_t)(k == 0 ? t->pdim0 : t->dims[k]); }

// child [ca, cb) of the node [pa, pb) whose tensor is T: into out (a leaf: M_n, valid rows)
static int launch_node(ptg_ctx *ctx, const ptg_tensor *t, const float *T, int pa, int pb, int ca, int cb,
                       const float *const *factors, int R, float *out, int64_t crows, cudaStream_t stream) {
  NodeArgs a{};
  a.T = T;
  a.R = R;
  a.out = out;
  a.crows = crows;
  for (int k = pa; k < pb; ++k) {
    a.ext[a.nm] = mode_ext(t, k);
    a.valid[a.nm] = (uint32_t)t->dims[k];
    a.fac[a.nm] = factors[k];
    a.nm++;
  }
  a.k0 = ca - pa;
  a.k1 = cb - pa;
  a.compact = (cb - ca == 1) ? 1 : 0;
  const int64_t n = crows * R;
  const int blocks = (int)std::min<int64_t>((n + 127) / 128, (int64_t)ctx->sm_count * 16);
  node_mttkrp_kernel<<<std::max(blocks, 1), 128, 0, stream>>>(a);
  PTG_CUDA(cudaGetLastError());
  count_launches(ctx, 1);
  return PTG_OK;
}

int DimTree::build(const ptg_tensor *t) {
  nodes.clear();
  N = t->order;
  // node [a, b) with b - a >= 2 splits at a + (1 + (b - a)) / 2, DIM_HALF_SIZE of
  // include/DimTrees.hpp:274-276 applied at every level
  std::vector<std::pair<int, int>> todo{{0, N}};
  nodes.push_back(Node{0, N, -1, {-1, -1}, 0, nullptr, -1});
  for (size_t i = 0; i < nodes.size(); ++i) {
    const int a = nodes[i].a, b = nodes[i].b;
    if (b - a < 2) continue;
    const int m = a + (1 + (b - a)) / 2;
    for (int side = 0; side < 2; ++side) {
      Node c{side == 0 ? a : m, side == 0 ? m : b, (int)i, {-1, -1}, 1, nullptr, -1};
      for (int k = c.a; k < c.b; ++k) c.rows *= mode_ext(t, k);
      nodes[i].child[side] = (int)nodes.size();
      nodes.push_back(c);
    }
  }
  deep = 0;
  for (const Node &nd : nodes)
    if (nd.parent > 0 && nd.b - nd.a >= 2) deep += (size_t)nd.rows;
  for (int k = 0; k < PTG_MAX_ORDER; ++k) last[k] = 0;
  step = 0;
  return PTG_OK;
}

void DimTree::bind(float *left, float *right, float *deep_base, int R) {
  for (Node &nd : nodes) nd.T = nullptr;
  nodes[nodes[0].child[0]].T = left;
  nodes[nodes[0].child[1]].T = right;
  size_t off = 0;
  for (Node &nd : nodes)
    if (nd.parent > 0 && nd.b - nd.a >= 2) {
      nd.T = deep_base + off * R;
      off += (size_t)nd.rows;
    }
}

void DimTree::new_sweep() {
  for (Node &nd : nodes) nd.at = -1;
}

void DimTree::updated(int mode) { last[mode] = ++step; }

// fresh: computed after the last change of every factor outside the node
bool DimTree::fresh(const Node &nd) const {
  if (nd.at < 0) return false;
  for (int k = 0; k < N; ++k)
    if ((k < nd.a || k >= nd.b) && last[k] > nd.at) return false;
  return true;
}

int DimTree::mttkrp(ptg_ctx *ctx, const ptg_tensor *X, const float *const *factors, int mode, int R, float *out,
                    cudaStream_t s) {
  // the path from the root's child that holds `mode` down to the leaf's parent; every stale
  // node on it is recomputed from its parent (UpdateTree, include/DimTrees.hpp:862-928)
  int i = nodes[0].child[mode >= nodes[nodes[0].child[0]].b ? 1 : 0];
  while (true) {
    Node &nd = nodes[i];
    // the root's children are stored even when they hold one mode (order 3: [2, 3) = M_2)
    if (nd.parent != 0 && nd.b - nd.a == 1) break;
    if (!fresh(nd)) {
      if (nd.parent == 0) {
        PTG_TRY(contraction_launch(ctx, X, node_contraction(X, factors, i == nodes[0].child[0]), R, nd.T, s));
      } else {
        const Node &p = nodes[nd.parent];
        PTG_TRY(launch_node(ctx, X, p.T, p.a, p.b, nd.a, nd.b, factors, R, nd.T, nd.rows, s));
      }
      nd.at = step;
    }
    if (nd.b - nd.a == 1) break;   // a one-mode child of the root: its tensor is M_n
    i = nd.child[mode >= nodes[nd.child[0]].b ? 1 : 0];
  }
  const Node &leaf = nodes[i];
  const Node &p = leaf.b - leaf.a == 1 && leaf.parent == 0 ? leaf : nodes[leaf.parent];
  return launch_node(ctx, X, p.T, p.a, p.b, mode, mode + 1, factors, R, out, X->dims[mode], s);
}

}  // namespace ptg
