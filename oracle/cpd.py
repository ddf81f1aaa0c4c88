"""FP64 CPU oracle for the dense CPD-ALS path -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy float64, the algorithm of Partensor's sequential and
OpenMP CPD drivers.  It is the checker the GPU kernels are compared against; nothing in
the product library imports or calls it.  Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may use it.

Parity status: the reference ships no golden vectors for this path (its examples use
time-seeded RNGs and print results).  The only numeric contract it pins is the MTTKRP
agreement test ``test/CPD_CUDA/test_mttkrp.cpp:101-109`` (||M_gpu - M_cpu||_F <= 1e-4
at 1000^3 R=100, factors in [-1,1]) and ``test/CPD_CUDA/test_batched_mttkrp.cpp:105-113``
(500^3 R=40).  Everything else here is "parity unpinned": it follows the cited reference
lines and is cross-checked against independent formulations (einsum MTTKRP, residual vs
Gram-form cost) and against the C restatement in ``oracle/cpd_omp.c``.

Every function cites the reference file:line it follows (paths are relative to the
reference project's root).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

# Constraint enum, include/Constants.hpp:40-55 (values in declaration order).
UNCONSTRAINED, NONNEGATIVITY, ORTHOGONALITY, SPARSITY, CONSTANT = 0, 1, 2, 3, 4


@dataclasses.dataclass
class Options:
    """Mirror of ``partensor::Options`` (include/PARTENSOR_basic.hpp:283-336) with the
    ``DefaultValues`` of include/PARTENSOR_basic.hpp:176-218."""
    order: int = 3
    constraints: Optional[List[int]] = None      # default nonnegativity on every mode
    threshold_error: float = 1e-3
    nesterov_delta_1: float = 1e-2
    nesterov_delta_2: float = 1e-2
    max_iter: int = 20
    accel_coeff: int = 3
    accel_fail: int = 0
    acceleration: bool = True
    normalization: bool = True

    def __post_init__(self):
        if self.constraints is None:
            self.constraints = [NONNEGATIVITY] * self.order


@dataclasses.dataclass
class Status:
    """Mirror of ``partensor::Status`` (include/PARTENSOR_basic.hpp:556-595) plus a
    per-sweep trace used by the tests."""
    options: Options
    factors: List[np.ndarray]
    frob_tns: float = 0.0
    f_value: float = 0.0
    rel_costFunction: float = 0.0
    ao_iter: int = 0
    trace: list = dataclasses.field(default_factory=list)


# --------------------------------------------------------------------------------------
# Unfolding and Khatri-Rao ordering
# --------------------------------------------------------------------------------------

def matricization(X: np.ndarray, mode: int) -> np.ndarray:
    """Mode-n unfolding, include/Matricization.hpp:65-75 (permute {n,0,..,n-1,n+1,..})
    and :101-124 (shuffle + ColMajor reshape).  ``X`` is indexed X[i0, i1, ...] with
    i0 fastest in memory (ColMajor, include/Tensor.hpp:64).  Column j of the result is
    j = sum_{k != n} i_k * prod_{l < k, l != n} I_l."""
    In = X.shape[mode]
    return np.moveaxis(X, mode, 0).reshape(In, -1, order="F")


def khatri_rao(*mats: np.ndarray) -> np.ndarray:
    """Column-wise Kronecker product with the FIRST argument varying slowest,
    include/KhatriRao.hpp:60-86 (kroneckerProduct of columns) and :134-140."""
    res = mats[-1]
    for m in reversed(mats[:-1]):
        R = m.shape[1]
        res = (m[:, None, :] * res[None, :, :]).reshape(-1, R)
    return res


def partial_khatri_rao(factors: Sequence[np.ndarray], mode: int) -> np.ndarray:
    """KhatriRao(A_{N-1}, ..., A_0) skipping ``mode``, include/PartialKhatriRao.hpp:59-233."""
    mats = [factors[k] for k in range(len(factors) - 1, -1, -1) if k != mode]
    return khatri_rao(*mats)


def partial_cwise_prod(grams: Sequence[np.ndarray], mode: int) -> np.ndarray:
    """Hadamard product of all Gramians except ``mode``, include/PartialCwiseProd.hpp:54-222
    with include/CwiseProd.hpp:48-63 (same operand order as PartialKhatriRao)."""
    out = None
    for k in range(len(grams) - 1, -1, -1):
        if k == mode:
            continue
        out = grams[k].copy() if out is None else out * grams[k]
    return out


def mttkrp(factors: Sequence[np.ndarray], X: np.ndarray, mode: int) -> np.ndarray:
    """Sequential MTTKRP, include/MTTKRP.hpp:60-69: krao = PartialKhatriRao(factors, mode);
    result = X_(mode) * krao."""
    return matricization(X, mode) @ partial_khatri_rao(factors, mode)


def mttkrp_einsum(factors: Sequence[np.ndarray], X: np.ndarray, mode: int) -> np.ndarray:
    """Independent formulation of the same contraction (used only to cross-check)."""
    N = X.ndim
    letters = "abcdefgh"[:N]
    spec = letters + "," + ",".join(f"{letters[k]}z" for k in range(N) if k != mode)
    spec += "->" + letters[mode] + "z"
    return np.einsum(spec, X, *[factors[k] for k in range(N) if k != mode], optimize=True)


def square_norm(X: np.ndarray) -> float:
    """include/TensorOperations.hpp:144-149."""
    return float(np.sum(X.astype(np.float64) ** 2))


# --------------------------------------------------------------------------------------
# Nesterov MNLS (dense), include/NesterovMNLS.hpp:45-234
# --------------------------------------------------------------------------------------

def compute_svd(Z: np.ndarray):
    """L, mu = largest / smallest singular value, include/NesterovMNLS.hpp:45-52."""
    s = np.linalg.svd(Z, compute_uv=False)
    return float(s.max()), float(s.min())


def glambda(mu: float, L: float):
    """include/NesterovMNLS.hpp:75-91.  Returns (L, mu, lambda, q) after the shift."""
    q = mu / L if L != 0 else 0.0
    inv_q = (1.0 / q) if q != 0 else math.inf
    if inv_q > 1e6:
        lam = 10.0 * mu
    elif inv_q > 1e3:
        lam = mu
    else:
        lam = mu / 10.0
    L += lam
    mu += lam
    q = mu / L
    return L, mu, lam, q


def update_alpha(alpha: float, q: float) -> float:
    """Positive root of a'^2 + (alpha^2 - q) a' - alpha^2 = 0, include/NesterovMNLS.hpp:103-113."""
    b = alpha * alpha - q
    c = -alpha * alpha
    D = b * b - 4.0 * c
    return (-b + math.sqrt(D)) / 2.0


def nesterov_betas(q: float, n: int) -> np.ndarray:
    """The beta sequence of include/NesterovMNLS.hpp:224-226; it depends on q only."""
    out = np.empty(n)
    alpha = 1.0
    for k in range(n):
        new_alpha = update_alpha(alpha, q)
        out[k] = alpha * (1.0 - alpha) / (alpha * alpha + new_alpha)
        alpha = new_alpha
    return out


NESTEROV_MAX_INNER = 50   # include/NesterovMNLS.hpp:187


def nesterov_mnls(Z: np.ndarray, W: np.ndarray, delta_1: float, delta_2: float,
                  A0: np.ndarray, return_info: bool = False):
    """Dense projected accelerated gradient, include/NesterovMNLS.hpp:181-234.

    Solves min_{A >= 0} with Hessian Z (R x R) and linear term W (I x R), proximal
    centre A0.  The stop test is global over the whole I x R block (lines 217-218)."""
    L, mu = compute_svd(Z)
    L, mu, lam, q = glambda(mu, L)
    R = Z.shape[0]
    Zt = Z + lam * np.eye(R)
    Wt = W + lam * A0
    alpha = 1.0
    A = A0.copy()
    Y = A0.copy()
    it = 0
    while True:
        grad = Y @ Zt - Wt
        if ((np.abs(grad * Y).max() <= delta_1 and grad.min() >= -delta_2)
                or it >= NESTEROV_MAX_INNER):
            break
        new_A = np.maximum(Y - grad / L, 0.0)
        new_alpha = update_alpha(alpha, q)
        beta = alpha * (1.0 - alpha) / (alpha * alpha + new_alpha)
        Y = (1.0 + beta) * new_A - beta * A
        A = new_A
        alpha = new_alpha
        it += 1
    if return_info:
        return A, dict(iters=it, L=L, mu=mu, lam=lam, q=q)
    return A


# --------------------------------------------------------------------------------------
# Normalisation, include/Normalize.hpp:53-174
# --------------------------------------------------------------------------------------

def choose_normalization_factor(constraints: Sequence[int]):
    """include/Normalize.hpp:53-67: first factor that is not orthogonal."""
    for i, c in enumerate(constraints):
        if c != ORTHOGONALITY:
            return False, i
    return True, 0


def normalize(weight: int, R: int, grams: List[np.ndarray], factors: List[np.ndarray]):
    """Literal restatement of include/Normalize.hpp:92-174, including its quirks: the
    column loop runs j < N-1 and skips j == weight (so the last factor is not
    normalised when weight < N-1), and ``nonZeroFlag`` reflects only the last j.
    Mutates ``grams`` and ``factors`` in place."""
    N = len(factors)
    last = N - 1
    pass_flag = 0
    cumul_power = 1.0
    non_zero = True
    norm_mats = [None] * N
    lambda_fac = [None] * last
    norm_factor = [0.0] * last
    for i in range(N):
        if i != weight:
            norm_factor[i - pass_flag] = 1.0
            lambda_fac[i - pass_flag] = np.diag(grams[i]).copy()
            norm_mats[i] = np.zeros((R, R))
        else:
            norm_mats[i] = np.ones((R, R))
            pass_flag = 1
    for i in range(R):
        for j in range(last):
            norm_factor[j] = math.sqrt(lambda_fac[j][i])
            non_zero = not (norm_factor[j] == 0)
        if not non_zero:
            for j in range(last):
                lambda_fac[j][i] = 1.0
        else:
            pass_flag = 0
            for j in range(last):
                if j == weight:
                    pass_flag = 1
                    continue
                with np.errstate(divide="ignore", invalid="ignore"):
                    factors[j][:, i] *= 1.0 / norm_factor[j - pass_flag]
                cumul_power *= norm_factor[j - pass_flag]
                lambda_fac[j - pass_flag][i] = norm_factor[j - pass_flag]
            factors[weight][:, i] *= cumul_power
            cumul_power = 1.0
    pass_flag = 0
    for i in range(last):
        if i == weight:
            pass_flag = 1
            continue
        lf = lambda_fac[i - pass_flag]
        norm_mats[i] = np.outer(lf, lf)
        norm_mats[weight] = norm_mats[weight] * norm_mats[i]
        with np.errstate(divide="ignore", invalid="ignore"):
            grams[i] = grams[i] / norm_mats[i]
    grams[weight] = grams[weight] * norm_mats[weight]


# --------------------------------------------------------------------------------------
# CPD-ALS driver, include/Cpd.hpp:131-356 (sequential) and include/CpdOpenMP.hpp:266-329
# --------------------------------------------------------------------------------------

def update_factor(idx: int, constraint: int, M: np.ndarray, Z: np.ndarray,
                  A: np.ndarray, delta_1: float, delta_2: float):
    """include/Cpd.hpp:189-228.  Returns (new_factor, info)."""
    info = {}
    if constraint == UNCONSTRAINED:
        A_new = M @ np.linalg.inv(Z)                                    # :196-199
    elif constraint == NONNEGATIVITY:
        A_new, info = nesterov_mnls(Z, M, delta_1, delta_2, A, return_info=True)  # :202-205
        if np.abs(A_new).sum(axis=0).min() == 0:                         # :206-207
            A_new = 0.9 * A_new + 0.1 * A
            info["repaired"] = True
    elif constraint == ORTHOGONALITY:
        w, V = np.linalg.eigh(M.T @ M)                                   # :210-217
        A_new = M @ (V @ np.diag(1.0 / np.sqrt(w)) @ V.T)
    else:                                                                # sparsity/constant
        A_new = A
    return A_new, info


def cpd_als(X: np.ndarray, R: int, options: Optional[Options] = None,
            factors_init: Optional[Sequence[np.ndarray]] = None,
            cost: str = "residual") -> Status:
    """Restates ``CPD<Tensor_, seq>::als`` (include/Cpd.hpp:288-356) with the
    ``factorsInit`` entry (include/Cpd.hpp:534-577).

    ``cost="residual"`` uses the explicit residual of include/Cpd.hpp:131-149;
    ``cost="gram"`` uses the Gram form of include/CUDA/CpdCUDA.hpp:137-142 (identical in
    exact arithmetic).  Acceleration follows include/Cpd.hpp:247-278 (its cost,
    include/Cpd.hpp:162-169, is <X, [[A_acc]]> through one more last-mode MTTKRP, as in
    include/CpdOpenMP.hpp:223-255)."""
    X = np.asarray(X, dtype=np.float64)
    N = X.ndim
    last = N - 1
    if options is None:
        options = Options(order=N)
    opts = dataclasses.replace(options, constraints=list(options.constraints))
    st = Status(options=opts, factors=[np.array(f, dtype=np.float64, copy=True) for f in factors_init])
    grams = [f.T @ f for f in st.factors]                               # :292-296
    all_orth, weight = True, 0
    if opts.normalization:
        all_orth, weight = choose_normalization_factor(opts.constraints)  # :303-306
    st.frob_tns = square_norm(X)                                         # :309
    Xl = matricization(X, last)
    st.f_value = math.sqrt(((Xl - st.factors[last] @ partial_khatri_rao(st.factors, last).T) ** 2).sum())
    st.rel_costFunction = st.f_value / math.sqrt(st.frob_tns)
    old_factors = None
    while True:
        st.ao_iter += 1                                                  # :316
        sweep = dict(iter=st.ao_iter, nesterov_iters=[], accel=None)
        for i in range(N):
            M = mttkrp(st.factors, X, i)                                 # :322
            Z = partial_cwise_prod(grams, i)                             # :323
            A_new, info = update_factor(i, opts.constraints[i], M, Z, st.factors[i],
                                        opts.nesterov_delta_1, opts.nesterov_delta_2)
            st.factors[i] = A_new
            grams[i] = A_new.T @ A_new                                   # :227
            sweep["nesterov_iters"].append(info.get("iters", 0))
            if i == last:                                                # :329-330
                if cost == "residual":
                    KR = partial_khatri_rao(st.factors, last)
                    st.f_value = math.sqrt(((Xl - A_new @ KR.T) ** 2).sum())
                else:
                    f2 = st.frob_tns - 2.0 * (M * A_new).sum() + (Z * grams[last]).sum()
                    st.f_value = math.sqrt(max(f2, 0.0))
        st.rel_costFunction = st.f_value / math.sqrt(st.frob_tns)        # :333
        if opts.normalization and not all_orth:                          # :334-335
            normalize(weight, R, grams, st.factors)
        sweep["f_value"] = st.f_value
        sweep["rel"] = st.rel_costFunction
        if st.rel_costFunction < opts.threshold_error or st.ao_iter >= opts.max_iter:  # :339
            st.trace.append(sweep)
            break
        if opts.acceleration:                                            # :346-354
            norm_factors = [f.copy() for f in st.factors]
            if st.ao_iter > 1:
                sweep["accel"] = _line_search_accel(X, st, old_factors, grams)
            old_factors = norm_factors
        st.trace.append(sweep)
    return st


def _line_search_accel(X, st: Status, old_factors, grams):
    """include/Cpd.hpp:247-278."""
    opts = st.options
    N = len(st.factors)
    last = N - 1
    step = (st.ao_iter + 1) ** (1.0 / opts.accel_coeff)
    acc = [old_factors[i] + step * (st.factors[i] - old_factors[i]) for i in range(N)]
    acc_g = [a.T @ a for a in acc]
    M = mttkrp(acc, X, last)
    f2 = st.frob_tns + (partial_cwise_prod(acc_g, last) * acc_g[last]).sum() - 2.0 * (M * acc[last]).sum()
    f_acc = math.sqrt(max(f2, 0.0))
    ok = st.f_value > f_acc
    if ok:
        st.factors = acc
        for i in range(N):
            grams[i] = acc_g[i]
        st.f_value = f_acc
    else:
        opts.accel_fail += 1
    if opts.accel_fail == 5:
        opts.accel_fail = 0
        opts.accel_coeff += 1
    return dict(step=step, f_accel=f_acc, accepted=ok)


def cost_from_factors(X: np.ndarray, factors: Sequence[np.ndarray]) -> float:
    """||X - [[A_0..A_{N-1}]]||_F, used to score a result independently of the solver."""
    last = X.ndim - 1
    Xl = matricization(np.asarray(X, np.float64), last)
    return math.sqrt(((Xl - factors[last] @ partial_khatri_rao(factors, last).T) ** 2).sum())


def congruence(A: Sequence[np.ndarray], B: Sequence[np.ndarray]) -> float:
    """Factor congruence after optimal column permutation (Hungarian assignment on the
    product of per-mode absolute cosine matrices); the mean over columns is returned."""
    from scipy.optimize import linear_sum_assignment
    R = A[0].shape[1]
    C = np.ones((R, R))
    for a, b in zip(A, B):
        an = a / np.maximum(np.linalg.norm(a, axis=0), 1e-300)
        bn = b / np.maximum(np.linalg.norm(b, axis=0), 1e-300)
        C *= np.abs(an.T @ bn)
    r, c = linear_sum_assignment(-C)
    return float(C[r, c].mean())


# --------------------------------------------------------------------------------------
# Dimension-tree CPD, include/CpdDimTree.hpp:317-401 with include/DimTrees.hpp
# --------------------------------------------------------------------------------------

def dimtree_split(order: int) -> int:
    """Labels of the root's left child: the first (1 + L)/2 modes (DIM_HALF_SIZE,
    include/DimTrees.hpp:274-276); 4-way gives {0,1} | {2,3}."""
    return (1 + order) // 2


def dimtree_partial(factors: Sequence[np.ndarray], X: np.ndarray, keep: Sequence[int]) -> np.ndarray:
    """Partial MTTKRP of a tree node: X contracted with the factors of every mode not in
    ``keep`` (TreeMode_N_Product + TTVs, include/DimTrees.hpp:669-800), returned as an
    array of shape [I_keep..., R]."""
    N = X.ndim
    letters = "abcdefgh"[:N]
    spec = letters + "," + ",".join(f"{letters[k]}z" for k in range(N) if k not in keep)
    spec += "->" + "".join(letters[k] for k in keep) + "z"
    return np.einsum(spec, X, *[factors[k] for k in range(N) if k not in keep], optimize=True)


def dimtree_leaf_mttkrp(T: np.ndarray, factors: Sequence[np.ndarray], keep: Sequence[int], mode: int):
    """Leaf step: the node tensor T [I_keep..., R] contracted with the node's other
    factors (TTVs with TensorPartialProduct_R, include/TensorOperations.hpp:196-213)."""
    if len(keep) == 1:
        return T
    letters = "abcdefgh"[:len(keep)]
    pos = list(keep).index(mode)
    spec = letters + "z," + ",".join(f"{letters[i]}z" for i, k in enumerate(keep) if k != mode)
    spec += "->" + letters[pos] + "z"
    return np.einsum(spec, T, *[factors[k] for k in keep if k != mode], optimize=True)


def cpd_dimtree_als(X: np.ndarray, R: int, options: Optional[Options] = None,
                    factors_init: Optional[Sequence[np.ndarray]] = None) -> Status:
    """CPD_DIMTREE::als (include/CpdDimTree.hpp:317-401): the same ALS sweep as cpd_als with
    each MTTKRP taken from the node tensor of its half of the tree (the left node is
    recomputed before mode 0 from the current right-half factors, the right node before the
    first right-half mode from the updated left-half factors), the Gram-form cost
    (include/CpdDimTree.hpp:156-160) and the dimension-tree Normalize
    (include/Normalize.hpp:200-303, same arithmetic as Normalize)."""
    X = np.asarray(X, dtype=np.float64)
    N = X.ndim
    last = N - 1
    h = dimtree_split(N)
    left, right = list(range(h)), list(range(h, N))
    if options is None:
        options = Options(order=N)
    opts = dataclasses.replace(options, constraints=list(options.constraints))
    st = Status(options=opts, factors=[np.array(f, dtype=np.float64, copy=True) for f in factors_init])
    grams = [f.T @ f for f in st.factors]
    all_orth, weight = True, 0
    if opts.normalization:
        all_orth, weight = choose_normalization_factor(opts.constraints)
    st.frob_tns = square_norm(X)
    st.f_value = cost_from_factors(X, st.factors)                      # CpdGen, :333-338
    st.rel_costFunction = st.f_value / math.sqrt(st.frob_tns)
    old_factors = None
    while True:
        st.ao_iter += 1
        sweep = dict(iter=st.ao_iter, nesterov_iters=[], accel=None)
        T = None
        for i in range(N):
            if i == 0:
                T = dimtree_partial(st.factors, X, left)
            elif i == h:
                T = dimtree_partial(st.factors, X, right)
            keep = left if i < h else right
            M = dimtree_leaf_mttkrp(T, st.factors, keep, i)
            Z = partial_cwise_prod(grams, i)
            A_new, info = update_factor(i, opts.constraints[i], M, Z, st.factors[i],
                                        opts.nesterov_delta_1, opts.nesterov_delta_2)
            st.factors[i] = A_new
            grams[i] = A_new.T @ A_new
            sweep["nesterov_iters"].append(info.get("iters", 0))
            if i == last:
                f2 = st.frob_tns - 2.0 * (M * A_new).sum() + (Z * grams[last]).sum()
                st.f_value = math.sqrt(max(f2, 0.0))
        st.rel_costFunction = st.f_value / math.sqrt(st.frob_tns)
        if opts.normalization and not all_orth:
            normalize(weight, R, grams, st.factors)
        sweep["f_value"] = st.f_value
        sweep["rel"] = st.rel_costFunction
        if st.ao_iter >= opts.max_iter or st.rel_costFunction < opts.threshold_error:
            st.trace.append(sweep)
            break
        if opts.acceleration:
            norm_factors = [f.copy() for f in st.factors]
            if st.ao_iter > 1:
                sweep["accel"] = _line_search_accel(X, st, old_factors, grams)
            old_factors = norm_factors
        st.trace.append(sweep)
    return st
