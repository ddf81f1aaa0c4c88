"""FP64 CPU oracle for sparse tensor completion (GTC) -- TEST INFRASTRUCTURE ONLY.

Restates in numpy float64 (paths relative to the reference project's root):
  - the per-mode sparse matricisation: sort by SortRows (include/TensorOperations.hpp:622-666)
    then FillSparseMatricization (:432-487) into a column-compressed matrix whose column is
    i_n and whose row is the linear index of the other modes (first other mode fastest);
    calculate_offsets (include/Gtc.hpp:259-273);
  - SparseMTTKRP (include/MTTKRP.hpp:229-267), which writes -M_n^T;
  - local_L::NesterovMNLS (include/NesterovMNLS.hpp:777-873) with PowerMethod (:131-160);
  - the GTC cost (include/Gtc.hpp:184-214) and aogtc (include/Gtc.hpp:430-490);
  - dynamic_blocksize::StochasticNesterovMNLS (include/NesterovMNLS.hpp:431-547) and
    aogtc_stochastic (include/GtcStochastic.hpp:409-481).

Deliberate restatement choices (the reference's versions are not reproducible):
  - PowerMethod starts from the all-ones vector instead of Matrix::Random (time-seeded);
  - the stochastic pivot is a counter-based hash of (seed, outer iteration, mode, inner
    iteration, row) instead of std::rand() after std::srand(time(nullptr));
  - no BalanceDataset permutation (include/TensorOperations.hpp:679-748): it is a random
    relabelling of indices for load balance and does not change the algorithm.
Parity status: unpinned (the reference ships no GTC fixtures and cannot be built here).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class SparseOptions:
    """partensor::SparseOptions fields the GTC loop reads (include/PARTENSOR_basic.hpp:341-418)
    with SparseDefaultValues (:221-270)."""
    order: int = 3
    threshold_error: float = 1e-3
    max_nesterov_iter: int = 20
    max_iter: int = 20
    c_stochastic_perc: float = 0.5
    lambdas: Optional[List[float]] = None
    seed: int = 0
    constraints: Optional[List[int]] = None   # Constraint values (include/Constants.hpp:49-57)

    def __post_init__(self):
        if self.lambdas is None:
            self.lambdas = [0.01] * self.order
        if self.constraints is None:
            self.constraints = [NONNEGATIVITY] * self.order


UNCONSTRAINED, NONNEGATIVITY = 0, 1


@dataclasses.dataclass
class ModeMatrix:
    """One mode's column-compressed matricisation: nonzeros ordered by (i_n, linear other
    index); column i_n spans [ptr[i], ptr[i+1])."""
    mode: int
    ptr: np.ndarray        # int64 [I_n + 1]
    other: np.ndarray      # int64 [nnz, N-1] other-mode indices, modes in increasing order
    lin: np.ndarray        # int64 [nnz] linear other index
    vals: np.ndarray       # float64 [nnz]
    perm: np.ndarray       # int64 [nnz] position in the input of each sorted entry


def other_strides(dims: Sequence[int], mode: int) -> List[int]:
    """offsets of calculate_offsets (include/Gtc.hpp:259-273) and of the matr_mapping rows
    of FillSparseMatricization (include/TensorOperations.hpp:438-457)."""
    out, s = [], 1
    for k in range(len(dims)):
        if k == mode:
            continue
        out.append(s)
        s *= dims[k]
    return out


def sort_key(idx: np.ndarray, dims: Sequence[int], mode: int) -> np.ndarray:
    """Key whose ascending order is SortRows<N, mode>: i_mode first, then the other modes
    from the highest to the lowest (ties are impossible without duplicates)."""
    N = len(dims)
    lin = np.zeros(idx.shape[1], dtype=np.int64)
    for s, k in zip(other_strides(dims, mode), [k for k in range(N) if k != mode]):
        lin += idx[k].astype(np.int64) * s
    J = int(np.prod([dims[k] for k in range(N) if k != mode], dtype=np.int64))
    return idx[mode].astype(np.int64) * J + lin, lin


def matricize(idx: np.ndarray, vals: np.ndarray, dims: Sequence[int], mode: int) -> ModeMatrix:
    """sort_ratings_base_util<mode> (include/Gtc.hpp:69-110): std::sort with SortRows then
    FillSparseMatricization; duplicates (same index) keep the first entry (:481-485)."""
    key, lin = sort_key(idx, dims, mode)
    order = np.argsort(key, kind="stable")
    k_sorted = key[order]
    keep = np.ones(len(order), dtype=bool)
    keep[1:] = k_sorted[1:] != k_sorted[:-1]
    order = order[keep]
    rows = idx[mode][order].astype(np.int64)
    ptr = np.zeros(dims[mode] + 1, dtype=np.int64)
    np.add.at(ptr, rows + 1, 1)
    ptr = np.cumsum(ptr)
    others = np.stack([idx[k][order] for k in range(len(dims)) if k != mode], axis=1).astype(np.int64)
    return ModeMatrix(mode, ptr, others, lin[order], vals[order].astype(np.float64), order)


def kr_rows(factors: Sequence[np.ndarray], mm: ModeMatrix) -> np.ndarray:
    """Hadamard product of the factor rows of every other mode for each nonzero, in the
    reference's multiplication order (last mode first, include/MTTKRP.hpp:248-259)."""
    N = len(factors)
    others = [k for k in range(N) if k != mm.mode]
    out = np.ones((len(mm.vals), factors[0].shape[1]))
    for j in range(len(others) - 1, -1, -1):
        out = out * factors[others[j]][mm.other[:, j]]
    return out


def sparse_mttkrp(factors: Sequence[np.ndarray], mm: ModeMatrix) -> np.ndarray:
    """M_n (I_n x R) = sum over the column's nonzeros of x * kr; the reference stores
    -M_n^T (include/MTTKRP.hpp:263)."""
    kr = kr_rows(factors, mm) * mm.vals[:, None]
    I = len(mm.ptr) - 1
    rows = np.repeat(np.arange(I), np.diff(mm.ptr))
    M = np.zeros((I, factors[0].shape[1]))
    np.add.at(M, rows, kr)
    return M


def power_method(H: np.ndarray, eps: float) -> float:
    """Largest eigenvalue, include/NesterovMNLS.hpp:131-160, from the all-ones vector."""
    x = np.ones(H.shape[0])
    it = 0
    while True:
        Ax = H @ x
        x_new = Ax / (np.linalg.norm(Ax) + 1e-12)
        if np.linalg.norm(x_new - x) <= eps or it >= 10000:
            return float(x_new @ (H @ x_new))
        x = x_new
        it += 1


def row_hessians(factors: Sequence[np.ndarray], mm: ModeMatrix) -> np.ndarray:
    kr = kr_rows(factors, mm)
    I = len(mm.ptr) - 1
    R = kr.shape[1]
    H = np.zeros((I, R, R))
    for i in range(I):
        K = kr[mm.ptr[i]:mm.ptr[i + 1]]
        H[i] = K.T @ K
    return H


def local_L_nesterov(factors: List[np.ndarray], mm: ModeMatrix, M: np.ndarray, max_iter: int,
                     lam: float) -> np.ndarray:
    """local_L::NesterovMNLS (include/NesterovMNLS.hpp:777-873).  Row i: H_i = sum kr kr^T,
    L_i = PowerMethod(H_i, 1e-3) + lambda (:821-855); each iteration
    grad = H_i y - m_i + lambda y (the reference forms H_i y as sum (kr.y) kr), a' =
    max(y - grad / L_i, 0), beta = (1 - sqrt(lambda/L_i)) / (1 + sqrt(lambda/L_i)),
    y = (1 + beta) a' - beta a, a = a'.  No stop test: max_iter iterations."""
    A = factors[mm.mode].copy()
    H = row_hessians(factors, mm)
    I, R = A.shape
    Ls = np.array([power_method(H[i], 1e-3) + lam for i in range(I)])
    Y = A.copy()
    for _ in range(max_iter):
        grad = np.einsum("irs,is->ir", H, Y) - M + lam * Y
        new_A = np.maximum(Y - grad / Ls[:, None], 0.0)
        sq = np.sqrt(lam / Ls)
        beta = (1.0 - sq) / (1.0 + sq)
        Y = (1.0 + beta[:, None]) * new_A - beta[:, None] * A
        A = new_A
    return A


def ridge_update(factors: List[np.ndarray], mm: ModeMatrix, M: np.ndarray, lam: float) -> np.ndarray:
    """unconstraint_update (include/Gtc.hpp:275-315): row i = (H_i + lambda I)^{-1} m_i with
    H_i = sum kr kr^T and m_i = sum x kr over the row's entries."""
    H = row_hessians(factors, mm)
    R = H.shape[1]
    return np.stack([np.linalg.solve(H[i] + lam * np.eye(R), M[i]) for i in range(H.shape[0])])


def gtc_cost(factors: Sequence[np.ndarray], idx: np.ndarray, vals: np.ndarray) -> float:
    """sum over observed entries of (x - sum_r prod_k A_k(i_k, r))^2, include/Gtc.hpp:184-214."""
    pred = np.ones((idx.shape[1], factors[0].shape[1]))
    for k in range(len(factors) - 1, -1, -1):
        pred = pred * factors[k][idx[k]]
    return float(((vals - pred.sum(axis=1)) ** 2).sum())


@dataclasses.dataclass
class SparseStatus:
    factors: List[np.ndarray]
    frob_tns: float = 0.0
    f_value: float = 0.0
    rel_costFunction: float = 0.0
    ao_iter: int = 0
    trace: list = dataclasses.field(default_factory=list)


def gtc(idx: np.ndarray, vals: np.ndarray, dims: Sequence[int], R: int, options: SparseOptions,
        factors_init: Sequence[np.ndarray]) -> SparseStatus:
    """aogtc (include/Gtc.hpp:430-490, OpenMP form include/GtcOpenMP.hpp:381-543) with
    nonnegativity on every mode; acceleration off (SparseDefaultValues)."""
    N = len(dims)
    mms = [matricize(idx, vals, dims, n) for n in range(N)]
    st = SparseStatus(factors=[np.array(f, dtype=np.float64, copy=True) for f in factors_init])
    st.frob_tns = float((mms[0].vals ** 2).sum())
    st.f_value = gtc_cost(st.factors, idx, vals)
    st.rel_costFunction = st.f_value / st.frob_tns
    while True:
        st.ao_iter += 1
        for n in range(N):
            # update_factor's switch (include/Gtc.hpp:330-355): unconstrained -> ridge solve,
            # nonnegativity -> local_L Nesterov, every other constraint keeps the factor
            con = options.constraints[n]
            if con not in (UNCONSTRAINED, NONNEGATIVITY):
                continue
            M = sparse_mttkrp(st.factors, mms[n])
            if con == UNCONSTRAINED:
                st.factors[n] = ridge_update(st.factors, mms[n], M, options.lambdas[n])
            else:
                st.factors[n] = local_L_nesterov(st.factors, mms[n], M, options.max_nesterov_iter,
                                                 options.lambdas[n])
        st.f_value = gtc_cost(st.factors, idx, vals)
        st.rel_costFunction = st.f_value / st.frob_tns
        st.trace.append(dict(f_value=st.f_value, rel=st.rel_costFunction))
        if st.rel_costFunction < options.threshold_error or st.ao_iter >= options.max_iter:
            break
    return st


# ---- stochastic variant -------------------------------------------------------------

def pivot_hash(seed: int, outer: int, mode: int, inner: int, row: int) -> int:
    """Counter-based 64-bit mix (splitmix64 finaliser) of the draw coordinates; replaces
    std::rand() (include/NesterovMNLS.hpp:460,482).  Same arithmetic as the GPU sampler."""
    M64 = (1 << 64) - 1
    z = (seed * 0x9E3779B97F4A7C15 + outer * 0xBF58476D1CE4E5B9 + mode * 0x94D049BB133111EB
         + inner * 0x2545F4914F6CDD1D + row * 0x632BE59BD9B4E019) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def stochastic_nesterov(factors: List[np.ndarray], mm: ModeMatrix, c: float, max_iter: int, lam: float,
                        seed: int, outer: int) -> np.ndarray:
    """dynamic_blocksize::StochasticNesterovMNLS (include/NesterovMNLS.hpp:431-547).  Row i
    with nnz_i entries: b_i = floor(c * nnz_i); if b_i > 0, every inner iteration takes the
    contiguous block [pivot, pivot + b_i) of the row's sorted entries with
    pivot = draw % (nnz_i - b_i + 1) (:481-494), grad = sum (kr.y - x) kr + lambda (y + a)
    (literally, :516,525), H = sum kr kr^T of the block, L = PowerMethod(H, 1e-3) + lambda
    (:519-529), then the same projected step and beta as local_L."""
    n = mm.mode
    A = factors[n].copy()
    Y = A.copy()
    kr_all = kr_rows(factors, mm)
    I = len(mm.ptr) - 1
    for it in range(max_iter):
        for i in range(I):
            p0, p1 = int(mm.ptr[i]), int(mm.ptr[i + 1])
            nz = p1 - p0
            b = int(c * nz)
            if b <= 0:
                continue
            pivot = pivot_hash(seed, outer, n, it, i) % (nz - b + 1)
            K = kr_all[p0 + pivot:p0 + pivot + b]
            x = mm.vals[p0 + pivot:p0 + pivot + b]
            y = Y[i]
            grad = K.T @ (K @ y - x) + lam * (y + A[i])
            H = K.T @ K
            L = power_method(H, 1e-3) + lam
            new_a = np.maximum(y - grad / L, 0.0)
            sq = math.sqrt(lam / L)
            beta = (1.0 - sq) / (1.0 + sq)
            Y[i] = (1.0 + beta) * new_a - beta * A[i]
            A[i] = new_a
    return A


def gtc_stochastic(idx: np.ndarray, vals: np.ndarray, dims: Sequence[int], R: int, options: SparseOptions,
                   factors_init: Sequence[np.ndarray]) -> SparseStatus:
    """aogtc_stochastic (include/GtcStochastic.hpp:409-481): one outer iteration updates every
    mode with the stochastic solver; the cost is evaluated once per epoch,
    epoch = floor(nnz / (blocksize_0 * I_0)) + 1 with blocksize_n = floor(c * nnz / I_n) + 1
    (:431, :590); max_iter counts epochs."""
    N = len(dims)
    mms = [matricize(idx, vals, dims, n) for n in range(N)]
    nnz = len(mms[0].vals)
    st = SparseStatus(factors=[np.array(f, dtype=np.float64, copy=True) for f in factors_init])
    st.frob_tns = float((mms[0].vals ** 2).sum())
    st.f_value = gtc_cost(st.factors, idx, vals)
    st.rel_costFunction = st.f_value / st.frob_tns
    block0 = int(options.c_stochastic_perc * nnz / dims[0]) + 1
    epoch = int(nnz / (block0 * dims[0])) + 1
    epochs = 0
    while True:
        st.ao_iter += 1
        for n in range(N):
            # the stochastic update_factor (include/GtcStochastic.hpp:325-345) updates only the
            # nonnegative modes; every other constraint, unconstrained included, keeps the factor
            if options.constraints[n] != NONNEGATIVITY:
                continue
            st.factors[n] = stochastic_nesterov(st.factors, mms[n], options.c_stochastic_perc,
                                                options.max_nesterov_iter, options.lambdas[n],
                                                options.seed, st.ao_iter)
        if st.ao_iter % epoch == 0:
            epochs += 1
            st.f_value = gtc_cost(st.factors, idx, vals)
            st.rel_costFunction = st.f_value / st.frob_tns
            st.trace.append(dict(f_value=st.f_value, rel=st.rel_costFunction, iter=st.ao_iter))
        if st.rel_costFunction < options.threshold_error or epochs >= options.max_iter:
            break
    return st


def make_gtc_problem(dims: Sequence[int], nnz: int, R: int, seed: int, noise_rel: float = 0.1,
                     holdout: float = 0.0):
    """Seeded synthetic completion problem: entries sampled uniformly without replacement,
    values from a rank-R nonnegative U[0,1] model plus relative Gaussian noise."""
    rng = np.random.default_rng(seed)
    total = int(np.prod(dims, dtype=np.int64))
    flat = rng.choice(total, size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims, order="F")).astype(np.int64)
    A = [rng.random((I, R)) for I in dims]
    pred = np.ones((nnz, R))
    for k in range(len(dims) - 1, -1, -1):
        pred = pred * A[k][idx[k]]
    clean = pred.sum(axis=1)
    vals = clean * (1.0 + noise_rel * rng.standard_normal(nnz))
    return idx, vals, A
