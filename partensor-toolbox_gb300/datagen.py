"""Seeded synthetic CPD problems (the counterpart of the reference's DataGeneration.hpp).

The reference seeds every generator from the clock (include/DataGeneration.hpp:60,86),
so its data cannot be reproduced; these generators are seeded instead.  They run on any
torch device: on a GPU the tensor is built in place in HBM (no host round trip), on the
CPU they produce the same shapes for the tests.

A tensor is returned as a flat, contiguous float64 buffer in ColMajor order (i0 fastest),
which is the memory layout of ``partensor::Tensor<N>`` (include/Tensor.hpp:64).  Factor k
is an I_k x R matrix; ``factors_colmajor`` flattens it the way Eigen's MatrixXd stores it.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import List, Sequence

import torch


@dataclasses.dataclass
class CpdProblem:
    dims: List[int]
    rank: int
    X: torch.Tensor                 # flat float64, ColMajor
    true_factors: List[torch.Tensor]
    init_factors: List[torch.Tensor]
    noise_rel: float                # ||noise||_F / ||X||_F, the best achievable relative error
    frob: float                     # ||X||_F^2


def full_tensor(factors: Sequence[torch.Tensor]) -> torch.Tensor:
    """[[A_0, ..., A_{N-1}]] as a flat ColMajor buffer: X[i0 + I0*j] = sum_r A0[i0,r] KR[j,r]
    with KR = KhatriRao(A_{N-1}, ..., A_1) (first argument slowest)."""
    kr = factors[-1]
    for A in reversed(factors[1:-1]):
        kr = (kr[:, None, :] * A[None, :, :]).reshape(-1, kr.shape[1])
    # row-major (J, I0) == ColMajor (I0, J)
    return (kr @ factors[0].T).reshape(-1)


def _rand(shape, g, device):
    return torch.rand(shape, generator=g, device=device, dtype=torch.float64)


def make_cpd_problem(dims: Sequence[int], rank: int, seed: int, snr_db: float,
                     init_seed: int | None = None, equalize_columns: bool = False,
                     collinearity: float | None = None, device="cpu") -> CpdProblem:
    """Ground truth i.i.d. U[0,1] factors (seed ``seed``); X = [[A]] + Gaussian noise at
    ``snr_db`` dB SNR, sigma^2 = ||[[A]]||^2 / (prod(I) * 10^(snr/10)); initial factors
    i.i.d. U[0,1] (seed ``init_seed``, default seed+1).

    ``equalize_columns`` rescales every column of a factor to the same norm (the mean
    column norm of the draw, so the entries keep the U[0,1] scale that the reference's
    absolute Nesterov tolerance, include/PARTENSOR_basic.hpp:188, is tuned for).
    ``collinearity=c`` makes the columns of each factor share a common component so the
    expected cosine between two columns is about c."""
    dims = [int(d) for d in dims]
    g = torch.Generator(device=device).manual_seed(int(seed))
    facs = []
    for I in dims:
        A = _rand((I, rank), g, device)
        if collinearity is not None:
            common = _rand((I, 1), g, device)
            # mix weight w so that the cosine of two columns is ~c (U[0,1] columns already
            # have cosine ~0.75; blend the centred part with a shared column)
            Ac = A - A.mean(0, keepdim=True)
            w = math.sqrt(collinearity / max(1e-12, 1.0 - collinearity))
            A = Ac + w * (common - common.mean()) * (Ac.norm(dim=0, keepdim=True) /
                                                      (common - common.mean()).norm())
            A = A - A.min(0, keepdim=True).values      # back to nonnegative
        if equalize_columns:
            # every column rescaled to the mean column norm of the draw (keeps the U[0,1] scale)
            nrm = A.norm(dim=0, keepdim=True)
            A = A * (nrm.mean() / nrm)
        facs.append(A)
    T = full_tensor(facs)
    t2 = float((T * T).sum())
    sigma = math.sqrt(t2 / (T.numel() * 10.0 ** (snr_db / 10.0)))
    noise = torch.randn(T.shape, generator=g, device=device, dtype=torch.float64) * sigma
    X = T + noise
    del T
    n2 = float((noise * noise).sum())
    del noise
    x2 = float((X * X).sum())
    gi = torch.Generator(device=device).manual_seed(int(seed + 1 if init_seed is None else init_seed))
    init = [_rand((I, rank), gi, device) for I in dims]
    return CpdProblem(dims, rank, X, facs, init, math.sqrt(n2 / x2), x2)


@dataclasses.dataclass
class HostCpdProblem:
    dims: List[int]
    rank: int
    X: "np.ndarray"                 # flat float64, ColMajor
    true_factors: list              # numpy I_k x R
    init_factors: list              # numpy I_k x R
    noise_rel: float
    frob: float


NOISE_CHUNKS = 64   # fixed, so the draw does not depend on the number of host threads


def make_cpd_problem_host(dims: Sequence[int], rank: int, seed: int, snr_db: float,
                          init_seed: int | None = None, equalize_columns: bool = False,
                          threads: int | None = None) -> HostCpdProblem:
    """The problem of ``make_cpd_problem`` drawn with numpy's PCG64 on the host, so the same
    seed gives the same tensor on every machine (x86 or Arm, any core count): factors
    i.i.d. U[0,1] from ``seed`` (columns equalised on request), X = [[A]] + Gaussian noise at
    ``snr_db`` dB, the noise drawn in NOISE_CHUNKS contiguous pieces from child seeds of
    ``SeedSequence([seed, 1])`` (filled by a thread pool; the pieces do not depend on the
    pool size), initial factors U[0,1] from ``init_seed`` (default seed + 1)."""
    import concurrent.futures as cf
    import numpy as np
    dims = [int(d) for d in dims]
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    facs = []
    for I in dims:
        A = rng.random((I, rank))
        if equalize_columns:
            nrm = np.linalg.norm(A, axis=0, keepdims=True)
            A = A * (nrm.mean() / nrm)
        facs.append(A)
    kr = facs[-1]
    for A in reversed(facs[1:-1]):
        kr = (kr[:, None, :] * A[None, :, :]).reshape(-1, rank)
    total = int(np.prod(dims))
    X = np.empty(total, dtype=np.float64)
    Xv = X.reshape(-1, dims[0])                       # row-major (J, I0) == ColMajor (I0, J)
    rows_per = max(1, (kr.shape[0] + 63) // 64)
    nthr = threads or os.cpu_count() or 1

    def build(j0):
        j1 = min(kr.shape[0], j0 + rows_per)
        np.matmul(kr[j0:j1], facs[0].T, out=Xv[j0:j1])
        seg = Xv[j0:j1].reshape(-1)
        return float(np.dot(seg, seg))

    with cf.ThreadPoolExecutor(nthr) as ex:
        t2 = sum(ex.map(build, range(0, kr.shape[0], rows_per)))
    del kr
    sigma = math.sqrt(t2 / (total * 10.0 ** (snr_db / 10.0)))
    children = np.random.SeedSequence([int(seed), 1]).spawn(NOISE_CHUNKS)
    step = (total + NOISE_CHUNKS - 1) // NOISE_CHUNKS

    def noise(c):
        lo, hi = c * step, min(total, (c + 1) * step)
        if lo >= hi:
            return 0.0, 0.0
        g = np.random.Generator(np.random.PCG64(children[c]))
        n = g.standard_normal(hi - lo)
        n *= sigma
        seg = X[lo:hi]
        seg += n
        return float(np.dot(n, n)), float(np.dot(seg, seg))

    with cf.ThreadPoolExecutor(nthr) as ex:
        parts = list(ex.map(noise, range(NOISE_CHUNKS)))
    n2 = sum(p[0] for p in parts)
    x2 = sum(p[1] for p in parts)
    gi = np.random.Generator(np.random.PCG64(int(seed + 1 if init_seed is None else init_seed)))
    init = [gi.random((I, rank)) for I in dims]
    return HostCpdProblem(dims, rank, X, facs, init, math.sqrt(n2 / x2), x2)


def factors_colmajor(A: torch.Tensor) -> torch.Tensor:
    """Eigen ColMajor storage of an I x R matrix: element (i, r) at i + I*r."""
    return A.t().contiguous().reshape(-1)


def from_colmajor(buf: torch.Tensor, rows: int, cols: int) -> torch.Tensor:
    return buf.reshape(cols, rows).t()


@dataclasses.dataclass
class BatchInstance:
    X: "np.ndarray"                 # float64 [I0, I1, I2]
    rank: int
    init_factors: list
    true_factors: list
    noise_rel: float


def make_fmri_batch(n: int = 256, seed: int = 4, snr_db: float = 15.0,
                    voxels=(32, 128), time=(100, 400), trials=(16, 64), ranks=(8, 12, 16, 24),
                    init_seed: int | None = None) -> list:
    """Uneven fMRI-like CPD instances (voxels x time x subjects-trials): per instance the
    dims are drawn uniformly from the three ranges and the rank from ``ranks``; spatial
    maps are nonnegative and sparse (Bernoulli(0.2) x U[0,1]), temporal factors are white
    noise filtered by a Gaussian kernel of width 5 (shifted to be nonnegative), trial
    loadings are U[0,1]; Gaussian noise at ``snr_db``.  Initial factors U[0,1] from
    ``init_seed`` (default seed + 1).  Seeded numpy generators; host FP64 tensors."""
    import numpy as np
    rng = np.random.default_rng(seed)
    rng_init = np.random.default_rng(seed + 1 if init_seed is None else init_seed)
    t = np.arange(-15, 16)
    kern = np.exp(-0.5 * (t / 5.0) ** 2)
    kern /= kern.sum()
    out = []
    for _ in range(n):
        I0 = int(rng.integers(voxels[0], voxels[1] + 1))
        I1 = int(rng.integers(time[0], time[1] + 1))
        I2 = int(rng.integers(trials[0], trials[1] + 1))
        R = int(ranks[int(rng.integers(0, len(ranks)))])
        S = (rng.random((I0, R)) < 0.2) * rng.random((I0, R))
        # a column that drew no voxel gets one, so every component is present
        for r in np.nonzero(S.sum(0) == 0)[0]:
            S[int(rng.integers(0, I0)), r] = rng.random()
        W = rng.standard_normal((I1 + len(t) - 1, R))
        Tm = np.stack([np.convolve(W[:, r], kern, mode="valid") for r in range(R)], axis=1)
        Tm = Tm - Tm.min(0, keepdims=True)
        C = rng.random((I2, R))
        X = np.einsum("ir,jr,kr->ijk", S, Tm, C)
        sigma = np.sqrt((X ** 2).sum() / (X.size * 10 ** (snr_db / 10)))
        noise = sigma * rng.standard_normal(X.shape)
        Xn = np.asfortranarray(X + noise)   # ColMajor, the layout the C ABI reads without a copy
        noise_rel = float(np.linalg.norm(noise) / np.linalg.norm(Xn))
        init = [rng_init.random((I, R)) for I in (I0, I1, I2)]
        out.append(BatchInstance(Xn, R, init, [S, Tm, C], noise_rel))
    return out
