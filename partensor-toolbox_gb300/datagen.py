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


def factors_colmajor(A: torch.Tensor) -> torch.Tensor:
    """Eigen ColMajor storage of an I x R matrix: element (i, r) at i + I*r."""
    return A.t().contiguous().reshape(-1)


def from_colmajor(buf: torch.Tensor, rows: int, cols: int) -> torch.Tensor:
    return buf.reshape(cols, rows).t()
