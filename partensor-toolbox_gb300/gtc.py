"""Host-side mirror of Partensor's sparse completion interface on top of libptg.

``gtc(Ratings_Base_T, options)`` follows ``partensor::gtc(execution::cuda, Ratings_Base_T,
options)`` and ``gtc_stochastic`` (include/Gtc.hpp:655-757, include/GtcStochastic.hpp:640-742):
the (N+1) x nnz FP64 matrix holds the indices (as doubles) and, in its last row, the values;
``SparseOptions`` carries the fields of include/PARTENSOR_basic.hpp:341-418 with the
defaults of :221-270.  The solve runs in libptg (``ptg_gtc``) on the GPU.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GtcOptions, GtcResult, SweepTrace, check
from .cpd import Context, default_context


@dataclasses.dataclass
class SparseOptions:
    order: int = 3
    rank: int = 2
    tnsDims: Optional[List[int]] = None
    nonZeros: int = 0
    threshold_error: float = 1e-3
    max_nesterov_iter: int = 20
    max_iter: int = 20
    c_stochastic_perc: float = 0.5
    lambdas: Optional[List[float]] = None
    seed: int = 0
    factorsInit: Optional[List[np.ndarray]] = None
    constraints: Optional[List[int]] = None   # default nonnegativity on every mode

    def __post_init__(self):
        if self.lambdas is None:
            self.lambdas = [0.01] * self.order
        if self.constraints is None:
            self.constraints = [1] * self.order


@dataclasses.dataclass
class SparseStatus:
    options: SparseOptions
    factors: List[np.ndarray]
    frob_tns: float = 0.0
    f_value: float = 0.0
    rel_costFunction: float = 0.0
    ao_iter: int = 0
    epochs: int = 0
    seconds_setup: float = 0.0
    seconds: float = 0.0
    trace: list = dataclasses.field(default_factory=list)


def _run(idx, vals, options: SparseOptions, stochastic: bool, ctx: Optional[Context],
         device_ptrs: Optional[tuple] = None) -> SparseStatus:
    ctx = ctx or default_context()
    lib = ctx._lib
    N = options.order
    dims = [int(d) for d in options.tnsDims]
    R = int(options.rank)
    if device_ptrs is None:
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float32)
        nnz = vals.shape[0]
        p_idx, p_vals, on_dev = idx.ctypes.data_as(ctypes.c_void_p), vals.ctypes.data_as(ctypes.c_void_p), 0
    else:
        p_idx, p_vals, nnz = device_ptrs
        p_idx, p_vals, on_dev = ctypes.c_void_p(int(p_idx)), ctypes.c_void_p(int(p_vals)), 1
    o = GtcOptions()
    lib.ptg_gtc_default_options(N, ctypes.byref(o))
    o.threshold_error = options.threshold_error
    o.max_nesterov_iter = options.max_nesterov_iter
    o.max_iter = options.max_iter
    o.c_stochastic_perc = options.c_stochastic_perc
    for k in range(N):
        o.lambdas[k] = options.lambdas[k]
        o.constraints[k] = int(options.constraints[k])
    o.stochastic = int(stochastic)
    o.seed = options.seed
    if options.factorsInit is None:
        rng = np.random.default_rng(options.seed)
        inits = [rng.random((I, R)) for I in dims]
    else:
        inits = options.factorsInit
    inits = [np.asfortranarray(np.asarray(f, dtype=np.float64)) for f in inits]
    outs = [np.zeros((dims[k], R), order="F") for k in range(N)]
    dp = ctypes.POINTER(ctypes.c_double)
    ip = (dp * N)(*[a.ctypes.data_as(dp) for a in inits])
    op = (dp * N)(*[a.ctypes.data_as(dp) for a in outs])
    res = GtcResult()
    trace = (SweepTrace * options.max_iter)()
    d = (ctypes.c_int64 * N)(*dims)
    check(lib.ptg_gtc(ctx.handle, N, d, int(nnz), p_idx, p_vals, on_dev, R, ctypes.byref(o), ip, op,
                      ctypes.byref(res), trace))
    st = SparseStatus(options=options, factors=outs, frob_tns=res.frob_tns, f_value=res.f_value,
                      rel_costFunction=res.rel_costFunction, ao_iter=res.ao_iter, epochs=res.epochs,
                      seconds_setup=res.seconds_setup, seconds=res.seconds_total)
    n_ev = res.epochs if stochastic else res.ao_iter
    for i in range(min(n_ev, options.max_iter)):
        st.trace.append(dict(f_value=trace[i].f_value, rel=trace[i].rel_costFunction, seconds=trace[i].seconds))
    return st


def _split(Ratings_Base_T: np.ndarray, order: int):
    M = np.asarray(Ratings_Base_T, dtype=np.float64)
    return M[:order].astype(np.int64), M[order]


def gtc(Ratings_Base_T: np.ndarray, options: SparseOptions, ctx: Optional[Context] = None) -> SparseStatus:
    """partensor::gtc(execution::cuda, Ratings_Base_T, options)."""
    idx, vals = _split(Ratings_Base_T, options.order)
    return _run(idx, vals, options, False, ctx)


def gtc_stochastic(Ratings_Base_T: np.ndarray, options: SparseOptions, ctx: Optional[Context] = None) -> SparseStatus:
    """partensor::gtc_stochastic(execution::cuda, Ratings_Base_T, options)."""
    idx, vals = _split(Ratings_Base_T, options.order)
    return _run(idx, vals, options, True, ctx)


def gtc_coo(idx: np.ndarray, vals: np.ndarray, options: SparseOptions, stochastic: bool = False,
            ctx: Optional[Context] = None) -> SparseStatus:
    """Same solve from int32 COO indices [N][nnz] and FP32 values (the device-native form)."""
    return _run(idx, vals, options, stochastic, ctx)


def gtc_device(idx_dev_ptr: int, vals_dev_ptr: int, nnz: int, options: SparseOptions, stochastic: bool = False,
               ctx: Optional[Context] = None) -> SparseStatus:
    """Same solve from device-resident int32 COO indices [N][nnz] and FP32 values (no host copy)."""
    return _run(None, None, options, stochastic, ctx, device_ptrs=(idx_dev_ptr, vals_dev_ptr, nnz))


def sort_mode(ctx: Context, idx_dev_ptr: int, dims: Sequence[int], nnz: int, mode: int, perm_dev_ptr: int):
    """Mode-n order of the entries (``ptg_gtc_sort_mode``), device pointers."""
    d = (ctypes.c_int64 * len(dims))(*dims)
    check(ctx._lib.ptg_gtc_sort_mode(ctx.handle, len(dims), d, nnz, ctypes.c_void_p(idx_dev_ptr), mode,
                                     ctypes.c_void_p(perm_dev_ptr)))
