"""Host-side mirror of Partensor's dense CPD interface on top of libptg.

``cpd(tnsX, R, options, factorsInit)`` follows ``partensor::cpd(execution::cuda, ...)``
(include/Cpd.hpp:893-1171): same argument meaning, same ``Options`` fields and defaults
(include/PARTENSOR_basic.hpp:176-218, 283-336), a ``Status`` with the fields of
include/PARTENSOR_basic.hpp:556-595.  Tensors are float64 in ColMajor order (a numpy
array with ``order='F'`` of shape dims, or a flat buffer plus ``dims``); factor matrices
are I_k x R float64.  All compute runs in libptg on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os
import dataclasses
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import CpdInstance, CpdOptions, CpdResult, SweepTrace, check

UNCONSTRAINED, NONNEGATIVITY, ORTHOGONALITY, SPARSITY, CONSTANT = 0, 1, 2, 3, 4
DTYPES = {"f32": _lib.PTG_F32, "fp32": _lib.PTG_F32, "bf16": _lib.PTG_BF16, "fp8": _lib.PTG_FP8E4M3}


@dataclasses.dataclass
class Options:
    """partensor::Options (include/PARTENSOR_basic.hpp:283-336) plus the GB300 knobs."""
    order: int = 3
    constraints: Optional[List[int]] = None
    threshold_error: float = 1e-3
    nesterov_delta_1: float = 1e-2
    nesterov_delta_2: float = 1e-2
    max_iter: int = 20
    accel_coeff: int = 3
    accel_fail: int = 0
    acceleration: bool = True
    normalization: bool = True
    writeToFile: bool = False     # write the final factors (row-major FP64) when the loop stops
    final_factors_paths: Optional[List[str]] = None   # default "final_<k>.bin"
    # GB300 extensions
    precision: str = "f32"        # storage of the tensor in HBM: "f32", "bf16" or "fp8" (e4m3, slab scales)
    refine_sweeps: int = 0        # FP32 sweeps after the main loop (bf16 / fp8 storage)
    warm_start: bool = False      # learned warm start of the NNLS rows (needs warm_model)
    warm_model: object = None     # a WarmStartModel
    warm_log_sweeps: int = 5      # sweeps that log training pairs before the network is trained
    warm_train_steps: int = 200
    verify_fp32: bool = False     # report the final cost on an FP32 copy (bf16 / fp8 storage, no refinement)

    def __post_init__(self):
        if self.constraints is None:
            self.constraints = [NONNEGATIVITY] * self.order

    def to_c(self) -> CpdOptions:
        o = CpdOptions()
        _lib.load().ptg_cpd_default_options(self.order, ctypes.byref(o))
        for k in range(self.order):
            o.constraints[k] = int(self.constraints[k])
        o.threshold_error = self.threshold_error
        o.nesterov_delta_1 = self.nesterov_delta_1
        o.nesterov_delta_2 = self.nesterov_delta_2
        o.max_iter = int(self.max_iter)
        o.accel_coeff = int(self.accel_coeff)
        o.accel_fail = int(self.accel_fail)
        o.acceleration = int(bool(self.acceleration))
        o.normalization = int(bool(self.normalization))
        o.refine_sweeps = int(self.refine_sweeps)
        o.warm_start = int(bool(self.warm_start))
        o.warm_model = self.warm_model.handle if self.warm_model is not None else None
        o.warm_log_sweeps = int(self.warm_log_sweeps)
        o.warm_train_steps = int(self.warm_train_steps)
        o.verify_fp32 = int(bool(self.verify_fp32))
        o.write_to_file = int(bool(self.writeToFile))
        # the encoded paths must outlive the call that reads the struct: kept on the struct
        o._paths = [os.fsencode(p) if p is not None else None for p in (self.final_factors_paths or [])]
        for k, p in enumerate(o._paths[:_lib.MAX_ORDER]):
            o.final_factors_paths[k] = p
        return o


@dataclasses.dataclass
class Status:
    """partensor::Status (include/PARTENSOR_basic.hpp:556-595) plus a per-sweep trace."""
    options: Options
    factors: List[np.ndarray]
    frob_tns: float = 0.0
    f_value: float = 0.0
    rel_costFunction: float = 0.0
    ao_iter: int = 0
    refine_sweeps_done: int = 0
    nesterov_iters_total: int = 0
    seconds: float = 0.0
    trace: list = dataclasses.field(default_factory=list)


class Context:
    """A libptg context on one device (streams, events, workspace)."""

    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.ptg_ctx_create(int(device), ctypes.byref(h)))
        self.handle = h
        self.device = device

    def set_stream(self, stream_ptr: int | None):
        check(self._lib.ptg_ctx_set_stream(self.handle, ctypes.c_void_p(stream_ptr or 0)))

    def synchronize(self):
        check(self._lib.ptg_ctx_synchronize(self.handle))

    def set_mttkrp_impl(self, impl: str):
        """"auto" (tensor cores for BF16 storage), "cuda_cores" or "tensor_cores"."""
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_MTTKRP_IMPL, _lib.MTTKRP_IMPLS[impl]))

    def set_nnls_cluster(self, size: int):
        """CTAs of the NNLS cluster: 0 (auto), 2, 4, 8 or 16."""
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_NNLS_CLUSTER, int(size)))

    def set_gtc_rows(self, solver: str):
        """Row solver of the sparse completion's nonnegative modes: "auto" (one warp per row
        for rank <= 32, the row Hessian on the tensor cores when rank % 4 == 0), "cta" (one
        CTA per row) or "warp_fma" (one warp per row, the Hessian on the FMA pipe: the same
        bits as "cta")."""
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_GTC_ROWS,
                                           {"auto": 0, "cta": 1, "warp_fma": 2}[solver]))

    def set_spin_limit(self, polls: int):
        """Polls of the tensor-core kernels' bounded waits before they give up with
        PTG_ERR_TIMEOUT: -1 the default, 0 at once (exercises the failure path)."""
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_SPIN_LIMIT, int(polls)))

    def set_alloc_limit(self, nbytes: int):
        """Largest single device allocation the context may make (0: no limit); a larger
        one fails with PTG_ERR_OOM."""
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_ALLOC_LIMIT, int(nbytes)))

    def set_host_read(self, mode: str):
        """How a host FP64 source reaches the conversion kernels: "auto" (page-locked memory
        read in place by the BF16/FP32 conversion, everything else staged), "staged" (copied
        through device chunks) or "in_place" (read in place wherever the device can address
        the buffer, pageable memory included where the device walks the host's page tables).
        All store the same bits."""
        modes = {"auto": 0, "staged": 1, "in_place": 2}
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_HOST_READ, modes[mode]))

    def set_batched_impl(self, impl: str):
        """cpd_batched: "persistent" (one launch for the whole batch, the default) or "graphs"
        (one launch per ALS phase, each sweep a replayed CUDA graph)."""
        check(self._lib.ptg_ctx_set_option(self.handle, _lib.PTG_OPT_BATCHED_IMPL,
                                           {"persistent": 0, "graphs": 1}[impl]))

    def enable_stats(self, on: bool = True):
        check(self._lib.ptg_ctx_enable_stats(self.handle, int(on)))

    def reset_stats(self):
        check(self._lib.ptg_ctx_reset_stats(self.handle))

    def stats(self) -> dict:
        s = _lib.Stats()
        check(self._lib.ptg_ctx_get_stats(self.handle, ctypes.byref(s)))
        return dict(launches=s.launches, mttkrp_launches=s.mttkrp_launches, mttkrp_ms=s.mttkrp_ms,
                    mttkrp_bytes=s.mttkrp_bytes, mttkrp_flops=s.mttkrp_flops, tc_launches=s.tc_launches,
                    tc_ms=s.tc_ms, tc_bytes=s.tc_bytes, batch_pass_launches=s.batch_pass_launches,
                    batch_pass_ms=s.batch_pass_ms, batch_pass_bytes=s.batch_pass_bytes)

    def close(self):
        if self.handle:
            self._lib.ptg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Tensor:
    """A dense tensor resident in HBM (``ptg_tensor_create``).

    ``src`` is either a float64 numpy array (ColMajor: Fortran-ordered of shape ``dims``,
    or flat with ``dims`` given) or a ``(device_pointer, dims)`` pair of a float64
    ColMajor buffer already on the GPU."""

    def __init__(self, ctx: Context, src, dims: Sequence[int] | None = None, precision: str = "f32"):
        self.ctx = ctx
        self._lib = ctx._lib
        if isinstance(src, tuple):
            ptr, dims = src
            on_dev, p = 1, ctypes.cast(ctypes.c_void_p(int(ptr)), ctypes.POINTER(ctypes.c_double))
            self._keep = None
        else:
            a = np.asarray(src, dtype=np.float64)
            if dims is None:
                dims = a.shape
                a = np.asfortranarray(a).reshape(-1, order="F")
            else:
                a = np.ascontiguousarray(a.reshape(-1))
            on_dev, p = 0, _dptr(a)
            self._keep = a
        self.dims = [int(d) for d in dims]
        self.precision = precision
        d = (ctypes.c_int64 * len(self.dims))(*self.dims)
        h = ctypes.c_void_p()
        check(self._lib.ptg_tensor_create(ctx.handle, len(self.dims), d, DTYPES[precision], p, on_dev,
                                          ctypes.byref(h)))
        self.handle = h
        self._keep = None

    def norms(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        check(self._lib.ptg_tensor_norms(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def storage(self):
        """(device address of the stored entries, padded mode-0 extent, device address of the
        FP8 slab scales or None)"""
        d, s = ctypes.c_void_p(), ctypes.c_void_p()
        p0 = ctypes.c_int64()
        check(self._lib.ptg_tensor_storage(self.handle, ctypes.byref(d), ctypes.byref(p0), ctypes.byref(s)))
        return d.value, p0.value, s.value

    def close(self):
        if getattr(self, "handle", None):
            self._lib.ptg_tensor_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WarmStartModel:
    """The learned NNLS warm start (``ptg_mlp_*``): a 2 x 128 ReLU MLP on the device."""

    def __init__(self, ctx: Context, rank: int, seed: int = 0):
        self.ctx = ctx
        self._lib = ctx._lib
        h = ctypes.c_void_p()
        check(self._lib.ptg_mlp_create(ctx.handle, int(rank), int(seed), ctypes.byref(h)))
        self.handle = h
        self.rank = rank
        self.n = int(self._lib.ptg_mlp_num_params(h))

    def params(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.float32)
        check(self._lib.ptg_mlp_get_params(self.ctx.handle, self.handle, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self._lib.ptg_mlp_set_params(self.ctx.handle, self.handle, p.ctypes.data_as(ctypes.c_void_p)))

    def forward(self, X_ptr: int, rows: int, Y_ptr: int):
        check(self._lib.ptg_mlp_forward(self.ctx.handle, self.handle, ctypes.c_void_p(X_ptr), rows,
                                        ctypes.c_void_p(Y_ptr)))

    def loss_grad(self, X_ptr: int, T_ptr: int, rows: int, G_ptr: int) -> float:
        loss = ctypes.c_double()
        check(self._lib.ptg_mlp_loss_grad(self.ctx.handle, self.handle, ctypes.c_void_p(X_ptr),
                                          ctypes.c_void_p(T_ptr), rows, ctypes.byref(loss), ctypes.c_void_p(G_ptr)))
        return loss.value

    def train(self, X_ptr: int, T_ptr: int, rows: int, steps: int, batch: int = 256, lr: float = 1e-3,
              seed: int = 0) -> float:
        loss = ctypes.c_double()
        check(self._lib.ptg_mlp_train(self.ctx.handle, self.handle, ctypes.c_void_p(X_ptr), ctypes.c_void_p(T_ptr),
                                      rows, steps, batch, lr, seed, ctypes.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "handle", None):
            self._lib.ptg_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mttkrp(ctx: Context, X: Tensor, factor_ptrs: Sequence[int], rank: int, mode: int, out_ptr: int):
    """Device-level MTTKRP (``ptg_mttkrp``): factor_ptrs are device pointers to row-major
    FP32 [I_k][R] matrices, out_ptr a device row-major FP32 [I_mode][R] buffer."""
    arr = (ctypes.c_void_p * len(factor_ptrs))(*[ctypes.c_void_p(int(p)) for p in factor_ptrs])
    check(ctx._lib.ptg_mttkrp(ctx.handle, X.handle, arr, int(rank), int(mode), ctypes.c_void_p(int(out_ptr))))


def _status_from(opts: Options, outs, res: CpdResult, trace, ntrace) -> Status:
    st = Status(options=opts, factors=outs, frob_tns=res.frob_tns, f_value=res.f_value,
                rel_costFunction=res.rel_costFunction, ao_iter=res.ao_iter,
                refine_sweeps_done=res.refine_sweeps_done,
                nesterov_iters_total=int(res.nesterov_iters_total), seconds=res.seconds_total)
    st.options = dataclasses.replace(opts, accel_coeff=res.accel_coeff, accel_fail=res.accel_fail)
    for i in range(ntrace):
        t = trace[i]
        st.trace.append(dict(f_value=t.f_value, rel=t.rel_costFunction, f_accel=t.f_accel,
                             accel_accepted=bool(t.accel_accepted),
                             nesterov_iters=list(t.nesterov_iters)[:opts.order], seconds=t.seconds))
    return st


def cpd_resident(ctx: Context, X: Tensor, R: int, options: Options, factorsInit: Sequence[np.ndarray],
                 refine: Optional[Tensor] = None, dimtree: bool = False) -> Status:
    """CPD-ALS on an HBM-resident tensor (``ptg_cpd_als``; ``ptg_cpd_dimtree_als`` when
    ``dimtree``)."""
    N = len(X.dims)
    inits = [np.asfortranarray(np.asarray(f, dtype=np.float64)) for f in factorsInit]
    outs = [np.zeros((X.dims[k], R), order="F") for k in range(N)]
    ip = (ctypes.POINTER(ctypes.c_double) * N)(*[_dptr(a) for a in inits])
    op = (ctypes.POINTER(ctypes.c_double) * N)(*[_dptr(a) for a in outs])
    res = CpdResult()
    ntr = options.max_iter + max(0, options.refine_sweeps)
    trace = (SweepTrace * ntr)()
    fn = ctx._lib.ptg_cpd_dimtree_als if dimtree else ctx._lib.ptg_cpd_als
    check(fn(ctx.handle, X.handle, refine.handle if refine else None, int(R),
             ctypes.byref(options.to_c()), ip, op, ctypes.byref(res), trace))
    return _status_from(options, outs, res, trace, res.ao_iter + res.refine_sweeps_done)


def cpd(tnsX, R: int, options: Optional[Options] = None, factorsInit: Optional[Sequence[np.ndarray]] = None,
        dims: Sequence[int] | None = None, ctx: Optional[Context] = None, _dimtree: bool = False) -> Status:
    """partensor::cpd(execution::cuda, tnsX, R[, options][, factorsInit]) with a host
    FP64 tensor (``ptg_cpd``: upload, convert, solve, download in one call).

    Without ``factorsInit`` the initial factors are U[0,1] like makeFactors
    (include/DataGeneration.hpp:564-581) but from a seeded generator."""
    ctx = ctx or default_context()
    a = np.asarray(tnsX, dtype=np.float64)
    if dims is None:
        dims = a.shape
        flat = np.asfortranarray(a).reshape(-1, order="F")
    else:
        flat = np.ascontiguousarray(a.reshape(-1))
    dims = [int(d) for d in dims]
    N = len(dims)
    options = options or Options(order=N)
    if factorsInit is None:
        rng = np.random.default_rng(0)
        factorsInit = [rng.random((I, R)) for I in dims]
    inits = [np.asfortranarray(np.asarray(f, dtype=np.float64)) for f in factorsInit]
    outs = [np.zeros((dims[k], R), order="F") for k in range(N)]
    ip = (ctypes.POINTER(ctypes.c_double) * N)(*[_dptr(x) for x in inits])
    op = (ctypes.POINTER(ctypes.c_double) * N)(*[_dptr(x) for x in outs])
    d = (ctypes.c_int64 * N)(*dims)
    res = CpdResult()
    ntr = options.max_iter + max(0, options.refine_sweeps)
    trace = (SweepTrace * ntr)()
    fn = ctx._lib.ptg_cpd_dimtree if _dimtree else ctx._lib.ptg_cpd
    check(fn(ctx.handle, N, d, _dptr(flat), DTYPES[options.precision], int(R),
             ctypes.byref(options.to_c()), ip, op, ctypes.byref(res), trace))
    return _status_from(options, outs, res, trace, res.ao_iter + res.refine_sweeps_done)


def cpdDimTree(tnsX, R: int, options: Optional[Options] = None,
               factorsInit: Optional[Sequence[np.ndarray]] = None, dims: Sequence[int] | None = None,
               ctx: Optional[Context] = None) -> Status:
    """partensor::cpdDimTree(execution::cuda, tnsX, R[, options][, factorsInit])
    (include/CpdDimTree.hpp:809-1362) with a host FP64 tensor (``ptg_cpd_dimtree``)."""
    return cpd(tnsX, R, options, factorsInit, dims=dims, ctx=ctx, _dimtree=True)


def cpd_batched(problems: Sequence[tuple], options: Optional[Options] = None,
                ctx: Optional[Context] = None) -> tuple[list[Status], np.ndarray]:
    """Many independent nonnegative CPDs in one call (``ptg_cpd_batched``): ``problems`` is a
    sequence of (tnsX, R, factorsInit) or (tnsX, R, factorsInit, threshold_error) with host
    FP64 tensors of the same order (the optional 4th item is that instance's stop target,
    otherwise ``options.threshold_error``).  Returns
    the per-instance Status list (``seconds``: from the call's start until the instance's
    stop test passed) and the same times counted from the start of the ALS loop, once every
    tensor is resident.  The reference has no batched form; this is the
    loop ``for p in problems: partensor::cpd(p...)`` (include/Cpd.hpp:534-577) in one call."""
    ctx = ctx or default_context()
    n = len(problems)
    if n == 0:
        return [], np.zeros(0)
    keep = []
    insts = (CpdInstance * n)()
    outs_all = []
    N = None
    for i, prob in enumerate(problems):
        X, R, init = prob[:3]
        insts[i].threshold_error = float(prob[3]) if len(prob) > 3 else 0.0
        a = np.asarray(X, dtype=np.float64)
        N = a.ndim if N is None else N
        flat = np.asfortranarray(a).reshape(-1, order="F")
        inits = [np.asfortranarray(np.asarray(f, dtype=np.float64)) for f in init]
        outs = [np.zeros((a.shape[k], R), order="F") for k in range(a.ndim)]
        ip = (ctypes.POINTER(ctypes.c_double) * a.ndim)(*[_dptr(x) for x in inits])
        op = (ctypes.POINTER(ctypes.c_double) * a.ndim)(*[_dptr(x) for x in outs])
        keep += [flat, inits, ip, op]
        outs_all.append(outs)
        insts[i].order = a.ndim
        for k in range(a.ndim):
            insts[i].dims[k] = a.shape[k]
        insts[i].tensor = _dptr(flat)
        insts[i].rank = int(R)
        insts[i].init_factors = ctypes.cast(ip, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)))
        insts[i].out_factors = ctypes.cast(op, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)))
    options = options or Options(order=N)
    res = (CpdResult * n)()
    secs = np.zeros(n)
    check(ctx._lib.ptg_cpd_batched(ctx.handle, n, insts, ctypes.byref(options.to_c()), res,
                                   secs.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return [_status_from(options, outs_all[i], res[i], None, 0) for i in range(n)], secs


def cpd_file(tnsDims: Sequence[int], R: int, path, options: Optional[Options] = None, skip: int = 0,
             seed: int = 0, ctx: Optional[Context] = None, dimtree: bool = False) -> Status:
    """partensor::cpd(tnsDims, R, path[, options]) and cpd(tnsDims, R, paths[, options])
    (include/Cpd.hpp:591-850): ``path`` is the tensor file (prod(dims) FP64 values, ColMajor,
    after ``skip`` values), or a sequence [tensor path, factor paths...] whose factor files
    hold I_k x R FP64 row-major matrices (the format of include/ReadWrite.hpp).  Without
    factor files the initial factors are U[0,1] from ``seed`` (``ptg_cpd_file``)."""
    ctx = ctx or default_context()
    dims = [int(d) for d in tnsDims]
    N = len(dims)
    options = options or Options(order=N)
    if isinstance(path, (str, bytes)):
        tpath, fpaths = path, None
    else:
        tpath, fpaths = path[0], list(path[1:])
        if len(fpaths) != N:
            raise ValueError("paths must hold the tensor path and one factor path per mode")
    enc = lambda p: p.encode() if isinstance(p, str) else p
    fp = None
    if fpaths is not None:
        fp = (ctypes.c_char_p * N)(*[enc(p) for p in fpaths])
    outs = [np.zeros((dims[k], R), order="F") for k in range(N)]
    op = (ctypes.POINTER(ctypes.c_double) * N)(*[_dptr(x) for x in outs])
    d = (ctypes.c_int64 * N)(*dims)
    res = CpdResult()
    ntr = options.max_iter + max(0, options.refine_sweeps)
    trace = (SweepTrace * ntr)()
    fn = ctx._lib.ptg_cpd_dimtree_file if dimtree else ctx._lib.ptg_cpd_file
    check(fn(ctx.handle, N, d, enc(tpath), int(skip), fp, int(seed), DTYPES[options.precision], int(R),
             ctypes.byref(options.to_c()), op, ctypes.byref(res), trace))
    return _status_from(options, outs, res, trace, res.ao_iter + res.refine_sweeps_done)


def write_tensor_file(path, X: np.ndarray):
    """Writes X in the reference's tensor file format (FP64, ColMajor)."""
    np.asfortranarray(np.asarray(X, dtype=np.float64)).reshape(-1, order="F").tofile(path)


def write_factor_file(path, A: np.ndarray):
    """Writes an I x R factor in the reference's factor file format (FP64, row-major)."""
    np.ascontiguousarray(np.asarray(A, dtype=np.float64)).tofile(path)
