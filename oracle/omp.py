"""ctypes wrapper of oracle/cpd_omp.c and oracle/gtc_omp.c -- TEST INFRASTRUCTURE ONLY (CPU
baselines and second restatements of the reference's CpdOpenMP driver,
include/CpdOpenMP.hpp:266-329, and of its OpenMP GTC row solvers,
include/NesterovMNLS.hpp:553-663,878-976)."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libptg_oracle.so")
MAXN = 8


class Options(ctypes.Structure):
    _fields_ = [("constraints", ctypes.c_int * MAXN), ("threshold_error", ctypes.c_double),
                ("nesterov_delta_1", ctypes.c_double), ("nesterov_delta_2", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("accel_coeff", ctypes.c_int),
                ("accel_fail", ctypes.c_int), ("acceleration", ctypes.c_int),
                ("normalization", ctypes.c_int), ("nthreads", ctypes.c_int)]


class Status(ctypes.Structure):
    _fields_ = [("frob_tns", ctypes.c_double), ("f_value", ctypes.c_double),
                ("rel_costFunction", ctypes.c_double), ("ao_iter", ctypes.c_int),
                ("accel_coeff", ctypes.c_int), ("accel_fail", ctypes.c_int),
                ("seconds_mttkrp", ctypes.c_double), ("seconds_total", ctypes.c_double)]


def build(force: bool = False) -> str:
    """Compile oracle/cpd_omp.c and oracle/gtc_omp.c with gcc (portable flags: they also
    build on the Arm host)."""
    srcs = [os.path.join(HERE, "cpd_omp.c"), os.path.join(HERE, "gtc_omp.c")]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(s) for s in srcs):
        os.makedirs(os.path.dirname(LIB), exist_ok=True)
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB, *srcs, "-lm"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        _lib.ptgo_mttkrp.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), dp,
                                     ctypes.POINTER(dp), ctypes.c_int, ctypes.c_int, dp, ctypes.c_int]
        _lib.ptgo_cpd_als.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), dp, ctypes.c_int,
                                      ctypes.POINTER(Options), ctypes.POINTER(dp),
                                      ctypes.POINTER(Status), dp]
        _lib.ptgo_cpd_als.restype = ctypes.c_int
        _lib.ptgo_gtc_rows.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                       ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), dp, ctypes.POINTER(dp),
                                       ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
        _lib.ptgo_gtc_rows.restype = ctypes.c_int
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def mttkrp(X_flat: np.ndarray, dims, factors, mode: int, nthreads: int = 0) -> np.ndarray:
    """X_flat: ColMajor float64; factors: list of I_k x R arrays.  Returns I_mode x R."""
    N = len(dims)
    R = factors[0].shape[1]
    d = (ctypes.c_int64 * N)(*dims)
    fs = [np.asfortranarray(f, dtype=np.float64) for f in factors]
    arr = (ctypes.POINTER(ctypes.c_double) * N)(*[_dp(f) for f in fs])
    out = np.zeros((dims[mode], R), order="F")
    lib().ptgo_mttkrp(N, d, _dp(np.ascontiguousarray(X_flat, dtype=np.float64)), arr, R, mode,
                      _dp(out), nthreads)
    return out


def cpd_als(X_flat: np.ndarray, dims, R: int, factors_init, constraints=None,
            threshold_error=1e-3, delta=1e-2, max_iter=20, acceleration=True,
            normalization=True, nthreads: int = 0):
    N = len(dims)
    o = Options()
    for k in range(N):
        o.constraints[k] = 1 if constraints is None else int(constraints[k])
    o.threshold_error = threshold_error
    o.nesterov_delta_1 = o.nesterov_delta_2 = delta
    o.max_iter = max_iter
    o.accel_coeff, o.accel_fail = 3, 0
    o.acceleration, o.normalization, o.nthreads = int(acceleration), int(normalization), nthreads
    st = Status()
    fs = [np.asfortranarray(np.array(f, dtype=np.float64)) for f in factors_init]
    arr = (ctypes.POINTER(ctypes.c_double) * N)(*[_dp(f) for f in fs])
    trace = np.zeros(3 * max_iter)
    d = (ctypes.c_int64 * N)(*dims)
    X = np.ascontiguousarray(X_flat, dtype=np.float64)
    lib().ptgo_cpd_als(N, d, _dp(X), R, ctypes.byref(o), arr, ctypes.byref(st), _dp(trace))
    return fs, st, trace.reshape(-1, 3)[: st.ao_iter]


def gtc_rows(ptr: np.ndarray, other: np.ndarray, vals: np.ndarray, factors, mode: int, stochastic: bool,
             c: float, max_inner: int, lam: float, seed: int = 0, outer: int = 1, nthreads: int = 0):
    """One GTC update of factor `mode` over the rows of a column-compressed matricisation
    (ptr [nrows + 1], other [nnz, N - 1] int32, vals [nnz]); factors are I_k x R arrays, the
    updated rows of factors[mode] are returned (the others are not changed)."""
    N = len(factors)
    R = factors[0].shape[1]
    fs = [np.ascontiguousarray(f, dtype=np.float64).copy() for f in factors]
    arr = (ctypes.POINTER(ctypes.c_double) * N)(*[_dp(f) for f in fs])
    p = np.ascontiguousarray(ptr, dtype=np.int64)
    o = np.ascontiguousarray(other, dtype=np.int32)
    v = np.ascontiguousarray(vals, dtype=np.float64)
    rc = lib().ptgo_gtc_rows(N, R, mode, p.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(p) - 1,
                             o.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dp(v), arr, int(stochastic),
                             float(c), int(max_inner), float(lam), int(seed), int(outer), int(nthreads))
    if rc != 0:
        raise RuntimeError("ptgo_gtc_rows failed")
    return fs[mode][: len(p) - 1]
