"""GPU parity of the FP32 tensor-core MTTKRP (tcgen05 kind::tf32 with the three-term split)
against the FP64 oracle, through the C ABI (ptg_mttkrp with PTG_OPT_MTTKRP_IMPL = 2 on an
FP32 tensor).

Bar: 1e-5 relative (Frobenius) at these contraction lengths (<= ~4e4 terms), within 5x the
CUDA-core FP32 kernel's error; a single-term TF32 product would miss it by two orders of
magnitude (TF32 keeps 10 mantissa bits).  The accumulation in TMEM is not round-to-nearest
(it drifts low by ~2^-25 of the running sum per accumulate step), so the kernel drains each
accumulator every two K-blocks into FP32 registers; at 10^6 terms per output the bias stays
below 2e-6 relative."""
import numpy as np
import pytest

from oracle import cpd as oc
from test_gpu_mttkrp import _run

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,R", [((23, 19, 17), 5), ((64, 33, 40), 16), ((40, 48, 56), 32),
                                    ((31, 17, 29), 40), ((20, 24, 18), 64), ((130, 70, 9), 24),
                                    ((7, 6, 5, 4), 3), ((10, 9, 8, 7), 33), ((5, 4, 3, 3, 2), 4)])
def test_mttkrp_fp32_tensor_cores_all_modes(pkg, ctx, dims, R):
    rng = np.random.default_rng(sum(dims) + R + 1)
    X = rng.standard_normal(dims)
    f = [rng.uniform(-1, 1, (I, R)) for I in dims]
    for mode in range(len(dims)):
        got = _run(pkg, ctx, X, f, R, mode, impl="tensor_cores")
        ref = oc.mttkrp(f, X, mode)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-5, (mode, err)


def test_mttkrp_fp32_tensor_cores_large_split_k(pkg, ctx):
    """Enough K-blocks for several splits and several q-tiles per CTA (R = 40, factors in
    [-1, 1] like the reference's own MTTKRP test, scaled down)."""
    rng = np.random.default_rng(5)
    dims, R = (200, 150, 120), 40
    X = rng.uniform(-1, 1, dims)
    f = [rng.uniform(-1, 1, (I, R)) for I in dims]
    for mode in range(3):
        got = _run(pkg, ctx, X, f, R, mode, impl="tensor_cores")
        ref = oc.mttkrp(f, X, mode)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5, mode
        # and as close to the FP64 product as the CUDA-core FP32 kernel
        simt = _run(pkg, ctx, X, f, R, mode, impl="cuda_cores")
        assert np.linalg.norm(got - ref) <= 5.0 * np.linalg.norm(simt - ref) + 1e-12, mode


def test_cpd_fp32_tensor_cores_follows_oracle(pkg, ctx):
    """A whole FP32 ALS run with the tensor-core MTTKRP follows the FP64 oracle per sweep."""
    rng = np.random.default_rng(3)
    dims, R = (40, 36, 32), 6
    A = [rng.random((I, R)) for I in dims]
    T = np.einsum("ir,jr,kr->ijk", *A)
    X = T + np.sqrt((T ** 2).mean() / 100.0) * rng.standard_normal(dims)
    init = [np.random.default_rng(9).random((I, R)) for I in dims]
    ctx.set_mttkrp_impl("tensor_cores")
    try:
        st = pkg.cpd(X, R, pkg.Options(order=3, max_iter=15), init, ctx=ctx)
    finally:
        ctx.set_mttkrp_impl("auto")
    ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=15), init)
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([s["rel"] for s in ref.trace])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 1e-4


def test_mttkrp_fp32_tensor_cores_long_contraction(pkg, ctx):
    """10^6 terms per output (mode 0 of 64 x 1000 x 1000, the contraction length of the
    1000^3 modes), uniform [0, 1) data and factors, so that a one-signed drift of the
    accumulation cannot cancel.  Each TMEM accumulator chain spans two K-blocks (16
    accumulate steps, ~2^-25 drift each) before it is drained into FP32 registers, so the
    relative bias stays below 2e-6 (it was -1.9e-5 with 64-K-block chains and ~-5e-5 with
    one chain per CTA)."""
    rng = np.random.default_rng(11)
    dims, R = (64, 1000, 1000), 32
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    for mode in (0, 1):
        got = _run(pkg, ctx, X, f, R, mode, impl="tensor_cores")
        ref = oc.mttkrp(f, X, mode)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        bias = float(np.mean((got - ref) / ref))
        print(f"mode {mode}: error {err:.3e}, bias {bias:.3e}")
        assert err < 4e-6 and -2e-6 < bias < 1e-6, (mode, err, bias)
        simt = _run(pkg, ctx, X, f, R, mode, impl="cuda_cores")
        assert np.linalg.norm(simt - ref) / np.linalg.norm(ref) < 1e-5, mode
