"""GPU parity of the tcgen05 (tensor-core) MTTKRP, BF16 storage.

The kernel rounds the tensor to BF16 at upload and each Khatri-Rao tile entry
(an FP32 product of factor entries) to BF16 before the BF16 x BF16 -> FP32 MMA.
``emulate`` reproduces exactly that rounding on the CPU and sums in FP64, so a layout,
swizzle or descriptor error shows up as a large mismatch while the only tolerated
difference is FP32 accumulation order (bound 2e-5 relative).  Against the unrounded FP64
oracle the stated BF16 bound is 4e-3 relative (Frobenius)."""
import numpy as np
import pytest
import torch

from oracle import cpd as oc

pytestmark = pytest.mark.gpu


def _bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.bfloat16).to(torch.float64).numpy()


def _kr_side_f32(factors, modes, dims):
    """Khatri-Rao rows over `modes` (first mode fastest), FP32 products accumulated in the
    kernel's order (1.0f * A_first * A_next ...)."""
    R = factors[0].shape[1]
    out = np.ones((1, R), dtype=np.float32)
    for k in modes:
        A = factors[k].astype(np.float32)
        # new index = old + len(old) * i_k  (earlier modes fastest)
        out = (out[None, :, :] * A[:, None, :]).reshape(-1, R).astype(np.float32)
    return out


def emulate(X, factors, mode):
    dims = X.shape
    N = len(dims)
    before = list(range(mode))
    after = list(range(mode + 1, N))
    Ka = _kr_side_f32(factors, after, dims)            # [S, R]
    Kb = _kr_side_f32(factors, before, dims)           # [P, R]
    T = (Ka[None, :, :] * Kb[:, None, :]).astype(np.float32)   # [P, S, R] = va * vb
    T = _bf16(T)
    P, S = Kb.shape[0], Ka.shape[0]
    Xb = _bf16(X)
    # X viewed as [P, Q, S] in ColMajor order
    Xv = Xb.reshape(-1, order="F").reshape(S, dims[mode], P).transpose(2, 1, 0)   # [P, Q, S]
    return np.einsum("pqs,psr->qr", Xv, T, optimize=True)


def _run(pkg, ctx, X, factors, R, mode, impl="tensor_cores"):
    ctx.set_mttkrp_impl(impl)
    try:
        T = pkg.Tensor(ctx, np.asfortranarray(X), precision="bf16")
        dev = [torch.tensor(np.ascontiguousarray(f), dtype=torch.float32, device="cuda:0") for f in factors]
        out = torch.full((X.shape[mode], R), float("nan"), dtype=torch.float32, device="cuda:0")
        pkg.mttkrp(ctx, T, [d.data_ptr() for d in dev], R, mode, out.data_ptr())
        ctx.synchronize()
        T.close()
    finally:
        ctx.set_mttkrp_impl("auto")
    return out.cpu().double().numpy()


@pytest.mark.parametrize("dims,R", [((40, 48, 56), 32), ((23, 19, 17), 5), ((130, 20, 24), 16),
                                    ((64, 70, 9), 64), ((16, 300, 8), 32), ((24, 20, 18, 10), 24)])
def test_tc_mttkrp_matches_emulation(pkg, ctx, dims, R):
    rng = np.random.default_rng(sum(dims) * R)
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    for mode in range(len(dims)):
        got = _run(pkg, ctx, X, f, R, mode)
        emu = emulate(X, f, mode)
        err = np.linalg.norm(got - emu) / np.linalg.norm(emu)
        assert err < 2e-5, (mode, err)
        ref = oc.mttkrp(f, X, mode)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 4e-3


def test_tc_mttkrp_signed_data(pkg, ctx):
    rng = np.random.default_rng(9)
    dims, R = (72, 40, 33), 32
    X = rng.standard_normal(dims)
    f = [rng.uniform(-1, 1, (I, R)) for I in dims]
    for mode in range(3):
        got = _run(pkg, ctx, X, f, R, mode)
        emu = emulate(X, f, mode)
        assert np.linalg.norm(got - emu) / np.linalg.norm(emu) < 1e-4


def test_tc_mttkrp_large_k_split(pkg, ctx):
    """Enough K-blocks that many CTAs split K and every q-tile group is exercised."""
    rng = np.random.default_rng(10)
    dims, R = (256, 200, 180), 32
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    for mode in range(3):
        got = _run(pkg, ctx, X, f, R, mode)
        ref = oc.mttkrp_einsum(f, X, mode)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 4e-3
        cuda = _run(pkg, ctx, X, f, R, mode, impl="cuda_cores")
        assert np.linalg.norm(got - cuda) / np.linalg.norm(cuda) < 4e-3


def test_tc_mttkrp_deterministic(pkg, ctx):
    rng = np.random.default_rng(11)
    dims, R = (128, 96, 80), 32
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    for mode in range(3):
        assert np.array_equal(_run(pkg, ctx, X, f, R, mode), _run(pkg, ctx, X, f, R, mode))
