"""GPU parity of FP8 (e4m3, per-slab scales) tensor storage and its tcgen05 MTTKRP.

* The stored codes and slab scales are bit-exact against oracle/fp8.py, for device sources
  and for host sources read in place (pageable memory where the device walks the host's page
  tables, page-locked memory) or staged through device chunks (stochastic rounding from a
  hash of each entry's position).
* The MTTKRP matches ``oracle.fp8.mttkrp`` -- the same FP8 codes and the same two-part
  e4m3 Khatri-Rao operand, summed in FP64 -- within 2e-5 relative (Frobenius): only the
  FP32 accumulation order of the MMA and of the split-K sum differs.
* Against the unrounded FP64 oracle the FP8 MTTKRP is within 5e-3 relative at these sizes;
  the error is the dither noise of the stored tensor, unbiased, and it falls as
  1/sqrt(contraction length).
* A CPD-ALS on FP8 storage with the fit verified on the FP32 copy ends within 1e-3 of the
  FP64 oracle's fit (the reference's bar)."""
import numpy as np
import pytest
import torch

from oracle import cpd as oc
from oracle import fp8 as of

pytestmark = pytest.mark.gpu


def _stored(T, dims):
    """Codes (unpadded, flat ColMajor) and slab scales read back from the device."""
    ptr, p0, sptr = T.storage()
    n_fib = int(np.prod(dims[1:]))
    torch.cuda.synchronize()
    # the device buffers, seen through the CUDA array interface, copied to the host
    codes = _from_ptr(ptr, n_fib * p0, torch.uint8).cpu()
    scales = _from_ptr(sptr, dims[-1], torch.float32).cpu()
    c = codes.numpy().reshape(n_fib, p0)
    return c[:, : dims[0]].reshape(-1), c[:, dims[0]:], scales.cpu().numpy()


class _Iface:
    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (int(ptr), False), "version": 3}


def _from_ptr(ptr, n, dtype):
    typestr = {torch.uint8: "|u1", torch.float32: "<f4"}[dtype]
    return torch.as_tensor(_Iface(ptr, n, typestr), device="cuda:0")


def _tensor(rng, dims, scale_per_slab=True):
    X = rng.random(dims) * 3.0 - 0.5                      # signs, and values near zero
    if scale_per_slab:                                     # slabs of very different magnitudes
        X = X * np.logspace(-3, 4, dims[-1]).reshape((1,) * (len(dims) - 1) + (-1,))
        X[..., dims[-1] // 2] = 0.0                        # an all-zero slab
    return X


@pytest.mark.parametrize("dims", [(23, 19, 17), (40, 48, 56), (16, 9, 5, 7), (130, 3, 6), (5, 4, 3)])
@pytest.mark.parametrize("source", ["host", "host_in_place", "pinned", "pinned_in_place", "device"])
def test_fp8_encode_bit_exact(pkg, ctx, dims, source):
    rng = np.random.default_rng(sum(dims))
    X = _tensor(rng, dims)
    if source in ("host", "host_in_place"):
        ctx.set_host_read("in_place" if source == "host_in_place" else "auto")
        try:
            T = pkg.Tensor(ctx, np.asfortranarray(X), precision="fp8")
        finally:
            ctx.set_host_read("auto")
    elif source in ("pinned", "pinned_in_place"):
        host = torch.empty(X.size, dtype=torch.float64, pin_memory=True)
        host.numpy()[:] = X.reshape(-1, order="F")
        ctx.set_host_read("in_place" if source == "pinned_in_place" else "auto")
        try:
            T = pkg.Tensor(ctx, host.numpy(), dims=dims, precision="fp8")
        finally:
            ctx.set_host_read("auto")
    else:
        dev = torch.tensor(X.reshape(-1, order="F"), dtype=torch.float64, device="cuda:0")
        T = pkg.Tensor(ctx, (dev.data_ptr(), dims), precision="fp8")
    codes, pads, scales = _stored(T, dims)
    f64, fst = T.norms()
    T.close()
    ref_codes, ref_scales, vals = of.encode_tensor(X)
    assert np.array_equal(scales, ref_scales)
    assert np.array_equal(codes, ref_codes), np.flatnonzero(codes != ref_codes)[:10]
    assert not pads.any()
    assert f64 == pytest.approx(float((X.astype(np.float32).astype(np.float64) ** 2).sum()), rel=1e-6)
    assert fst == pytest.approx(float((vals ** 2).sum()), rel=1e-6)


def test_fp8_storage_is_unbiased(pkg, ctx):
    """Mean of stored - x over many entries of one value is zero within its sampling error."""
    dims = (256, 128, 4)
    X = np.full(dims, 1.03)
    T = pkg.Tensor(ctx, np.asfortranarray(X), precision="fp8")
    codes, _, scales = _stored(T, dims)
    T.close()
    vals = of.decode(codes) * scales[0]
    # 1.03 sits at t = 0.24 of an e4m3 interval 0.125 wide (in data units): each entry is
    # 1 + 0.125 * Bernoulli(0.24), whose mean has standard deviation 0.125 sqrt(t (1 - t) / n)
    t = (np.float32(1.03) - 1.0) / 0.125
    sd = 0.125 * np.sqrt(t * (1 - t) / vals.size)
    assert set(np.unique(vals)) == {1.0, 1.125}
    assert abs(vals.mean() - np.float32(1.03)) < 5 * sd


def _run(pkg, ctx, X, factors, R, mode):
    T = pkg.Tensor(ctx, np.asfortranarray(X), precision="fp8")
    codes, _, scales = _stored(T, X.shape)
    dev = [torch.tensor(np.ascontiguousarray(f), dtype=torch.float32, device="cuda:0") for f in factors]
    out = torch.full((X.shape[mode], R), float("nan"), dtype=torch.float32, device="cuda:0")
    pkg.mttkrp(ctx, T, [d.data_ptr() for d in dev], R, mode, out.data_ptr())
    ctx.synchronize()
    T.close()
    return out.cpu().double().numpy(), codes, scales


@pytest.mark.parametrize("dims,R", [((40, 48, 56), 32), ((23, 19, 17), 5), ((130, 20, 24), 16),
                                    ((64, 70, 9), 64), ((16, 300, 8), 32), ((24, 20, 18, 10), 24),
                                    ((33, 17, 29), 100), ((20, 24, 18), 128)])
def test_fp8_mttkrp_matches_emulation(pkg, ctx, dims, R):
    rng = np.random.default_rng(sum(dims) * R)
    X = _tensor(rng, dims)
    f = [rng.random((I, R)) * 2.0 - 0.3 for I in dims]
    for mode in range(len(dims)):
        got, codes, scales = _run(pkg, ctx, X, f, R, mode)
        ref = of.mttkrp(codes, scales, dims, f, mode)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 2e-5, (mode, err)


@pytest.mark.parametrize("dims,R", [((60, 50, 40), 32), ((30, 28, 26, 12), 16)])
def test_fp8_mttkrp_fp64_bound(pkg, ctx, dims, R):
    rng = np.random.default_rng(7)
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    for mode in range(len(dims)):
        got, _, _ = _run(pkg, ctx, X, f, R, mode)
        ref = oc.mttkrp(f, X, mode)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 5e-3, (mode, err)


def _problem(dims, R, seed, snr_db):
    rng = np.random.default_rng(seed)
    A = [rng.random((I, R)) for I in dims]
    T = np.einsum("ir,jr,kr->ijk", *A) if len(dims) == 3 else np.einsum("ir,jr,kr,lr->ijkl", *A)
    sigma = np.sqrt((T ** 2).sum() / (T.size * 10 ** (snr_db / 10)))
    X = T + sigma * rng.standard_normal(dims)
    init = [np.random.default_rng(seed + 1).random((I, R)) for I in dims]
    return X, init


@pytest.mark.parametrize("dimtree", [False, True])
def test_fp8_cpd_fit_matches_oracle(pkg, ctx, dimtree):
    dims = (64, 56, 48) if not dimtree else (24, 22, 20, 18)
    R = 8
    X, init = _problem(dims, R, 11, 25.0)
    opts = pkg.Options(order=len(dims), max_iter=25, precision="fp8", verify_fp32=True)
    fn = pkg.cpdDimTree if dimtree else pkg.cpd
    st = fn(X, R, opts, init, ctx=ctx)
    ref = oc.cpd_als(X, R, oc.Options(order=len(dims), max_iter=25), init)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3, (st.rel_costFunction, ref.rel_costFunction)
    # the reported cost is that of the returned factors on the data
    assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=1e-4)
