"""Failure paths of the GPU code, made to happen without a GPU fault.

* A bounded wait that gives up: with the context's spin limit at 0 every bounded wait of the
  tensor-core MTTKRP kernels gives up at its first poll, before any TMA copy or MMA is
  issued.  The kernel returns early, the error word carries PTG_ERR_TIMEOUT to the host,
  and the context computes correctly once the limit is restored.
* An allocation that fails: with the context's allocation limit below a request, tensor
  storage and solve buffers fail with PTG_ERR_OOM before cudaMalloc is called, and the
  context works again once the limit is lifted.
The reference has no status codes (failures print and continue, include/CUDA/CUDAMTTKRP.hpp:
171-175); these are the library's own error conventions."""
import numpy as np
import pytest
import torch

from oracle import cpd as oc

pytestmark = pytest.mark.gpu


def _mttkrp(pkg, ctx, T, f, R, mode):
    dev = [torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda:0") for a in f]
    out = torch.zeros((T.dims[mode], R), dtype=torch.float32, device="cuda:0")
    pkg.mttkrp(ctx, T, [d.data_ptr() for d in dev], R, mode, out.data_ptr())
    return out


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_bounded_wait_gives_up_and_reports_timeout(pkg, ctx, precision):
    rng = np.random.default_rng(0)
    dims, R = (48, 40, 36), 16
    X = rng.random(dims)
    f = [rng.random((I, R)) for I in dims]
    T = pkg.Tensor(ctx, np.asfortranarray(X), precision=precision)
    ctx.set_spin_limit(0)
    try:
        for mode in range(3):
            _mttkrp(pkg, ctx, T, f, R, mode)
            with pytest.raises(pkg.PtgError) as ei:
                ctx.synchronize()
            assert ei.value.code == pkg._lib.PTG_ERR_TIMEOUT
    finally:
        ctx.set_spin_limit(-1)
    # the context still computes, and the error word was cleared by the report
    for mode in range(3):
        out = _mttkrp(pkg, ctx, T, f, R, mode)
        ctx.synchronize()
        ref = oc.mttkrp(f, X, mode)
        err = np.linalg.norm(out.cpu().double().numpy() - ref) / np.linalg.norm(ref)
        assert err < 5e-3, (mode, err)
    T.close()


def test_allocation_limit_reports_oom_and_context_recovers(pkg, ctx):
    rng = np.random.default_rng(1)
    dims, R = (40, 30, 20), 5
    X = rng.random(dims)
    init = [rng.random((I, R)) for I in dims]
    ctx.set_alloc_limit(4096)
    try:
        with pytest.raises(pkg.PtgError) as ei:
            pkg.Tensor(ctx, np.asfortranarray(X), precision="f32")
        assert ei.value.code == pkg._lib.PTG_ERR_OOM
        with pytest.raises(pkg.PtgError) as ei:
            pkg.cpd(X, R, pkg.Options(order=3, max_iter=3), init, ctx=ctx)
        assert ei.value.code == pkg._lib.PTG_ERR_OOM
    finally:
        ctx.set_alloc_limit(0)
    st = pkg.cpd(X, R, pkg.Options(order=3, max_iter=3), init, ctx=ctx)
    ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=3), init)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-4
