"""Host FP64 sources reach the conversion kernels in one of two ways (PTG_OPT_HOST_READ):
read in place where the device can address the buffer (page-locked memory through its mapped
device pointer; pageable memory where the device walks the host's page tables, as over
NVLink-C2C), or staged through 64 MB device chunks.  The test runs each route under each
mode: auto, staged and in place.  Every route must store the same bits as a
device source, for every storage type, including a tensor that spans more than one staging
chunk (FP8 chunks hold whole slabs)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


class _Iface:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (int(ptr), False), "version": 3}


def _bytes(T, dims, esz):
    ptr, p0, sptr = T.storage()
    torch.cuda.synchronize()
    n = int(np.prod(dims[1:])) * p0 * esz
    raw = torch.as_tensor(_Iface(ptr, n), device="cuda:0").cpu().numpy().copy()
    scales = None
    if sptr:
        scales = torch.as_tensor(_Iface(sptr, dims[-1] * 4), device="cuda:0").cpu().numpy().copy()
    return raw, scales


@pytest.mark.parametrize("precision,esz", [("f32", 4), ("bf16", 2), ("fp8", 1)])
@pytest.mark.parametrize("dims", [(37, 29, 23), (260, 200, 210)])   # the second spans two 64 MB chunks
def test_host_routes_store_the_same_bits(pkg, ctx, precision, esz, dims):
    rng = np.random.default_rng(len(precision) + dims[0])
    X = rng.random(dims) * 4.0 - 1.0
    flat = X.reshape(-1, order="F")
    dev = torch.from_numpy(flat).to("cuda:0")
    ref_T = pkg.Tensor(ctx, (dev.data_ptr(), dims), precision=precision)
    ref = _bytes(ref_T, dims, esz)
    ref_norms = ref_T.norms()
    ref_T.close()
    del dev
    host = torch.empty(flat.size, dtype=torch.float64, pin_memory=True)
    host.numpy()[:] = flat
    routes = {f"{kind}_{mode}": (mode, src) for kind, src in (("pageable", flat), ("pinned", host.numpy()))
              for mode in ("auto", "staged", "in_place")}
    for name, (mode, src) in routes.items():
        ctx.set_host_read(mode)
        try:
            T = pkg.Tensor(ctx, src, dims=dims, precision=precision)
        finally:
            ctx.set_host_read("auto")
        got = _bytes(T, dims, esz)
        norms = T.norms()
        T.close()
        assert np.array_equal(got[0], ref[0]), (name, np.flatnonzero(got[0] != ref[0])[:8])
        if precision == "fp8":
            assert np.array_equal(got[1], ref[1]), name
        # the norms are sums of per-chunk partials: equal up to the summation order
        assert norms[0] == pytest.approx(ref_norms[0], rel=1e-12), name
        assert norms[1] == pytest.approx(ref_norms[1], rel=1e-12), name


def test_host_read_option_is_checked(pkg, ctx):
    lib = pkg._lib
    assert ctx._lib.ptg_ctx_set_option(ctx.handle, lib.PTG_OPT_HOST_READ, 3) == lib.PTG_ERR_INVALID
    assert b"host read" in ctx._lib.ptg_last_error()
    assert ctx._lib.ptg_ctx_set_option(ctx.handle, lib.PTG_OPT_HOST_READ, 0) == 0
