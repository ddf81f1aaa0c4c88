"""ptg_mttkrp_noalloc: the MTTKRP entry point that allocates no device memory.

It exists for callers that may not call cudaMalloc when they need an MTTKRP (an
application allocator that owns all of HBM, code that must not synchronise the device,
latency-bound loops).  This test calls it through the C ABI, twice in a row per case so
the second call runs on the scratch block the first one left behind, and compares each
result with the regular entry point (ptg_mttkrp) within the FP32 MTTKRP tolerance used by
the other tests (1e-5 relative, Frobenius).  It also checks the size limit is refused
with a clear error.  The file name makes pytest collect it last; it passes alone in a fresh
process as well."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(lib, X_dev, dims, ld0, facs, R, mode, out):
    N = len(dims)
    d = (ctypes.c_int64 * N)(*dims)
    arr = (ctypes.c_void_p * N)(*[ctypes.c_void_p(f.data_ptr()) for f in facs])
    stream = torch.cuda.current_stream().cuda_stream
    return lib.ptg_mttkrp_noalloc(ctypes.c_void_p(X_dev.data_ptr()), N, d, ld0, arr, R, mode,
                                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))


def _padded(X, ld0):
    """Device FP32 ColMajor copy of X with mode-0 stride ld0 (pads zero)."""
    dims = X.shape
    rest = int(np.prod(dims[1:]))
    buf = np.zeros((rest, ld0), dtype=np.float32)
    buf[:, : dims[0]] = X.reshape(dims[0], rest, order="F").T
    return torch.from_numpy(buf.reshape(-1)).cuda()


@pytest.mark.parametrize("dims,R", [((37, 29, 23), 7), ((64, 48, 40), 32), ((20, 12, 10, 8), 40)])
def test_noalloc_matches_regular_entry_point(pkg, ctx, dims, R):
    lib = pkg._lib.load()
    rng = np.random.default_rng(sum(dims) + R)
    X = rng.random(dims)
    facs_np = [rng.random((I, R)) for I in dims]
    facs = [torch.tensor(f, dtype=torch.float32, device="cuda") for f in facs_np]
    ld0 = (dims[0] + 7) // 8 * 8
    Xd = _padded(X, ld0)
    T = pkg.Tensor(ctx, np.asfortranarray(X), precision="f32")
    for mode in range(len(dims)):
        ref = torch.empty(dims[mode], R, device="cuda")
        pkg.mttkrp(ctx, T, [f.data_ptr() for f in facs], R, mode, ref.data_ptr())
        ctx.synchronize()
        for call in range(2):   # two calls in a row on the shared scratch block
            out = torch.full((dims[mode], R), float("nan"), device="cuda")
            rc = _noalloc(lib, Xd, list(dims), ld0, facs, R, mode, out)
            assert rc == 0, lib.ptg_last_error().decode()
            torch.cuda.synchronize()
            err = (torch.linalg.norm(out.double() - ref.double()) / torch.linalg.norm(ref.double())).item()
            assert err < 1e-5, (mode, call, err)
    T.close()


def test_noalloc_rejects_sizes_beyond_the_block(pkg):
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = pkg._lib.load()
    dims, R = [70000, 8, 8], 32        # I_0 x 32 columns > 2,097,152 floats
    ld0 = 70000
    X = torch.zeros(ld0 * 64, device="cuda")
    facs = [torch.zeros(I, R, device="cuda") for I in dims]
    out = torch.zeros(dims[0], R, device="cuda")
    rc = _noalloc(lib, X, dims, ld0, facs, R, 0, out)
    assert rc == pkg._lib.PTG_ERR_UNSUPPORTED
    assert b"2097152" in lib.ptg_last_error()
    # a misaligned stride is refused too
    rc = _noalloc(lib, X, [7, 8, 8], 7, facs, R, 1, out)
    assert rc == pkg._lib.PTG_ERR_INVALID
    # mode 0 is limited by the padded stride: 65536 x 32 columns fits, 65544 x 32 does not
    X2 = torch.zeros(65544 * 64, device="cuda")
    facs2 = [torch.zeros(I, R, device="cuda") for I in (65536, 8, 8)]
    out2 = torch.zeros(65536, R, device="cuda")
    assert _noalloc(lib, X2, [65536, 8, 8], 65536, facs2, R, 0, out2) == 0, lib.ptg_last_error().decode()
    torch.cuda.synchronize()
    rc = _noalloc(lib, X2, [65536, 8, 8], 65544, facs2, R, 0, out2)
    assert rc == pkg._lib.PTG_ERR_UNSUPPORTED
    # host memory is refused
    host = torch.zeros(ld0 * 64)
    assert _noalloc(lib, host, dims, ld0, facs, R, 1, out) == pkg._lib.PTG_ERR_INVALID


def test_noalloc_allocates_nothing(pkg):
    """After a first call (which looks up the block's address), calls of several shapes leave
    the device's free memory and torch's allocated bytes unchanged."""
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = pkg._lib.load()
    rng = np.random.default_rng(5)
    cases = []
    for dims, R in [((37, 29, 23), 7), ((64, 48, 40), 32), ((20, 12, 10, 8), 40), ((128, 16, 9), 100)]:
        X = rng.random(dims)
        ld0 = (dims[0] + 7) // 8 * 8
        facs = [torch.tensor(rng.random((I, R)), dtype=torch.float32, device="cuda") for I in dims]
        outs = [torch.empty(dims[m], R, device="cuda") for m in range(len(dims))]
        cases.append((_padded(X, ld0), list(dims), ld0, facs, R, outs))
    Xd, dims, ld0, facs, R, outs = cases[0]
    assert _noalloc(lib, Xd, dims, ld0, facs, R, 0, outs[0]) == 0
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for Xd, dims, ld0, facs, R, outs in cases:
        for m in range(len(dims)):
            assert _noalloc(lib, Xd, dims, ld0, facs, R, m, outs[m]) == 0, lib.ptg_last_error().decode()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0
