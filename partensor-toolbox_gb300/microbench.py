"""MTTKRP micro-benchmark: time one mode-n MTTKRP of a random dense tensor on cuda:0.

    python partensor-toolbox_gb300/microbench.py --dims 640 640 640 --rank 32 \
        --precision bf16 --impl auto --mode all --iters 10

Prints one JSON line per mode with the mean CUDA-event time of a launch and the
achieved HBM bandwidth from the algorithmic bytes (prod(I)*s_x + sum_{k != n} I_k*R*4 +
I_n*R*4).  Used for kernel tuning and for the ncu captures of the MTTKRP kernels.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys


def _pkg():
    here = os.path.dirname(os.path.abspath(__file__))
    name = "partensor_toolbox_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(here, "__init__.py"),
                                                  submodule_search_locations=[here])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def main():
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs="+", default=[640, 640, 640])
    ap.add_argument("--rank", type=int, default=32)
    ap.add_argument("--precision", default="bf16", choices=["bf16", "f32"])
    ap.add_argument("--impl", default="auto", choices=["auto", "cuda_cores", "tensor_cores"])
    ap.add_argument("--mode", default="all")
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    a = ap.parse_args()
    pkg = _pkg()
    dims, R = a.dims, a.rank
    g = torch.Generator(device="cuda").manual_seed(0)
    numel = 1
    for d in dims:
        numel *= d
    X = torch.rand(numel, generator=g, device="cuda", dtype=torch.float64)
    ctx = pkg.Context(0)
    ctx.set_mttkrp_impl(a.impl)
    T = pkg.Tensor(ctx, (X.data_ptr(), dims), precision=a.precision)
    del X
    torch.cuda.synchronize()
    facs = [torch.rand(I, R, generator=g, device="cuda", dtype=torch.float32) for I in dims]
    s = torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)
    modes = range(len(dims)) if a.mode == "all" else [int(a.mode)]
    esz = 2 if a.precision == "bf16" else 4
    for mode in modes:
        out = torch.empty(dims[mode], R, device="cuda")
        ptrs = [f.data_ptr() for f in facs]
        for _ in range(a.warmup):
            pkg.mttkrp(ctx, T, ptrs, R, mode, out.data_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(a.iters):
            pkg.mttkrp(ctx, T, ptrs, R, mode, out.data_ptr())
        e1.record(s)
        e1.synchronize()
        ctx.synchronize()
        ms = e0.elapsed_time(e1) / max(1, a.iters)
        nbytes = numel * esz + sum(I * R * 4 for k, I in enumerate(dims) if k != mode) + dims[mode] * R * 4
        print(json.dumps({"mode": mode, "dims": dims, "rank": R, "precision": a.precision, "impl": a.impl,
                          "ms": ms, "GBps": nbytes / ms / 1e6, "TFLOPs": 2.0 * numel * R / ms / 1e9}),
              flush=True)
    T.close()
    ctx.close()


if __name__ == "__main__":
    main()
