"""The reference-side C++ binding (include/partensor_gb300.hpp) compiled against a
project-written stand-in of Partensor's types (tests/cpp/partensor_standin.hpp; the
reference needs Eigen, which is not installed), linked against libptg.so and, on a GPU,
run: cpd(execution::cuda, ...)'s dispatch target, the cpdDimTree and gtc cuda branches,
and the writeToFile output, each against the Python mirror of the same call and the FP64
oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "partensor-toolbox_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "binding_driver.cpp")


def _compile(out, link=True):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "tests", "cpp"), SRC]
    if link:
        cmd += ["-L", LIBDIR, "-lptg", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)]
    else:
        cmd += ["-c", "-o", str(out)]
    subprocess.run(cmd, check=True)


def test_binding_compiles_and_links(tmp_path):
    link = os.path.exists(os.path.join(LIBDIR, "libptg.so"))
    _compile(tmp_path / ("driver" if link else "driver.o"), link=link)


def _problem(dims, R, seed):
    rng = np.random.default_rng(seed)
    A = [rng.random((I, R)) for I in dims]
    T = np.einsum("ir,jr,kr->ijk", *A)
    X = T + 0.05 * T.std() * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    return X, init


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["cpd", "dimtree"])
def test_binding_runs_cpd(pkg, ctx, tmp_path, mode):
    from oracle import cpd as oc
    exe = tmp_path / "driver"
    _compile(exe)
    dims, R = (30, 26, 22), 4
    X, init = _problem(dims, R, 3)
    np.asfortranarray(X).reshape(-1, order="F").tofile(tmp_path / "x.bin")
    for k, f in enumerate(init):
        np.asfortranarray(f).reshape(-1, order="F").tofile(tmp_path / f"init{k}.bin")
    out = subprocess.run([str(exe), mode, *map(str, dims), str(R), str(tmp_path / "x.bin"),
                          str(tmp_path / "init"), str(tmp_path / "out")], check=True, capture_output=True,
                         text=True).stdout.split()
    rel, iters = float(out[1]), int(out[3])
    facs = [np.fromfile(tmp_path / f"out{k}.bin").reshape(dims[k], R, order="F") for k in range(3)]
    # writeToFile: factor k row-major FP64 (the reference writes the transpose)
    written = [np.fromfile(tmp_path / f"outfinal_{k}.bin").reshape(dims[k], R) for k in range(3)]
    for a, b in zip(facs, written):
        assert np.array_equal(a, b)
    # the same call through the Python mirror gives the same bits
    fn = pkg.cpd if mode == "cpd" else pkg.cpdDimTree
    st = fn(X, R, pkg.Options(order=3, max_iter=15), init, ctx=ctx)
    assert iters == st.ao_iter == 15
    assert rel == st.rel_costFunction
    for a, b in zip(facs, st.factors):
        assert np.array_equal(a, b)
    ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=15), init)
    assert abs(rel - ref.rel_costFunction) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["gtc", "gtc_stochastic"])
def test_binding_runs_gtc(pkg, ctx, tmp_path, mode):
    exe = tmp_path / "driver"
    _compile(exe)
    dims, R, nnz = (40, 35, 30), 3, 6000
    rng = np.random.default_rng(9)
    flat = rng.choice(int(np.prod(dims)), nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims, order="F"))
    A = [rng.random((I, R)) for I in dims]
    vals = (A[0][idx[0]] * A[1][idx[1]] * A[2][idx[2]]).sum(1)
    rb = np.vstack([idx.astype(np.float64), vals[None, :]])          # (N+1) x nnz Ratings_Base_T
    np.asfortranarray(rb).reshape(-1, order="F").tofile(tmp_path / "ratings.bin")
    init = [rng.random((I, R)) for I in dims]
    for k, f in enumerate(init):
        np.asfortranarray(f).reshape(-1, order="F").tofile(tmp_path / f"init{k}.bin")
    out = subprocess.run([str(exe), mode, *map(str, dims), str(R), str(nnz), str(tmp_path / "ratings.bin"),
                          str(tmp_path / "init")], check=True, capture_output=True, text=True).stdout.split()
    rel = float(out[1])
    so = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), nonZeros=nnz, max_iter=3, threshold_error=0.0,
                           lambdas=[1e-3] * 3, c_stochastic_perc=0.1, factorsInit=init)
    st = (pkg.gtc if mode == "gtc" else pkg.gtc_stochastic)(rb, so, ctx=ctx)
    assert rel == st.rel_costFunction
