"""GPU parity of the full CPD-ALS loop (ptg_cpd / ptg_cpd_als) against the FP64 oracle
(oracle/cpd.py, a restatement of include/Cpd.hpp:288-356) on the same tensor and the
same initial factors.

Bars (FP32 path): the per-sweep relative cost follows the oracle within 1e-4 absolute,
the final relative fit error is within 1e-3 of the oracle's and the factor congruence
after permutation and scaling is >= 0.99."""
import numpy as np
import pytest
import torch

from oracle import cpd as oc

pytestmark = pytest.mark.gpu


def _cfg1_like(dims, R, seed=0, snr_db=20.0):
    """Config-1 recipe at a size the oracle runs in seconds: U[0,1] ground truth (seed),
    Gaussian noise at snr_db, U[0,1] initial factors (seed+1)."""
    rng = np.random.default_rng(seed)
    A = [rng.random((I, R)) for I in dims]
    T = np.einsum("ir,jr,kr->ijk", *A)
    sigma = np.sqrt((T ** 2).sum() / (T.size * 10 ** (snr_db / 10)))
    X = T + sigma * rng.standard_normal(dims)
    rng1 = np.random.default_rng(seed + 1)
    init = [rng1.random((I, R)) for I in dims]
    return X, A, init


def test_cpd_fp32_matches_oracle_config1_shape_small(pkg, ctx):
    X, A, init = _cfg1_like((40, 36, 32), 6)
    opts = pkg.Options(order=3, max_iter=20)
    st = pkg.cpd(X, 6, opts, init, ctx=ctx)
    ref = oc.cpd_als(X, 6, oc.Options(order=3, max_iter=20), init)
    assert st.ao_iter == ref.ao_iter == 20
    rel_gpu = [t["rel"] for t in st.trace]
    rel_ref = [s["rel"] for s in ref.trace]
    assert np.max(np.abs(np.array(rel_gpu) - np.array(rel_ref))) < 1e-4, (rel_gpu, rel_ref)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3
    assert oc.congruence(st.factors, ref.factors) >= 0.99
    # the reported cost is the cost of the returned factors
    assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=1e-4)


def test_one_sweep_parity(pkg, ctx):
    """One FP32 sweep against the FP64 oracle: every factor within 1e-5 relative (Frobenius),
    the bar the reference's double-precision path sets for the FP32 form."""
    X, _, init = _cfg1_like((30, 28, 26), 5, seed=3)
    opts = pkg.Options(order=3, max_iter=1)
    st = pkg.cpd(X, 5, opts, init, ctx=ctx)
    ref = oc.cpd_als(X, 5, oc.Options(order=3, max_iter=1), init)
    assert st.trace[0]["nesterov_iters"] == ref.trace[0]["nesterov_iters"]
    for k in range(3):
        err = np.linalg.norm(st.factors[k] - ref.factors[k]) / np.linalg.norm(ref.factors[k])
        assert err < 1e-5, (k, err)
    assert st.rel_costFunction == pytest.approx(ref.rel_costFunction, rel=1e-5)


def test_cpd_config1_full_size(pkg, ctx):
    """Config 1 at its own size: 200^3, R=10, 20 dB, 20 outer iterations.  Compared with the
    FP64 oracle: the MTTKRP of every mode (1e-5 relative), the relative cost of every sweep
    (1e-4 absolute), the final fit (1e-3) and the factors (congruence >= 0.99)."""
    X, A, init = _cfg1_like((200, 200, 200), 10, seed=0)
    T = pkg.Tensor(ctx, np.asfortranarray(X))
    dev = [torch.tensor(np.ascontiguousarray(f), dtype=torch.float32, device="cuda:0") for f in init]
    for mode in range(3):
        out = torch.empty((200, 10), dtype=torch.float32, device="cuda:0")
        pkg.mttkrp(ctx, T, [d.data_ptr() for d in dev], 10, mode, out.data_ptr())
        ctx.synchronize()
        ref_m = oc.mttkrp(init, X, mode)
        err = np.linalg.norm(out.cpu().double().numpy() - ref_m) / np.linalg.norm(ref_m)
        assert err < 1e-5, (mode, err)
    T.close()
    st = pkg.cpd(X, 10, pkg.Options(order=3, max_iter=20), init, ctx=ctx)
    ref = oc.cpd_als(X, 10, oc.Options(order=3, max_iter=20), init, cost="gram")
    assert st.ao_iter == ref.ao_iter == 20
    rel_gpu = np.array([t["rel"] for t in st.trace][:20])
    rel_ref = np.array([s["rel"] for s in ref.trace][:20])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 1e-4, (rel_gpu, rel_ref)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3
    assert oc.congruence(st.factors, ref.factors) >= 0.99


def test_cpd_bf16_with_refinement(pkg, ctx):
    X, A, init = _cfg1_like((48, 40, 36), 6, seed=5, snr_db=30.0)
    ref = oc.cpd_als(X, 6, oc.Options(order=3, max_iter=25), init)
    st = pkg.cpd(X, 6, pkg.Options(order=3, max_iter=25, precision="bf16", refine_sweeps=1), init, ctx=ctx)
    assert st.refine_sweeps_done == 1
    # the refined cost is measured on the FP32 copy and is the cost of the returned factors
    assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=1e-3)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3


def test_cpd_deterministic(pkg, ctx):
    X, _, init = _cfg1_like((33, 29, 25), 4, seed=9)
    a = pkg.cpd(X, 4, pkg.Options(order=3, max_iter=8), init, ctx=ctx)
    b = pkg.cpd(X, 4, pkg.Options(order=3, max_iter=8), init, ctx=ctx)
    for k in range(3):
        assert np.array_equal(a.factors[k], b.factors[k])
    assert a.f_value == b.f_value


@pytest.mark.parametrize("R", [40, 64])
def test_wide_rank_one_sweep_parity_and_determinism(pkg, ctx, R):
    """Ranks above 32: the tridiagonal of the eigenvalue-bound kernel spans two warps and the
    NNLS solves two columns per lane.  Two one-sweep solves give the same bits, and the sweep
    matches the FP64 oracle (the small-rank one-sweep bar, widened to 1e-3 for the R-term
    gradients of 50 FP32 Nesterov steps)."""
    X, _, init = _cfg1_like((90, 80, 70), R, seed=R)
    opts = pkg.Options(order=3, max_iter=1)
    a = pkg.cpd(X, R, opts, init, ctx=ctx)
    b = pkg.cpd(X, R, opts, init, ctx=ctx)
    for k in range(3):
        assert np.array_equal(a.factors[k], b.factors[k]), k
    ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=1), init)
    assert a.trace[0]["nesterov_iters"] == ref.trace[0]["nesterov_iters"]
    for k in range(3):
        err = np.linalg.norm(a.factors[k] - ref.factors[k]) / np.linalg.norm(ref.factors[k])
        assert err < 1e-3, (k, err)
    assert a.rel_costFunction == pytest.approx(ref.rel_costFunction, rel=1e-4)


def test_cpd_4way(pkg, ctx):
    rng = np.random.default_rng(11)
    dims, R = (12, 11, 10, 9), 3
    A = [rng.random((I, R)) for I in dims]
    X = np.einsum("ir,jr,kr,lr->ijkl", *A) + 0.01 * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    st = pkg.cpd(X, R, pkg.Options(order=4, max_iter=15), init, ctx=ctx)
    ref = oc.cpd_als(X, R, oc.Options(order=4, max_iter=15), init)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3


def test_cpd_error_paths(pkg, ctx):
    X, _, init = _cfg1_like((10, 9, 8), 3, seed=2)
    bad = [f.copy() for f in init]
    bad[1][0, 0] = np.nan
    with pytest.raises(pkg._lib.PtgError) as e:
        pkg.cpd(X, 3, pkg.Options(order=3, max_iter=2), bad, ctx=ctx)
    assert e.value.code == pkg._lib.PTG_ERR_NUMERIC
    with pytest.raises(pkg._lib.PtgError) as e:
        big = [np.ones((I, 65)) for I in X.shape]
        pkg.cpd(X, 65, pkg.Options(order=3, max_iter=2), big, ctx=ctx)
    assert e.value.code == pkg._lib.PTG_ERR_UNSUPPORTED
    # the context is still usable afterwards
    st = pkg.cpd(X, 3, pkg.Options(order=3, max_iter=2), init, ctx=ctx)
    assert np.isfinite(st.f_value)


def test_cpd_dimtree_matches_oracle(pkg, ctx):
    """cpdDimTree (include/CpdDimTree.hpp:317-401) on a 4-way tensor, split {0,1}|{2,3}."""
    rng = np.random.default_rng(21)
    dims, R = (20, 18, 16, 14), 5
    A = [rng.random((I, R)) for I in dims]
    X = np.einsum("ir,jr,kr,lr->ijkl", *A) + 0.05 * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    st = pkg.cpdDimTree(X, R, pkg.Options(order=4, max_iter=12), init, ctx=ctx)
    ref = oc.cpd_dimtree_als(X, R, oc.Options(order=4, max_iter=12), init)
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([s["rel"] for s in ref.trace])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 1e-4
    assert oc.congruence(st.factors, ref.factors) >= 0.99


@pytest.mark.parametrize("precision", ["f32", "bf16"])
def test_cpd_dimtree_equals_cpd(pkg, ctx, precision):
    """The dimension tree is an exact reorganisation: same trajectory as cpd."""
    rng = np.random.default_rng(22)
    dims, R = (24, 20, 17, 13), 6
    A = [rng.random((I, R)) for I in dims]
    X = np.einsum("ir,jr,kr,lr->ijkl", *A) + 0.05 * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    o = pkg.Options(order=4, max_iter=8, precision=precision)
    a = pkg.cpdDimTree(X, R, o, init, ctx=ctx)
    b = pkg.cpd(X, R, o, init, ctx=ctx)
    tol = 1e-4 if precision == "f32" else 2e-3
    assert abs(a.rel_costFunction - b.rel_costFunction) < tol


def test_cpd_dimtree_3way(pkg, ctx):
    X, _, init = _cfg1_like((30, 26, 22), 4, seed=23)
    st = pkg.cpdDimTree(X, 4, pkg.Options(order=3, max_iter=10), init, ctx=ctx)
    ref = oc.cpd_dimtree_als(X, 4, oc.Options(order=3, max_iter=10), init)
    assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-4


def test_cpd_bf16_verify_fp32_reports_fp32_cost(pkg, ctx):
    """verify_fp32: after a BF16 main loop the reported cost is the final factors' cost on the
    FP32 copy (one CUDA-core FP32 MTTKRP, the Gram term from FP64 Grams), so it equals the FP64
    residual of the returned factors to what FP32 arithmetic allows.  The Gram form cancels:
    f^2 = ||X||^2 - 2<M, A> + ..., with f^2 ~ 1e-3 ||X||^2 at 30 dB, so a relative error e of
    the FP32 <M, A> moves f by ~1100 e; the bar, 5e-5 on f, is e < 4.5e-8, below FP32's unit
    roundoff (6e-8)."""
    X, A, init = _cfg1_like((48, 40, 36), 6, seed=6, snr_db=30.0)
    st = pkg.cpd(X, 6, pkg.Options(order=3, max_iter=12, precision="bf16", verify_fp32=True), init, ctx=ctx)
    assert st.refine_sweeps_done == 0
    assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=5e-5)
    plain = pkg.cpd(X, 6, pkg.Options(order=3, max_iter=12, precision="bf16"), init, ctx=ctx)
    # the same factors; only where the cost is measured differs
    for k in range(3):
        assert np.array_equal(st.factors[k], plain.factors[k])


U_, N_, O_, S_, C_ = oc.UNCONSTRAINED, oc.NONNEGATIVITY, oc.ORTHOGONALITY, oc.SPARSITY, oc.CONSTANT


@pytest.mark.parametrize("cons", [(U_, U_, U_), (O_, N_, N_), (N_, U_, N_), (C_, N_, N_), (S_, N_, U_),
                                  (U_, O_, N_)])
def test_constraints_match_oracle(pkg, ctx, cons):
    """update_factor for every constraint (include/Cpd.hpp:189-228): unconstrained A = M Z^-1,
    orthogonality A = M (M^T M)^-1/2, sparsity/constant keep the factor; normalisation and
    acceleration as the reference applies them.  Per-sweep relative cost within 1e-4 of the
    FP64 oracle for 8 sweeps."""
    X, A, init = _cfg1_like((36, 30, 28), 5, seed=11)
    o = pkg.Options(order=3, max_iter=8, constraints=list(cons))
    st = pkg.cpd(X, 5, o, init, ctx=ctx)
    ref = oc.cpd_als(X, 5, oc.Options(order=3, max_iter=8, constraints=list(cons)), init)
    assert st.ao_iter == ref.ao_iter
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([s["rel"] for s in ref.trace])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 1e-4, (rel_gpu, rel_ref)
    for k in range(3):
        if cons[k] in (C_, S_):
            assert np.array_equal(st.factors[k], np.asarray(init[k], dtype=np.float32).astype(np.float64)) or \
                oc.congruence([st.factors[k]], [ref.factors[k]]) > 0.999
    assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=1e-4)


def test_orthogonal_factor_is_orthonormal(pkg, ctx):
    X, A, init = _cfg1_like((40, 30, 28), 4, seed=12)
    # (the line-search extrapolation of include/Cpd.hpp:247-278 mixes two orthonormal factors,
    # so it is off here)
    st = pkg.cpd(X, 4, pkg.Options(order=3, max_iter=3, constraints=[O_, N_, N_], normalization=False,
                                   acceleration=False), init, ctx=ctx)
    Q = st.factors[0]
    assert np.abs(Q.T @ Q - np.eye(4)).max() < 1e-4


def test_cpd_from_files_matches_in_memory(pkg, ctx, tmp_path):
    """cpd(tnsDims, R, paths[, options]) with the reference's file formats (ColMajor FP64
    tensor after `skip` values, row-major FP64 factors): the same result as the in-memory call."""
    X, _, init = _cfg1_like((30, 26, 22), 4, seed=31)
    tpath = tmp_path / "x.bin"
    # 5 leading values to skip, as read(path, size, skip, ...) allows
    np.concatenate([np.full(5, 7.0), np.asfortranarray(X).reshape(-1, order="F")]).tofile(tpath)
    fpaths = []
    for k, A in enumerate(init):
        fpaths.append(str(tmp_path / f"a{k}.bin"))
        pkg.write_factor_file(fpaths[-1], A)
    o = pkg.Options(order=3, max_iter=6)
    st_f = pkg.cpd_file(X.shape, 4, [str(tpath)] + fpaths, o, skip=5, ctx=ctx)
    st_m = pkg.cpd(X, 4, o, init, ctx=ctx)
    for k in range(3):
        assert np.array_equal(st_f.factors[k], st_m.factors[k])
    assert st_f.f_value == st_m.f_value
    # the tensor alone, with seeded initial factors: a valid run, reproducible
    pkg.write_tensor_file(tmp_path / "y.bin", X)
    a = pkg.cpd_file(X.shape, 4, str(tmp_path / "y.bin"), o, seed=3, ctx=ctx)
    b = pkg.cpd_file(X.shape, 4, str(tmp_path / "y.bin"), o, seed=3, ctx=ctx)
    assert np.array_equal(a.factors[0], b.factors[0]) and np.isfinite(a.f_value)
    with pytest.raises(pkg.PtgError):
        pkg.cpd_file((31, 26, 22), 4, str(tmp_path / "y.bin"), o, ctx=ctx)   # file too short


def _nway_problem(dims, R, seed):
    rng = np.random.default_rng(seed)
    A = [rng.random((I, R)) for I in dims]
    sub = "abcdefgh"[:len(dims)]
    X = np.einsum(",".join(c + "r" for c in sub) + "->" + sub, *A)
    X = X + 0.02 * X.std() * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    return X, init


@pytest.mark.parametrize("dims", [(9, 8, 7, 6, 5), (6, 5, 5, 4, 4, 3), (4, 4, 3, 3, 3, 3, 2), (3, 3, 3, 3, 2, 2, 2, 2)])
def test_cpd_orders_5_to_8_match_oracle(pkg, ctx, dims):
    """Orders 5-8 (the reference supports 3-8): cpd and cpdDimTree (split at (1+N)/2) follow
    the FP64 oracle per sweep."""
    N, R = len(dims), 3
    X, init = _nway_problem(dims, R, 40 + N)
    o = pkg.Options(order=N, max_iter=6)
    ref = oc.cpd_als(X, R, oc.Options(order=N, max_iter=6), init)
    rel_ref = np.array([s["rel"] for s in ref.trace])
    for fn in (pkg.cpd, pkg.cpdDimTree):
        st = fn(X, R, o, init, ctx=ctx)
        rel = np.array([t["rel"] for t in st.trace])
        assert st.ao_iter == ref.ao_iter
        assert np.max(np.abs(rel - rel_ref)) < 1e-4, (fn.__name__, rel, rel_ref)


@pytest.mark.parametrize("case", ["clustered", "large_scale"])
def test_eigen_bounds_hard_z(pkg, ctx, case):
    """The FP64 eigenvalue bounds (L, mu) of Z = Hadamard of the Grams where the FP32 bracket
    cannot be trusted.  clustered: two nearly equal columns in every initial factor make
    cond(Z) >= 1e6, where GLambda switches lambda to 10 mu (include/NesterovMNLS.hpp:75-91);
    large_scale: initial factors of size 1e6 put Z's tridiagonal squares beyond FP32 range.
    One sweep against the FP64 oracle: same inner iteration counts, same cost, factors within
    1e-4 (clustered: 1e-3, the ill-conditioned directions move little in 50 steps)."""
    rng = np.random.default_rng(21)
    dims, R = (40, 36, 32), 6
    X, _, _ = _cfg1_like(dims, R, seed=21)
    init = [rng.random((I, R)) for I in dims]
    if case == "clustered":
        for f in init:
            f[:, 1] = f[:, 0] * (1 + 1e-3 * rng.standard_normal(f.shape[0]))
        Z = (init[1].T @ init[1]) * (init[2].T @ init[2])
        w = np.linalg.eigvalsh(Z)
        assert w.max() / w.min() >= 1e6
        bar = 1e-3
    else:
        init = [f * 1e6 for f in init]
        bar = 1e-4
    st = pkg.cpd(X, R, pkg.Options(order=3, max_iter=1, acceleration=False), init, ctx=ctx)
    ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=1, acceleration=False), init)
    assert st.trace[0]["nesterov_iters"] == ref.trace[0]["nesterov_iters"]
    assert st.rel_costFunction == pytest.approx(ref.rel_costFunction, rel=1e-4)
    for k in range(3):
        err = np.linalg.norm(st.factors[k] - ref.factors[k]) / np.linalg.norm(ref.factors[k])
        assert err < bar, (k, err)


def test_dimtree_order5_mixed_constraints_matches_direct(pkg, ctx):
    """Order 5: the tree splits [0,5) -> [0,3) [3,5) -> [0,2) [2,3) ..., so modes 0 and 1 come
    from a node recomputed from its parent (include/DimTrees.hpp:862-928).  With an
    unconstrained and an orthogonal mode among nonnegative ones, cpdDimTree follows the
    direct cpd per sweep (the same algorithm, another summation order) and the oracle."""
    dims, R = (9, 8, 7, 6, 5), 3
    X, init = _nway_problem(dims, R, 77)
    cons = [pkg.UNCONSTRAINED, pkg.NONNEGATIVITY, pkg.ORTHOGONALITY, pkg.NONNEGATIVITY, pkg.NONNEGATIVITY]
    o = pkg.Options(order=5, max_iter=6, constraints=cons)
    st_t = pkg.cpdDimTree(X, R, o, init, ctx=ctx)
    st_d = pkg.cpd(X, R, o, init, ctx=ctx)
    ref = oc.cpd_als(X, R, oc.Options(order=5, max_iter=6, constraints=cons), init)
    rel_t = np.array([t["rel"] for t in st_t.trace])
    rel_d = np.array([t["rel"] for t in st_d.trace])
    rel_r = np.array([s["rel"] for s in ref.trace])
    assert st_t.ao_iter == st_d.ao_iter == ref.ao_iter
    assert np.max(np.abs(rel_t - rel_d)) < 1e-5, (rel_t, rel_d)
    assert np.max(np.abs(rel_t - rel_r)) < 1e-4, (rel_t, rel_r)
