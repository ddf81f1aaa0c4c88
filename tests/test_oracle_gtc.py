"""CPU tests of the GTC oracle (oracle/gtc.py) and of the warm-start MLP oracle."""
import functools

import numpy as np
import pytest

from oracle import cpd as oc
from oracle import gtc as og
from oracle import mlp as om


def sort_rows_literal(N, mode):
    """SortRows<N, mode> (include/TensorOperations.hpp:622-666) restated line by line as a
    comparator: sort_direction = {mode, last (or last-1), then downwards skipping mode}."""
    direction = [mode, N - 1 if mode < N - 1 else N - 2]
    for i in range(2, N):
        d = direction[i - 1] - 1
        if d == mode:
            d -= 1
        direction.append(d)

    def less(v1, v2):
        prev_equal = False
        for i in range(N):
            a, b = v1[direction[i]], v2[direction[i]]
            if i == 0:
                if a < b:
                    return True
                prev_equal = a == b
            else:
                if prev_equal and a < b:
                    return True
                prev_equal = prev_equal and a == b
        return False

    return lambda x, y: -1 if less(x, y) else (1 if less(y, x) else 0)


@pytest.mark.parametrize("dims", [(7, 5, 4), (4, 3, 5, 2)])
def test_sort_key_equals_sortrows(dims):
    idx, vals, _ = og.make_gtc_problem(dims, 60, 2, seed=1)
    N = len(dims)
    rows = [list(idx[:, e]) + [e] for e in range(idx.shape[1])]
    for mode in range(N):
        ref = sorted(rows, key=functools.cmp_to_key(sort_rows_literal(N, mode)))
        got = og.matricize(idx, vals, dims, mode).perm
        assert [r[-1] for r in ref] == list(got)


def test_sparse_mttkrp_matches_dense():
    dims, R = (9, 8, 7), 3
    idx, vals, _ = og.make_gtc_problem(dims, 150, R, seed=2)
    rng = np.random.default_rng(3)
    f = [rng.random((I, R)) for I in dims]
    Xd = np.zeros(dims)
    Xd[tuple(idx)] = vals
    for n in range(3):
        assert np.allclose(og.sparse_mttkrp(f, og.matricize(idx, vals, dims, n)), oc.mttkrp(f, Xd, n))


def test_power_method_reaches_top_eigenvalue():
    rng = np.random.default_rng(4)
    K = rng.random((50, 6))
    H = K.T @ K
    assert og.power_method(H, 1e-9) == pytest.approx(np.linalg.eigvalsh(H).max(), rel=1e-8)


def test_gtc_decreases_cost_and_stochastic_is_deterministic():
    dims, R = (20, 18, 16), 3
    idx, vals, _ = og.make_gtc_problem(dims, 1500, R, seed=5)
    rng = np.random.default_rng(6)
    init = [rng.random((I, R)) for I in dims]
    st = og.gtc(idx, vals, dims, R, og.SparseOptions(order=3, max_iter=4, lambdas=[1e-3] * 3), init)
    rels = [t["rel"] for t in st.trace]
    assert rels[-1] < rels[0]
    o = og.SparseOptions(order=3, max_iter=1, c_stochastic_perc=0.2, lambdas=[1e-3] * 3, seed=9)
    a = og.gtc_stochastic(idx, vals, dims, R, o, init)
    b = og.gtc_stochastic(idx, vals, dims, R, o, init)
    for k in range(3):
        assert np.array_equal(a.factors[k], b.factors[k])


def test_pivot_hash_known_values():
    # splitmix64 finaliser of the mixed coordinates (the GPU sampler uses the same arithmetic)
    assert og.pivot_hash(0, 0, 0, 0, 0) == 0
    assert og.pivot_hash(1, 2, 3, 4, 5) == og.pivot_hash(1, 2, 3, 4, 5)
    assert og.pivot_hash(1, 2, 3, 4, 5) != og.pivot_hash(1, 2, 3, 4, 6)


def test_mlp_gradient_finite_differences():
    din, h, dout = 5, 8, 3
    rng = np.random.default_rng(7)
    theta = om.init(din, h, dout, 2) + 0.01 * rng.standard_normal(om.nparams(din, h, dout))
    X, T = rng.standard_normal((6, din)), rng.standard_normal((6, dout))
    _, g = om.loss_and_grad(theta, X, T, din, h, dout)
    for i in range(len(theta)):
        e = np.zeros_like(theta)
        e[i] = 1e-6
        fd = (om.loss_and_grad(theta + e, X, T, din, h, dout)[0] - om.loss_and_grad(theta - e, X, T, din, h, dout)[0]) / 2e-6
        assert fd == pytest.approx(g[i], rel=1e-4, abs=1e-9)


def test_ridge_update_minimises_the_row_objective():
    """unconstraint_update (include/Gtc.hpp:275-315): each row minimises
    sum over its entries (x - kr.a)^2 + lambda ||a||^2, so H a - m + lambda a = 0 and a equals
    the least-squares solution of the stacked system [K; sqrt(lambda) I] a = [x; 0]."""
    dims, R, lam = (12, 10, 9), 4, 1e-2
    idx, vals, _ = og.make_gtc_problem(dims, 600, R, seed=41)
    rng = np.random.default_rng(42)
    factors = [rng.random((I, R)) for I in dims]
    for mode in range(3):
        mm = og.matricize(idx, vals, dims, mode)
        M = og.sparse_mttkrp(factors, mm)
        A = og.ridge_update(factors, mm, M, lam)
        H = og.row_hessians(factors, mm)
        kr = og.kr_rows(factors, mm)
        for i in range(dims[mode]):
            grad = H[i] @ A[i] - M[i] + lam * A[i]
            assert np.abs(grad).max() < 1e-10 * max(1.0, np.abs(M[i]).max())
            K = kr[mm.ptr[i]:mm.ptr[i + 1]]
            x = mm.vals[mm.ptr[i]:mm.ptr[i + 1]]
            stacked = np.vstack([K, np.sqrt(lam) * np.eye(R)])
            ls = np.linalg.lstsq(stacked, np.concatenate([x, np.zeros(R)]), rcond=None)[0]
            assert np.allclose(A[i], ls, rtol=1e-9, atol=1e-12)


def test_local_l_nesterov_reaches_row_kkt():
    """local_L::NesterovMNLS (include/NesterovMNLS.hpp:777-873) run long: every row meets the
    KKT conditions of min (1/2) a^T (H + lambda I) a - m^T a over a >= 0."""
    dims, R, lam = (10, 9, 8), 3, 1e-3
    idx, vals, _ = og.make_gtc_problem(dims, 500, R, seed=43)
    rng = np.random.default_rng(44)
    factors = [rng.random((I, R)) for I in dims]
    mm = og.matricize(idx, vals, dims, 0)
    M = og.sparse_mttkrp(factors, mm)
    A = og.local_L_nesterov(factors, mm, M, 3000, lam)
    H = og.row_hessians(factors, mm)
    assert (A >= 0).all()
    for i in range(dims[0]):
        grad = H[i] @ A[i] - M[i] + lam * A[i]
        scale = max(1.0, np.abs(M[i]).max())
        assert grad.min() > -1e-6 * scale                       # dual feasibility
        assert np.abs(grad * A[i]).max() < 1e-6 * scale ** 2    # complementarity


@pytest.mark.parametrize("stochastic", [False, True])
def test_c_restatement_matches_numpy_oracle(stochastic):
    """oracle/gtc_omp.c (the CPU baseline of the sparse workload) against oracle/gtc.py, one
    factor update of every mode: local_L (NesterovMNLS.hpp:878-976) or the stochastic block
    solver (:553-663)."""
    from oracle import gtc as og
    from oracle import omp
    dims, R = [30, 25, 20], 5
    idx, vals, _ = og.make_gtc_problem(dims, 3000, R, seed=1)
    init = [np.random.default_rng(k).random((I, R)) for k, I in enumerate(dims)]
    for n in range(3):
        mm = og.matricize(idx, vals, dims, n)
        if stochastic:
            ref = og.stochastic_nesterov(init, mm, 0.3, 20, 1e-3, 7, 3)
        else:
            ref = og.local_L_nesterov(init, mm, og.sparse_mttkrp(init, mm), 20, 1e-3)
        got = omp.gtc_rows(mm.ptr, mm.other, mm.vals, init, n, stochastic, 0.3, 20, 1e-3, seed=7, outer=3)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
