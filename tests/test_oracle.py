"""CPU tests of the FP64 oracle: the restatement must agree with independent
formulations and with the C restatement (oracle/cpd_omp.c) before it may judge the GPU."""
import math

import numpy as np
import pytest

from oracle import cpd as oc
from oracle import omp


def _problem(dims, R, seed=0, noise=0.01):
    rng = np.random.default_rng(seed)
    A = [rng.random((I, R)) for I in dims]
    T = np.einsum("ir,jr,kr->ijk", *A) if len(dims) == 3 else np.einsum("ir,jr,kr,lr->ijkl", *A)
    X = T + noise * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    return X, A, init


def test_matricization_order():
    # X_(n)[i_n, j] with j = sum_{k != n} i_k prod_{l<k, l != n} I_l  (Matricization.hpp:65-124)
    dims = (3, 4, 5)
    X = np.arange(60, dtype=float).reshape(dims, order="F")
    for n in range(3):
        Xn = oc.matricization(X, n)
        others = [k for k in range(3) if k != n]
        for idx in np.ndindex(*dims):
            j = idx[others[0]] + dims[others[0]] * idx[others[1]]
            assert Xn[idx[n], j] == X[idx]


def test_khatri_rao_first_argument_slowest():
    rng = np.random.default_rng(1)
    A, B = rng.random((3, 2)), rng.random((4, 2))
    K = oc.khatri_rao(A, B)
    for ia in range(3):
        for ib in range(4):
            assert np.allclose(K[ib + 4 * ia], A[ia] * B[ib])


@pytest.mark.parametrize("dims", [(7, 5, 3), (6, 5, 4, 3), (9, 1, 4)])
def test_mttkrp_matches_einsum_and_c(dims):
    rng = np.random.default_rng(2)
    R = 3
    X = rng.standard_normal(dims)
    f = [rng.standard_normal((I, R)) for I in dims]
    flat = X.reshape(-1, order="F")
    for n in range(len(dims)):
        a = oc.mttkrp(f, X, n)
        b = oc.mttkrp_einsum(f, X, n)
        c = omp.mttkrp(flat, list(dims), f, n)
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
        assert np.allclose(a, c, rtol=1e-12, atol=1e-12)


def test_glambda_branches():
    # include/NesterovMNLS.hpp:75-91
    L, mu, lam, q = oc.glambda(1.0, 10.0)       # 1/q = 10 -> lambda = mu/10
    assert lam == pytest.approx(0.1) and L == pytest.approx(10.1) and q == pytest.approx(1.1 / 10.1)
    _, _, lam, _ = oc.glambda(1e-4, 10.0)       # 1/q = 1e5 -> lambda = mu
    assert lam == pytest.approx(1e-4)
    _, _, lam, _ = oc.glambda(1e-8, 10.0)       # 1/q = 1e9 -> lambda = 10 mu
    assert lam == pytest.approx(1e-7)


def test_update_alpha_is_positive_root():
    for alpha, q in [(1.0, 0.1), (0.5, 1e-3), (0.2, 0.9)]:
        a = oc.update_alpha(alpha, q)
        assert a > 0
        assert a * a + (alpha * alpha - q) * a - alpha * alpha == pytest.approx(0.0, abs=1e-12)


def test_nesterov_reaches_nnls_kkt():
    rng = np.random.default_rng(3)
    B = rng.random((40, 6))
    Z = B.T @ B
    W = rng.random((10, 6)) * 5
    A0 = rng.random((10, 6))
    A, info = oc.nesterov_mnls(Z, W, 1e-9, 1e-9, A0, return_info=True)
    assert info["iters"] <= oc.NESTEROV_MAX_INNER
    assert (A >= 0).all()


def test_normalize_quirk_last_factor_untouched():
    # include/Normalize.hpp:127-157: with weight 0 and N=3 only factor 1 is normalised
    rng = np.random.default_rng(4)
    f = [rng.random((5, 3)) * 3 for _ in range(3)]
    g = [a.T @ a for a in f]
    f2 = [a.copy() for a in f]
    g2 = [a.copy() for a in g]
    oc.normalize(0, 3, g2, f2)
    assert np.allclose(np.linalg.norm(f2[1], axis=0), 1.0)
    assert np.allclose(f2[2], f[2])
    # model unchanged and Grams consistent with the rescaled factors
    assert np.allclose(np.einsum("ir,jr,kr->ijk", *f2), np.einsum("ir,jr,kr->ijk", *f))
    for a, gg in zip(f2, g2):
        assert np.allclose(a.T @ a, gg)


def test_normalize_zero_last_column_skips():
    rng = np.random.default_rng(5)
    f = [rng.random((5, 2)) for _ in range(3)]
    f[2][:, 1] = 0.0
    g = [a.T @ a for a in f]
    f2 = [a.copy() for a in f]
    oc.normalize(0, 2, g, f2)
    assert np.allclose(f2[1][:, 1], f[1][:, 1])   # column 1 not rescaled (nonZeroFlag false)
    assert np.allclose(np.linalg.norm(f2[1][:, 0]), 1.0)


@pytest.mark.parametrize("accel", [True, False])
def test_als_numpy_vs_c(accel):
    X, _, init = _problem((14, 12, 10), 4, seed=6)
    flat = X.reshape(-1, order="F")
    st = oc.cpd_als(X, 4, oc.Options(order=3, max_iter=12, acceleration=accel), init)
    fs, cs, tr = omp.cpd_als(flat, [14, 12, 10], 4, init, max_iter=12, acceleration=accel)
    assert cs.ao_iter == st.ao_iter
    assert cs.rel_costFunction == pytest.approx(st.rel_costFunction, rel=1e-9)
    for k in range(3):
        assert np.allclose(fs[k], st.factors[k], rtol=1e-8, atol=1e-10)
    assert [bool(x) for x in tr[:, 2]] == [bool((s["accel"] or {}).get("accepted")) for s in st.trace]


def test_residual_and_gram_cost_agree():
    X, _, init = _problem((10, 9, 8), 3, seed=7)
    a = oc.cpd_als(X, 3, oc.Options(order=3, max_iter=6), init, cost="residual")
    b = oc.cpd_als(X, 3, oc.Options(order=3, max_iter=6), init, cost="gram")
    assert a.f_value == pytest.approx(b.f_value, rel=1e-9)


def test_als_4way():
    X, _, init = _problem((6, 5, 4, 3), 2, seed=8)
    st = oc.cpd_als(X, 2, oc.Options(order=4, max_iter=10), init)
    flat = X.reshape(-1, order="F")
    fs, cs, _ = omp.cpd_als(flat, [6, 5, 4, 3], 2, init, max_iter=10)
    assert cs.rel_costFunction == pytest.approx(st.rel_costFunction, rel=1e-9)
    assert math.isclose(oc.cost_from_factors(X, st.factors), st.f_value, rel_tol=1e-6)
