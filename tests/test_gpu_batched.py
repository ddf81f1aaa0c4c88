"""GPU parity of the batched many-instance CPD (ptg_cpd_batched) against the FP64 oracle
(oracle/cpd.py, include/Cpd.hpp:288-356 restated) instance by instance, and against the
single-instance GPU path (ptg_cpd) on the same inputs.

Bars: one sweep matches the oracle to 1e-4 relative per factor; after 15 sweeps each
instance's relative error is within 1e-3 of the oracle's with factor congruence >= 0.99;
each instance's sweep count, stop decision and cost equal the single-instance path's.
Every test runs both solvers: the persistent one (one launch for the batch) and the
per-phase graphs."""
import numpy as np
import pytest

from oracle import cpd as oc

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["persistent", "graphs"], autouse=True)
def impl(request, ctx):
    ctx.set_batched_impl(request.param)
    yield request.param
    ctx.set_batched_impl("persistent")


def _instance(dims, R, seed, snr_db=20.0):
    rng = np.random.default_rng(seed)
    A = [rng.random((I, R)) for I in dims]
    T = np.einsum("ir,jr,kr->ijk", *A)
    sigma = np.sqrt((T ** 2).sum() / (T.size * 10 ** (snr_db / 10)))
    X = T + sigma * rng.standard_normal(dims)
    init = [np.random.default_rng(seed + 100).random((I, R)) for I in dims]
    return X, R, init


UNEVEN = [((21, 30, 17), 3, 1), ((40, 26, 33), 7, 2), ((13, 45, 20), 5, 3), ((32, 32, 32), 8, 4),
          ((50, 12, 29), 4, 5)]


def test_batched_one_sweep_matches_oracle(pkg, ctx):
    probs = [_instance(d, R, s) for d, R, s in UNEVEN]
    sts, _ = pkg.cpd_batched(probs, pkg.Options(order=3, max_iter=1), ctx=ctx)
    for (X, R, init), st in zip(probs, sts):
        ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=1), init)
        assert st.ao_iter == 1
        for k in range(3):
            err = np.linalg.norm(st.factors[k] - ref.factors[k]) / np.linalg.norm(ref.factors[k])
            assert err < 1e-4, (X.shape, k, err)
        assert st.rel_costFunction == pytest.approx(ref.rel_costFunction, rel=1e-5)


def test_batched_matches_oracle_and_single_path(pkg, ctx):
    probs = [_instance(d, R, s) for d, R, s in UNEVEN]
    opts = pkg.Options(order=3, max_iter=15)
    sts, secs = pkg.cpd_batched(probs, opts, ctx=ctx)
    assert np.all(secs > 0)
    for (X, R, init), st in zip(probs, sts):
        ref = oc.cpd_als(X, R, oc.Options(order=3, max_iter=15), init)
        assert st.ao_iter == ref.ao_iter == 15
        assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3
        assert oc.congruence(st.factors, ref.factors) >= 0.99
        # the reported cost is the cost of the returned factors
        assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=1e-4)
        one = pkg.cpd(X, R, opts, init, ctx=ctx)
        assert one.ao_iter == st.ao_iter
        assert st.rel_costFunction == pytest.approx(one.rel_costFunction, abs=1e-4)


def test_instances_stop_independently(pkg, ctx):
    """A threshold that some instances reach early: each stops on its own test, with the
    sweep count the single-instance path gives it."""
    probs = [_instance(d, R, s, snr_db=40.0) for d, R, s in UNEVEN]
    opts = pkg.Options(order=3, max_iter=60, threshold_error=0.02)
    sts, secs = pkg.cpd_batched(probs, opts, ctx=ctx)
    iters = [st.ao_iter for st in sts]
    singles = [pkg.cpd(X, R, opts, init, ctx=ctx) for X, R, init in probs]
    for st, one in zip(sts, singles):
        assert st.ao_iter == one.ao_iter
        if st.ao_iter < 60:
            assert st.rel_costFunction < 0.02
    assert len(set(iters)) > 1, iters
    # an instance that stopped earlier finished no later
    order = np.argsort(iters)
    assert secs[order[0]] <= secs[order[-1]]


def test_fmri_batch_shape(pkg, ctx):
    """The fMRI-like generator (sparse spatial maps, smooth time courses, uneven dims and
    ranks) at reduced count: every instance's reported cost is the cost of its returned
    factors and matches the single-instance path on a sample."""
    batch = pkg.datagen.make_fmri_batch(12, seed=4)
    probs = [(b.X, b.rank, b.init_factors) for b in batch]
    opts = pkg.Options(order=3, max_iter=40, threshold_error=0.0)
    sts, _ = pkg.cpd_batched(probs, opts, ctx=ctx)
    for (X, R, init), st in zip(probs, sts):
        assert oc.cost_from_factors(X, st.factors) == pytest.approx(st.f_value, rel=1e-3)
    for i in (0, 5, 11):
        X, R, init = probs[i]
        one = pkg.cpd(X, R, opts, init, ctx=ctx)
        assert sts[i].rel_costFunction == pytest.approx(one.rel_costFunction, abs=1e-4)


def test_batched_rejects_unsupported(pkg, ctx):
    X, R, init = _instance((10, 11, 12), 3, 0)
    X4 = np.random.default_rng(0).random((4, 5, 6, 7))
    with pytest.raises(pkg.PtgError):
        pkg.cpd_batched([(X, R, init), (X4, 2, [np.ones((I, 2)) for I in X4.shape])], pkg.Options(order=3),
                        ctx=ctx)
    Xb, Rb, initb = _instance((10, 11, 12), 40, 0)
    with pytest.raises(pkg.PtgError):
        pkg.cpd_batched([(Xb, Rb, initb)], pkg.Options(order=3), ctx=ctx)


def test_persistent_and_graph_solvers_agree(pkg, ctx, impl):
    """The same batch through both solvers: the same sweeps per instance and the same fit to
    FP32 summation-order differences (the MTTKRP K-splits differ)."""
    if impl != "persistent":
        pytest.skip("compares the two solvers once")
    batch = pkg.datagen.make_fmri_batch(24, seed=9)
    probs = [(b.X, b.rank, b.init_factors) for b in batch]
    opts = pkg.Options(order=3, max_iter=30, threshold_error=0.0)
    per, _ = pkg.cpd_batched(probs, opts, ctx=ctx)
    ctx.set_batched_impl("graphs")
    gra, _ = pkg.cpd_batched(probs, opts, ctx=ctx)
    for a, b in zip(per, gra):
        assert a.ao_iter == b.ao_iter == 30
        assert a.rel_costFunction == pytest.approx(b.rel_costFunction, abs=2e-5)
        assert oc.congruence(a.factors, b.factors) >= 0.999


def test_batched_order4_matches_single_path(pkg, ctx, impl):
    """A batch of 4-way instances (the solvers take orders 3-8): the same sweeps as the single-
    instance path, the fit within 1e-4 of it and within 1e-3 of the FP64 oracle."""
    probs = []
    for s, (dims, R) in enumerate([((12, 10, 9, 8), 3), ((9, 14, 7, 10), 5), ((16, 8, 8, 6), 4)]):
        rng = np.random.default_rng(40 + s)
        A = [rng.random((I, R)) for I in dims]
        X = np.einsum("ir,jr,kr,lr->ijkl", *A)
        X = X + 0.05 * np.sqrt((X ** 2).mean()) * rng.standard_normal(dims)
        init = [np.random.default_rng(140 + s).random((I, R)) for I in dims]
        probs.append((X, R, init))
    opts = pkg.Options(order=4, max_iter=12)
    sts, _ = pkg.cpd_batched(probs, opts, ctx=ctx)
    for (X, R, init), st in zip(probs, sts):
        one = pkg.cpd(X, R, opts, init, ctx=ctx)
        assert st.ao_iter == one.ao_iter == 12
        assert st.rel_costFunction == pytest.approx(one.rel_costFunction, abs=1e-4)
        ref = oc.cpd_als(X, R, oc.Options(order=4, max_iter=12), init)
        assert abs(st.rel_costFunction - ref.rel_costFunction) < 1e-3
