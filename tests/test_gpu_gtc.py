"""GPU parity of sparse tensor completion (ptg_gtc) against the FP64 oracle (oracle/gtc.py).

The index sort is bit-exact (the permutation must equal the oracle's SortRows order).  The
solves run in FP32 on the GPU: the relative cost per iteration must follow the oracle
within 2e-4 absolute (rel is a ratio of squared norms ~1e-2 here) and the factors must be
congruent >= 0.99."""
import numpy as np
import pytest
import torch

from oracle import cpd as oc
from oracle import gtc as og

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,nnz", [((60, 50, 40), 20000), ((31, 17, 23, 9), 15000), ((300, 7, 5), 3000)])
def test_sort_is_bitexact(pkg, ctx, dims, nnz):
    idx, vals, _ = og.make_gtc_problem(dims, nnz, 3, seed=nnz)
    d_idx = torch.tensor(idx.astype(np.int32), device="cuda").contiguous()
    for mode in range(len(dims)):
        perm = torch.zeros(nnz, dtype=torch.int32, device="cuda")
        pkg.gtc_sort_mode(ctx, d_idx.data_ptr(), list(dims), nnz, mode, perm.data_ptr())
        got = perm.cpu().numpy().astype(np.int64)
        ref = og.matricize(idx, vals, dims, mode).perm
        assert np.array_equal(got, ref), mode


def _problem(dims, nnz, R, seed):
    idx, vals, A = og.make_gtc_problem(dims, nnz, R, seed=seed)
    rng = np.random.default_rng(seed + 1)
    init = [rng.random((I, R)) for I in dims]
    return idx, vals, init


def test_gtc_matches_oracle(pkg, ctx):
    dims, R = (60, 50, 40), 4
    idx, vals, init = _problem(dims, 20000, R, 5)
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=8, lambdas=[1e-3] * 3,
                          factorsInit=init)
    st = pkg.gtc_coo(idx, vals, o, ctx=ctx)
    ref = og.gtc(idx, vals, dims, R, og.SparseOptions(order=3, max_iter=8, lambdas=[1e-3] * 3), init)
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([t["rel"] for t in ref.trace])
    assert len(rel_gpu) == len(rel_ref) == 8
    assert np.max(np.abs(rel_gpu - rel_ref)) < 2e-4, (rel_gpu, rel_ref)
    assert oc.congruence(st.factors, ref.factors) >= 0.99
    # the reported cost is the cost of the returned factors
    f = og.gtc_cost(st.factors, idx, vals)
    assert f == pytest.approx(st.f_value, rel=1e-3)


def test_gtc_ratings_base_interface(pkg, ctx):
    dims, R = (30, 25, 20), 3
    idx, vals, init = _problem(dims, 4000, R, 7)
    ratings = np.vstack([idx.astype(np.float64), vals[None, :]])     # (N+1) x nnz
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=3, factorsInit=init)
    a = pkg.gtc(ratings, o, ctx=ctx)
    b = pkg.gtc_coo(idx, vals, o, ctx=ctx)
    for k in range(3):
        assert np.array_equal(a.factors[k], b.factors[k])


def test_gtc_stochastic_matches_oracle(pkg, ctx):
    dims, R = (40, 30, 20), 3
    idx, vals, init = _problem(dims, 12000, R, 9)
    c = 0.1
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=2, c_stochastic_perc=c,
                          lambdas=[1e-3] * 3, seed=11, factorsInit=init)
    st = pkg.gtc_coo(idx, vals, o, stochastic=True, ctx=ctx)
    ref = og.gtc_stochastic(idx, vals, dims, R,
                            og.SparseOptions(order=3, max_iter=2, c_stochastic_perc=c, lambdas=[1e-3] * 3,
                                             seed=11), init)
    assert st.ao_iter == ref.ao_iter
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([t["rel"] for t in ref.trace])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 1e-3, (rel_gpu, rel_ref)


def test_gtc_rejects_duplicates(pkg, ctx):
    dims, R = (10, 9, 8), 2
    idx, vals, init = _problem(dims, 200, R, 3)
    idx = np.concatenate([idx, idx[:, :1]], axis=1)
    vals = np.concatenate([vals, vals[:1]])
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=2, factorsInit=init)
    with pytest.raises(pkg._lib.PtgError) as e:
        pkg.gtc_coo(idx, vals, o, ctx=ctx)
    assert e.value.code == pkg._lib.PTG_ERR_INVALID


@pytest.mark.parametrize("cons", [(0, 0, 0), (1, 0, 1), (0, 4, 1)])
def test_gtc_constraints_match_oracle(pkg, ctx, cons):
    """update_factor of include/Gtc.hpp:330-355: unconstrained modes by the ridge solve
    (H_i + lambda I)^{-1} m_i (FP32 Cholesky here, FP64 inverse in the oracle), nonnegative modes
    by local_L Nesterov, a constant mode kept."""
    dims, R = (40, 36, 30), 4
    idx, vals, init = _problem(dims, 12000, R, 11)
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=5, lambdas=[1e-2] * 3,
                          factorsInit=init, constraints=list(cons))
    st = pkg.gtc_coo(idx, vals, o, ctx=ctx)
    ref = og.gtc(idx, vals, dims, R, og.SparseOptions(order=3, max_iter=5, lambdas=[1e-2] * 3,
                                                      constraints=list(cons)), init)
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([t["rel"] for t in ref.trace])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 2e-4 * max(1.0, rel_ref.max()), (rel_gpu, rel_ref)
    for k in range(3):
        if cons[k] == 4:
            assert np.allclose(st.factors[k], init[k], atol=1e-7)


def test_gtc_stochastic_keeps_unconstrained_modes(pkg, ctx):
    """The stochastic form updates only the nonnegative modes (include/GtcStochastic.hpp:325-345)."""
    dims, R = (30, 28, 26), 3
    idx, vals, init = _problem(dims, 8000, R, 13)
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=1, c_stochastic_perc=0.2,
                          lambdas=[1e-3] * 3, factorsInit=init, constraints=[1, 0, 1])
    st = pkg.gtc_coo(idx, vals, o, stochastic=True, ctx=ctx)
    assert np.allclose(st.factors[1], init[1], atol=1e-7)
    assert not np.allclose(st.factors[0], init[0], atol=1e-3)


@pytest.mark.parametrize("R", [3, 17, 32])
def test_gtc_stochastic_row_solvers_agree(pkg, ctx, R):
    """The stochastic row solver with one warp per row (rank <= 32: H_i in the lanes' registers,
    formed on the FMA pipe) and the one with one CTA per row do the same arithmetic in the same
    order: same bits."""
    dims = (70, 60, 50)
    idx, vals, init = _problem(dims, 30000, R, 21)
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=2, c_stochastic_perc=0.05,
                          lambdas=[1e-3] * 3, seed=3, factorsInit=init)
    out = {}
    for solver in ("warp_fma", "cta"):
        c = pkg.Context(0)
        try:
            c.set_gtc_rows(solver)
            out[solver] = pkg.gtc_coo(idx, vals, o, stochastic=True, ctx=c)
        finally:
            c.close()
    for k in range(3):
        assert np.array_equal(out["warp_fma"].factors[k], out["cta"].factors[k]), k
    assert out["warp_fma"].rel_costFunction == out["cta"].rel_costFunction


@pytest.mark.parametrize("R", [3, 17, 32])
def test_gtc_full_row_solvers_agree(pkg, ctx, R):
    """local_L Nesterov with one warp per row (rank <= 32) and with one CTA per row: the same
    FMAs in the same order, the same bits (rows with no entries included)."""
    dims = (70, 60, 50)
    idx, vals, init = _problem(dims, 9000, R, 25)
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=3, lambdas=[1e-3] * 3,
                          factorsInit=init)
    out = {}
    for solver in ("warp_fma", "cta"):
        c = pkg.Context(0)
        try:
            c.set_gtc_rows(solver)
            out[solver] = pkg.gtc_coo(idx, vals, o, ctx=c)
        finally:
            c.close()
    for k in range(3):
        assert np.array_equal(out["warp_fma"].factors[k], out["cta"].factors[k]), k
    assert out["warp_fma"].rel_costFunction == out["cta"].rel_costFunction


@pytest.mark.parametrize("R", [32, 40])
def test_gtc_stochastic_matches_oracle_rank(pkg, ctx, R):
    """Stochastic form at rank 32 (one warp per row) and 40 (one CTA per row) against the oracle.
    Each sampled block holds >= 150 entries (> R), so the row problems are well posed: the oracle
    moves by < 1e-7 under a 1e-6 perturbation of its initial factors here, while 30-entry blocks
    at rank 32 move it by 5e-3 and say nothing about the kernel."""
    dims = (40, 30, 20)
    idx, vals, init = _problem(dims, 20000, R, 23)
    c = 0.3
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=2, c_stochastic_perc=c,
                          lambdas=[1e-2] * 3, seed=5, factorsInit=init)
    st = pkg.gtc_coo(idx, vals, o, stochastic=True, ctx=ctx)
    ref = og.gtc_stochastic(idx, vals, dims, R,
                            og.SparseOptions(order=3, max_iter=2, c_stochastic_perc=c, lambdas=[1e-2] * 3,
                                             seed=5), init)
    assert st.ao_iter == ref.ao_iter
    rel_gpu = np.array([t["rel"] for t in st.trace])
    rel_ref = np.array([t["rel"] for t in ref.trace])
    assert np.max(np.abs(rel_gpu - rel_ref)) < 2e-4, (rel_gpu, rel_ref)
    assert oc.congruence(st.factors, ref.factors) >= 0.99


@pytest.mark.parametrize("R", [6, 8])
def test_gtc_4way_row_solvers(pkg, ctx, R):
    """Order 4 (three other modes per entry; R = 8 gathers float4 rows, R = 6 scalars): the
    warp-per-row and one-CTA solvers give the same bits in both forms, and the full form
    follows the oracle within 2e-4 per iteration."""
    dims = (16, 14, 12, 10)
    idx, vals, init = _problem(dims, 6000, R, 31)
    for stochastic in (False, True):
        o = pkg.SparseOptions(order=4, rank=R, tnsDims=list(dims), max_iter=3, lambdas=[1e-3] * 4,
                              c_stochastic_perc=0.2, seed=7, factorsInit=init)
        out = {}
        for solver in ("warp_fma", "cta"):
            c = pkg.Context(0)
            try:
                c.set_gtc_rows(solver)
                out[solver] = pkg.gtc_coo(idx, vals, o, stochastic=stochastic, ctx=c)
            finally:
                c.close()
        for k in range(4):
            assert np.array_equal(out["warp_fma"].factors[k], out["cta"].factors[k]), (stochastic, k)
        if not stochastic:
            ref = og.gtc(idx, vals, dims, R, og.SparseOptions(order=4, max_iter=3, lambdas=[1e-3] * 4), init)
            rel_gpu = np.array([t["rel"] for t in out["warp_fma"].trace])
            rel_ref = np.array([t["rel"] for t in ref.trace])
            assert np.max(np.abs(rel_gpu - rel_ref)) < 2e-4, (rel_gpu, rel_ref)


@pytest.mark.parametrize("R", [8, 16, 32])
def test_gtc_tensor_core_hessian_matches_fma(pkg, ctx, R):
    """The default warp solver forms H_i on the tensor cores (mma.sync TF32, three-term split):
    the local_L solve equals the FMA-pipe warp solver's up to FP32 summation order.  (The
    stochastic form is compared with the oracle elsewhere: on problems this small its result
    moves by ~0.02 in rel under a 1e-6 perturbation of the initial factors on either path, as
    its power method stops at a 1e-3 tolerance, so two summation orders need not agree.)"""
    dims = (70, 60, 50)
    idx, vals, init = _problem(dims, 30000, R, 29)
    o = pkg.SparseOptions(order=3, rank=R, tnsDims=list(dims), max_iter=2, lambdas=[1e-3] * 3, seed=3,
                          factorsInit=init)
    out = {}
    for solver in ("auto", "warp_fma"):
        c = pkg.Context(0)
        try:
            c.set_gtc_rows(solver)
            out[solver] = pkg.gtc_coo(idx, vals, o, stochastic=False, ctx=c)
        finally:
            c.close()
    for k in range(3):
        a, b = out["auto"].factors[k], out["warp_fma"].factors[k]
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-4, k
    assert abs(out["auto"].rel_costFunction - out["warp_fma"].rel_costFunction) < 1e-5
