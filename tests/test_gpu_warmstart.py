"""GPU tests of the learned NNLS warm start (ptg_mlp_*): the network's forward pass and
gradient against the FP64 oracle (oracle/mlp.py), training on the GPU, a warm-started CPD
that must reach the same fit as the plain one, and the gain of a network trained on earlier
instances of a problem family: on new instances of a 4-way collinear family, at the
reference's Nesterov tolerance (1e-2) with line-search acceleration on, the warm-started
solves must need at least 20 % fewer sweeps and inner iterations in total than the plain
ones, every one reaching the same target.  (Where every row subproblem hits the 50-iteration
cap in every sweep, as at 1000^3 R=32, no start can save iterations; the bench reports that
case beside the headline.)"""
import numpy as np
import pytest
import torch

from oracle import cpd as oc
from oracle import mlp as om

pytestmark = pytest.mark.gpu


def _dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device="cuda")


def test_forward_and_gradient_match_oracle(pkg, ctx):
    R = 8
    din, h, dout = R + 8, 128, R
    model = pkg.WarmStartModel(ctx, R, seed=3)
    theta = om.init(din, h, dout, 3)
    # the device initialises the same He-uniform values (FP32)
    assert np.allclose(model.params(), theta, atol=1e-6)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((200, din))
    T = rng.standard_normal((200, dout))
    Xd, Td = _dev(X), _dev(T)
    Y = torch.zeros(200, dout, device="cuda")
    model.forward(Xd.data_ptr(), 200, Y.data_ptr())
    torch.cuda.synchronize()
    y_ref, _ = om.forward(model.params().astype(np.float64), X, din, h, dout)
    assert np.abs(Y.cpu().numpy() - y_ref).max() < 1e-4 * max(1.0, np.abs(y_ref).max())
    G = torch.zeros(model.n, device="cuda")
    loss = model.loss_grad(Xd.data_ptr(), Td.data_ptr(), 200, G.data_ptr())
    loss_ref, g_ref = om.loss_and_grad(model.params().astype(np.float64), X, T, din, h, dout)
    assert loss == pytest.approx(loss_ref, rel=1e-5)
    g = G.cpu().numpy()
    assert np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref) < 1e-4


def test_gradient_matches_finite_differences_of_oracle(pkg, ctx):
    """The oracle's analytic gradient itself checked against central differences."""
    din, h, dout = 6, 16, 3
    rng = np.random.default_rng(1)
    theta = om.init(din, h, dout, 5) + 0.01 * rng.standard_normal(om.nparams(din, h, dout))
    X = rng.standard_normal((7, din))
    T = rng.standard_normal((7, dout))
    _, g = om.loss_and_grad(theta, X, T, din, h, dout)
    for i in rng.choice(len(theta), 25, replace=False):
        e = np.zeros_like(theta)
        e[i] = 1e-6
        fd = (om.loss_and_grad(theta + e, X, T, din, h, dout)[0] - om.loss_and_grad(theta - e, X, T, din, h, dout)[0]) / 2e-6
        assert fd == pytest.approx(g[i], rel=1e-4, abs=1e-9)


def test_training_reduces_loss(pkg, ctx):
    R = 8
    din = R + 8
    model = pkg.WarmStartModel(ctx, R, seed=1)
    rng = np.random.default_rng(2)
    X = rng.standard_normal((2048, din))
    W = rng.standard_normal((din, R)) / np.sqrt(din)
    T = np.maximum(X @ W, 0.0)
    Xd, Td = _dev(X), _dev(T)
    G = torch.zeros(model.n, device="cuda")
    l0 = model.loss_grad(Xd.data_ptr(), Td.data_ptr(), 2048, G.data_ptr())
    model.train(Xd.data_ptr(), Td.data_ptr(), 2048, steps=400, batch=256, lr=1e-3)
    l1 = model.loss_grad(Xd.data_ptr(), Td.data_ptr(), 2048, G.data_ptr())
    assert l1 < 0.2 * l0, (l0, l1)


def _collinear_problem(dims, R, seed, snr_db=25.0, cos=0.6):
    """Factors U[0,1] mixed with one shared column (expected cosine ~cos), Gaussian noise at
    snr_db; returns the tensor, U[0,1] initial factors and ||noise|| / ||X||."""
    rng = np.random.default_rng(seed)
    A = []
    for I in dims:
        U = rng.random((I, R))
        c = rng.random((I, 1))
        A.append((1 - cos) * U + cos * c)
    X = np.einsum("ir,jr,kr,lr->ijkl", *A)
    noise = np.sqrt((X ** 2).mean() / 10 ** (snr_db / 10)) * rng.standard_normal(dims)
    X = X + noise
    init = [rng.random((I, R)) for I in dims]
    return X, init, float(np.linalg.norm(noise) / np.linalg.norm(X))


def warm_vs_plain(pkg, ctx, delta=10.0):
    """Same dimension-tree CPD with and without the learned warm start (log sweeps 1-5,
    train, infer from sweep 6).  Returns both statuses."""
    dims, R = (40, 40, 40, 40), 8
    X, init, _ = _collinear_problem(dims, R, seed=3)
    base = dict(order=4, max_iter=12, nesterov_delta_1=delta, nesterov_delta_2=delta, acceleration=False)
    plain = pkg.cpdDimTree(X, R, pkg.Options(**base), init, ctx=ctx)
    model = pkg.WarmStartModel(ctx, R, seed=7)
    warm = pkg.cpdDimTree(X, R, pkg.Options(**base, warm_start=True, warm_model=model, warm_log_sweeps=5,
                                            warm_train_steps=300), init, ctx=ctx)
    return plain, warm, X


def test_warm_start_keeps_the_fit_and_reports_iterations(pkg, ctx):
    plain, warm, X = warm_vs_plain(pkg, ctx)
    # identical until the network is used
    for s in range(5):
        assert plain.trace[s]["nesterov_iters"] == warm.trace[s]["nesterov_iters"]
    # the warm-started solve is not worse than the plain one (it may escape a stall of the
    # plain solver, whose loose delta lets every NNLS stop at once late in the run)
    assert warm.rel_costFunction <= plain.rel_costFunction + 1e-3
    assert oc.cost_from_factors(X, warm.factors) == pytest.approx(warm.f_value, rel=1e-3)
    it_plain = sum(sum(t["nesterov_iters"]) for t in plain.trace[5:])
    it_warm = sum(sum(t["nesterov_iters"]) for t in warm.trace[5:])
    print(f"inner Nesterov iterations in sweeps 6-12: plain {it_plain}, warm start {it_warm}")


def test_network_trained_on_a_family_saves_sweeps_and_iterations(pkg, ctx):
    """Train on every sweep of 12-sweep solves of four instances, then solve six new instances
    of the family from sweep 1 with the network, against the plain solver from the same
    initial factors: reference tolerance, acceleration on, stop at noise floor + 1e-3."""
    dims, R, delta = (30, 30, 30, 30), 8, 1e-2
    model = pkg.WarmStartModel(ctx, R, seed=7)
    for s in range(4):
        X, init, _ = _collinear_problem(dims, R, seed=100 + s)
        pkg.cpdDimTree(X, R, pkg.Options(order=4, max_iter=12, threshold_error=0.0, nesterov_delta_1=delta,
                                         nesterov_delta_2=delta, warm_start=True, warm_model=model,
                                         warm_log_sweeps=12, warm_train_steps=400), init, ctx=ctx)
    sweeps = {"plain": 0, "warm": 0}
    inner = {"plain": 0, "warm": 0}
    for s in range(4, 10):
        X, init, nr = _collinear_problem(dims, R, seed=100 + s)
        base = dict(order=4, max_iter=100, threshold_error=nr + 1e-3, nesterov_delta_1=delta,
                    nesterov_delta_2=delta)
        runs = {"plain": pkg.cpdDimTree(X, R, pkg.Options(**base), init, ctx=ctx),
                "warm": pkg.cpdDimTree(X, R, pkg.Options(**base, warm_start=True, warm_model=model,
                                                         warm_log_sweeps=0), init, ctx=ctx)}
        for k, st in runs.items():
            assert st.ao_iter < 100 and st.rel_costFunction < nr + 1e-3, (k, s, st.ao_iter, st.rel_costFunction)
            sweeps[k] += st.ao_iter
            inner[k] += sum(sum(t["nesterov_iters"]) for t in st.trace)
    print(f"sweeps plain {sweeps['plain']} warm {sweeps['warm']}; inner iterations plain {inner['plain']} "
          f"warm {inner['warm']}")
    assert sweeps["warm"] <= 0.8 * sweeps["plain"], sweeps
    assert inner["warm"] <= 0.8 * inner["plain"], inner
