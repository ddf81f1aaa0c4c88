"""GPU tests of the learned NNLS warm start (ptg_mlp_*): the network's forward pass and
gradient against the FP64 oracle (oracle/mlp.py), training on the GPU, and a warm-started
CPD that must reach the same fit as the plain one.  The effect on the inner Nesterov
iterations is measured and returned, not assumed (the reference's own start -- the
previous factor -- is hard to beat late in ALS)."""
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
    rng = np.random.default_rng(seed)
    A = []
    for I in dims:
        U = rng.random((I, R))
        c = rng.random((I, 1))
        A.append((1 - cos) * U + cos * c)
    X = np.einsum("ir,jr,kr,lr->ijkl", *A)
    X = X + np.sqrt((X ** 2).mean() / 10 ** (snr_db / 10)) * rng.standard_normal(dims)
    init = [rng.random((I, R)) for I in dims]
    return X, init


def warm_vs_plain(pkg, ctx, delta=10.0):
    """Same dimension-tree CPD with and without the learned warm start (log sweeps 1-5,
    train, infer from sweep 6).  Returns both statuses."""
    dims, R = (40, 40, 40, 40), 8
    X, init = _collinear_problem(dims, R, seed=3)
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
