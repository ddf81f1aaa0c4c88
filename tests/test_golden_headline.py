"""The FP64 reference fixture of the 1000^3 R=32 headline solve (tests/golden/, made by
tests/golden/make_headline_fp64.py with the FP64 OpenMP restatement of the reference's ALS
under its default stopping rule) and the host generator that reproduces its tensor."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "headline_1000cubed_r32_fp64.npz")


def test_fixture_is_the_reference_stopping_rule_run():
    fx = np.load(FIX)
    assert list(fx["dims"]) == [1000, 1000, 1000] and int(fx["rank"]) == 32
    # default options: threshold 1e-3 is never met at 30 dB, so the run stops at max_iter 20
    assert int(fx["ao_iter"]) == 20
    tr = fx["trace"]
    assert tr.shape == (20, 3)
    assert float(tr[-1, 1]) == pytest.approx(float(fx["rel_fp64"]), rel=1e-12)
    # the fit improves over the run and ends a little above the noise floor
    assert tr[-1, 1] < tr[0, 1]
    assert float(fx["noise_rel"]) - 1e-4 < float(fx["rel_fp64"]) < float(fx["noise_rel"]) + 1e-3
    f = fx["factors"]
    assert f.shape == (3, 1000, 32) and (f >= 0).all()
    if "long_trace" in fx:
        # the 20-sweep fit is within 1e-3 of where a longer run of the same solve ends
        assert abs(float(fx["long_trace"][-1, 1]) - float(fx["rel_fp64"])) < 1e-3


def test_host_generator_does_not_depend_on_threads(pkg):
    from partensor_toolbox_gb300 import datagen as dg
    a = dg.make_cpd_problem_host([37, 23, 11], 4, seed=2, init_seed=3, snr_db=30.0, equalize_columns=True,
                                 threads=1)
    b = dg.make_cpd_problem_host([37, 23, 11], 4, seed=2, init_seed=3, snr_db=30.0, equalize_columns=True,
                                 threads=5)
    assert np.array_equal(a.X, b.X)
    assert all(np.array_equal(x, y) for x, y in zip(a.init_factors, b.init_factors))
    assert a.frob == b.frob and a.noise_rel == b.noise_rel
    c = dg.make_cpd_problem_host([37, 23, 11], 4, seed=3, snr_db=30.0)
    assert not np.array_equal(a.X, c.X)
    # the noise is at the requested SNR
    T = np.einsum("ir,jr,kr->ijk", *a.true_factors).reshape(-1, order="F")
    snr = 10 * np.log10((T ** 2).sum() / ((a.X - T) ** 2).sum())
    assert abs(snr - 30.0) < 0.5
