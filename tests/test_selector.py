"""Precision selector, CPU side: the network oracle is pinned by finite
differences; label ladder, class weights and the eigenvalue tool used for
the shifted training instances are checked against known answers."""
import math

import numpy as np

from oracle import selector_oracle as so
from uhm_gb300 import selector as S


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    P = S.init_params(3).astype(np.float64)
    X = rng.standard_normal((40, 12))
    y = rng.integers(0, 3, 40)
    w = np.array([2.0, 1.0, 0.5])
    _, g = so.loss_and_grad(P, X, y, w)
    for i in rng.choice(so.N_PARAMS, 40, replace=False):
        e = np.zeros_like(P)
        e[i] = 1e-6
        num = (so.loss_and_grad(P + e, X, y, w)[0] - so.loss_and_grad(P - e, X, y, w)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, num, g[i])


def test_parameter_layout_matches_library(native_lib):
    from uhm_gb300 import api
    assert api.mlp_n_params() == so.N_PARAMS == S.init_params(0).size
    assert api.mlp_n_features() == so.F


def test_ladder_assigns_by_depth():
    depth = np.array([0, 1, 1, 2, 2, 2, 3])
    by_name = {r[0]: r for r in S.LADDER}
    assert S.ladder_classes(by_name["bf16"], depth).tolist() == [2] * 7
    assert S.ladder_classes(by_name["fp32@top2"], depth).tolist() == [1, 1, 1, 2, 2, 2, 2]
    assert S.ladder_classes(by_name["fp64@top1"], depth).tolist() == [0, 1, 1, 1, 1, 1, 1]
    assert S.ladder_classes(by_name["fp64"], depth).tolist() == [0] * 7


def test_class_weights_balance_counts():
    y = np.array([0] * 10 + [1] * 30 + [2] * 60)
    counts = np.bincount(y)
    w = S.class_weights(y, power=1.0)                 # fully balanced
    assert np.allclose(w * counts, (w * counts)[0], rtol=1e-6)
    w = S.class_weights(y)                            # square-root balanced
    assert np.allclose(w * np.sqrt(counts), (w * np.sqrt(counts))[0], rtol=1e-6)


def test_lambda_min_of_the_unit_cube():
    inst = S.Instance(seed=1, n=4, p_lo=4, p_hi=4, contrast=1.0, shift=0.0)
    lam = S.lambda_min(inst)
    assert abs(lam - 3 * math.pi ** 2) < 1e-3 * 3 * math.pi ** 2
