"""Precision selector on the device: training and inference kernels against
the CPU oracle, training progress, and the per-front features.

Tolerances: FP32 kernels vs the float64 oracle, loss within 1e-5 relative,
gradient within 1e-4 of its norm, probabilities within 1e-5."""
import numpy as np
import pytest

from oracle import selector_oracle as so
from uhm_gb300 import api, hpfem
from uhm_gb300 import selector as S

pytestmark = pytest.mark.gpu


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, 12)).astype(np.float32)
    y = rng.integers(0, 3, n).astype(np.int32)
    return X, y


def test_gradient_matches_oracle(native_lib):
    X, y = _data(300, 1)
    P = S.init_params(5)
    P[768:832] = 0.1          # non-zero biases exercise every term
    w = np.array([3.0, 1.0, 0.5], np.float32)
    loss, g = api.mlp_gradient(X, y, P, w)
    loss_ref, g_ref = so.loss_and_grad(P.astype(np.float64), X.astype(np.float64), y, w.astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert np.abs(g - g_ref).max() <= 1e-4 * np.linalg.norm(g_ref)


def test_predict_matches_oracle(native_lib):
    X, _ = _data(500, 2)
    P = S.init_params(6)
    cls, prob = api.mlp_predict(X, P)
    _, _, z = so.forward(P.astype(np.float64), X.astype(np.float64))
    pr = np.exp(z - z.max(1, keepdims=True))
    pr /= pr.sum(1, keepdims=True)
    assert np.abs(prob - pr).max() < 1e-5
    clear = np.sort(pr, 1)[:, -1] - np.sort(pr, 1)[:, -2] > 1e-4
    assert np.array_equal(cls[clear], pr.argmax(1)[clear])


def test_training_learns_a_separable_rule(native_lib):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((4096, 12)).astype(np.float32)
    y = np.where(X[:, 0] + 0.5 * X[:, 3] > 0.5, 0, np.where(X[:, 1] > 0, 1, 2)).astype(np.int32)
    P0 = S.init_params(7)
    P, hist = api.mlp_train(X, y, P0, epochs=30, batch=256, lr=3e-3, seed=1)
    assert hist[-1] < 0.3 * hist[0]
    cls, _ = api.mlp_predict(X, P)
    assert (cls == y).mean() > 0.95


def test_front_features(native_lib):
    spec = hpfem.poisson3d(8, 4, seed=2)
    m = api.load_spec(spec)
    eid, gen, fs, ss = m.fronts()
    F = m.front_features()
    assert F.shape == (len(eid), 12) and np.isfinite(F).all()
    n = fs + ss
    root = np.argmin(gen)
    assert F[root, 3] == 0.0                                   # depth of the root
    assert np.array_equal(F[:, 4] == 1.0, n >= 512)            # tensor-core eligible
    assert np.allclose(F[:, 0], np.log2(n + 1.0) / 14, atol=1e-6)
    assert F[root, 10] == pytest.approx(F[root, 5], abs=1e-6)              # whole mesh = root subtree
    assert np.ptp(F[:, 9]) == 0.0 and np.ptp(F[:, 10]) == 0.0              # mesh-wide features
    assert F[root, 9] == pytest.approx(F[:, 7].min(), abs=1e-6)
