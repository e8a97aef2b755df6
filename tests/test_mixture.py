"""GaussianMixture's host-side helpers (Evaluate, ComputePosteriors,
Classify, NormalizeWeights, FindLargestConditionNumber) against scipy's
multivariate normal in FP64; no GPU."""
import os

import numpy as np
import pytest

from fastem_gb300 import GaussianMixture

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def mixture():
    z = np.load(os.path.join(GOLDEN, "em_small.npz"))
    return GaussianMixture(z["pi"], z["mu"], z["sigma"]), z["X"]


def test_evaluate_posteriors_classify_against_scipy():
    st = pytest.importorskip("scipy.stats")
    G, X = mixture()
    X = X[:500]
    dens = np.stack([G.weights[j] * st.multivariate_normal(G.means[j], G.covs[j]).pdf(X.astype(np.float64))
                     for j in range(G.GetComponentCount())], axis=1)
    np.testing.assert_allclose(G.Evaluate(X), dens.sum(1), rtol=1e-10)
    assert G.Evaluate(X[3]) == pytest.approx(dens[3].sum(), rel=1e-10)
    np.testing.assert_allclose(G.ComputePosteriors(X), dens / dens.sum(1, keepdims=True), rtol=1e-9, atol=1e-15)
    np.testing.assert_array_equal(G.Classify(X), np.argmax(dens, axis=1))
    assert G.Classify(X[7]) == int(np.argmax(dens[7]))


def test_classify_far_row_and_ties():
    """A row far from every component: the reference's densities underflow to
    0 and give class 0; the log-domain comparison gives the component of
    largest log(pi_j N(x)).  Identical components: the lowest index, as the
    reference's strict comparison."""
    st = pytest.importorskip("scipy.stats")
    G, _ = mixture()
    far = G.means[2] * 1e4
    logd = [np.log(G.weights[j]) + st.multivariate_normal(G.means[j], G.covs[j]).logpdf(far)
            for j in range(G.GetComponentCount())]
    assert G.Evaluate(far) == 0.0                # every density underflows
    assert G.Classify(far) == int(np.argmax(logd)) != 0
    twin = GaussianMixture([0.5, 0.5], [[0.0, 0.0], [0.0, 0.0]], [np.eye(2), np.eye(2)])
    assert twin.Classify(np.array([0.3, -0.2])) == 0


def test_normalize_weights_and_condition_number():
    G, _ = mixture()
    G.weights *= 3.0
    G.NormalizeWeights()
    assert G.weights.sum() == pytest.approx(1.0, abs=1e-15)
    ev = [np.linalg.eigvalsh(S) for S in G.covs]
    assert G.FindLargestConditionNumber() == pytest.approx(max(abs(e[-1] / e[0]) for e in ev), rel=1e-12)
    iso = GaussianMixture([1.0], [[0.0, 0.0]], [np.eye(2) * 4.0])
    assert iso.FindLargestConditionNumber() == 1.0
