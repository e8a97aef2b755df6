"""ComputePosterriorCorrelation (R^T R of the last E-step's posteriors) on the
device against numpy on the posteriors read back, for every precision."""
import numpy as np
import pytest

from fastem_gb300 import CudaMatrixEM, GaussianMixture, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,d,n,k,rtol", [("fp64", 8, 30001, 10, 1e-12), ("fp32", 8, 30001, 70, 1e-5),
                                                   ("mixed", 64, 20000 + 3, 128, 1e-5)])
def test_posterior_correlation(gpu_lib, precision, d, n, k, rtol):
    if d == 64:
        X, _ = synth.em_large(seed=3, n=n, d=d, k=k)
    else:
        X, _ = synth.kmeans_blobs(seed=4, n=n, d=d, k=k, spread=5.0, sigma=1.0)
    init = synth.dsquared_init(X, k, seed=2)
    with CudaMatrixEM(d, n, k, precision=precision) as em:
        em.CopyDataset(X)
        em.SetMixture(GaussianMixture(*init))
        em.InitDensities()
        em.PrecomputeDensityMatrix()
        P = em.Posteriors()
        C = em.ComputePosterriorCorrelation()
    ref = P.T @ P
    assert C.shape == (k, k)
    np.testing.assert_allclose(C, ref, rtol=rtol, atol=rtol * np.abs(ref).max())
    assert np.allclose(C, C.T, rtol=1e-12, atol=0)
