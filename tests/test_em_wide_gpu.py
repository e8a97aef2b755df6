"""Split-precision tensor-core EM for 64 < d <= 256 (csrc/em_wide.cu) against
the FP64 GPU path, which test_em_gpu.py pins to the oracle at d = 256.

Tolerances: |dlogL/N| <= 1e-5 per sweep (the metric's bound); posteriors
within 2e-3 absolute (FP16 hi + lo storage is exact to ~2^-22; the rest is
the Mahalanobis error of ~1e-3 on points that sit between components);
means within 1e-6 relative to their norm and covariances within 1e-4 in
relative Frobenius norm after the sweeps (the whitened sums round z to FP16
once per point, an error of ~2^-12 / sqrt(N_j))."""
import numpy as np
import pytest

from fastem_gb300 import CudaMatrixEM, GaussianMixture, synth

pytestmark = pytest.mark.gpu


def train(X, init, precision, sweeps, reg):
    n, d = X.shape
    with CudaMatrixEM(d, n, len(init[0]), precision=precision) as em:
        em.SetParameters(sweeps, 0.0, 1e12, reg)
        G = GaussianMixture(*init)
        em.Train(X, G)
        return em.logl_trace.copy(), G, em.Posteriors(), em.RetrieveClasses()


def one_estep(X, init, precision):
    n, d = X.shape
    with CudaMatrixEM(d, n, len(init[0]), precision=precision) as em:
        em.SetParameters(1, 0.0, 1e12)
        em.CopyDataset(X)
        em.SetMixture(GaussianMixture(*init))
        em.InitDensities()
        ll = em.PrecomputeDensityMatrix()
        return ll, em.Posteriors()


def compare(t64, tmx, G64, Gmx, n):
    dl = np.abs(tmx - t64) / n
    assert len(tmx) == len(t64)
    assert dl.max() <= 1e-5, dl
    np.testing.assert_allclose(Gmx.weights, G64.weights, rtol=0, atol=1e-6)
    for j in range(len(G64.weights)):
        dm = np.linalg.norm(Gmx.means[j] - G64.means[j]) / np.linalg.norm(G64.means[j])
        dc = np.linalg.norm(Gmx.covs[j] - G64.covs[j]) / np.linalg.norm(G64.covs[j])
        assert dm <= 1e-6 and dc <= 1e-4, (j, dm, dc)
    return dl


def test_wide_estep_matches_fp64(gpu_lib):
    """One E-step at the condition-1e6 workload's initial mixture (means
    offset by 0.1 in every dimension: ~13 standard deviations in the
    smallest eigen-direction)."""
    n, d, k = 1 << 15, 256, 4
    X, info = synth.em_illcond(seed=5, n=n, d=d, k=k)
    init = (info["weights"], info["means"] + 0.1, info["covs"] * 1.05)
    l64, P64 = one_estep(X, init, "fp64")
    lmx, Pmx = one_estep(X, init, "mixed")
    assert abs(lmx - l64) / n <= 2e-6, (lmx, l64)
    assert np.abs(Pmx - P64).max() <= 2e-3
    np.testing.assert_allclose(Pmx.sum(1), 1.0, atol=1e-5)


def test_wide_illcond_sweeps_match_fp64(gpu_lib):
    """15 sweeps at d = 256, condition 1e6, RegCoef 1e-6 (the workload's
    setting), N = 2^16 over 8 components."""
    n, d, k = 1 << 16, 256, 8
    X, info = synth.em_illcond(seed=5, n=n, d=d, k=k)
    init = (info["weights"], info["means"] + 0.1, info["covs"] * 1.05)
    t64, G64, P64, c64 = train(X, init, "fp64", 15, 1e-6)
    tmx, Gmx, Pmx, cmx = train(X, init, "mixed", 15, 1e-6)
    compare(t64, tmx, G64, Gmx, n)
    assert np.abs(Pmx - P64).max() <= 2e-3
    sure = P64.max(1) > 0.99
    assert np.array_equal(cmx[sure], c64[sure])


@pytest.mark.parametrize("d", [100, 150, 192])
def test_wide_padded_dimensions(gpu_lib, d):
    """d that is not a multiple of 64 (zero padding to 128 / 192) and d with
    rows that are not 16-byte multiples (150: scalar row loads)."""
    n, k = 1 << 15, 3
    X, info = synth.em_illcond(seed=11, n=n, d=d, k=k)
    init = (info["weights"], info["means"] + 0.05, info["covs"] * 1.02)
    t64, G64, _, _ = train(X, init, "fp64", 5, 1e-6)
    tmx, Gmx, _, _ = train(X, init, "mixed", 5, 1e-6)
    compare(t64, tmx, G64, Gmx, n)


def test_wide_ragged_tiles_and_blocks(gpu_lib):
    """N not a multiple of the 128-point tile or the 64-point block, more
    components than CTAs need (several components per CTA range)."""
    n, d, k = 20_000 + 37, 128, 24
    X, info = synth.em_illcond(seed=3, n=n, d=d, k=k)
    w = np.full(k, 1.0 / k)
    init = (w, info["means"] + 0.05, info["covs"] * 1.02)
    t64, G64, _, _ = train(X, init, "fp64", 4, 1e-3)
    tmx, Gmx, _, _ = train(X, init, "mixed", 4, 1e-3)
    dl = np.abs(tmx - t64) / n
    assert dl.max() <= 1e-5, dl
    np.testing.assert_allclose(Gmx.weights, G64.weights, rtol=0, atol=1e-6)
