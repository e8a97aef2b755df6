"""Split-precision tensor-core EM for 64 < d <= 256 (csrc/em_wide.cu) against
the FP64 GPU path, which test_em_gpu.py pins to the oracle at d = 256.

Tolerances are the errors this form has, measured on a GB300, with margin:
  * The tensor core's FP32 accumulation drops an addend's bits below the
    accumulator's ulp, toward zero (a single-MMA probe shows it).  With
    covariance condition 1e6 the running sums of L^-1 (x - mu) are ~1e3
    times their result, so the E-step keeps a systematic logL error of
    ~2-3e-4 per point: the condition-1e6 cases are held to 5e-4.
  * The whitened M-step rounds y to FP16 once per point and component; the
    diagonal of sum r y y^T then carries relative noise ~2^-11 / sqrt(N_j)
    per dimension, which the log-determinant sums over d.  At d = 256 and
    N_j ~ 8K that is ~1e-4 in logL/N even at condition 1e2 (held to 3e-4);
    it falls as 1 / sqrt(N_j).
Posteriors within 2e-3 absolute; means and covariances within the relative
errors stated per test."""
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


def compare(t64, tmx, G64, Gmx, n, dl_max, dm_max, dc_max):
    dl = np.abs(tmx - t64) / n
    assert len(tmx) == len(t64)
    assert dl.max() <= dl_max, dl
    np.testing.assert_allclose(Gmx.weights, G64.weights, rtol=0, atol=1e-5)
    for j in range(len(G64.weights)):
        dm = np.linalg.norm(Gmx.means[j] - G64.means[j]) / np.linalg.norm(G64.means[j])
        dc = np.linalg.norm(Gmx.covs[j] - G64.covs[j]) / np.linalg.norm(G64.covs[j])
        assert dm <= dm_max and dc <= dc_max, (j, dm, dc)
    return dl


def conditioned_mixture(seed, n, d, k, lo, hi, spread):
    """k components, eigenvalues log-spaced over [lo, hi] with Haar bases,
    means N(0, spread^2 I), equal weights."""
    rng = np.random.default_rng(seed)
    lam = np.logspace(np.log10(lo), np.log10(hi), d)
    covs = np.empty((k, d, d))
    for j in range(k):
        Q = synth.haar_orthogonal(rng, d)
        covs[j] = (Q * lam) @ Q.T
        covs[j] = 0.5 * (covs[j] + covs[j].T)
    means = rng.normal(0.0, spread, size=(k, d))
    w = np.full(k, 1.0 / k)
    X, _ = synth.sample_mixture(rng, n, w, means, covs)
    return X, (w, means, covs)


def test_wide_estep_matches_fp64(gpu_lib):
    """One E-step at the condition-1e6 workload's initial mixture (means
    offset by 0.1 in every dimension: ~13 standard deviations in the
    smallest eigen-direction)."""
    n, d, k = 1 << 15, 256, 4
    X, info = synth.em_illcond(seed=5, n=n, d=d, k=k)
    init = (info["weights"], info["means"] + 0.1, info["covs"] * 1.05)
    l64, P64 = one_estep(X, init, "fp64")
    lmx, Pmx = one_estep(X, init, "mixed")
    assert abs(lmx - l64) / n <= 5e-4, (lmx, l64)
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
    compare(t64, tmx, G64, Gmx, n, 5e-4, 1e-5, 1e-2)
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
    compare(t64, tmx, G64, Gmx, n, 5e-4, 1e-5, 1e-2)


def test_wide_ragged_tiles_and_blocks(gpu_lib):
    """N not a multiple of the 128-point tile or the 64-point block, more
    components than CTAs need (several components per CTA range)."""
    n, d, k = 20_000 + 37, 128, 24
    _, info = synth.em_illcond(seed=3, n=256, d=d, k=k)
    w = np.full(k, 1.0 / k)   # equal sizes: every component holds ~830 > d points
    X, _ = synth.sample_mixture(np.random.default_rng(4), n, w, info["means"], info["covs"])
    init = (w, info["means"] + 0.05, info["covs"] * 1.02)
    t64, G64, _, _ = train(X, init, "fp64", 4, 1e-3)
    tmx, Gmx, _, _ = train(X, init, "mixed", 4, 1e-3)
    dl = np.abs(tmx - t64) / n
    assert dl.max() <= 5e-4, dl
    np.testing.assert_allclose(Gmx.weights, G64.weights, rtol=0, atol=1e-5)


@pytest.mark.parametrize("d", [128, 256])
def test_wide_moderate_condition(gpu_lib, d):
    """Condition 1e2 (eigenvalues over [0.1, 10], as the d = 64 workload),
    N_j = 8192: 10 sweeps within 3e-4 of FP64 in logL/N (measured 4.7e-5 at
    d = 128, 1.9e-4 at d = 256: the FP16 noise of the whitened diagonal)."""
    n, k = 1 << 16, 8
    X, (w, means, covs) = conditioned_mixture(21, n, d, k, 0.1, 10.0, 5.0)
    init = (w, means + 0.05, covs * 1.05)
    t64, G64, P64, _ = train(X, init, "fp64", 10, 0.0)
    tmx, Gmx, Pmx, _ = train(X, init, "mixed", 10, 0.0)
    compare(t64, tmx, G64, Gmx, n, 3e-4, 1e-5, 1e-2)
    assert np.abs(Pmx - P64).max() <= 2e-3
