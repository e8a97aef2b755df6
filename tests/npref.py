"""Independent numpy/scipy FP64 statement of the EM and k-means iterations.

Written from the mathematics (full-covariance Gaussian mixture EM; Lloyd
k-means with lowest-index tie break), not from the oracle's code, so that
agreement between the two pins the oracle at small sizes.
"""
import numpy as np
from scipy.linalg import cholesky, solve_triangular
from scipy.special import logsumexp


def em_step(X, pi, mu, sigma):
    """One E-step + M-step.  Returns (logL at the old parameters,
    posteriors, new pi, mu, sigma)."""
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    k = len(pi)
    logp = np.empty((n, k))
    for j in range(k):
        L = cholesky(sigma[j], lower=True)
        z = solve_triangular(L, (X - mu[j]).T, lower=True)
        maha = np.sum(z * z, axis=0)
        logdet = 2.0 * np.sum(np.log(np.diag(L)))
        logp[:, j] = np.log(pi[j]) - 0.5 * (d * np.log(2 * np.pi) + logdet + maha)
    lse = logsumexp(logp, axis=1)
    R = np.exp(logp - lse[:, None])
    Nk = R.sum(axis=0)
    new_mu = (R.T @ X) / Nk[:, None]
    new_sigma = np.empty((k, d, d))
    for j in range(k):
        D = X - new_mu[j]
        new_sigma[j] = (D * R[:, j:j + 1]).T @ D / Nk[j]
    return lse.sum(), R, Nk / n, new_mu, new_sigma


def em_run(X, pi, mu, sigma, sweeps):
    lls = []
    for _ in range(sweeps):
        ll, _, pi, mu, sigma = em_step(X, pi, mu, sigma)
        lls.append(ll)
    return np.array(lls), pi, mu, sigma


def km_step(X, C):
    """One Lloyd iteration in FP64 difference form (argmin ties -> lowest
    index).  Returns (fit/N, new centroids (empty clusters keep NaN),
    counts, labels)."""
    X = np.asarray(X, dtype=np.float64)
    D = ((X[:, None, :] - C[None, :, :]) ** 2).sum(axis=2)
    lab = np.argmin(D, axis=1)
    fit = D[np.arange(len(X)), lab].sum() / len(X)
    k = C.shape[0]
    counts = np.bincount(lab, minlength=k)
    S = np.zeros_like(C)
    np.add.at(S, lab, X)
    with np.errstate(invalid="ignore", divide="ignore"):
        newC = S / counts[:, None]
    return fit, newC, counts, lab.astype(np.int32)
