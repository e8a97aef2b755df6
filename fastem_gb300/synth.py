"""Seeded synthetic workloads with the shapes and value distributions of the
FastEM benchmark configurations.

The reference measures on EMNIST-PCA300 (INSTALL.md:55), which is not
available; these generators stand in for it.  Every generator is a pure
function of its seed (numpy PCG64), so the CUDA path and the CPU oracle see
identical bytes within one process.

Workloads (N points, d dims, K components):
  em_small     N=100,000  d=8   K=10   weights~Dir(1), means~U[-10,10]^d,
                                        covariances A A^T + 0.5 I
  kmeans_blobs N=2^24     d=32  K=256  equal-size isotropic blobs, sigma=1,
                                        centres ~U[-20,20]^d
  em_large     N=2^23     d=64  K=128  weights~Dir(2), means~N(0,25 I),
                                        covariances Q diag(l) Q^T, Q Haar,
                                        l log-uniform in [0.1, 10]
  em_batched   512 fits   N log-uniform [2e3,2e5], d in {4,8,16,32},
                          K~U[2,32], blobs as kmeans_blobs, per-fit seeds
  em_illcond   N=2^21     d=256 K=64   eigenvalues log-spaced [1e-3,1e3]
                                        (cond 1e6), Haar bases,
                                        means~N(0,100 I), weights~Dir(1)
"""
import numpy as np

__all__ = [
    "haar_orthogonal", "sample_mixture", "em_small", "em_large", "em_illcond",
    "kmeans_blobs", "em_batched", "forgy_init", "identity_init",
]


def haar_orthogonal(rng, d):
    """Haar-distributed orthogonal matrix (QR of a Gaussian, sign-fixed)."""
    A = rng.standard_normal((d, d))
    Q, R = np.linalg.qr(A)
    return Q * np.sign(np.diag(R))[None, :]


def sample_mixture(rng, n, weights, means, covs, shuffle=True):
    """Draw n float32 points from a Gaussian mixture.  Component sizes are
    multinomial(n, weights); rows are shuffled unless shuffle=False."""
    k, d = means.shape
    counts = rng.multinomial(n, weights)
    X = np.empty((n, d), dtype=np.float32)
    labels = np.empty(n, dtype=np.int32)
    pos = 0
    for j in range(k):
        c = int(counts[j])
        if c == 0:
            continue
        L = np.linalg.cholesky(covs[j])
        Z = rng.standard_normal((c, d))
        X[pos:pos + c] = (means[j] + Z @ L.T).astype(np.float32)
        labels[pos:pos + c] = j
        pos += c
    if shuffle:
        perm = rng.permutation(n)
        X = X[perm]
        labels = labels[perm]
    return X, labels


def em_small(seed=1, n=100_000, d=8, k=10):
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(k))
    means = rng.uniform(-10.0, 10.0, size=(k, d))
    covs = np.empty((k, d, d))
    for j in range(k):
        A = rng.standard_normal((d, d))
        covs[j] = A @ A.T + 0.5 * np.eye(d)
    X, lab = sample_mixture(rng, n, w, means, covs)
    return X, dict(weights=w, means=means, covs=covs, labels=lab)


def em_large(seed=3, n=2 ** 23, d=64, k=128):
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.full(k, 2.0))
    means = rng.normal(0.0, 5.0, size=(k, d))
    covs = np.empty((k, d, d))
    for j in range(k):
        Q = haar_orthogonal(rng, d)
        lam = np.exp(rng.uniform(np.log(0.1), np.log(10.0), size=d))
        covs[j] = (Q * lam) @ Q.T
        covs[j] = 0.5 * (covs[j] + covs[j].T)
    X, lab = sample_mixture(rng, n, w, means, covs)
    return X, dict(weights=w, means=means, covs=covs, labels=lab)


def em_illcond(seed=5, n=2 ** 21, d=256, k=64):
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(k))
    means = rng.normal(0.0, 10.0, size=(k, d))
    lam = np.logspace(-3.0, 3.0, d)
    covs = np.empty((k, d, d))
    for j in range(k):
        Q = haar_orthogonal(rng, d)
        covs[j] = (Q * lam) @ Q.T
        covs[j] = 0.5 * (covs[j] + covs[j].T)
    X, lab = sample_mixture(rng, n, w, means, covs)
    return X, dict(weights=w, means=means, covs=covs, labels=lab)


def kmeans_blobs(seed=2, n=2 ** 24, d=32, k=256, spread=20.0, sigma=1.0):
    """Equal-size isotropic blobs (sizes differ by at most one when k does
    not divide n), rows shuffled."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-spread, spread, size=(k, d))
    sizes = np.full(k, n // k)
    sizes[: n % k] += 1
    lab = np.repeat(np.arange(k, dtype=np.int32), sizes)
    rng.shuffle(lab)
    X = np.empty((n, d), dtype=np.float32)
    step = 1 << 20
    for s in range(0, n, step):
        e = min(n, s + step)
        X[s:e] = (centres[lab[s:e]] + sigma * rng.standard_normal((e - s, d))).astype(np.float32)
    return X, dict(centres=centres, labels=lab)


def em_batched(seed=4, fits=512, n_lo=2_000, n_hi=200_000, dims=(4, 8, 16, 32), k_lo=2, k_hi=32):
    """Per-fit shapes and seeds of the batched workload; data is produced
    lazily by kmeans_blobs(seed_f, n_f, d_f, k_f)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), size=fits)).astype(np.int64)
    ds = rng.choice(np.asarray(dims), size=fits)
    ks = rng.integers(k_lo, k_hi + 1, size=fits)
    seeds = rng.integers(1, 2 ** 31 - 1, size=fits)
    return [dict(n=int(ns[f]), d=int(ds[f]), k=int(ks[f]), seed=int(seeds[f])) for f in range(fits)]


def forgy_init(X, k, seed):
    """k distinct rows as means (numpy-seeded), identity covariances and
    uniform weights."""
    rng = np.random.default_rng(seed)
    n, d = X.shape
    rows = rng.choice(n, size=k, replace=False)
    return identity_init(X[rows].astype(np.float64))


def dsquared_init(X, k, seed, sample=1 << 16):
    """Means by D^2 sampling (k-means++ rule) on a seeded row sample, with
    identity covariances and uniform weights.  A harness initialisation:
    numpy-seeded, cheap at any N (the reference's own seeders with its
    mt19937_64 stream live in the oracle and the C++ host library)."""
    rng = np.random.default_rng(seed)
    n, d = X.shape
    idx = rng.choice(n, size=min(n, sample), replace=False)
    S = X[idx].astype(np.float64)
    means = np.empty((k, d))
    means[0] = S[rng.integers(len(S))]
    dist = ((S - means[0]) ** 2).sum(axis=1)
    for i in range(1, k):
        p = dist / dist.sum()
        means[i] = S[rng.choice(len(S), p=p)]
        dist = np.minimum(dist, ((S - means[i]) ** 2).sum(axis=1))
    return identity_init(means)


def identity_init(means):
    k, d = means.shape
    return (np.full(k, 1.0 / k), np.array(means, dtype=np.float64, copy=True),
            np.broadcast_to(np.eye(d), (k, d, d)).copy())
