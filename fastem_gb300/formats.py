"""The reference's file formats, for tests and tooling.

  .bin      MultithreadedDataset (Util/MultithreadedDataset.cpp:119-134): int32
            rows and int32 cols (or int32 -1, int32 cols, int64 rows), then the
            rows of float32
  .cmp      GaussianMixture::Write / read (EM2/GaussianMixture.cpp:155-171,
            228-244): int32 K, int32 d, per component the d x d covariance
            (row-major), the mean and the weight as float64, then one float64
            log-likelihood
  classes   GaussianMixture::WriteClasses (EM2/GaussianMixture.cpp:112-122):
            int32 row count, then int32 1-based classes
"""
import numpy as np

from .em import GaussianMixture


def write_bin(fname, X):
    X = np.ascontiguousarray(X, dtype=np.float32)
    n, d = X.shape
    with open(fname, "wb") as f:
        if n <= np.iinfo(np.int32).max:
            np.array([n, d], dtype=np.int32).tofile(f)
        else:
            np.array([-1, d], dtype=np.int32).tofile(f)
            np.array([n], dtype=np.int64).tofile(f)
        X.tofile(f)


def read_bin(fname):
    with open(fname, "rb") as f:
        n, d = np.fromfile(f, dtype=np.int32, count=2)
        if n == -1:
            n = int(np.fromfile(f, dtype=np.int64, count=1)[0])
        X = np.fromfile(f, dtype=np.float32, count=int(n) * int(d))
    if X.size != int(n) * int(d):
        raise IOError("truncated .bin file")
    return X.reshape(int(n), int(d))


def write_cmp(fname, G, loglike=0.0):
    k, d = G.means.shape
    with open(fname, "wb") as f:
        np.array([k, d], dtype=np.int32).tofile(f)
        for j in range(k):
            np.ascontiguousarray(G.covs[j], dtype=np.float64).tofile(f)
            np.ascontiguousarray(G.means[j], dtype=np.float64).tofile(f)
            np.array([G.weights[j]], dtype=np.float64).tofile(f)
        np.array([loglike], dtype=np.float64).tofile(f)


def read_cmp(fname):
    """Returns (GaussianMixture, stored log-likelihood)."""
    with open(fname, "rb") as f:
        k, d = (int(v) for v in np.fromfile(f, dtype=np.int32, count=2))
        w, mu, sg = np.zeros(k), np.zeros((k, d)), np.zeros((k, d, d))
        for j in range(k):
            sg[j] = np.fromfile(f, dtype=np.float64, count=d * d).reshape(d, d)
            mu[j] = np.fromfile(f, dtype=np.float64, count=d)
            w[j] = np.fromfile(f, dtype=np.float64, count=1)[0]
        ll = np.fromfile(f, dtype=np.float64, count=1)
    if ll.size != 1:
        raise IOError("truncated .cmp file")
    return GaussianMixture(w, mu, sg), float(ll[0])


def read_classes(fname):
    """A classes file (GaussianMixture::WriteClasses, EM2/GaussianMixture.cpp;
    read as ReadAssignment, Util/MultithreadedDataset.cpp:371-386): an int32
    count, or -1 and an int64 count, then the 1-based int32 classes, returned
    as stored (1-based)."""
    with open(fname, "rb") as f:
        n = int(np.fromfile(f, dtype=np.int32, count=1)[0])
        if n == -1:
            n = int(np.fromfile(f, dtype=np.int64, count=1)[0])
        c = np.fromfile(f, dtype=np.int32, count=n)
    if len(c) != n:
        raise ValueError("%s: %d of %d classes" % (fname, len(c), n))
    return c
