"""Generate the golden fixtures of tests/golden/ from the FP64 oracle, and
km_ref.npz from the reference itself.

Every oracle fixture is produced by oracle/fem_oracle.cpp on one thread and
checked against the independent numpy statement in tests/npref.py before it
is written.  km_ref.npz is written by the reference's own NaiveKMA
(oracle/_ref/ref_kmeans, built from the reference's sources by
`make -C oracle ref`; skipped when that binary is absent) and checked against
the oracle before it is written.  The inputs are stored in the fixture, so it does not depend on the
numpy version that generated them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from fastem_gb300 import synth  # noqa: E402
import npref  # noqa: E402


def em_fixture():
    X, _ = synth.em_small(seed=11, n=3000, d=4, k=3)
    O.rng_seed(2)
    mu0 = O.kmeans_plusplus(X, 3)
    pi0, mu0, s0 = synth.identity_init(mu0)
    st, U0, ld0, _ = O.init_densities(s0)
    post0, ll0 = O.estep(X, pi0, mu0, U0, ld0, nthreads=1)
    r = O.em_train(X, pi0, mu0, s0, 12, eps=0.0, nthreads=1)
    assert r["status"] == 0 and len(r["logl"]) == 12
    ll, pi, mu, sg = npref.em_run(X, pi0, mu0, s0, 12)
    assert np.allclose(r["logl"], ll, rtol=1e-12, atol=0)
    assert np.allclose(r["mu"], mu, rtol=1e-10, atol=1e-12)
    assert np.allclose(r["sigma"], sg, rtol=1e-10, atol=1e-12)
    np.savez_compressed(os.path.join(HERE, "em_small.npz"), X=X, pi0=pi0, mu0=mu0, sigma0=s0,
                        U0=U0, logdet0=ld0, post0=post0, logl0=ll0, logl=r["logl"], e=r["e"],
                        pi=r["pi"], mu=r["mu"], sigma=r["sigma"])


def km_fixture():
    X, _ = synth.kmeans_blobs(seed=12, n=4096, d=8, k=8, spread=3.0)
    C0 = O.kmeans_oror(X, 8, seed=3, nthreads=1)
    C = C0.copy()
    labels, fits, cents, counts = [], [], [], []
    for _ in range(6):
        f2, C2, c2, l2 = npref.km_step(X, C)
        fit, C, cnt, lab = O.km_iterate(X, C, nthreads=1)
        assert (lab == l2).all() and (cnt == c2).all() and abs(fit - f2) <= 1e-12 * f2
        labels.append(lab)
        fits.append(fit)
        cents.append(C.copy())
        counts.append(cnt)
    np.savez_compressed(os.path.join(HERE, "km_blobs.npz"), X=X, C0=C0, labels=np.array(labels),
                        fits=np.array(fits), centroids=np.array(cents), counts=np.array(counts))


def km_ties_fixture():
    # rows exactly equidistant from two or more centroids: the lowest index wins
    X = np.array([[0, 0], [0, 0], [1, 1], [-1, -1], [2, 0], [0, 2], [3, 3], [-3, -3]],
                 dtype=np.float32)
    C0 = np.array([[1.0, -1.0], [-1.0, 1.0], [2.0, 2.0], [-2.0, -2.0]])
    fit, C1, cnt, lab = O.km_iterate(X, C0, repair=False, nthreads=1)
    f2, C2, c2, l2 = npref.km_step(X, C0)
    assert (lab == l2).all()
    np.savez_compressed(os.path.join(HERE, "km_ties.npz"), X=X, C0=C0, labels=lab, fit=fit,
                        counts=cnt, C1=C1)


def km_ref_fixture():
    # d = 32 (the tensor-core assignment's shape), overlapping blobs so that
    # many rows are near ties, and one centroid far from every row so that the
    # first iteration repairs an empty cluster with the generator (seed 17)
    X, _ = synth.kmeans_blobs(seed=31, n=8192, d=32, k=31, spread=2.5)
    C0 = np.vstack([X[::256][:31].astype(np.float64), np.full((1, 32), 1e3)])
    seed, iters = 17, 5
    out = O.ref_kmeans(X, C0, iters, seed, nthreads=1)
    if out is None:
        print("oracle/_ref/ref_kmeans not built: km_ref.npz not written")
        return
    fits, labels, cents = out
    O.rng_seed(seed)
    C = C0.copy()
    for i in range(iters):
        fit, C, cnt, lab = O.km_iterate(X, C, repair=True, nthreads=1)
        assert (lab == labels[i]).all() and np.allclose(C, cents[i], rtol=1e-13, atol=1e-13)
        assert abs(fit - fits[i]) <= 1e-13 * fits[i]
    np.savez_compressed(os.path.join(HERE, "km_ref.npz"), X=X, C0=C0, seed=seed, labels=labels, fits=fits,
                        centroids=cents)


def rng_fixture():
    O.rng_seed(42)
    u42 = np.array([O.rng_uniform() for _ in range(8)])
    np.savez_compressed(os.path.join(HERE, "rng.npz"), seed42_uniform=u42)


if __name__ == "__main__":
    O.build()
    em_fixture()
    km_fixture()
    km_ties_fixture()
    km_ref_fixture()
    rng_fixture()
    print("golden fixtures written to", HERE)
