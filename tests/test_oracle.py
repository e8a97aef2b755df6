"""CPU tests of the FP64 oracle: known answers, golden fixtures and the
independent numpy statement (tests/npref.py)."""
import os

import numpy as np
import pytest

import npref
from fastem_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_rng_known_answer(oracle):
    # C++ [rand.predef]: the 10000th output of a default-constructed
    # mt19937_64 (seed 5489) is 9981545732273789042; uniform_real_distribution
    # <double> divides the 53-bit-rounded draw by 2^64 (Util/Rand.cpp:7-18)
    oracle.rng_seed(5489)
    for _ in range(9999):
        oracle.rng_uniform()
    assert oracle.rng_uniform() == float(9981545732273789042) / 2.0 ** 64


REF_RAND = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "ref_rand")


@pytest.mark.parametrize("seed", [0, 2, 3, 11, 637563561, 4294967295])
def test_rng_matches_reference_rand(oracle, seed):
    """The oracle's generator against the reference's own Util/Rand.cpp
    (compiled in place into oracle/_ref where the reference sources are
    present): SRand(seed), then Rand() and RandInt(n) bit for bit."""
    import subprocess
    if not os.access(REF_RAND, os.X_OK):
        pytest.skip("oracle/_ref/ref_rand not built (reference sources absent)")
    count, n = 2000, 1000003
    try:
        out = subprocess.run([REF_RAND, str(seed), str(count), str(n)], capture_output=True, text=True,
                             timeout=60)
    except OSError as e:                       # built for another CPU architecture
        pytest.skip(str(e))
    vals = out.stdout.split()
    ref_u = [float(v) for v in vals[:count]]
    ref_i = [int(v) for v in vals[count:]]
    oracle.rng_seed(seed)
    got_u = [oracle.rng_uniform() for _ in range(count)]
    got_i = [int(oracle.rng_uniform() * n) for _ in range(count)]
    assert got_u == ref_u
    assert got_i == ref_i


def _ref_kmeans_or_skip(oracle, *args, **kw):
    try:
        out = oracle.ref_kmeans(*args, **kw)
    except OSError as e:                       # built for another CPU architecture
        pytest.skip(str(e))
    if out is None:
        pytest.skip("oracle/_ref/ref_kmeans not built (reference sources absent)")
    return out


def _oracle_iterations(oracle, X, C0, iters, seed):
    oracle.rng_seed(seed)
    C = C0.copy()
    fits, labels, cents = [], [], []
    for _ in range(iters):
        fit, C, _, lab = oracle.km_iterate(X, C, repair=True, nthreads=1)
        fits.append(fit)
        labels.append(lab)
        cents.append(C.copy())
    return np.array(fits), np.array(labels), np.array(cents)


def _km_pin_cases():
    z = np.load(os.path.join(GOLDEN, "km_blobs.npz"))
    yield "km_blobs golden", z["X"], z["C0"], 6
    t = np.load(os.path.join(GOLDEN, "km_ties.npz"))
    yield "km_ties golden", t["X"], t["C0"], 2
    X, _ = synth.kmeans_blobs(seed=6, n=1000, d=4, k=3)
    yield "empty cluster (random repair)", X, np.vstack([X[:3].astype(np.float64), np.full((1, 4), 1e6)]), 3
    X, _ = synth.kmeans_blobs(seed=21, n=6000, d=32, k=24, spread=1.0)
    yield "d = 32 blobs, overlapping", X, X[::250][:24].astype(np.float64), 5


@pytest.mark.parametrize("threads", [1, 4])
def test_kmeans_matches_reference_naive_kma(oracle, threads):
    """The oracle's Lloyd iteration against the reference's own
    NaiveKMA::ComputeMSEAndCorrect (Clust/KMAlgorithm.cpp:205-255, compiled
    in place into oracle/_ref with CentroidVector, OpenMPKMAReducer and
    CentroidRandomRepair): labels and repair draws bit-exact, centroids and fit
    equal up to the order of the reference's per-thread sums."""
    for name, X, C0, iters in _km_pin_cases():
        rf, rl, rc = _ref_kmeans_or_skip(oracle, X, C0, iters, seed=17, nthreads=threads)
        of, ol, oc = _oracle_iterations(oracle, X, C0, iters, seed=17)
        assert np.array_equal(rl, ol), name
        np.testing.assert_allclose(oc, rc, rtol=1e-13, atol=1e-13, err_msg=name)
        np.testing.assert_allclose(of, rf, rtol=1e-13, err_msg=name)


def test_kmeans_golden_made_by_reference(oracle):
    """tests/golden/km_ref.npz was written by the reference's own NaiveKMA
    (tests/golden/make_golden.py); where the reference binary is built, it
    still gives those bytes."""
    z = np.load(os.path.join(GOLDEN, "km_ref.npz"))
    rf, rl, rc = _ref_kmeans_or_skip(oracle, z["X"], z["C0"], len(z["fits"]), seed=int(z["seed"]), nthreads=1)
    assert np.array_equal(rl, z["labels"])
    np.testing.assert_allclose(rc, z["centroids"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(rf, z["fits"], rtol=1e-13)


def test_rng_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "rng.npz"))
    oracle.rng_seed(42)
    got = np.array([oracle.rng_uniform() for _ in range(8)])
    assert np.array_equal(got, z["seed42_uniform"])


def test_em_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "em_small.npz"))
    st, U, ld, _ = oracle.init_densities(z["sigma0"])
    assert st == 0
    np.testing.assert_allclose(U, z["U0"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(ld, z["logdet0"], rtol=1e-13)
    post, ll = oracle.estep(z["X"], z["pi0"], z["mu0"], U, ld, nthreads=1)
    np.testing.assert_allclose(post, z["post0"], rtol=1e-12, atol=1e-300)
    assert abs(ll - z["logl0"]) <= 1e-12 * abs(ll)
    r = oracle.em_train(z["X"], z["pi0"], z["mu0"], z["sigma0"], 12, eps=0.0, nthreads=1)
    np.testing.assert_allclose(r["logl"], z["logl"], rtol=1e-13)
    np.testing.assert_allclose(r["mu"], z["mu"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(r["sigma"], z["sigma"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(r["pi"], z["pi"], rtol=1e-11)


def test_km_golden(oracle):
    z = np.load(os.path.join(GOLDEN, "km_blobs.npz"))
    C = z["C0"].copy()
    for it in range(len(z["fits"])):
        fit, C, cnt, lab = oracle.km_iterate(z["X"], C, nthreads=1)
        assert np.array_equal(lab, z["labels"][it])
        assert np.array_equal(cnt, z["counts"][it])
        assert fit == z["fits"][it]
        np.testing.assert_array_equal(C, z["centroids"][it])


def test_km_ties_lowest_index(oracle):
    z = np.load(os.path.join(GOLDEN, "km_ties.npz"))
    fit, C1, cnt, lab = oracle.km_iterate(z["X"], z["C0"], repair=False, nthreads=1)
    assert np.array_equal(lab, z["labels"])
    assert lab[0] == 0 and lab[1] == 0  # equidistant from centroids 0 and 1


def test_em_vs_numpy(oracle):
    X, _ = synth.em_small(seed=7, n=6000, d=8, k=5)
    oracle.rng_seed(2)
    pi0, mu0, s0 = synth.identity_init(oracle.kmeans_plusplus(X, 5))
    r = oracle.em_train(X, pi0, mu0, s0, 15, eps=0.0, nthreads=3)
    ll, pi, mu, sg = npref.em_run(X, pi0, mu0, s0, 15)
    np.testing.assert_allclose(r["logl"], ll, rtol=1e-12)
    np.testing.assert_allclose(r["mu"], mu, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(r["sigma"], sg, rtol=1e-9, atol=1e-11)


def test_cachedem_order_matches_simple_matrix_em(oracle):
    """CachedEM (EM2/CachedEM.cpp:120-170) sums rank-1 updates weighted by the
    unscaled posteriors and divides by the posterior sum after the reduction;
    SimpleMatrixEM (EM2/MatrixEM.cpp:53-67,90-99) scales every point by
    sqrt(r / N_j) first.  The library runs the second order for both
    algorithms; the two differ by rounding only: the same IterCounter and
    LogL traces within 1e-12 per point, here and with the Eps rule."""
    X, _ = synth.em_small(seed=11, n=8000, d=8, k=5)
    oracle.rng_seed(3)
    pi0, mu0, s0 = synth.identity_init(oracle.kmeans_plusplus(X, 5))
    a = oracle.em_train(X, pi0, mu0, s0, 25, eps=0.0, nthreads=3)
    b = oracle.em_train(X, pi0, mu0, s0, 25, eps=0.0, nthreads=3, cached=True)
    assert a["status"] == b["status"] == 0 and a["iter_counter"] == b["iter_counter"]
    assert np.max(np.abs(a["logl"] - b["logl"])) / len(X) < 1e-12
    np.testing.assert_allclose(b["mu"], a["mu"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(b["sigma"], a["sigma"], rtol=1e-9, atol=1e-12)
    # one M-step from the same posteriors: rounding-level differences only
    st, U, logdet, _ = oracle.init_densities(s0)
    assert st == 0
    post, _ = oracle.estep(X, pi0, mu0, U, logdet)
    ps, ms, ss = oracle.mstep(X, post)
    pc, mc, sc = oracle.mstep_cached(X, post)
    np.testing.assert_array_equal(pc, ps)
    np.testing.assert_array_equal(mc, ms)
    np.testing.assert_allclose(sc, ss, rtol=1e-12, atol=1e-14)
    # with the convergence rule the sweep counts agree too
    c = oracle.em_train(X, pi0, mu0, s0, 500, eps=1e-7, nthreads=2)
    e = oracle.em_train(X, pi0, mu0, s0, 500, eps=1e-7, nthreads=2, cached=True)
    assert c["iter_counter"] == e["iter_counter"]
    np.testing.assert_allclose(e["final_logl"], c["final_logl"], rtol=1e-12)


def test_em_thread_count_independent(oracle):
    X, _ = synth.em_small(seed=8, n=5000, d=4, k=3)
    pi0, mu0, s0 = synth.forgy_init(X, 3, seed=1)
    a = oracle.em_train(X, pi0, mu0, s0, 8, eps=0.0, nthreads=1)
    b = oracle.em_train(X, pi0, mu0, s0, 8, eps=0.0, nthreads=4)
    np.testing.assert_allclose(a["logl"], b["logl"], rtol=1e-13)


def test_em_convergence_rule(oracle):
    # TrainNoCopy stops when |dL/L| < Eps and reports IterCounter one past the last sweep
    X, _ = synth.em_small(seed=9, n=4000, d=4, k=2)
    pi0, mu0, s0 = synth.forgy_init(X, 2, seed=3)
    r = oracle.em_train(X, pi0, mu0, s0, 500, eps=1e-6, nthreads=2)
    assert r["status"] == 0
    n = len(r["logl"])
    assert r["iter_counter"] == n + 1
    assert r["e"][-1] < 1e-6 and np.all(r["e"][:-1] >= 1e-6)


def test_em_regularization(oracle):
    s = np.stack([np.diag([1.0, 4.0, 9.0])] * 2)
    out = oracle.regularize(s, 0.25)
    tr = 14.0
    np.testing.assert_allclose(out[0], 0.75 * s[0] + 0.25 * tr / 3 * np.eye(3))


def test_cholesky_failure_status(oracle):
    s = np.stack([np.eye(3), np.array([[1.0, 2.0, 0], [2.0, 1.0, 0], [0, 0, 1.0]])])
    st, U, ld, failed = oracle.init_densities(s)
    assert st == oracle.ORC_ERR_CHOLESKY and failed == 1


def test_cond_number(oracle):
    rng = np.random.default_rng(0)
    Q = synth.haar_orthogonal(rng, 6)
    lam = np.logspace(-2, 3, 6)
    S = (Q * lam) @ Q.T
    assert abs(oracle.cond_number(S) / 1e5 - 1.0) < 1e-9


def test_km_vs_numpy_and_threads(oracle):
    X, _ = synth.kmeans_blobs(seed=5, n=20000, d=16, k=12)
    C0 = oracle.kmeans_oror(X, 12, seed=3)
    f1, C1, c1, l1 = oracle.km_iterate(X, C0, nthreads=1)
    f4, C4, c4, l4 = oracle.km_iterate(X, C0, nthreads=4)
    f2, C2, c2, l2 = npref.km_step(X, C0)
    assert np.array_equal(l1, l2) and np.array_equal(l1, l4)
    assert abs(f1 - f2) <= 1e-12 * f2
    np.testing.assert_allclose(C1, C2, rtol=1e-13)


def test_km_empty_cluster_repair(oracle):
    X, _ = synth.kmeans_blobs(seed=6, n=1000, d=4, k=3)
    C0 = np.vstack([X[:3].astype(np.float64), np.full((1, 4), 1e6)])
    oracle.rng_seed(17)
    fit, C1, cnt, lab = oracle.km_iterate(X, C0, nthreads=2)
    assert cnt[3] == 0
    oracle.rng_seed(17)
    src = int(oracle.rng_uniform() * len(X))
    np.testing.assert_array_equal(C1[3], X[src].astype(np.float64))


def test_km_run_stopping_rule(oracle):
    X, _ = synth.kmeans_blobs(seed=4, n=8000, d=8, k=6)
    C0 = oracle.kmeans_forgy(X, 6, seed=1)
    best, C, it = oracle.km_run(X, C0, min_rel=-1.0, max_iter=50)
    # max_iter bounds the sweeps at max_iter - 1
    assert 1 <= it <= 49
    C = C0.copy()
    fits = []
    for _ in range(it):
        f, C, _, _ = oracle.km_iterate(X, C)
        fits.append(f)
    assert best == min(fits)


def test_seeders_deterministic(oracle):
    X, _ = synth.kmeans_blobs(seed=3, n=5000, d=8, k=10)
    a = oracle.kmeans_oror(X, 10, seed=3, nthreads=1)
    b = oracle.kmeans_oror(X, 10, seed=3, nthreads=4)
    np.testing.assert_array_equal(a, b)
    p = oracle.kmeans_plusplus(X, 10, seed=2)
    q = oracle.kmeans_plusplus(X, 10, seed=2)
    np.testing.assert_array_equal(p, q)
    # every seed is a data row
    rows = {tuple(r) for r in X.astype(np.float64)}
    assert all(tuple(r) in rows for r in p)


def test_blas_sweep_matches_oracle(oracle):
    """The BLAS-organised sweep used for CPU timing gives the oracle's sweep."""
    if oracle.openblas() is None:
        pytest.skip("scipy's bundled OpenBLAS not found")
    from fastem_gb300 import synth
    X, _ = synth.em_large(seed=3, n=4000, d=16, k=6)
    pi, mu, sg = synth.dsquared_init(X, 6, seed=5)
    ll, pi2, mu2, sg2 = oracle.em_sweep_blas(X, pi, mu, sg)
    ref = oracle.em_train(X, pi, mu, sg, 1, eps=0.0)
    assert abs(ll - ref["logl"][0]) <= 1e-11 * abs(ref["logl"][0])
    np.testing.assert_allclose(pi2, ref["pi"], rtol=1e-11)
    np.testing.assert_allclose(mu2, ref["mu"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(sg2, ref["sigma"], rtol=1e-9, atol=1e-12)


def test_blas_sweeps_match_oracle_train(oracle):
    """Several sweeps in one call (buffers sized once, as the reference arm
    times them) follow the scalar oracle's TrainNoCopy trace."""
    if oracle.openblas() is None:
        pytest.skip("scipy's bundled OpenBLAS not found")
    from fastem_gb300 import synth
    X, _ = synth.em_large(seed=3, n=5000, d=16, k=6)
    pi, mu, sg = synth.dsquared_init(X, 6, seed=5)
    ll, sec, pi2, mu2, sg2 = oracle.em_sweeps_blas(X, pi, mu, sg, 4, nthreads=2)
    ref = oracle.em_train(X, pi, mu, sg, 4, eps=0.0)
    assert len(ref["logl"]) == 4 and np.all(sec > 0)
    np.testing.assert_allclose(ll, ref["logl"], rtol=1e-10)
    np.testing.assert_allclose(pi2, ref["pi"], rtol=1e-9)
    np.testing.assert_allclose(sg2, ref["sigma"], rtol=1e-7, atol=1e-10)
