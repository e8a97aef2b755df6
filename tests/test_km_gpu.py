"""GPU parity of the Lloyd iteration: assignments bit-exact to the FP64
oracle, centroids and fit within FP64 rounding."""
import os

import numpy as np
import pytest

from fastem_gb300 import CudaKMA, synth

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def iterate_both(oracle, X, C0, iters, precision, repair=True, seed=0):
    n, d = X.shape
    k = C0.shape[0]
    Cg = np.array(C0, dtype=np.float64, copy=True)
    Co = Cg.copy()
    out = []
    with CudaKMA(d, n, k, precision=precision, seed=seed, repair=repair) as km:
        km.SetDataset(X)
        oracle.rng_seed(seed)
        for _ in range(iters):
            fg, cg = km.ComputeMSEAndCorrectCounts(Cg)
            lg = km.Assignment()
            fo, Co, co, lo = oracle.km_iterate(X, Co, repair=repair)
            out.append((fg, cg, lg, Cg.copy(), fo, co, lo, Co.copy(), km.Stats()))
    return out


def check_iters(out):
    for it, (fg, cg, lg, Cg, fo, co, lo, Co, st) in enumerate(out):
        assert np.array_equal(lg, lo), "labels differ at iteration %d (%d rows)" % (it, (lg != lo).sum())
        assert np.array_equal(cg, co)
        assert abs(fg - fo) <= 1e-11 * abs(fo)
        np.testing.assert_allclose(Cg, Co, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_km_blobs_30_iterations(gpu_lib, oracle, precision):
    """kmeans_blobs shape at reduced N (d=32, K=64), k-means|| seed 3, 30 iterations."""
    X, _ = synth.kmeans_blobs(seed=2, n=1 << 17, d=32, k=64)
    C0 = oracle.kmeans_oror(X, 64, seed=3)
    out = iterate_both(oracle, X, C0, 30, precision)
    check_iters(out)
    print("rechecked rows per iteration:", [o[-1]["rechecked"] for o in out])


@pytest.mark.parametrize("precision", ["fp32"])
def test_km_golden_fixture(gpu_lib, precision):
    z = np.load(os.path.join(GOLDEN, "km_blobs.npz"))
    C = z["C0"].copy()
    with CudaKMA(8, len(z["X"]), 8, precision=precision) as km:
        km.SetDataset(z["X"])
        for it in range(len(z["fits"])):
            fit, cnt = km.ComputeMSEAndCorrectCounts(C)
            assert np.array_equal(km.Assignment(), z["labels"][it])
            assert np.array_equal(cnt, z["counts"][it])
            assert abs(fit - z["fits"][it]) <= 1e-12 * z["fits"][it]
            np.testing.assert_allclose(C, z["centroids"][it], rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_km_matches_reference_fixture(gpu_lib, precision):
    """Against tests/golden/km_ref.npz, written by the reference's own
    NaiveKMA::ComputeMSEAndCorrect (Clust/KMAlgorithm.cpp:205-255, built from
    its sources): d = 32 overlapping blobs with many near ties and an empty
    cluster repaired from the generator (CentroidRandomRepair, seed 17) in the
    first iteration.  Labels bit-exact, centroids and fit within FP64
    summation order."""
    z = np.load(os.path.join(GOLDEN, "km_ref.npz"))
    X, C = z["X"], z["C0"].copy()
    n, d = X.shape
    with CudaKMA(d, n, C.shape[0], precision=precision, seed=int(z["seed"]), repair=True) as km:
        km.SetDataset(X)
        for it in range(len(z["fits"])):
            fit = km.ComputeMSEAndCorrect(C)
            lab = km.Assignment()
            assert np.array_equal(lab, z["labels"][it]), "iteration %d: %d labels differ" % (
                it, (lab != z["labels"][it]).sum())
            np.testing.assert_allclose(C, z["centroids"][it], rtol=1e-13, atol=1e-13)
            assert abs(fit - z["fits"][it]) <= 1e-12 * z["fits"][it]


def test_km_exact_ties_lowest_index(gpu_lib):
    z = np.load(os.path.join(GOLDEN, "km_ties.npz"))
    C = z["C0"].copy()
    with CudaKMA(2, len(z["X"]), 4, precision="fp32", repair=False) as km:
        km.SetDataset(z["X"])
        fit, cnt = km.ComputeMSEAndCorrectCounts(C)
        assert np.array_equal(km.Assignment(), z["labels"])
        assert np.array_equal(cnt, z["counts"])
        assert km.Stats()["rechecked"] >= 2


def test_km_empty_cluster_repair(gpu_lib, oracle):
    X, _ = synth.kmeans_blobs(seed=6, n=1000, d=4, k=3)
    C0 = np.vstack([X[:3].astype(np.float64), np.full((1, 4), 1e6)])
    out = iterate_both(oracle, X, C0, 2, "fp32", seed=17)
    assert out[0][1][3] == 0
    check_iters(out)


def test_km_deterministic_repair(gpu_lib, oracle):
    """repair="next" (CentroidDeterministicRepair, Clust/CentroidRepair.cpp:
    30-43): empty clusters take rows 0, 1, 2, ... in index order, the counter
    carried from one iteration to the next; the other centroids as without
    repair."""
    X, _ = synth.kmeans_blobs(seed=6, n=1000, d=4, k=3)
    C0 = np.vstack([X[:3].astype(np.float64), np.full((2, 4), 1e6)])
    with CudaKMA(4, len(X), 5, precision="fp32", repair="next") as km:
        km.SetDataset(X)
        C = C0.copy()
        _, counts = km.ComputeMSEAndCorrectCounts(C)
        _, Co, co, _ = oracle.km_iterate(X, C0, repair=False)
        assert list(counts[3:]) == [0, 0] and np.array_equal(counts, co)
        np.testing.assert_array_equal(C[3:], X[:2].astype(np.float64))
        np.testing.assert_allclose(C[:3], Co[:3], rtol=1e-13, atol=1e-13)
        C[4] = 1e6
        _, counts = km.ComputeMSEAndCorrectCounts(C)
        assert counts[4] == 0
        np.testing.assert_array_equal(C[4], X[2].astype(np.float64))


@pytest.mark.parametrize("n", [1, 255, 257, 10001])
def test_km_ragged(gpu_lib, oracle, n):
    X, _ = synth.kmeans_blobs(seed=8, n=max(n, 16), d=16, k=5)
    X = X[:n]
    C0 = X[np.arange(5) % n].astype(np.float64) + 0.5
    check_iters(iterate_both(oracle, X, C0, 2, "fp32", repair=False))


def test_km_run_matches_oracle(gpu_lib, oracle):
    X, _ = synth.kmeans_blobs(seed=4, n=30000, d=8, k=10)
    C0 = oracle.kmeans_forgy(X, 10, seed=1)
    best_o, Co, it_o = oracle.km_run(X, C0, min_rel=1e-4, max_iter=30)
    Cg = C0.copy()
    with CudaKMA(8, len(X), 10, precision="fp32") as km:
        km.SetDataset(X)
        best_g = km.RunKMeans(Cg, MinRel=1e-4, MaxIter=30)
        assert km.IterCount == it_o
    assert abs(best_g - best_o) <= 1e-11 * best_o
    np.testing.assert_allclose(Cg, Co, rtol=1e-13, atol=1e-13)


# ---------------------------------------------------------------- tensor-core path (d = 32)

@pytest.mark.parametrize("n,k", [(1, 5), (127, 5), (129, 17), (10001, 200), (1 << 16, 256)])
def test_km_tc_ragged_and_padded_k(gpu_lib, oracle, n, k):
    """Rows past N (partial 128-row tiles) and K not a multiple of 16 / 32
    (padded MMA columns) are ignored; labels bit-exact to the oracle."""
    X, _ = synth.kmeans_blobs(seed=9, n=max(n, k), d=32, k=k)
    X = X[:n]
    rng = np.random.default_rng(3)
    C0 = X[rng.integers(0, n, size=k)].astype(np.float64) + rng.standard_normal((k, 32))
    check_iters(iterate_both(oracle, X, C0, 3, "mixed", repair=False))


def test_km_tc_duplicate_centroids_recheck(gpu_lib, oracle):
    """Exact ties (a centroid repeated) cannot be separated by the bound: the
    rows are re-decided in FP64 and the lowest index wins."""
    X, _ = synth.kmeans_blobs(seed=10, n=20000, d=32, k=16)
    C0 = oracle.kmeans_forgy(X, 16, seed=2)
    C0[9] = C0[3]
    C0[15] = C0[3]
    with CudaKMA(32, len(X), 16, precision="mixed", repair=False) as km:
        km.SetDataset(X)
        C = C0.copy()
        km.ComputeMSEAndCorrect(C)
        lg = km.Assignment()
        st = km.Stats()
    fo, Co, co, lo = oracle.km_iterate(X, C0.copy(), repair=False)
    assert np.array_equal(lg, lo)
    assert (lg == 9).sum() == 0 and (lg == 15).sum() == 0
    assert st["rechecked"] >= (lo == 3).sum()
    np.testing.assert_allclose(C, Co, rtol=1e-13, atol=1e-13)


def test_km_tc_far_from_origin(gpu_lib, oracle):
    """Blobs offset by 3e3 (||x|| ~ 2e4, so the error of ||c||^2 - 2 x.c grows
    with ||x|| ||c||): the bound must still hold; labels bit-exact."""
    X, _ = synth.kmeans_blobs(seed=12, n=1 << 16, d=32, k=64, spread=20.0, sigma=1.0)
    X = (X + 3000.0).astype(np.float32)
    C0 = oracle.kmeans_forgy(X, 64, seed=4)
    out = iterate_both(oracle, X, C0, 4, "mixed", repair=False)
    check_iters(out)
    print("rechecked rows per iteration:", [o[-1]["rechecked"] for o in out])


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_km_correct_without_mse(gpu_lib, oracle, precision):
    """NaiveKMA::CorrectWithoutMSE: the same iteration without the fit,
    reporting whether any label changed since the previous one (all zero
    before the first); run until nothing changes, as KMeansWithoutMSE does."""
    X, _ = synth.kmeans_blobs(seed=11, n=20000, d=32, k=12, spread=6.0)
    C0 = X[np.random.default_rng(3).choice(len(X), 12, replace=False)].astype(np.float64)
    Cg, Co = C0.copy(), C0.copy()
    prev = np.zeros(len(X), dtype=np.int32)
    with CudaKMA(32, len(X), 12, precision=precision, repair=True) as km:
        km.SetDataset(X)
        km.InitDataStructures()
        for it in range(60):
            changed = km.CorrectWithoutMSE(Cg)
            _, Co, _, lo = oracle.km_iterate(X, Co, repair=True)
            assert np.array_equal(km.Assignment(), lo), it
            np.testing.assert_allclose(Cg, Co, rtol=1e-13, atol=1e-13)
            assert changed == bool(np.any(lo != prev)), it
            prev = lo.copy()
            if not changed:
                break
        assert not changed and it > 1
