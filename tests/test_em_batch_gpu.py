"""GPU parity of the batched EM engine (fem_em_batch_*): every fit against
the FP64 oracle run on that fit alone, and against the single-fit FP32 path;
per-fit convergence, Cholesky and condition-number stops."""
import numpy as np
import pytest

from fastem_gb300 import CudaBatchEM, CudaMatrixEM, GaussianMixture, synth
from fastem_gb300 import _capi as C

pytestmark = pytest.mark.gpu

# (d, n, k, data seed): every dimension class, d below its class (zero
# padding), k spanning several staged component groups and covariance unit
# ranges; none of these fits collapses in the FP64 oracle
SHAPES = [(2, 3000, 3, 200), (4, 5000, 7, 201), (5, 2500, 4, 202), (8, 12000, 12, 203), (13, 4000, 9, 204),
          (16, 20000, 20, 205), (21, 6000, 6, 206), (32, 30000, 32, 207), (32, 9000, 40, 208),
          (24, 16000, 64, 214), (16, 2022, 2, 210), (8, 1500, 31, 211), (28, 20000, 48, 213)]


def fits(shapes=SHAPES, seed_shift=0):
    out = []
    for i, (d, n, k, seed) in enumerate(shapes):
        X, _ = synth.kmeans_blobs(seed=seed + seed_shift, n=n, d=d, k=k, spread=8.0)
        out.append((X, synth.dsquared_init(X, k, seed=seed % 100)))
    return out


def train_batch(data, sweeps, eps=0.0, abort_thr=1e12, reg=0.0, svd=False, tuning="table", precision="fp32"):
    shapes = [(X.shape[1], X.shape[0], len(init[0])) for X, init in data]
    with CudaBatchEM(shapes, tuning=tuning, precision=precision) as B:
        B.SetParameters(sweeps, eps, abort_thr, reg)
        st, it, ll = B.Train([X for X, _ in data], [GaussianMixture(*init) for _, init in data], svd=svd)
        traces = [B.Trace(i) for i in range(len(data))]
        mix = [B.GetMixture(i) for i in range(len(data))]
        fail = [B.FailedComponent(i) for i in range(len(data))]
    return dict(status=st, iters=it, logl=ll, traces=traces, mix=mix, fail=fail)


# item sizes: the library defaults, the smallest and the largest the autotuner
# tries, and its committed table
TUNINGS = {"default": None, "small": {"means_chunk": [512] * 4, "cov_chunk": [1024] * 4},
           "large": {"means_chunk": [8192] * 4, "cov_chunk": [8192] * 4}, "table": "table"}


@pytest.mark.parametrize("tuning", list(TUNINGS) + ["mixed"])
def test_batch_matches_oracle(gpu_lib, oracle, tuning):
    """10 sweeps of every fit: |dlogL/N| <= 1e-5 per sweep against the FP64
    oracle (FP32 per-point terms, FP64 sums), same IterCounter, means and
    weights close -- whatever the work-item sizes, and with the tensor-core
    E-step of the d > 16 fits (mixed)."""
    data = fits()
    if tuning == "mixed":
        got = train_batch(data, 10, precision="mixed")
    else:
        got = train_batch(data, 10, tuning=TUNINGS[tuning])
    for i, (X, init) in enumerate(data):
        ref = oracle.em_train(X, *init, 10, eps=0.0, abort_thr=1e12)
        assert ref["status"] == 0
        assert got["status"][i] == 0 and got["iters"][i] == ref["iter_counter"] == 11
        ll, ee = got["traces"][i]
        err = np.max(np.abs(ll - ref["logl"])) / len(X)
        print(i, X.shape, len(init[0]), "|dlogL/N| =", err)
        assert err <= 1e-5, (i, err)
        G = got["mix"][i]
        np.testing.assert_allclose(G.weights, ref["pi"], rtol=1e-3, atol=1e-6)
        scale = np.max(np.abs(ref["mu"]))
        assert np.max(np.abs(G.means - ref["mu"])) <= 1e-4 * scale
        cs = np.max(np.abs(ref["sigma"]))
        assert np.max(np.abs(G.covs - ref["sigma"])) <= 1e-3 * cs


def test_batch_matches_single_fit_fp32(gpu_lib):
    """The batch and the single-fit FP32 handle agree fit by fit (both FP32
    with FP64 sums; only the summation order differs)."""
    data = fits(SHAPES[:6])
    got = train_batch(data, 6)
    for i, (X, init) in enumerate(data):
        d = X.shape[1]
        with CudaMatrixEM(d, len(X), len(init[0]), precision="fp32") as em:
            em.SetParameters(6, 0.0, 1e12)
            em.Train(X, GaussianMixture(*init))
            ref = em.logl_trace
        np.testing.assert_allclose(got["traces"][i][0], ref, rtol=2e-6)


def test_batch_convergence_per_fit(gpu_lib):
    """eps > 0: each fit stops on its own at the first sweep with e < Eps
    (IterCounter = sweeps + 1), the others keep sweeping."""
    data = fits(SHAPES[:8])
    eps = 1e-4
    got = train_batch(data, 200, eps=eps)
    iters = []
    for i in range(len(data)):
        assert got["status"][i] == 0
        ll, ee = got["traces"][i]
        assert len(ll) == got["iters"][i] - 1 >= 1
        assert ee[-1] < eps and np.all(ee[:-1] >= eps)
        assert got["logl"][i] == ll[-1]
        iters.append(got["iters"][i])
    assert len(set(iters)) > 1        # the fits did stop at different sweeps


def test_batch_failures_stop_only_their_fit(gpu_lib, oracle):
    """A fit with a singular initial covariance fails before the first sweep
    (IterCounter 0), a fit whose components collapse fails in the sweep the
    oracle fails in; the other fits train to the end unchanged."""
    good = fits(SHAPES[:3])
    # 26 components on 2536 8-d points: a component collapses in sweep 2
    X, _ = synth.kmeans_blobs(seed=637563561, n=2536, d=8, k=26)
    collapse = (X, synth.dsquared_init(X, 26, seed=637563561 % 1000))
    Xs, _ = synth.kmeans_blobs(seed=7, n=3000, d=4, k=3)
    pi, mu, _ = synth.dsquared_init(Xs, 3, seed=1)
    singular = (Xs, (pi, mu, np.zeros((3, 4, 4))))
    data = good + [collapse, singular]
    got = train_batch(data, 8)
    ref = oracle.em_train(collapse[0], *collapse[1], 8, eps=0.0, abort_thr=1e12)
    assert ref["status"] == C.FEM_ERR_CHOLESKY
    # the sweep in which a collapsing covariance stops being positive definite
    # depends on rounding: FP32 sums may cross it one sweep apart from FP64
    assert got["status"][3] == C.FEM_ERR_CHOLESKY and abs(got["iters"][3] - ref["iter_counter"]) <= 1
    m = min(len(got["traces"][3][0]), len(ref["logl"]))
    assert np.max(np.abs(got["traces"][3][0][:m] - ref["logl"][:m])) / len(collapse[0]) <= 1e-5
    assert got["status"][4] == C.FEM_ERR_CHOLESKY and got["iters"][4] == 0 and got["fail"][4] == 0
    alone = train_batch(good, 8)
    for i in range(3):
        assert got["status"][i] == 0 and got["iters"][i] == 9
        np.testing.assert_array_equal(got["traces"][i][0], alone["traces"][i][0])


def test_batch_condition_check(gpu_lib, oracle):
    """svd on: a fit whose covariance condition exceeds AbortThr stops with
    FEM_ERR_COND_ABORT; below it the check changes nothing."""
    data = fits(SHAPES[:4])
    base = train_batch(data, 4)
    chk = train_batch(data, 4, svd=True)
    for i in range(4):
        assert chk["status"][i] == 0
        np.testing.assert_array_equal(chk["traces"][i][0], base["traces"][i][0])
    ab = train_batch(data, 4, abort_thr=1.0 + 1e-9, svd=True)
    for i, (X, init) in enumerate(data):
        ref = oracle.em_train(X, *init, 4, eps=0.0, abort_thr=1.0 + 1e-9, svd=True)
        assert ab["status"][i] == ref["status"] == C.FEM_ERR_COND_ABORT
        assert ab["iters"][i] == ref["iter_counter"]


def test_batch_regularization(gpu_lib, oracle):
    """RegCoef > 0 (EMAlgorithm::RegularizeCovariances) in every sweep."""
    data = fits(SHAPES[3:7])
    got = train_batch(data, 5, reg=0.05)
    for i, (X, init) in enumerate(data):
        ref = oracle.em_train(X, *init, 5, eps=0.0, abort_thr=1e12, reg_coef=0.05)
        err = np.max(np.abs(got["traces"][i][0] - ref["logl"])) / len(X)
        assert err <= 1e-5, (i, err)


def test_batch_rejects_unsupported_shapes(gpu_lib):
    for shape in [(33, 1000, 4), (8, 1000, 65)]:
        with pytest.raises(C.FemError, match="batched fits need"):
            CudaBatchEM([(4, 1000, 2), shape])


def test_batch_edge_shapes(gpu_lib, oracle):
    """d = 1, K = 1, fits smaller than one E-step item (512 points) or just
    over it, n barely above d, 64 components in 2 dimensions: each fit's
    trace against the FP64 oracle."""
    shapes = [(1, 500, 1, 701), (1, 1000, 3, 702), (3, 40, 2, 703), (32, 200, 1, 704), (7, 513, 2, 705),
              (2, 5000, 64, 706)]
    data = []
    for d, n, k, seed in shapes:
        X, _ = synth.kmeans_blobs(seed=seed, n=n, d=d, k=k, spread=6.0)
        data.append((X, synth.dsquared_init(X, k, seed=seed - 700)))
    got = train_batch(data, 6)
    for i, (X, init) in enumerate(data):
        ref = oracle.em_train(X, *init, 6, eps=0.0, abort_thr=1e12)
        assert ref["status"] == 0 and got["status"][i] == 0 and got["iters"][i] == ref["iter_counter"]
        err = np.max(np.abs(got["traces"][i][0] - ref["logl"])) / len(X)
        assert err <= 1e-5, (shapes[i], err)


def test_batch_mixed_mixes_classes_and_ragged_tiles(gpu_lib, oracle):
    """mixed: fits of every class in one batch, the d > 16 ones with n not a
    multiple of the 128-point tile and k not a multiple of 4 (padding
    components), against the oracle and against the FP32 batch"""
    shapes = [(20, 1000 + 37, 5, 301), (32, 777, 9, 302), (8, 3000, 6, 303), (17, 4321, 13, 304),
              (4, 2000, 3, 305), (30, 129, 2, 306)]
    data = fits(shapes)
    got = train_batch(data, 6, precision="mixed")
    f32 = train_batch(data, 6)
    for i, (X, init) in enumerate(data):
        ref = oracle.em_train(X, *init, 6, eps=0.0, abort_thr=1e12)
        if ref["status"] != 0:
            continue
        ll, _ = got["traces"][i]
        err = np.max(np.abs(ll - ref["logl"])) / len(X)
        print(i, X.shape, "mixed |dlogL/N| =", err)
        assert err <= 1e-5, (i, err)
        if X.shape[1] <= 16:
            # the same CUDA-core kernels as the FP32 batch
            np.testing.assert_array_equal(ll, f32["traces"][i][0])
