"""fem_km_classify_noalloc -- k-means classification on caller-owned device
buffers with a fixed static scratch array -- against the handle API
(fem_km_compute_mse_and_correct + fem_km_get_assignment) on the same inputs.

Labels must be identical (both are the FP64 difference-form argmin, lowest
index on ties); the fit is the same sum of FP64 distances formed in another
order (per-CTA partials here, cluster sums through the data mean there), so
it is compared to 1e-10 relative.  The file name sorts last so that the test
also runs after every other GPU test of the session."""
import ctypes

import numpy as np
import pytest

from fastem_gb300 import CudaKMA, synth
from fastem_gb300 import _capi as C

pytestmark = pytest.mark.gpu

FIT_RTOL = 1e-10


def noalloc_fn():
    return C.lib().fem_km_classify_noalloc


def handle_reference(X, cent, oracle=None):
    """Labels and fit of `cent` from the handle API; where its shared-memory
    centroid table cannot hold k x d (the size limits of the no-alloc entry
    point go further), from the FP64 oracle's NaiveKMA restatement."""
    n, d = X.shape
    k = cent.shape[0]
    if oracle is not None and k * d * 12 + 256 * (d + 1) * 4 + k * 8 + 1024 > 220 * 1024:
        fit, _, _, labels = oracle.km_iterate(X, cent, repair=False)
        return labels, fit
    with CudaKMA(d, n, k, precision="fp32", repair=False) as km:
        km.SetDataset(X)
        km.InitDataStructures()
        fit = km.ComputeMSEAndCorrect(cent.copy())   # fit and labels refer to `cent`
        labels = km.Assignment()
    return labels, fit


@pytest.mark.parametrize("n,d,k", [(200_003, 32, 96), (65_536 + 17, 64, 128), (1000, 8, 3),
                                   # the size limits: k * d = 32768 and k = 1024 fill the scratch and
                                   # the largest shared-memory layouts (~200 KB)
                                   (20_000 + 3, 64, 512), (20_000 + 5, 32, 1024), (5_000 + 1, 2, 1024),
                                   # d = 4, 16: a partial last tile of 256 rows
                                   (300, 4, 5), (777, 16, 33)])
def test_classify_noalloc_matches_handle(gpu_lib, oracle, n, d, k):
    torch = pytest.importorskip("torch")
    X, _ = synth.kmeans_blobs(seed=11, n=n, d=d, k=k)
    rng = np.random.default_rng(5)
    cent = np.ascontiguousarray(X[rng.choice(n, size=k, replace=False)].astype(np.float64) +
                                rng.standard_normal((k, d)) * 0.5)
    labels_ref, fit_ref = handle_reference(X, cent, oracle)

    f = noalloc_fn()
    dX = torch.from_numpy(X).cuda()
    dC = torch.from_numpy(cent).cuda()
    dL = torch.empty(n, dtype=torch.int32, device="cuda")
    dF = torch.empty(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):                      # two calls in a row share the scratch
        dL.fill_(-7)
        dF.fill_(float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        C.check(f(d, n, k, dX.data_ptr(), dC.data_ptr(), dL.data_ptr(), dF.data_ptr(),
                  torch.cuda.current_device(), stream))
        torch.cuda.synchronize()
        if call == 1:
            # after the first call's set-up, a call allocates no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        labels = dL.cpu().numpy()
        fit = dF.item()
        print("no-alloc call %d: n=%d d=%d k=%d fit %.17g vs %.17g" % (call, n, d, k, fit, fit_ref))
        assert np.array_equal(labels, labels_ref)
        assert abs(fit - fit_ref) <= FIT_RTOL * abs(fit_ref)


def test_classify_noalloc_nan_row(gpu_lib):
    """A row of NaN is closer to no centroid: label -1 and DBL_MAX added to
    the fit, as CentroidVector::ClassifyDataset / ComputeMSE leave it
    (Clust/CentroidVector.cpp:8-34,56-94); every other row as the handle API
    labels it without that row."""
    torch = pytest.importorskip("torch")
    n, d, k = 3000, 8, 6
    X, _ = synth.kmeans_blobs(seed=13, n=n, d=d, k=k)
    cent = np.ascontiguousarray(X[:k].astype(np.float64) + 0.25)
    bad = 1234
    keep = np.arange(n) != bad
    labels_ref, fit_ref = handle_reference(np.ascontiguousarray(X[keep]), cent)
    Xn = X.copy()
    Xn[bad] = np.nan
    dX = torch.from_numpy(Xn).cuda()
    dC = torch.from_numpy(cent).cuda()
    dL = torch.empty(n, dtype=torch.int32, device="cuda")
    dF = torch.empty(1, dtype=torch.float64, device="cuda")
    C.check(noalloc_fn()(d, n, k, dX.data_ptr(), dC.data_ptr(), dL.data_ptr(), dF.data_ptr(),
                         torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    labels = dL.cpu().numpy()
    assert labels[bad] == -1
    assert np.array_equal(labels[keep], labels_ref)
    assert dF.item() == pytest.approx((fit_ref * (n - 1) + np.finfo(np.float64).max) / n, rel=1e-12)


def test_classify_noalloc_rejects_oversize(gpu_lib):
    f = noalloc_fn()
    one = ctypes.c_void_p(16)                  # never dereferenced: the size check comes first
    st = f(32, 1000, 2048, one, one, one, one, 0, None)
    assert st == 1                             # FEM_ERR_BAD_ARG
    assert b"scratch" in C.lib().fem_last_error()
    assert f(64, 1000, 600, one, one, one, one, 0, None) == 1
    assert f(12, 1000, 4, one, one, one, one, 0, None) == 8   # FEM_ERR_UNSUPPORTED
