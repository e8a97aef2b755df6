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


def handle_reference(X, cent):
    n, d = X.shape
    k = cent.shape[0]
    with CudaKMA(d, n, k, precision="fp32", repair=False) as km:
        km.SetDataset(X)
        km.InitDataStructures()
        fit = km.ComputeMSEAndCorrect(cent.copy())   # fit and labels refer to `cent`
        labels = km.Assignment()
    return labels, fit


@pytest.mark.parametrize("n,d,k", [(200_003, 32, 96), (65_536 + 17, 64, 128), (1000, 8, 3)])
def test_classify_noalloc_matches_handle(gpu_lib, n, d, k):
    torch = pytest.importorskip("torch")
    X, _ = synth.kmeans_blobs(seed=11, n=n, d=d, k=k)
    rng = np.random.default_rng(5)
    cent = np.ascontiguousarray(X[rng.choice(n, size=k, replace=False)].astype(np.float64) +
                                rng.standard_normal((k, d)) * 0.5)
    labels_ref, fit_ref = handle_reference(X, cent)

    f = noalloc_fn()
    dX = torch.from_numpy(X).cuda()
    dC = torch.from_numpy(cent).cuda()
    dL = torch.empty(n, dtype=torch.int32, device="cuda")
    dF = torch.empty(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):                      # two calls in a row share the scratch
        dL.fill_(-7)
        dF.fill_(float("nan"))
        C.check(f(d, n, k, dX.data_ptr(), dC.data_ptr(), dL.data_ptr(), dF.data_ptr(),
                  torch.cuda.current_device(), stream))
        torch.cuda.synchronize()
        labels = dL.cpu().numpy()
        fit = dF.item()
        print("no-alloc call %d: n=%d d=%d k=%d fit %.17g vs %.17g" % (call, n, d, k, fit, fit_ref))
        assert np.array_equal(labels, labels_ref)
        assert abs(fit - fit_ref) <= FIT_RTOL * abs(fit_ref)


def test_classify_noalloc_rejects_oversize(gpu_lib):
    f = noalloc_fn()
    one = ctypes.c_void_p(16)                  # never dereferenced: the size check comes first
    st = f(32, 1000, 2048, one, one, one, one, 0, None)
    assert st == 1                             # FEM_ERR_BAD_ARG
    assert b"scratch" in C.lib().fem_last_error()
    assert f(64, 1000, 600, one, one, one, one, 0, None) == 1
    assert f(12, 1000, 4, one, one, one, one, 0, None) == 8   # FEM_ERR_UNSUPPORTED
