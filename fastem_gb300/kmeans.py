"""Python mirror of the reference's k-means interface on top of the C-ABI.

  CudaKMA   KMeansAlgorithm / NaiveKMA (Clust/KMAlgorithm.h:29-117): Lloyd
            iterations on one GB300 with assignments bit-exact to an FP64
            difference-form argmin (lowest index wins ties).
Centroids use the CentroidVector layout (Clust/CentroidVector.h:11-17):
K consecutive rows of d doubles.
"""
import ctypes

import numpy as np

from . import _capi as C


class CudaKMA:
    def __init__(self, ncols, nrows, nclusters, precision="mixed", device=0, seed=0, repair=True):
        cfg = C.KmConfig()
        C.lib().fem_km_config_default(ctypes.byref(cfg))
        cfg.precision = C.PREC[precision]
        cfg.device = device
        cfg.seed = int(seed)
        # True / "random": CentroidRandomRepair; "next": CentroidDeterministicRepair;
        # False / "none": empty clusters keep their centroid
        cfg.repair = {False: 0, True: 1, "none": 0, "random": 1, "next": 2}[repair]
        h = ctypes.c_void_p()
        C.check(C.lib().fem_km_create(int(ncols), int(nrows), int(nclusters), ctypes.byref(cfg),
                                      ctypes.byref(h)))
        self._h = h
        self.ncols, self.nrows, self.nclusters = int(ncols), int(nrows), int(nclusters)
        self.precision = precision
        self.IterCount = 0

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            C.lib().fem_km_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def SetDataset(self, X):
        X = C.f32rows(X)
        assert X.shape == (self.nrows, self.ncols)
        C.check(C.lib().fem_km_upload(self._h, C.ptr(X), X.shape[1]))

    def SetDatasetDevice(self, dev_ptr, ld=None):
        C.check(C.lib().fem_km_upload_device(self._h, ctypes.c_void_p(dev_ptr),
                                             int(ld or self.ncols)))

    def Seed(self, seed):
        C.check(C.lib().fem_km_seed(self._h, int(seed)))

    def InitDataStructures(self, vec=None):
        C.check(C.lib().fem_km_init_data_structures(self._h))

    def ComputeMSEAndCorrect(self, vec):
        """vec: (K, d) float64 array updated in place.  Returns fit / N."""
        assert vec.dtype == np.float64 and vec.flags.c_contiguous
        fit = ctypes.c_double(np.nan)
        C.check(C.lib().fem_km_compute_mse_and_correct(self._h, C.ptr(vec), ctypes.byref(fit),
                                                       None))
        return fit.value

    def CorrectWithoutMSE(self, vec):
        """NaiveKMA::CorrectWithoutMSE (Clust/KMAlgorithm.cpp:148-202): vec
        updated in place; True when some label changed since the previous
        iteration."""
        assert vec.dtype == np.float64 and vec.flags.c_contiguous
        changed = ctypes.c_int(0)
        C.check(C.lib().fem_km_correct_without_mse(self._h, C.ptr(vec), ctypes.byref(changed)))
        return bool(changed.value)

    def ComputeMSEAndCorrectCounts(self, vec):
        assert vec.dtype == np.float64 and vec.flags.c_contiguous
        fit = ctypes.c_double(np.nan)
        counts = np.zeros(self.nclusters, dtype=np.int64)
        C.check(C.lib().fem_km_compute_mse_and_correct(self._h, C.ptr(vec), ctypes.byref(fit),
                                                       C.ptr(counts)))
        return fit.value, counts

    def RunKMeans(self, vec, verbosity=0, MinRel=-1.0, MaxIter=0):
        assert vec.dtype == np.float64 and vec.flags.c_contiguous
        best = ctypes.c_double(0)
        it = ctypes.c_int(0)
        C.check(C.lib().fem_km_run(self._h, C.ptr(vec), float(MinRel), int(MaxIter),
                                   ctypes.byref(best), ctypes.byref(it)))
        self.IterCount += it.value
        return best.value

    def Assignment(self):
        out = np.zeros(self.nrows, dtype=np.int32)
        C.check(C.lib().fem_km_get_assignment(self._h, C.ptr(out)))
        return out

    def Stats(self):
        r, a, u = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        C.check(C.lib().fem_km_stats(self._h, ctypes.byref(r), ctypes.byref(a), ctypes.byref(u)))
        return dict(rechecked=r.value, assign_ms=a.value, update_ms=u.value)
