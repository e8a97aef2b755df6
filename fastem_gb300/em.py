"""Python mirror of the reference's EM interface on top of the C-ABI.

  GaussianMixture   EM2/GaussianMixture.h:17-58 (weights, means, covariances;
                    .cmp read/write in fastem_gb300.formats)
  CudaMatrixEM      EMAlgorithm / SimpleMatrixEM (EM2/EMAlgorithm.h:26-79,
                    EM2/MatrixEM.h:83-100) running on one GB300
"""
import ctypes

import numpy as np

from . import _capi as C


class GaussianMixture:
    """K weights, K x d means and K x d x d covariances (FP64)."""

    def __init__(self, weights, means, covs):
        self.weights = np.array(weights, dtype=np.float64, copy=True)
        self.means = np.array(means, dtype=np.float64, copy=True, order="C")
        self.covs = np.array(covs, dtype=np.float64, copy=True, order="C")
        k, d = self.means.shape
        assert self.weights.shape == (k,) and self.covs.shape == (k, d, d)

    def GetComponentCount(self):
        return self.means.shape[0]

    def GetDimension(self):
        return self.means.shape[1]

    def GetWeight(self, j):
        return self.weights[j]

    def GetMean(self, j):
        return self.means[j].copy()

    def GetCovariance(self, j):
        return self.covs[j].copy()

    def Init(self, weights, covs, means):
        self.__init__(weights, means, covs)

    def copy(self):
        return GaussianMixture(self.weights, self.means, self.covs)

    def _log_terms(self, X):
        """log(pi_j N(x; mu_j, Sigma_j)) for the rows of X (n x K, FP64 on the
        host), through the Cholesky factor of each covariance's lower triangle
        as NormalDensity::Init (EM2/NormalDensity.cpp:43-65) forms it."""
        X = np.atleast_2d(np.asarray(X, dtype=np.float64))
        k, d = self.means.shape
        out = np.empty((X.shape[0], k))
        for j in range(k):
            L = np.linalg.cholesky(np.tril(self.covs[j]) + np.tril(self.covs[j], -1).T)
            y = np.linalg.solve(L, (X - self.means[j]).T)
            logdet = 2.0 * np.log(np.diag(L)).sum()
            out[:, j] = (np.log(self.weights[j]) - 0.5 * d * np.log(2.0 * np.pi) - 0.5 * logdet
                         - 0.5 * np.einsum("ij,ij->j", y, y))
        return out

    def Evaluate(self, x):
        """GaussianMixture::Evaluate (EM2/GaussianMixture.cpp:54-60): the
        mixture density sum_j pi_j N(x), summed in the log domain (the same
        value where the densities do not underflow).  One row -> a float,
        n rows -> n values."""
        lt = self._log_terms(x)
        m = lt.max(axis=1, keepdims=True)
        v = (np.exp(m[:, 0]) * np.exp(lt - m).sum(axis=1))
        return float(v[0]) if np.ndim(x) == 1 else v

    def ComputePosteriors(self, x):
        """GaussianMixture::ComputePosteriors (EM2/GaussianMixture.cpp:62-69):
        pi_j N(x) / sum, per row."""
        lt = self._log_terms(x)
        p = np.exp(lt - lt.max(axis=1, keepdims=True))
        p /= p.sum(axis=1, keepdims=True)
        return p[0] if np.ndim(x) == 1 else p

    def Classify(self, x):
        """GaussianMixture::Classify (EM2/GaussianMixture.cpp:86-98): the
        component of largest pi_j N(x), lowest index on ties; compared in the
        log domain, so a row far from every component still gets its nearest
        one where the reference's densities underflow to 0 and give 0."""
        c = np.argmax(self._log_terms(x), axis=1)
        return int(c[0]) if np.ndim(x) == 1 else c

    def NormalizeWeights(self):
        """GaussianMixture::NormalizeWeights (EM2/GaussianMixture.cpp:71-79)."""
        self.weights *= 1.0 / self.weights.sum()

    def FindLargestConditionNumber(self):
        """GaussianMixture::FindLargestConditionNumber (EM2/GaussianMixture.cpp:
        125-135): max(1, |lambda_max / lambda_min|) over the covariances."""
        cond = 1.0
        for S in self.covs:
            ev = np.linalg.eigvalsh(S, UPLO="L")
            cond = max(cond, abs(ev[-1] / ev[0]))
        return cond


class CudaMatrixEM:
    """EMAlgorithm with every sweep on the GPU.

    precision: "mixed" (tcgen05 FP16 hi/lo split contractions, FP32 accumulation, FP64
    factorisation / logdet / logL), "fp32" (CUDA cores) or "fp64"."""

    def __init__(self, ncols, nrows, ncl, precision="mixed", device=0, svd=False):
        cfg = C.EmConfig()
        C.lib().fem_em_config_default(ctypes.byref(cfg))
        cfg.precision = C.PREC[precision]
        cfg.device = device
        cfg.svd = int(bool(svd))
        h = ctypes.c_void_p()
        C.check(C.lib().fem_em_create(int(ncols), int(nrows), int(ncl), ctypes.byref(cfg),
                                      ctypes.byref(h)))
        self._h = h
        self.nCols, self.nRows, self.K = int(ncols), int(nrows), int(ncl)
        self.precision = precision
        self.IterCounter = 0
        self.logl_trace = np.zeros(0)
        self.e_trace = np.zeros(0)
        self._max_sweeps = 1000000

    def close(self):
        if getattr(self, "_h", None):
            C.lib().fem_em_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # EMAlgorithm::SetParameters
    def SetParameters(self, max_sweeps, eps, abort_thr, reg_coef=0.0):
        self._max_sweeps = int(max_sweeps)
        C.check(C.lib().fem_em_set_parameters(self._h, int(max_sweeps), float(eps),
                                              float(abort_thr), float(reg_coef)))

    # EMAlgorithm::CopyDataset
    def CopyDataset(self, X):
        X = C.f32rows(X)
        assert X.shape == (self.nRows, self.nCols)
        C.check(C.lib().fem_em_upload(self._h, C.ptr(X), X.shape[1]))

    def CopyDatasetDevice(self, dev_ptr, ld=None):
        C.check(C.lib().fem_em_upload_device(self._h, ctypes.c_void_p(dev_ptr),
                                             int(ld or self.nCols)))

    def SetMixture(self, G):
        C.check(C.lib().fem_em_set_params(self._h, C.ptr(C.f64(G.weights)), C.ptr(C.f64(G.means)),
                                          C.ptr(C.f64(G.covs))))

    def GetMixture(self):
        k, d = self.K, self.nCols
        pi, mu, sg = np.zeros(k), np.zeros((k, d)), np.zeros((k, d, d))
        C.check(C.lib().fem_em_get_params(self._h, C.ptr(pi), C.ptr(mu), C.ptr(sg)))
        return GaussianMixture(pi, mu, sg)

    # EMAlgorithm::Train / TrainNoCopy
    def Train(self, X, G, verbosity=0, svd=False):
        self.CopyDataset(X)
        return self.TrainNoCopy(G, verbosity, svd)

    def TrainNoCopy(self, G, verbosity=0, svd=False):
        self.SetMixture(G)
        cap = max(1, min(self._max_sweeps, 1 << 20))
        ll = np.full(cap, np.nan)
        ee = np.full(cap, np.nan)
        it = ctypes.c_int(0)
        logl = ctypes.c_double(np.nan)
        st = C.lib().fem_em_train(self._h, int(bool(svd)), C.ptr(ll), C.ptr(ee), cap,
                                  ctypes.byref(it), ctypes.byref(logl))
        self.IterCounter = it.value
        sweeps = max(0, min(it.value - 1, cap))
        self.logl_trace, self.e_trace = ll[:sweeps], ee[:sweeps]
        if verbosity > 1:
            for i in range(sweeps):
                print("iter: %d LogL: %10.6f e: %g" % (i + 1, ll[i], ee[i]))
        C.check(st)
        R = self.GetMixture()
        G.Init(R.weights, R.covs, R.means)
        return logl.value

    def GetIterCounter(self):
        return self.IterCounter

    # single pieces of a sweep
    def InitDensities(self):
        failed = ctypes.c_int(-1)
        C.check(C.lib().fem_em_init_densities(self._h, ctypes.byref(failed)))

    def PrecomputeDensityMatrix(self):
        v = ctypes.c_double(np.nan)
        C.check(C.lib().fem_em_precompute(self._h, ctypes.byref(v)))
        self._logl = v.value
        return v.value

    def ComputeLogLike(self):
        return self._logl

    def MStep(self):
        C.check(C.lib().fem_em_mstep(self._h))

    def FindLargestConditionNumber(self):
        v = ctypes.c_double(0)
        C.check(C.lib().fem_em_max_condition(self._h, ctypes.byref(v)))
        return v.value

    def Posteriors(self):
        out = np.zeros((self.nRows, self.K))
        C.check(C.lib().fem_em_get_posteriors(self._h, C.ptr(out)))
        return out

    def RetrieveClasses(self):
        out = np.zeros(self.nRows, dtype=np.int32)
        C.check(C.lib().fem_em_retrieve_classes(self._h, C.ptr(out)))
        return out

    def ComputePosterriorCorrelation(self):
        """R^T R (K x K) of the last E-step's posteriors."""
        out = np.zeros((self.K, self.K))
        C.check(C.lib().fem_em_posterior_correlation(self._h, C.ptr(out)))
        return out

    def Factors(self):
        k, d = self.K, self.nCols
        U, ld = np.zeros((k, d, d)), np.zeros(k)
        C.check(C.lib().fem_em_get_factors(self._h, C.ptr(U), C.ptr(ld)))
        return U, ld

    # device-time diagnostics
    def TimingReset(self, enable=True):
        C.check(C.lib().fem_em_timing_reset(self._h, int(bool(enable))))

    def Timing(self):
        e, m, f = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        n = ctypes.c_int64()
        C.check(C.lib().fem_em_timing_get(self._h, ctypes.byref(e), ctypes.byref(m),
                                          ctypes.byref(f), ctypes.byref(n)))
        t, sw = ctypes.c_double(), ctypes.c_int64()
        C.check(C.lib().fem_em_timing_total(self._h, ctypes.byref(t), ctypes.byref(sw)))
        cov = ctypes.c_double()
        C.check(C.lib().fem_em_timing_covariance(self._h, ctypes.byref(cov)))
        return dict(estep_ms=e.value, mstep_ms=m.value, factor_ms=f.value, launches=n.value,
                    train_ms=t.value, sweeps=sw.value, cov_ms=cov.value)
