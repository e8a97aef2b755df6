"""Batched EM: many independent fits trained together on one GPU
(fem_em_batch_* in include/fastem_gpu.h).

There is no single reference counterpart -- the reference trains one mixture
per em2 run -- so each fit here behaves as CudaMatrixEM.Train would for that
fit alone (precision "fp32"; "mixed" runs the E-step of the fits with
16 < d <= 32 on the tensor cores): EMAlgorithm::TrainNoCopy
(EM2/EMAlgorithm.cpp:139-191) with its own convergence test, IterCounter and
Cholesky / condition-number failure.  The difference is the schedule: every
kernel of a sweep covers all fits still sweeping.
"""
import ctypes
import json
import os

import numpy as np

from . import _capi as C
from .em import GaussianMixture

# work-item sizes measured by fastem_gb300/autotune.py on a GB300
TUNING_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "batch_gb300.json")
CLASS_DIMS = (4, 8, 16, 32)


def load_tuning(path=TUNING_TABLE):
    """{"means_chunk": [4], "cov_chunk": [4]} from an autotuner table, or None
    when there is no table."""
    try:
        with open(path) as f:
            t = json.load(f)
    except OSError:
        return None
    return {"means_chunk": [int(v) for v in t["means_chunk"]], "cov_chunk": [int(v) for v in t["cov_chunk"]]}


def tuning_struct(tuning):
    t = C.BatchTuning()
    C.lib().fem_em_batch_tuning_default(ctypes.byref(t))
    if tuning:
        for c in range(4):
            t.means_chunk[c] = int(tuning["means_chunk"][c])
            t.cov_chunk[c] = int(tuning["cov_chunk"][c])
    return t


class CudaBatchEM:
    """shapes: sequence of (d, n, k) per fit (d <= 32, k <= 64).  tuning: "table"
    (the autotuner's table when present, else the library defaults), None (the
    library defaults) or {"means_chunk": [4], "cov_chunk": [4]}.  precision:
    "fp32" (CUDA cores) or "mixed" (the E-step of the fits with 16 < d <= 32 on
    the tensor cores in FP16 x 3 split products, everything else as "fp32")."""

    def __init__(self, shapes, device=0, max_sweeps=1000000, tuning="table", precision="fp32"):
        shapes = [(int(d), int(n), int(k)) for d, n, k in shapes]
        self.shapes = shapes
        self.nfits = len(shapes)
        d = np.array([s[0] for s in shapes], dtype=np.int32)
        n = np.array([s[1] for s in shapes], dtype=np.int64)
        k = np.array([s[2] for s in shapes], dtype=np.int32)
        cfg = C.EmConfig()
        C.lib().fem_em_config_default(ctypes.byref(cfg))
        cfg.precision = C.PREC[precision]
        cfg.device = device
        cfg.max_sweeps = int(max_sweeps)
        if isinstance(tuning, str):
            tuning = load_tuning() if tuning == "table" else load_tuning(tuning)
        t = tuning_struct(tuning)
        h = ctypes.c_void_p()
        C.check(C.lib().fem_em_batch_create_tuned(self.nfits, C.ptr(d), C.ptr(n), C.ptr(k), ctypes.byref(cfg),
                                                  ctypes.byref(t), ctypes.byref(h)))
        self._h = h
        self.status = np.zeros(self.nfits, dtype=np.int32)
        self.iters = np.zeros(self.nfits, dtype=np.int32)
        self.logl = np.full(self.nfits, np.nan)

    def Tuning(self):
        """the work-item sizes this batch was created with"""
        t = C.BatchTuning()
        C.check(C.lib().fem_em_batch_get_tuning(self._h, ctypes.byref(t)))
        return {"means_chunk": list(t.means_chunk), "cov_chunk": list(t.cov_chunk)}

    def close(self):
        if getattr(self, "_h", None):
            C.lib().fem_em_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # EMAlgorithm::SetParameters, for every fit
    def SetParameters(self, max_sweeps, eps, abort_thr, reg_coef=0.0):
        C.check(C.lib().fem_em_batch_set_parameters(self._h, int(max_sweeps), float(eps), float(abort_thr),
                                                    float(reg_coef)))

    def CopyDataset(self, i, X):
        X = C.f32rows(X)
        d, n, _ = self.shapes[i]
        assert X.shape == (n, d)
        C.check(C.lib().fem_em_batch_upload(self._h, int(i), C.ptr(X), X.shape[1]))

    def CopyDatasets(self, Xs):
        """every fit's rows in one call (packed on the host first)"""
        assert len(Xs) == self.nfits
        packed = np.concatenate([C.f32rows(X).reshape(-1) for X in Xs])
        C.check(C.lib().fem_em_batch_upload_packed(self._h, C.ptr(packed)))

    def CopyPacked(self, packed):
        """rows already packed one fit after another (float32, contiguous)"""
        packed = np.ascontiguousarray(packed, dtype=np.float32)
        C.check(C.lib().fem_em_batch_upload_packed(self._h, C.ptr(packed)))

    def SetMixture(self, i, G):
        C.check(C.lib().fem_em_batch_set_params(self._h, int(i), C.ptr(C.f64(G.weights)), C.ptr(C.f64(G.means)),
                                                C.ptr(C.f64(G.covs))))

    def GetMixture(self, i):
        d, _, k = self.shapes[i]
        pi, mu, sg = np.zeros(k), np.zeros((k, d)), np.zeros((k, d, d))
        C.check(C.lib().fem_em_batch_get_params(self._h, int(i), C.ptr(pi), C.ptr(mu), C.ptr(sg)))
        return GaussianMixture(pi, mu, sg)

    def TrainNoCopy(self, svd=False):
        """Trains every fit; returns the per-fit status (FEM_OK, FEM_ERR_CHOLESKY
        or FEM_ERR_COND_ABORT), IterCounter and LogL arrays."""
        st = C.lib().fem_em_batch_train(self._h, int(bool(svd)), C.ptr(self.status), C.ptr(self.iters),
                                        C.ptr(self.logl))
        C.check(st)
        return self.status.copy(), self.iters.copy(), self.logl.copy()

    def Train(self, Xs, mixtures, svd=False):
        self.CopyDatasets(Xs)
        for i, G in enumerate(mixtures):
            self.SetMixture(i, G)
        return self.TrainNoCopy(svd)

    def Trace(self, i):
        """(logl_trace, e_trace) of fit i's sweeps in the last train"""
        m = max(0, int(self.iters[i]) - 1)
        ll, ee = np.zeros(max(m, 1)), np.zeros(max(m, 1))
        C.check(C.lib().fem_em_batch_trace(self._h, int(i), C.ptr(ll), C.ptr(ee), m))
        return ll[:m], ee[:m]

    def FailedComponent(self, i):
        c = ctypes.c_int(-1)
        C.check(C.lib().fem_em_batch_fail_component(self._h, int(i), ctypes.byref(c)))
        return c.value

    def EnableTiming(self, on=True):
        C.check(C.lib().fem_em_batch_timing_enable(self._h, int(bool(on))))

    def Timing(self):
        ms = np.zeros(5)
        launches, sweeps = ctypes.c_int64(0), ctypes.c_int64(0)
        C.check(C.lib().fem_em_batch_timing(self._h, C.ptr(ms), ctypes.byref(launches), ctypes.byref(sweeps)))
        cls = np.zeros(12)
        C.check(C.lib().fem_em_batch_timing_classes(self._h, C.ptr(cls)))
        per = {D: dict(estep_ms=cls[c], means_ms=cls[4 + c], cov_ms=cls[8 + c]) for c, D in enumerate((4, 8, 16, 32))}
        return dict(estep_ms=ms[0], means_ms=ms[1], cov_ms=ms[2], factor_ms=ms[3], loop_ms=ms[4],
                    launches=launches.value, sweeps=sweeps.value, classes=per)
