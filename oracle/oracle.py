"""ctypes wrapper of the FP64 CPU oracle (oracle/fem_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs, never by the fastem_gb300 package.

PARITY UNPINNED for the EM and k-means arithmetic: the reference
(wkwedlo/fastem) cannot be built here (Eigen, MKL, libnuma and MPI are
absent) and ships no golden vectors; the oracle is cross-checked against an
independent numpy FP64 computation instead (tests/test_oracle.py).  The
generator stream is pinned against the reference's own Util/Rand.cpp,
compiled in place (`make -C oracle ref`) where its sources are present.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

ORC_OK = 0
ORC_ERR_CHOLESKY = 3
ORC_ERR_COND_ABORT = 4


def build():
    """Compile liboracle.so in place (make; a few seconds).  A library left
    over from another CPU architecture is rebuilt."""
    import platform
    so = os.path.join(_HERE, "liboracle.so")
    want = {"x86_64": 62, "aarch64": 183}.get(platform.machine())
    if os.path.exists(so) and want is not None:
        with open(so, "rb") as f:
            head = f.read(20)
        if head[:4] == b"\x7fELF" and int.from_bytes(head[18:20], "little") != want:
            os.remove(so)
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    # the reference's own generator and k-means, where its sources are present
    # (optional: the tests that use them skip without them)
    ref = os.environ.get("FEM_REFERENCE_DIR") or ("/root/reference" if os.path.isdir("/root/reference") else "")
    if ref:
        subprocess.run(["make", "-s", "-C", _HERE, "ref", "REF=" + ref], check=False, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        build()                       # make: a no-op when the library is up to date
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i32, i64, f64 = ctypes.c_int, ctypes.c_int64, ctypes.c_double
        L.orc_rng_seed.argtypes = [ctypes.c_uint64]
        L.orc_rng_uniform.restype = f64
        L.orc_em_init_densities.argtypes = [i32, i32, P, P, P, P]
        L.orc_em_regularize.argtypes = [i32, i32, f64, P]
        L.orc_cond_number.argtypes = [i32, P]
        L.orc_cond_number.restype = f64
        L.orc_em_estep.argtypes = [i32, i64, i32, P, P, P, P, P, P, P, i32]
        L.orc_em_mstep.argtypes = [i32, i64, i32, P, P, P, P, P, i32]
        L.orc_em_mstep_cached.argtypes = [i32, i64, i32, P, P, P, P, P, i32]
        L.orc_em_train.argtypes = [i32, i64, i32, P, P, P, P, i32, f64, f64, f64,
                                   i32, P, P, P, P, i32]
        L.orc_em_train_order.argtypes = [i32, i64, i32, P, P, P, P, i32, f64, f64, f64,
                                         i32, P, P, P, P, i32, i32]
        L.orc_km_iterate.argtypes = [i32, i64, i32, P, P, P, P, i32, i32]
        L.orc_km_iterate.restype = f64
        L.orc_km_run.argtypes = [i32, i64, i32, P, P, f64, i32, P, i32]
        L.orc_km_run.restype = f64
        L.orc_km_plusplus.argtypes = [i32, i64, i32, P, P, P]
        L.orc_km_oror.argtypes = [i32, i64, i32, P, f64, P, i32]
        L.orc_km_forgy.argtypes = [i32, i64, i32, P, P]
        L.orc_em_sweep_blas.argtypes = [i32, i64, i32, P, P, P, P, P, i32, P, P, P]
        L.orc_em_sweeps_blas.argtypes = [i32, i64, i32, P, P, P, P, i32, i32, f64, P, P, i32, P, P, P]
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(X):
    X = np.ascontiguousarray(X, dtype=np.float32)
    assert X.ndim == 2
    return X


def rng_seed(seed):
    lib().orc_rng_seed(int(seed))


def rng_uniform():
    return lib().orc_rng_uniform()


def init_densities(sigma):
    sigma = np.ascontiguousarray(sigma, dtype=np.float64)
    k, d, _ = sigma.shape
    U = np.zeros_like(sigma)
    logdet = np.zeros(k)
    failed = ctypes.c_int(-1)
    st = lib().orc_em_init_densities(d, k, _p(sigma), _p(U), _p(logdet), ctypes.byref(failed))
    return st, U, logdet, failed.value


def regularize(sigma, reg):
    sigma = np.array(sigma, dtype=np.float64, copy=True, order="C")
    k, d, _ = sigma.shape
    lib().orc_em_regularize(d, k, float(reg), _p(sigma))
    return sigma


def cond_number(sigma_j):
    s = np.ascontiguousarray(sigma_j, dtype=np.float64)
    return lib().orc_cond_number(s.shape[0], _p(s))


def estep(X, pi, mu, U, logdet, nthreads=0):
    X = _f32(X)
    n, d = X.shape
    k = len(pi)
    pi, mu, U, logdet = (np.ascontiguousarray(a, dtype=np.float64) for a in (pi, mu, U, logdet))
    post = np.zeros((n, k))
    logl = ctypes.c_double(0)
    lib().orc_em_estep(d, n, k, _p(X), _p(pi), _p(mu), _p(U), _p(logdet), _p(post),
                       ctypes.byref(logl), nthreads)
    return post, logl.value


def mstep(X, post, nthreads=0):
    X = _f32(X)
    n, d = X.shape
    post = np.ascontiguousarray(post, dtype=np.float64)
    k = post.shape[1]
    pi, mu, sigma = np.zeros(k), np.zeros((k, d)), np.zeros((k, d, d))
    lib().orc_em_mstep(d, n, k, _p(X), _p(post), _p(pi), _p(mu), _p(sigma), nthreads)
    return pi, mu, sigma


def mstep_cached(X, post, nthreads=0):
    """CachedEM::MStep order (orc_em_mstep_cached)."""
    X = _f32(X)
    n, d = X.shape
    post = np.ascontiguousarray(post, dtype=np.float64)
    k = post.shape[1]
    pi, mu, sigma = np.zeros(k), np.zeros((k, d)), np.zeros((k, d, d))
    lib().orc_em_mstep_cached(d, n, k, _p(X), _p(post), _p(pi), _p(mu), _p(sigma), nthreads)
    return pi, mu, sigma


def em_train(X, pi, mu, sigma, max_sweeps, eps=1e-5, abort_thr=1e5, reg_coef=0.0,
             svd=False, nthreads=0, cached=False):
    """EMAlgorithm::TrainNoCopy over SimpleMatrixEM (cached=True: CachedEM's
    M-step order).  Returns a dict with the final mixture, the per-sweep LogL /
    e traces, IterCounter and status."""
    X = _f32(X)
    n, d = X.shape
    pi = np.array(pi, dtype=np.float64, copy=True)
    mu = np.array(mu, dtype=np.float64, copy=True, order="C")
    sigma = np.array(sigma, dtype=np.float64, copy=True, order="C")
    k = len(pi)
    ll = np.full(max_sweeps, np.nan)
    ee = np.full(max_sweeps, np.nan)
    it = ctypes.c_int(0)
    fl = ctypes.c_double(np.nan)
    st = lib().orc_em_train_order(d, n, k, _p(X), _p(pi), _p(mu), _p(sigma), int(max_sweeps),
                                  float(eps), float(abort_thr), float(reg_coef), int(bool(svd)),
                                  _p(ll), _p(ee), ctypes.byref(it), ctypes.byref(fl), nthreads,
                                  int(bool(cached)))
    sweeps = max(0, min(it.value - 1, max_sweeps))
    return dict(status=st, pi=pi, mu=mu, sigma=sigma, logl=ll[:sweeps], e=ee[:sweeps],
                iter_counter=it.value, final_logl=fl.value)


def km_iterate(X, centroids, repair=True, nthreads=0):
    """One NaiveKMA::ComputeMSEAndCorrect.  Returns (fit, new_centroids,
    counts, labels)."""
    X = _f32(X)
    n, d = X.shape
    c = np.array(centroids, dtype=np.float64, copy=True, order="C")
    k = c.shape[0]
    counts = np.zeros(k, dtype=np.int64)
    labels = np.zeros(n, dtype=np.int32)
    fit = lib().orc_km_iterate(d, n, k, _p(X), _p(c), _p(counts), _p(labels), int(bool(repair)),
                               nthreads)
    return fit, c, counts, labels


def km_run(X, centroids, min_rel=-1.0, max_iter=0, nthreads=0):
    X = _f32(X)
    n, d = X.shape
    c = np.array(centroids, dtype=np.float64, copy=True, order="C")
    it = ctypes.c_int(0)
    best = lib().orc_km_run(d, n, c.shape[0], _p(X), _p(c), float(min_rel), int(max_iter),
                            ctypes.byref(it), nthreads)
    return best, c, it.value


def kmeans_plusplus(X, k, seed=None, weights=None):
    X = _f32(X)
    n, d = X.shape
    if seed is not None:
        rng_seed(seed)
    out = np.zeros((k, d))
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    lib().orc_km_plusplus(d, n, k, _p(X), _p(w), _p(out))
    return out


def kmeans_oror(X, k, seed=None, oversample=1.4, nthreads=0):
    X = _f32(X)
    n, d = X.shape
    if seed is not None:
        rng_seed(seed)
    out = np.zeros((k, d))
    lib().orc_km_oror(d, n, k, _p(X), float(oversample), _p(out), nthreads)
    return out


def kmeans_forgy(X, k, seed=None):
    X = _f32(X)
    n, d = X.shape
    if seed is not None:
        rng_seed(seed)
    out = np.zeros((k, d))
    lib().orc_km_forgy(d, n, k, _p(X), _p(out))
    return out


_BLAS = None


def openblas():
    """scipy's bundled OpenBLAS (CBLAS entry points named scipy_cblas_*), set
    to one thread (the oracle's OpenMP threads each call it); None if absent."""
    global _BLAS
    if _BLAS is None:
        import glob
        try:
            import scipy
        except ImportError:
            return None
        libs = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs",
                                             "libscipy_openblas*.so*")))
        for path in libs:
            try:
                B = ctypes.CDLL(path)
                fns = [ctypes.cast(getattr(B, "scipy_cblas_" + f), ctypes.c_void_p).value
                       for f in ("dtrmm", "dgemm", "dsyrk")]
            except (OSError, AttributeError):
                continue
            if hasattr(B, "scipy_openblas_set_num_threads"):
                B.scipy_openblas_set_num_threads(1)
            _BLAS = (B, fns)
            break
    return _BLAS


def em_sweep_blas(X, pi, mu, sigma, nthreads=0):
    """One FP64 sweep organised like SimpleMatrixEM with OpenBLAS level-3
    calls (orc_em_sweep_blas).  Returns (logL, pi, mu, sigma)."""
    blas = openblas()
    if blas is None:
        raise RuntimeError("scipy's bundled OpenBLAS was not found")
    X = _f32(X)
    n, d = X.shape
    pi = np.array(pi, dtype=np.float64, copy=True)
    mu = np.array(mu, dtype=np.float64, copy=True, order="C")
    sigma = np.array(sigma, dtype=np.float64, copy=True, order="C")
    ll = ctypes.c_double(np.nan)
    st = lib().orc_em_sweep_blas(d, n, len(pi), _p(X), _p(pi), _p(mu), _p(sigma), ctypes.byref(ll),
                                 int(nthreads), *[ctypes.c_void_p(f) for f in blas[1]])
    if st != ORC_OK:
        raise RuntimeError("orc_em_sweep_blas failed with status %d" % st)
    return ll.value, pi, mu, sigma


def em_sweeps_blas(X, pi, mu, sigma, sweeps, nthreads=0, svd=False, abort_thr=1e5):
    """`sweeps` FP64 sweeps in one call, organised like SimpleMatrixEM with
    OpenBLAS level-3 calls, buffers sized once as TrainNoCopy has them, with
    the condition-number check after each sweep when `svd`
    (orc_em_sweeps_blas).  Returns (logL per sweep, seconds per sweep, pi, mu,
    sigma)."""
    blas = openblas()
    if blas is None:
        raise RuntimeError("scipy's bundled OpenBLAS was not found")
    X = _f32(X)
    n, d = X.shape
    pi = np.array(pi, dtype=np.float64, copy=True)
    mu = np.array(mu, dtype=np.float64, copy=True, order="C")
    sigma = np.array(sigma, dtype=np.float64, copy=True, order="C")
    ll = np.full(sweeps, np.nan)
    sec = np.full(sweeps, np.nan)
    st = lib().orc_em_sweeps_blas(d, n, len(pi), _p(X), _p(pi), _p(mu), _p(sigma), int(sweeps), int(bool(svd)),
                                  float(abort_thr), _p(ll), _p(sec), int(nthreads),
                                  *[ctypes.c_void_p(f) for f in blas[1]])
    if st != ORC_OK:
        raise RuntimeError("orc_em_sweeps_blas failed with status %d" % st)
    return ll, sec, pi, mu, sigma


REF_KMEANS = os.path.join(_HERE, "_ref", "ref_kmeans")


def ref_kmeans(X, centroids, iterations, seed, nthreads=1):
    """Run the reference's own NaiveKMA (oracle/_ref/ref_kmeans, built from the
    reference's sources by `make -C oracle ref`) for `iterations`
    ComputeMSEAndCorrect calls from `centroids`, its generator seeded with
    `seed` (SRand, used by CentroidRandomRepair).  Returns (fits, labels per
    iteration, centroids after each iteration); None when the binary was not
    built."""
    import tempfile
    if not os.path.exists(REF_KMEANS):
        return None
    from fastem_gb300 import formats
    X = _f32(X)
    C = np.ascontiguousarray(centroids, dtype=np.float64)
    with tempfile.TemporaryDirectory() as d:
        formats.write_bin(os.path.join(d, "x.bin"), X)
        C.tofile(os.path.join(d, "c.f64"))
        env = dict(os.environ, OMP_NUM_THREADS=str(int(nthreads)))
        subprocess.run([REF_KMEANS, os.path.join(d, "x.bin"), os.path.join(d, "c.f64"), str(int(iterations)),
                        str(int(seed)), os.path.join(d, "o.bin")], check=True, env=env,
                       stdout=subprocess.DEVNULL)
        b = open(os.path.join(d, "o.bin"), "rb").read()
    it, n, k, dd = (int(v) for v in np.frombuffer(b[:16], dtype=np.int32))
    fits, labels, cents = [], [], []
    off = 16
    for _ in range(it):
        fits.append(float(np.frombuffer(b[off:off + 8], dtype=np.float64)[0]))
        off += 8
        labels.append(np.frombuffer(b[off:off + 4 * n], dtype=np.int32).copy())
        off += 4 * n
        cents.append(np.frombuffer(b[off:off + 8 * k * dd], dtype=np.float64).reshape(k, dd).copy())
        off += 8 * k * dd
    return np.array(fits), np.array(labels), np.array(cents)
