"""C++ host layer (fastem_gb300/host): the reference's .bin / .cmp formats
read and written by the C++ classes, checked against the Python readers and
numpy; and em2gpu end to end on the GPU against the FP64 oracle."""
import os
import subprocess

import numpy as np
import pytest

from fastem_gb300 import GaussianMixture, formats, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def em2gpu():
    from fastem_gb300 import build
    build.build_gpu()
    build.build_host()
    assert os.path.exists(build.EM2GPU)
    return build.EM2GPU


def info(exe, fname):
    out = subprocess.run([exe, "--info", fname], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    return dict(kv.split("=") for kv in out.stdout.split()[1:])


def test_bin_read_by_cpp(em2gpu, tmp_path):
    X = np.random.default_rng(1).standard_normal((1001, 7)).astype(np.float32)
    f = str(tmp_path / "x.bin")
    formats.write_bin(f, X)
    assert np.array_equal(formats.read_bin(f), X)
    d = info(em2gpu, f)
    assert int(d["rows"]) == 1001 and int(d["cols"]) == 7
    assert float(d["sum"]) == pytest.approx(X.astype(np.float64).sum(), rel=1e-12, abs=1e-9)
    tr = np.trace(np.cov(X.astype(np.float64).T))
    assert float(d["trace"]) == pytest.approx(tr, rel=1e-9)


def test_bin_long_header(em2gpu, tmp_path):
    """rows = -1 marks a 64-bit row count after the column count."""
    X = np.arange(15, dtype=np.float32).reshape(5, 3)
    f = str(tmp_path / "long.bin")
    with open(f, "wb") as fh:
        np.array([-1, 3], dtype=np.int32).tofile(fh)
        np.array([5], dtype=np.int64).tofile(fh)
        X.tofile(fh)
    assert np.array_equal(formats.read_bin(f), X)
    d = info(em2gpu, f)
    assert int(d["rows"]) == 5 and float(d["sum"]) == 105.0


def test_truncated_bin_rejected(em2gpu, tmp_path):
    f = str(tmp_path / "bad.bin")
    with open(f, "wb") as fh:
        np.array([10, 4], dtype=np.int32).tofile(fh)
        np.zeros(7, dtype=np.float32).tofile(fh)
    out = subprocess.run([em2gpu, "--info", f], capture_output=True, text=True, timeout=60)
    assert out.returncode != 0 and "bytes" in out.stderr


def test_cmp_read_by_cpp(em2gpu, tmp_path):
    z = np.load(os.path.join(GOLDEN, "em_small.npz"))
    G = GaussianMixture(z["pi"], z["mu"], z["sigma"])
    f = str(tmp_path / "g.cmp")
    formats.write_cmp(f, G, loglike=-123.5)
    G2, ll = formats.read_cmp(f)
    assert ll == -123.5
    assert np.array_equal(G2.covs, G.covs) and np.array_equal(G2.means, G.means)
    d = info(em2gpu, f)
    assert int(d["components"]) == 3 and int(d["dims"]) == 4
    assert float(d["sum_weights"]) == pytest.approx(G.weights.sum(), rel=1e-15)
    assert float(d["sum_covs"]) == pytest.approx(G.covs.sum(), rel=1e-12)


def test_classes_file_both_headers(tmp_path):
    """Classes files as ReadAssignment reads them: an int32 count, or -1 and
    an int64 count, then 1-based int32 classes; a short file is refused."""
    cls = np.array([1, 3, 2, 2, 1], dtype=np.int32)
    short, long_, bad = (str(tmp_path / n) for n in ("s.cls", "l.cls", "b.cls"))
    with open(short, "wb") as f:
        np.array([5], dtype=np.int32).tofile(f)
        cls.tofile(f)
    with open(long_, "wb") as f:
        np.array([-1], dtype=np.int32).tofile(f)
        np.array([5], dtype=np.int64).tofile(f)
        cls.tofile(f)
    with open(bad, "wb") as f:
        np.array([7], dtype=np.int32).tofile(f)
        cls.tofile(f)
    np.testing.assert_array_equal(formats.read_classes(short), cls)
    np.testing.assert_array_equal(formats.read_classes(long_), cls)
    with pytest.raises(ValueError):
        formats.read_classes(bad)


@pytest.mark.parametrize("opt,val,msg", [("-c", "0", "invalid value of -c option"),
                                          ("-r", "-1", "invalid value of -r option"),
                                          ("-m", "-2", "invalid value of -m option"),
                                          ("-b", "-1", "invalid value of -b option"),
                                          ("-v", "-1", "invalid value of -v option"),
                                          ("-f", "0", "argument to -f must be greater or than 0"),
                                          ("-a", "0.5", "argument to -a must be greater then 1.0"),
                                          ("-g", "1.5", "argument to -g must be small positive number")])
def test_em2gpu_option_values_checked_as_em2(em2gpu, opt, val, msg):
    """ProcessArgs' value checks (EM2/EMArgs.cpp:75-170), refused before the
    dataset is read."""
    out = subprocess.run([em2gpu, opt, val, "missing.bin"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "Invalid program argument: " + msg in out.stdout


def test_em2gpu_refuses_mismatched_initial_mixture(em2gpu, tmp_path):
    """-I file.cmp with another component count than -c, or another
    dimension than the dataset's, stops before any GPU work."""
    z = np.load(os.path.join(GOLDEN, "em_small.npz"))
    fb, fi = str(tmp_path / "x.bin"), str(tmp_path / "g.cmp")
    formats.write_bin(fb, z["X"])
    formats.write_cmp(fi, GaussianMixture(z["pi0"], z["mu0"], z["sigma0"]))   # 3 components, d = 4
    for c in ("2", "5"):
        out = subprocess.run([em2gpu, fb, "-c", c, "-I", fi, "-m", "2"], capture_output=True, text=True, timeout=60)
        assert out.returncode == 1 and "initial mixture has 3 components of dimension 4" in out.stderr
    fw = str(tmp_path / "w.bin")
    formats.write_bin(fw, np.zeros((50, 6), dtype=np.float32))
    out = subprocess.run([em2gpu, fw, "-c", "3", "-I", fi, "-m", "2"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "on 6 columns" in out.stderr


def test_usage_without_arguments(em2gpu):
    out = subprocess.run([em2gpu], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "Arguments" in out.stdout


@pytest.mark.gpu
def test_em2gpu_fp64_matches_oracle(em2gpu, oracle, tmp_path):
    """em2gpu -p fp64 from a .cmp initial mixture: per-sweep logL and the
    written mixture equal the FP64 oracle's; classes are 1-based."""
    z = np.load(os.path.join(GOLDEN, "em_small.npz"))
    X = z["X"]
    fb, fi, fo, fc = (str(tmp_path / n) for n in ("x.bin", "init.cmp", "out.cmp", "cls.bin"))
    formats.write_bin(fb, X)
    formats.write_cmp(fi, GaussianMixture(z["pi0"], z["mu0"], z["sigma0"]))
    # -f must be > 0 (as em2 requires): 1e-300 keeps all 8 sweeps, as eps = 0 in the oracle
    out = subprocess.run([em2gpu, fb, "-c", "3", "-I", fi, "-p", "fp64", "-m", "8", "-f", "1e-300", "-v", "2",
                          "-o", fo, "-O", fc], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    ll = [float(l.split("LogL:")[1].split()[0]) for l in out.stdout.splitlines() if l.startswith("iter:")]
    ref = oracle.em_train(X, z["pi0"], z["mu0"], z["sigma0"], 8, eps=0.0)
    assert len(ll) == len(ref["logl"])
    np.testing.assert_allclose(ll, ref["logl"], rtol=1e-9)   # printed with 6 decimals
    G, _ = formats.read_cmp(fo)
    np.testing.assert_allclose(G.weights, ref["pi"], rtol=1e-10)
    np.testing.assert_allclose(G.means, ref["mu"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(G.covs, ref["sigma"], rtol=1e-9, atol=1e-12)
    cls = formats.read_classes(fc)
    assert cls.shape == (len(X),) and cls.min() >= 1 and cls.max() <= 3
    # verbosity > 3 prints the fitted mixture (GaussianMixture::Dump) as em2 does
    loud = subprocess.run([em2gpu, fb, "-c", "3", "-I", fi, "-p", "fp64", "-m", "2", "-v", "4"],
                          capture_output=True, text=True, timeout=300)
    assert loud.returncode == 0 and loud.stdout.count("Covariance matrix\n") == 3
    assert "Condition number of the solution:" in loud.stdout


@pytest.mark.gpu
def test_em2gpu_kmeans_init_mixed_and_unsupported_width(em2gpu, tmp_path):
    X, _ = synth.kmeans_blobs(seed=3, n=20000, d=8, k=6)
    fb = str(tmp_path / "b.bin")
    formats.write_bin(fb, X)
    out = subprocess.run([em2gpu, fb, "-c", "6", "-I", "kmeans", "-p", "fp64", "-m", "5", "-r", "7"],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    final = float(out.stdout.split("Final loglikelihood:")[1].split()[0])
    assert np.isfinite(final)
    # mixed precision runs d <= 64 (zero-padded) and 64 < d <= 256 (the wide kernels)
    ok = subprocess.run([em2gpu, fb, "-c", "6", "-p", "mixed", "-m", "3", "-I", "kmeans"], capture_output=True,
                        text=True, timeout=300)
    assert ok.returncode == 0, ok.stdout + ok.stderr
    fw = str(tmp_path / "wide.bin")
    formats.write_bin(fw, np.random.default_rng(1).standard_normal((5000, 80)).astype(np.float32))
    wide = subprocess.run([em2gpu, fw, "-c", "4", "-p", "mixed", "-m", "2"], capture_output=True, text=True,
                          timeout=300)
    assert wide.returncode == 0, wide.stdout + wide.stderr
    assert np.isfinite(float(wide.stdout.split("Final loglikelihood:")[1].split()[0]))
    # values outside the FP16 operand range are refused with a message
    fh = str(tmp_path / "huge.bin")
    formats.write_bin(fh, (np.random.default_rng(2).standard_normal((5000, 80)) * 1e5).astype(np.float32))
    bad = subprocess.run([em2gpu, fh, "-c", "4", "-p", "mixed", "-m", "2"], capture_output=True, text=True,
                         timeout=300)
    assert bad.returncode == 1 and "mixed precision" in bad.stderr
    # the k-means|| EM initializer (KMeansOrOrEMInitializer)
    oror = subprocess.run([em2gpu, fb, "-c", "6", "-I", "kmeansoror", "-p", "fp32", "-m", "5", "-r", "7"],
                          capture_output=True, text=True, timeout=300)
    assert oror.returncode == 0, oror.stdout + oror.stderr
    assert np.isfinite(float(oror.stdout.split("Final loglikelihood:")[1].split()[0]))


def seed(exe, how, fname, k, s):
    out = subprocess.run([exe, "--seed", how, fname, str(k), str(s)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return np.array([[float(v) for v in ln.split()] for ln in out.stdout.strip().splitlines()])


@pytest.mark.parametrize("how,n,d,k,s", [("pp", 5000, 8, 10, 2), ("oror", 20000, 16, 12, 3), ("oror", 3000, 5, 40, 7)])
def test_host_seeders_match_oracle(em2gpu, oracle, tmp_path, how, n, d, k, s):
    """k-means++ and k-means|| in the C++ host library (the -I kmeans /
    kmeansoror initialisers) pick the same rows as the oracle's restatement of
    PlusPlusInitializer / KMeansOrOrInitializer from the same generator seed."""
    X, _ = synth.kmeans_blobs(seed=30 + s, n=n, d=d, k=k, spread=5.0)
    f = str(tmp_path / "x.bin")
    formats.write_bin(f, X)
    got = seed(em2gpu, how, f, k, s)
    ref = oracle.kmeans_plusplus(X, k, seed=s) if how == "pp" else oracle.kmeans_oror(X, k, seed=s)
    assert got.shape == (k, d)
    np.testing.assert_array_equal(got, ref)


def test_em2gpu_accepts_reference_cpu_options(em2gpu):
    """em2's CPU tuning options parse as in the reference (-N as
    ParseEMBlockParams, -A as CreateEMAlgorithm's names); -B has no GPU
    counterpart."""
    def run(*a):
        return subprocess.run([em2gpu, *a], capture_output=True, text=True, timeout=60)
    bad_n = run("-N", "3:x", "missing.bin")
    assert bad_n.returncode == 1 and "Bad value of MStepLoopParam" in bad_n.stderr
    bad_a = run("-A", "nosuchem", "missing.bin")
    assert bad_a.returncode == 1 and "Invalid EM algorithm name" in bad_a.stderr
    assert run("-B").returncode == 0
    # well-formed options get as far as opening the (missing) data file
    ok = run("-N", "automax:32", "-A", "simplematrixem", "-R", "log2", "-M", "simple", "missing.bin")
    assert ok.returncode != 0 and "MStepLoopParam" not in ok.stderr and "algorithm" not in ok.stderr


@pytest.fixture(scope="module")
def eminit(em2gpu):
    from fastem_gb300 import build
    assert os.path.exists(build.EMINITGPU)
    return build.EMINITGPU


def jain_rows(n, k, seed, oracle):
    """JainEMInitializer::Init's draws (EM2/EMInitializer.cpp:43-77) from the
    oracle's Rand(): a component keeps its first draw; further draws repeat
    until one misses the rows already taken."""
    oracle.rng_seed(seed)
    taken = []
    for _ in range(k):
        idx = int(oracle.rng_uniform() * n)
        # once every row is taken no draw can miss: the reference loops
        # forever there, the host library stops redrawing
        while len(set(taken)) < n and int(oracle.rng_uniform() * n) in taken:
            pass
        taken.append(idx)
    return taken


def test_eminit_jain(eminit, oracle, tmp_path):
    """eminitgpu -I jain: the reference's rows (a repeated row included, as
    its repeat test reads a shadowing variable), tr(Cov) / d / 10 I, 1 / K."""
    X, _ = synth.kmeans_blobs(seed=5, n=60, d=3, k=4)
    fb, fo = str(tmp_path / "j.bin"), str(tmp_path / "j.cmp")
    formats.write_bin(fb, X)
    out = subprocess.run([eminit, "-I", "jain", "-c", "7", "-r", "11", "-o", fo, fb], capture_output=True,
                         text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    G, _ = formats.read_cmp(fo)
    rows = jain_rows(len(X), 7, 11, oracle)
    assert len(set(rows)) < len(rows)          # this seed repeats a row
    np.testing.assert_array_equal(G.means, X[rows].astype(np.float64))
    cv = np.trace(np.cov(X.astype(np.float64).T)) / 3 / 10
    np.testing.assert_allclose(G.covs, np.broadcast_to(np.eye(3) * cv, (7, 3, 3)), rtol=1e-12)
    np.testing.assert_array_equal(G.weights, np.full(7, 1.0 / 7))


def test_eminit_jain_more_components_than_rows(eminit, oracle, tmp_path):
    """K > N: the reference's repeat loop never ends once every row is
    taken; here the draws stop there and the run completes."""
    X = np.arange(15, dtype=np.float32).reshape(5, 3)
    fb, fo = str(tmp_path / "s.bin"), str(tmp_path / "s.cmp")
    formats.write_bin(fb, X)
    out = subprocess.run([eminit, "-I", "jain", "-c", "8", "-r", "4", "-o", fo, fb], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    G, _ = formats.read_cmp(fo)
    np.testing.assert_array_equal(G.means, X[jain_rows(5, 8, 4, oracle)].astype(np.float64))


def test_eminit_file_dump_and_arguments(eminit, tmp_path):
    """-I file.cmp without -o prints the mixture as GaussianMixture::Dump,
    ending with the largest condition number; bad options are refused as
    eminit's ProcessArgs refuses them."""
    z = np.load(os.path.join(GOLDEN, "em_small.npz"))
    fb, fi = str(tmp_path / "x.bin"), str(tmp_path / "g.cmp")
    formats.write_bin(fb, z["X"])
    formats.write_cmp(fi, GaussianMixture(z["pi"], z["mu"], z["sigma"]))
    out = subprocess.run([eminit, "-I", fi, "-c", "3", fb], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "File EM initializer" in out.stdout and out.stdout.count("Covariance matrix\n") == 3
    cond = float(out.stdout.split("Condition number of the solution:")[1].split()[0])
    ev = [np.linalg.eigvalsh(s) for s in z["sigma"]]
    assert cond == pytest.approx(max(abs(e[-1] / e[0]) for e in ev), rel=1e-5)   # printed with %g
    for args, msg in [(["-c", "0", fb], "invalid value of -c option"), (["-r", "-2", fb], "invalid value of -r option"),
                      (["-c", "2"], "Missing dataset name")]:
        bad = subprocess.run([eminit] + args, capture_output=True, text=True, timeout=60)
        assert bad.returncode == 1 and "Invalid program argument: " + msg in bad.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,k,data_seed", [(5000, 8, 6, 3), (200, 4, 12, 4)])
def test_eminit_kmeans_matches_oracle(eminit, oracle, tmp_path, n, d, k, data_seed):
    """eminitgpu -I kmeans = KMeansEMInitializer::Init (EM2/EMInitializer.cpp:
    103-134): Forgy rows, RunKMeans(0, 1e-4, 30) with empty clusters repaired
    from the same Rand() stream, the classes of the final centroids, class
    covariances / (count - 1), weights count / N.  The second shape takes a
    seed whose Forgy rows repeat, so a repair draws from the stream."""
    X, _ = synth.kmeans_blobs(seed=data_seed, n=n, d=d, k=max(2, k // 2), spread=6.0)
    seed = 0
    while True:
        oracle.rng_seed(seed)
        rows = [int(oracle.rng_uniform() * n) for _ in range(k)]
        if (len(set(rows)) < k) == (n < 1000):
            break
        seed += 1
    fb, fo = str(tmp_path / "x.bin"), str(tmp_path / "g.cmp")
    formats.write_bin(fb, X)
    out = subprocess.run([eminit, "-I", "kmeans", "-c", str(k), "-r", str(seed), "-p", "fp32", "-o", fo, fb],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    G, _ = formats.read_cmp(fo)
    C = oracle.kmeans_forgy(X, k, seed=seed)
    _, C, _ = oracle.km_run(X, C, min_rel=1e-4, max_iter=30)
    _, _, counts, labels = oracle.km_iterate(X, C, repair=False)
    np.testing.assert_allclose(G.means, C, rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(G.weights, counts / n)
    X64 = X.astype(np.float64)
    for j in range(k):
        R = X64[labels == j] - C[j]
        np.testing.assert_allclose(G.covs[j], R.T @ R / (counts[j] - 1.0), rtol=1e-9, atol=1e-12)
