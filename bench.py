#!/usr/bin/env python3
"""EM iterations/s on one GB300: N = 2^23 points, d = 64, K = 128
(synthetic em_large workload, seeded), mixed precision (tcgen05 FP16
contractions, FP32 accumulation, FP64 factorisation / logdet / logL) against
the plain FP32 CUDA-core sweep, with the reference's CPU algorithm (the FP64
oracle port, OpenMP) timed on the host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --workload kmeans [...]

One step = one EM sweep (E-step + M-step + regularise/factorise) over all N
points, the body of EMAlgorithm::TrainNoCopy.  Prints one JSON line (rank 0).
`--workload kmeans` measures one Lloyd iteration (NaiveKMA::
ComputeMSEAndCorrect) at N = 2^24, d = 32, K = 256 instead (not the headline
metric; its roofline is HBM bandwidth).
Multi-GPU runs are independent replicas (the reference's data-parallel MPI
path is not part of this backend): value = all sweeps of all ranks / max time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EM iter/s N=8M d=64 K=128: mixed-prec vs FP32 GPU at |ΔlogL/N|≤1e-5"
UNIT = "iter/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
PROFILE_FILE = os.path.join(ROOT, "profiles", "em_sweep_n8m_d64_k128.md")
FALLBACK_TFLOPS = 1900.0  # GB300 bf16 dense burst, used only without measured peaks
PRECISION_NOTE = ("fp16x3 E-step / fp16 M-step (exact diagonal) tensor cores, fp32 accumulate, "
                  "fp64 factorisation, logdet and logL")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="em", choices=["em", "kmeans", "batched", "small", "illcond"])
    ap.add_argument("--n", type=int, default=None, help="points (default 2^23 EM, 2^24 k-means)")
    ap.add_argument("--k", type=int, default=128)
    ap.add_argument("--fits-d", type=int, default=None, choices=[4, 8, 16, 32],
                    help="batched workload: only the fits of this dimension (a smaller case for profiling)")
    ap.add_argument("--no-fp32", action="store_true", help="skip the FP32 CUDA-core comparison")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--acc-sweeps", type=int, default=20,
                    help="EM workload: sweeps of the accuracy check against the FP64 GPU path (0 = skip)")
    ap.add_argument("--no-svd", action="store_true",
                    help="EM workload: leave out the per-sweep condition-number check (the reference's -S)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barriers and max-over-ranks on the host (gloo); no data-path collective."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def measured_peak_tflops():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured (MEASURED_PEAKS bf16_tflops, burst)"
    except Exception:
        return FALLBACK_TFLOPS, "fallback 1.9 PFLOP/s"


def profiled_traffic(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summary."""
    try:
        for line in open(PROFILE_FILE):
            if line.startswith("traffic_bytes_per_launch") and kernel in line:
                return float(line.split("=")[-1])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.device)],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def workload(n, k):
    from fastem_gb300 import synth
    X, _ = synth.em_large(seed=3, n=n, d=64, k=k)
    init = synth.dsquared_init(X, k, seed=5)
    return X, init


def em_flops(n, d, k):
    """Algorithmic flop counts per sweep: TRMM and SYRK N K d(d+1) each
    (triangular, non-redundant), means GEMM 2 N K d."""
    tri = n * k * d * (d + 1)
    return dict(estep=tri, cov=tri, mstep=tri + 2 * n * k * d, total=2 * tri + 2 * n * k * d)


def time_device_sweeps(em, G, warmup, steps, dist, reg=0.0, svd=False):
    """Warm-up sweeps, then `steps` sweeps timed by CUDA events on the
    library's stream (max over ranks).  With `svd` every sweep ends with the
    condition-number check (the reference's default, EM2/EMArgs.cpp:40)."""
    import torch
    em.SetParameters(warmup, 0.0, 1e5, reg)
    em.TrainNoCopy(G, svd=svd)
    dist.barrier()
    torch.cuda.synchronize()
    em.TimingReset(True)
    em.SetParameters(steps, 0.0, 1e5, reg)
    em.TrainNoCopy(G, svd=svd)
    torch.cuda.synchronize()
    dist.barrier()
    t = em.Timing()
    em.TimingReset(False)
    return t


def cpu_sweep_seconds(X, init, sample, threads):
    """One FP64 sweep of the oracle on the first `sample` rows, organised like
    the reference's SimpleMatrixEM: OpenMP over row blocks, level-3 BLAS
    (scipy's OpenBLAS) inside each thread for the TRMM / GEMM / SYRK steps;
    the scalar oracle sweep when no OpenBLAS is found.  Returns (seconds, how)."""
    from oracle import oracle as O
    O.lib()
    Xs = np.ascontiguousarray(X[:sample])
    if O.openblas() is not None:
        t0 = time.perf_counter()
        O.em_sweep_blas(Xs, *init, nthreads=threads)
        return time.perf_counter() - t0, "FP64, OpenMP + OpenBLAS dtrmm/dgemm/dsyrk"
    t0 = time.perf_counter()
    O.em_train(Xs, *init, 1, eps=0.0, nthreads=threads)
    return time.perf_counter() - t0, "FP64, OpenMP scalar loops"


def cpu_full_sweeps(X, init, burn_in, timed, threads, svd):
    """`burn_in` + `timed` FP64 sweeps of the oracle over ALL rows in one call
    (buffers sized once, as EMAlgorithm::TrainNoCopy runs its sweeps),
    organised like the reference's SimpleMatrixEM: OpenMP over row blocks,
    single-threaded OpenBLAS dtrmm / dgemm / dsyrk inside each thread where the
    reference calls MKL; with `svd` the condition-number check after each
    sweep.  Returns (seconds of each timed sweep, logL trace, how)."""
    from oracle import oracle as O
    O.lib()
    if O.openblas() is None:
        raise RuntimeError("scipy's bundled OpenBLAS was not found: no CPU baseline")
    O.em_sweeps_blas(X[:4096], *init, 1, nthreads=threads)    # load the libraries, start the thread pool
    ll, sec, *_ = O.em_sweeps_blas(X, *init, burn_in + timed, nthreads=threads, svd=svd)
    how = "FP64, OpenMP + OpenBLAS dtrmm/dgemm/dsyrk" + (", condition check each sweep" if svd else "")
    return sec[burn_in:], ll, how


def em_config(n, d, k, world, svd):
    return {"workload": "em_large N=%d d=%d K=%d, one EM sweep per step" % (n, d, k),
            "n": n, "d": d, "k": k, "parallelism": "replicas" if world > 1 else "single",
            "svd": "off (-S)" if not svd else "on (the reference default: condition number of every "
                                               "covariance after each sweep, abort above 1e5)",
            "l2": "inputs larger than L2 (X 2.1 GB fp32 + 2.1 GB fp16 splits, posteriors 4.3 GB)"}


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU algorithm (the oracle's FP64
    restatement of SimpleMatrixEM, OpenMP with OpenBLAS level-3 calls where
    the reference calls MKL, all host cores) sweeping ALL N rows: `warmup`
    untimed sweeps, then `steps` timed sweeps, in one TrainNoCopy-like call.
    The reference itself cannot be compiled here (Eigen 3.4, MKL, libnuma and
    MPI are absent).  With svd on (the reference's default) every sweep ends
    with the condition check, as the GPU arm's sweeps do."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    n, d, k = args.n, 64, args.k
    X, init = workload(n, k)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    sec, ll, how = cpu_full_sweeps(X, init, args.warmup, args.steps, threads, not args.no_svd)
    wall = time.perf_counter() - t0
    per_sweep = float(np.mean(sec))
    value = 1.0 / per_sweep
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_sweep * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic em_large (seeded; Dirichlet(2) weights, N(0,25I) means, Haar-rotated "
                "covariances with eigenvalues log-uniform in [0.1,10])",
        "config": em_config(n, d, k, world, not args.no_svd),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "how": "%s, %d warm-up + %d timed sweeps over all %d rows" % (how, args.warmup,
                                                                                     args.steps, n),
                         "sweep_seconds": [round(float(x), 3) for x in sec], "wall_s": wall},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def accuracy_vs_fp64(X, init, sweeps, local):
    """The metric's |dlogL/N| <= 1e-5 clause, measured: `sweeps` sweeps from
    the same initial mixture through the FP64 GPU path (the parity path,
    equal to the oracle within 1e-10 over 50 sweeps in the tests), the mixed
    path and the FP32 path.  Per sweep |L - L_fp64| / N (the pre-M-step logL
    each sweep returns, EM2/EMAlgorithm.cpp:170-178), and the final mixture's
    largest differences from the FP64 one."""
    from fastem_gb300 import CudaMatrixEM, GaussianMixture
    n, d = X.shape
    k = len(init[0])
    tr, mix, secs = {}, {}, {}
    for prec in ("fp64", "mixed", "fp32"):
        with CudaMatrixEM(d, n, k, precision=prec, device=local) as em:
            em.CopyDataset(X)
            em.SetParameters(sweeps, 0.0, 1e12)
            G = GaussianMixture(*init)
            t0 = time.perf_counter()
            em.TrainNoCopy(G)
            secs[prec] = time.perf_counter() - t0
            tr[prec], mix[prec] = em.logl_trace.copy(), G
    out = {"vs": "fp64 GPU path (oracle-pinned)", "sweeps": sweeps, "n": n, "bound": 1e-5,
           "fp64_seconds": secs["fp64"]}
    ref = tr["fp64"]
    for prec in ("mixed", "fp32"):
        m = min(len(ref), len(tr[prec]))
        per = np.abs(tr[prec][:m] - ref[:m]) / n
        G, R = mix[prec], mix["fp64"]
        cov_rel = max(float(np.linalg.norm(G.covs[j] - R.covs[j]) / np.linalg.norm(R.covs[j]))
                      for j in range(k))
        out[prec] = {"max_dlogL_per_N": float(per.max()), "final_dlogL_per_N": float(per[-1]),
                     "per_sweep": [float("%.3g" % v) for v in per],
                     "within_bound": bool(per.max() <= 1e-5),
                     "final_max_dweight": float(np.max(np.abs(G.weights - R.weights))),
                     "final_max_dmean": float(np.max(np.abs(G.means - R.means))),
                     "final_max_cov_rel_frobenius": cov_rel}
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload == "kmeans":
        if args.n is None:
            args.n = 1 << 24
        run_kmeans(args, rank, world, local)
        return
    if args.workload == "batched":
        run_batched(args, rank, world, local)
        return
    if args.workload == "small":
        run_small(args, rank, world, local)
        return
    if args.workload == "illcond":
        run_illcond(args, rank, world, local)
        return
    if args.n is None:
        args.n = 1 << 23
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    from fastem_gb300 import CudaMatrixEM, GaussianMixture
    dist = Dist(world)
    torch.cuda.set_device(local)
    n, d, k = args.n, 64, args.k
    X, init = workload(n, k)
    fl = em_flops(n, d, k)

    # ---- mixed precision, inputs resident in HBM
    svd = not args.no_svd
    em = CudaMatrixEM(d, n, k, precision="mixed", device=local)
    em.CopyDataset(X)
    G = GaussianMixture(*init)
    clocks = Clocks(local)
    clocks.start()
    t = time_device_sweeps(em, G, args.warmup, args.steps, dist, svd=svd)
    clk = clocks.stop()
    train_ms = dist.max(t["train_ms"])
    sweeps = t["sweeps"]
    ms_step = train_ms / sweeps
    value = world * sweeps / (train_ms / 1e3)
    est_ms = t["estep_ms"] / sweeps
    mst_ms = t["mstep_ms"] / sweeps
    fac_ms = t["factor_ms"] / sweeps
    launches = t["launches"]

    cov_ms = t["cov_ms"] / sweeps

    # roofline of the dominant kernel (tensor-bound contractions): the
    # covariance rank update (SYRK, N K d(d+1) flop) or the E-step
    # triangular multiply (TRMM, N K d(d+1) flop), one launch per sweep
    peak, peak_src = measured_peak_tflops()
    if est_ms >= cov_ms:
        kern, dom_ms, dom_flops = "k_estep_tc", est_ms, fl["estep"]
    else:
        # the z x^T kernel unless FEM_COV_KERNEL=zz selects the z z^T one
        kern = "k_cov_tc" if os.environ.get("FEM_COV_KERNEL", "").startswith("zz") else "k_cov_zx"
        dom_ms, dom_flops = cov_ms, fl["cov"]
    achieved = dom_flops / (dom_ms / 1e3) / 1e12
    roof = {"kernel": kern, "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": peak_src, "traffic": profiled_traffic(kern),
            "algorithmic_flops_per_launch": dom_flops, "launch_ms": dom_ms,
            "estep_ms": est_ms, "mstep_ms": mst_ms, "cov_ms": cov_ms, "factor_ms": fac_ms,
            "estep_frac": fl["estep"] / (est_ms / 1e3) / 1e12 / peak,
            "cov_frac": fl["cov"] / (cov_ms / 1e3) / 1e12 / peak,
            "sweep_algorithmic_tflops": fl["total"] / (ms_step / 1e3) / 1e12}

    # ---- end to end through the C-ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hostX = torch.from_numpy(X).pin_memory()
        from fastem_gb300 import _capi as C
        steps = max(1, min(args.steps, 5))
        em.SetParameters(1, 0.0, 1e5)
        Ge = G.copy()
        # untimed: the first copies out of a freshly pinned buffer are slower
        for _ in range(max(args.warmup, 3)):
            C.check(C.lib().fem_em_upload(em.handle, ctypes.c_void_p(hostX.data_ptr()), d))
            em.TrainNoCopy(Ge, svd=svd)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            C.check(C.lib().fem_em_upload(em.handle, ctypes.c_void_p(hostX.data_ptr()), d))
            em.TrainNoCopy(Ge, svd=svd)  # uploads the mixture, 1 sweep, reads it back
        dt = dist.max(time.perf_counter() - t0)
        pbytes = k * (1 + d + d * d) * 8
        # where an end-to-end step goes: the upload alone, the train call alone
        t0 = time.perf_counter()
        for _ in range(steps):
            C.check(C.lib().fem_em_upload(em.handle, ctypes.c_void_p(hostX.data_ptr()), d))
        up = (time.perf_counter() - t0) / steps
        t0 = time.perf_counter()
        for _ in range(steps):
            em.TrainNoCopy(Ge, svd=svd)
        tr = (time.perf_counter() - t0) / steps
        e2e = {"value": world * steps / dt, "unit": UNIT, "h2d_bytes_per_step": n * d * 4 + pbytes,
               "d2h_bytes_per_step": pbytes + 8 + 16, "upload_ms": up * 1e3, "train_call_ms": tr * 1e3}
        del hostX
    em.close()

    # ---- plain FP32 CUDA-core sweep on the same workload
    fp32 = None
    if not args.no_fp32:
        e32 = CudaMatrixEM(d, n, k, precision="fp32", device=local)
        e32.CopyDataset(X)
        G32 = GaussianMixture(*init)
        s32 = max(2, args.steps // 3)
        t32 = time_device_sweeps(e32, G32, max(1, min(args.warmup, 2)), s32, dist, svd=svd)
        ms32 = dist.max(t32["train_ms"]) / t32["sweeps"]
        fp32 = {"value": world * 1e3 / ms32, "ms_per_step": ms32, "steps": t32["sweeps"],
                "estep_ms": t32["estep_ms"] / t32["sweeps"], "mstep_ms": t32["mstep_ms"] / t32["sweeps"],
                "cov_ms": t32["cov_ms"] / t32["sweeps"],
                "estep_fp32_frac": fl["estep"] / (t32["estep_ms"] / t32["sweeps"] / 1e3) / 1e12
                / (152 * 128 * 2 * (clk.get("sm_mhz") or 2070.0) * 1e6 / 1e12),
                "mstep_fp32_frac": fl["mstep"] / (t32["mstep_ms"] / t32["sweeps"] / 1e3) / 1e12
                / (152 * 128 * 2 * (clk.get("sm_mhz") or 2070.0) * 1e6 / 1e12),
                "fp32_peak_note": "fractions of the nominal FP32 CUDA-core rate (152 SMs x 128 lanes x 2 flop "
                                  "at the sampled SM clock)"}
        e32.close()

    # ---- the metric's accuracy clause, outside the timed region
    acc = accuracy_vs_fp64(X, init, args.acc_sweeps, local) if args.acc_sweeps > 0 else None

    # ---- CPU baseline: the oracle port, 1 burn-in + 2 timed sweeps over all rows (rank 0)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sec, _, how = cpu_full_sweeps(X, init, 1, 2, threads, svd)
        cpu = {"value": 1.0 / float(np.mean(sec)), "unit": UNIT, "cores": threads, "kind": "port",
               "how": "%s, 1 burn-in + 2 timed sweeps over all %d rows" % (how, n),
               "sweep_seconds": [round(float(x), 3) for x in sec]}

    dist.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": sweeps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16",
        "precision": PRECISION_NOTE,
        "data": "synthetic em_large (seeded; Dirichlet(2) weights, N(0,25I) means, Haar-rotated "
                "covariances with eigenvalues log-uniform in [0.1,10])",
        "config": em_config(n, d, k, world, svd),
        "accuracy": acc,
        "roofline": roof, "e2e": e2e, "fp32_plain": fp32,
        "speedup_vs_fp32_plain": (value / fp32["value"]) if fp32 else None,
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


BATCH_METRIC = "batched EM fits/s: 512 fits, N in [2e3,2e5], d in {4,8,16,32}, K in [2,32], 30 sweeps"
BATCH_SWEEPS = 30
BATCH_PROFILE_FILE = os.path.join(ROOT, "profiles", "batch_em_512fits.md")


def batched_workload():
    """512 fits: blob data per fit seed, D^2-sampled initial means."""
    from fastem_gb300 import synth
    fits = synth.em_batched()
    data = []
    for f in fits:
        X, _ = synth.kmeans_blobs(seed=f["seed"], n=f["n"], d=f["d"], k=f["k"])
        data.append((X, synth.dsquared_init(X, f["k"], seed=f["seed"] % 1000)))
    return fits, data


def batched_cpu_baseline(fits, data, sample_every=32, gpu_traces=None, mixed_traces=None, extra=None):
    """The oracle's TrainNoCopy (FP64, OpenMP over all host cores) on every
    `sample_every`-th fit, 30 sweeps each.  With `gpu_traces` ({fit: LogL
    trace}) the oracle's traces of the same fits check the GPU's:
    the largest per-fit |dlogL/N| (and the same for `mixed_traces` and for
    each {name: traces} of `extra`)."""
    from oracle import oracle as O
    O.lib()
    idx = list(range(0, len(fits), sample_every))
    t0 = time.perf_counter()
    refs = {}
    for i in idx:
        X, init = data[i]
        refs[i] = O.em_train(X, *init, BATCH_SWEEPS, eps=0.0, abort_thr=1e12, nthreads=os.cpu_count())
    dt = time.perf_counter() - t0
    def worst(traces):
        errs = []
        for i, tr in (traces or {}).items():
            ref = refs.get(i)
            if ref is not None and ref["status"] == 0 and tr is not None:
                m = min(len(tr), len(ref["logl"]))
                errs.append(float(np.max(np.abs(tr[:m] - ref["logl"][:m])) / fits[i]["n"]))
        return errs
    errs, merrs = worst(gpu_traces), worst(mixed_traces)
    out = {"value": len(idx) / dt, "unit": "fits/s", "cores": os.cpu_count(), "kind": "port",
           "sample": "%d of the %d fits (every %dth), %d sweeps each, %.1f s" % (len(idx), len(fits), sample_every,
                                                                                BATCH_SWEEPS, dt),
           "max_dlogL_per_N_vs_gpu": max(errs) if errs else None, "checked_fits": len(errs),
           "max_dlogL_per_N_vs_mixed_per_fit": max(merrs) if merrs else None, "checked_mixed_fits": len(merrs)}
    for name, traces in (extra or {}).items():
        e = worst(traces)
        out["max_dlogL_per_N_vs_" + name] = max(e) if e else None
    return out


def run_batched(args, rank, world, local):
    """512 independent fits trained together by the batched engine
    (fem_em_batch_*): every kernel of a sweep covers all fits still sweeping,
    the host waits every 8 sweeps.  A step is the whole batch (512 fits x 30
    sweeps, FP32 CUDA cores with FP64 sums / factorisation / LogL).  Per-fit
    |dlogL/N| against the FP64 oracle is reported for a sample of fits.
    With --gpus N each rank trains its own copy of the batch (replicas)."""
    fits, data = batched_workload()
    if args.fits_d:
        keep = [i for i, f in enumerate(fits) if f["d"] == args.fits_d]
        fits, data = [fits[i] for i in keep], [data[i] for i in keep]
    nf = len(fits)
    if args.impl == "reference":
        if rank == 0:
            cpu = batched_cpu_baseline(fits, data)
            print(json.dumps({"metric": BATCH_METRIC, "impl": "reference", "value": cpu["value"], "unit": "fits/s",
                              "n_gpus": world, "steps": 1, "warmup": 0, "higher_is_better": True,
                              "cpu_baseline": cpu, "e2e": {"value": cpu["value"], "unit": "fits/s",
                                                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                              "config": {"workload": "512 fits x 30 sweeps (em_batched, seed 4)"}}), flush=True)
        return
    import torch
    from fastem_gb300 import CudaBatchEM, CudaMatrixEM, GaussianMixture
    from fastem_gb300 import _capi as C
    dist = Dist(world)
    torch.cuda.set_device(local)
    shapes = [(X.shape[1], X.shape[0], len(init[0])) for X, init in data]
    mixtures = [GaussianMixture(*init) for _, init in data]
    packed = np.concatenate([X.reshape(-1) for X, _ in data])
    x_bytes = packed.nbytes
    from fastem_gb300.batch import TUNING_TABLE, load_tuning
    B = CudaBatchEM(shapes, device=local, max_sweeps=BATCH_SWEEPS)
    tuning = B.Tuning()
    tuning_src = ("autotuner table " + os.path.relpath(TUNING_TABLE, ROOT)) if load_tuning() else "library defaults"
    B.SetParameters(BATCH_SWEEPS, 0.0, 1e12)
    B.CopyPacked(packed)

    def set_all():
        for i, G in enumerate(mixtures):
            B.SetMixture(i, G)

    for _ in range(args.warmup):
        set_all()
        B.TrainNoCopy()
    clocks = Clocks(local)
    clocks.start()
    B.EnableTiming(True)
    total = 0.0
    dist.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        set_all()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, it, ll = B.TrainNoCopy()
        total += time.perf_counter() - t0
    clk = clocks.stop()
    tm = B.Timing()
    ms = dist.max(total * 1e3) / args.steps
    value = world * nf / (ms / 1e3)
    # the mixed form of the engine: the E-step of the d > 16 fits on the tensor cores
    mixed = None
    mixed_traces_batched = {}
    with CudaBatchEM(shapes, device=local, max_sweeps=BATCH_SWEEPS, precision="mixed") as BM:
        BM.SetParameters(BATCH_SWEEPS, 0.0, 1e12)
        BM.CopyPacked(packed)
        for _ in range(args.warmup):
            for i, G in enumerate(mixtures):
                BM.SetMixture(i, G)
            BM.TrainNoCopy()
        BM.EnableTiming(True)
        mtot = 0.0
        for _ in range(args.steps):
            for i, G in enumerate(mixtures):
                BM.SetMixture(i, G)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mst, _, _ = BM.TrainNoCopy()
            mtot += time.perf_counter() - t0
        mtm = BM.Timing()
        mms = dist.max(mtot * 1e3) / args.steps
        mixed_traces_batched = {i: BM.Trace(i)[0] for i in range(0, nf, 32) if mst[i] == 0}
        mixed = {"value": world * nf / (mms / 1e3), "unit": "fits/s", "ms_per_step": mms,
                 "failed_fits": int((mst != 0).sum()),
                 "estep_ms_d32_per_step": mtm["classes"][32]["estep_ms"] / args.steps,
                 "estep_ms_d32_per_step_fp32": tm["classes"][32]["estep_ms"] / args.steps}
    # end to end through the C-ABI: pinned host rows -> device, initial mixtures,
    # train, every fit's trained mixture and status back to the host
    e2e = None
    if not args.no_e2e:
        pinned = torch.from_numpy(packed).pin_memory()
        steps = max(1, min(args.steps, 3))
        p_bytes = sum(k * (1 + d + d * d) * 8 for d, n, k in shapes)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            C.check(C.lib().fem_em_batch_upload_packed(B._h, ctypes.c_void_p(pinned.data_ptr())))
            set_all()
            B.TrainNoCopy()
            for i in range(nf):
                B.GetMixture(i)
        dt = dist.max(time.perf_counter() - t0)
        e2e = {"value": world * nf * steps / dt, "unit": "fits/s", "h2d_bytes_per_step": x_bytes + p_bytes,
               "d2h_bytes_per_step": p_bytes + nf * 16}
    # one handle and stream per fit, 16 host threads: the FP32 form (the scheme
    # the batched engine replaced) and the mixed tensor-core form (the single-fit
    # tcgen05 kernels, d zero-padded to 64; not batched into one launch)
    per_fit, per_fit_mixed, mixed_traces = None, None, {}
    if not args.no_fp32:
        import concurrent.futures as cf

        def run(i, prec):
            X, init = data[i]
            d, n, k = shapes[i]
            with CudaMatrixEM(d, n, k, precision=prec, device=local) as em:
                em.SetParameters(BATCH_SWEEPS, 0.0, 1e12)
                try:
                    em.Train(X, GaussianMixture(*init))
                except Exception:
                    return None
                return em.logl_trace.copy()
        for prec in ("fp32", "mixed"):
            with cf.ThreadPoolExecutor(16) as ex:
                list(ex.map(lambda i: run(i, prec), range(8)))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                tr = list(ex.map(lambda i: run(i, prec), range(nf)))
                torch.cuda.synchronize()
                leg = {"value": nf / (time.perf_counter() - t0), "unit": "fits/s",
                       "scheme": "one %s handle and stream per fit, 16 host threads" % prec,
                       "failed_fits": int(sum(t is None for t in tr))}
            if prec == "fp32":
                per_fit = leg
            else:
                per_fit_mixed = leg
                mixed_traces = {i: tr[i] for i in range(0, nf, 32)}
    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        # the CPU baseline leg also checks the sampled fits' LogL traces
        traces = {i: B.Trace(i)[0] for i in range(0, nf, 32) if st[i] == 0}
        cpu = batched_cpu_baseline(fits, data, gpu_traces=traces, mixed_traces=mixed_traces,
                                   extra={"mixed_batched": mixed_traces_batched})
        if mixed is not None:
            mixed["max_dlogL_per_N_sampled"] = cpu["max_dlogL_per_N_vs_mixed_batched"]
        if per_fit_mixed is not None:
            per_fit_mixed["max_dlogL_per_N_sampled"] = cpu["max_dlogL_per_N_vs_mixed_per_fit"]
            per_fit_mixed["sampled_fits"] = cpu["checked_mixed_fits"]
    B.close()
    dist.close()
    if rank != 0:
        return
    # roofline: the largest kernel, the covariance sums of the d = 32 class
    # (k_b_cov<32>), FP32 CUDA-core flops N K d (d + 1) per fit and sweep against
    # the nominal FP32 rate at the sampled SM clock (152 SMs x 128 lanes x 2 flop);
    # traffic per launch from the committed ncu summary
    cov_flop = sum(n * k * d * (d + 1) for d, n, k in shapes if d > 16) * BATCH_SWEEPS
    cov_s = tm["classes"][32]["cov_ms"] / 1e3 / args.steps
    mhz = clk.get("sm_mhz") or 2070.0
    peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
    achieved = cov_flop / cov_s / 1e12 if cov_s > 0 else None
    traffic = None
    try:
        for ln in open(BATCH_PROFILE_FILE):
            if ln.startswith("traffic_bytes_per_launch k_b_cov<32>"):
                traffic = float(ln.split("=")[-1])
    except OSError:
        pass
    per_step = {k2: tm[k2] / args.steps for k2 in ("estep_ms", "means_ms", "cov_ms", "factor_ms", "loop_ms")}
    per_class = {"d<=%d" % D: {k2: v / args.steps for k2, v in tm["classes"][D].items()} for D in (4, 8, 16, 32)}
    line = {
        "metric": BATCH_METRIC, "value": value, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 (CUDA cores), fp64 sums / factorisation / logL",
        "data": "synthetic blobs per fit seed (synth.em_batched, seed 4)",
        "config": {"workload": ("%d fits x 30 sweeps per step, batched engine (every kernel covers all fits)" % nf)
                   + (", only the d = %d fits" % args.fits_d if args.fits_d else ""),
                   "total_points": int(sum(f["n"] for f in fits)), "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (rows %.2f GB, posteriors %.2f GB)" % (
                       x_bytes / 1e9, sum(n * k for d, n, k in shapes) * 4 / 1e9),
                   "work_items": dict(tuning, source=tuning_src)},
        "phase_ms_per_step": per_step, "class_ms_per_step": per_class,
        "roofline": {"kernel": "k_b_cov<32> (covariance sums, d = 32 fits)", "bound": "fp32", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                     "peak_source": "nominal FP32 CUDA-core rate at the sampled SM clock (no measured FP32 peak)",
                     "traffic": traffic, "algorithmic_flop_per_step": cov_flop,
                     "launch_ms": cov_s * 1e3 / BATCH_SWEEPS},
        "failed_fits": int((st != 0).sum()),
        "failed_fits_note": None if args.fits_d else "fits 282, 283, 385 also collapse in the FP64 oracle",
        "max_dlogL_per_N_sampled": cpu["max_dlogL_per_N_vs_gpu"] if cpu else None,
        "sampled_fits": cpu["checked_fits"] if cpu else 0,
        "per_fit_handles": per_fit, "speedup_vs_per_fit_handles": (value / per_fit["value"]) if per_fit else None,
        "mixed_per_fit_handles": per_fit_mixed,
        "mixed": mixed,
        "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": tm["launches"],
    }
    print(json.dumps(line), flush=True)


SMALL_METRIC = "EM iter/s N=1e5 d=8 K=10 (FP64 sweeps, per-sweep logL against the FP64 oracle)"
ILL_METRIC = "EM iter/s N=2^21 d=256 K=64, covariance condition 1e6: split-precision tensor cores vs FP32 plain, error vs FP64 stated"
FP64_NOMINAL_TFLOPS = 1.25   # GB300 FP64, nominal (no measured FP64 peak)
ILL_REG = 1e-6               # RegCoef of the ill-conditioned workload (-g 1e-6)


def l2_flush(buf):
    """Writes a buffer larger than L2 (129 MB) on the current stream."""
    buf.add_(1.0)


def time_single_sweeps(em, G, steps, dist, flush):
    """`steps` one-sweep trains, L2 flushed before each (outside the timed
    events on the library's stream); returns the summed sweep-loop ms."""
    import torch
    em.TimingReset(True)
    em.SetParameters(1, 0.0, 1e12)
    for _ in range(steps):
        flush()
        torch.cuda.synchronize()
        em.TrainNoCopy(G.copy())
    torch.cuda.synchronize()
    t = em.Timing()
    em.TimingReset(False)
    return dist.max(t["train_ms"]), t["launches"]


def run_small(args, rank, world, local):
    """N = 100,000, d = 8, K = 10 (em_small, seed 1): D^2-sampled means
    (seed 2), identity covariances, uniform weights.  A step is one sweep;
    `value` = FP64 sweeps/s (the reference's precision), FP32 and mixed
    beside it.  The inputs (3.2 MB) fit in L2, so every timed sweep is its own
    train call after an L2 flush.  The CPU baseline leg runs the oracle's 50
    sweeps and checks the GPU's FP64 LogL trace against them."""
    import torch
    from fastem_gb300 import CudaMatrixEM, GaussianMixture, synth
    from fastem_gb300 import _capi as C
    X, _ = synth.em_small()
    n, d, k = X.shape[0], X.shape[1], 10
    init = synth.dsquared_init(X, k, seed=2)
    if args.impl == "reference":
        if rank == 0:
            from oracle import oracle as O
            O.lib()
            t0 = time.perf_counter()
            O.em_train(X, *init, 50, eps=0.0, abort_thr=1e12, nthreads=os.cpu_count())
            v = 50 / (time.perf_counter() - t0)
            cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": "50 sweeps, all rows"}
            print(json.dumps({"metric": SMALL_METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": world,
                              "steps": 50, "warmup": 0, "higher_is_better": True, "cpu_baseline": cpu,
                              "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                              "config": {"workload": "em_small N=100000 d=8 K=10"}}), flush=True)
        return
    dist = Dist(world)
    torch.cuda.set_device(local)
    flush_buf = torch.zeros(128 << 20, dtype=torch.float32, device="cuda")   # 512 MB > L2
    G = GaussianMixture(*init)
    res, trace64 = {}, None
    clocks = Clocks(local)
    clocks.start()
    for prec in ("fp64", "fp32", "mixed"):
        with CudaMatrixEM(d, n, k, precision=prec, device=local) as em:
            em.CopyDataset(X)
            em.SetParameters(max(args.warmup, 3), 0.0, 1e12)
            em.TrainNoCopy(G.copy())
            ms, launches = time_single_sweeps(em, G, args.steps, dist, lambda: l2_flush(flush_buf))
            res[prec] = {"value": world * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                         "launches": launches}
            if prec == "fp64":
                em.SetParameters(50, 0.0, 1e12)
                Gt = G.copy()
                em.TrainNoCopy(Gt)
                trace64 = em.logl_trace.copy()
                # end to end through the C-ABI: host rows -> device, parameters, one sweep, parameters back
                steps = max(1, min(args.steps, 10))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(steps):
                    C.check(C.lib().fem_em_upload(em.handle, C.ptr(C.f32rows(X)), d))
                    em.SetParameters(1, 0.0, 1e12)
                    Ge = G.copy()
                    em.TrainNoCopy(Ge)
                e2e = {"value": world * steps / dist.max(time.perf_counter() - t0), "unit": UNIT,
                       "h2d_bytes_per_step": X.nbytes + k * (1 + d + d * d) * 8,
                       "d2h_bytes_per_step": k * (1 + d + d * d) * 8}
    clk = clocks.stop()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import oracle as O
        O.lib()
        t0 = time.perf_counter()
        ref = O.em_train(X, *init, 50, eps=0.0, abort_thr=1e12, nthreads=os.cpu_count())
        dt = time.perf_counter() - t0
        err = float(np.max(np.abs(trace64 - ref["logl"])) / n) if len(ref["logl"]) == len(trace64) else None
        cpu = {"value": 50 / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": "50 sweeps, all rows", "fp64_gpu_max_dlogL_per_N": err}
    dist.close()
    if rank != 0:
        return
    fl = em_flops(n, d, k)["total"]
    ms = res["fp64"]["ms_per_step"]
    achieved = fl / (ms / 1e3) / 1e12
    line = {
        "metric": SMALL_METRIC, "value": res["fp64"]["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic em_small (seeded: Dirichlet(1) weights, U[-10,10] means, A A^T + 0.5 I covariances)",
        "config": {"workload": "em_small N=100000 d=8 K=10, one EM sweep per step", "n": n, "d": d, "k": k,
                   "l2": "inputs 3.2 MB (below L2): 512 MB written between timed sweeps"},
        "fp32": res["fp32"], "mixed": res["mixed"],
        "roofline": {"kernel": "whole FP64 sweep", "bound": "fp64", "achieved": achieved,
                     "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s", "frac": achieved / FP64_NOMINAL_TFLOPS,
                     "peak_source": "nominal GB300 FP64 rate (no measured FP64 peak)", "traffic": None,
                     "algorithmic_flop_per_step": fl, "note": "launch- and latency-bound at this size"},
        "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": res["fp64"]["launches"],
    }
    print(json.dumps(line), flush=True)


def run_illcond(args, rank, world, local):
    """N = 2^21, d = 256, K = 64, eigenvalues log-spaced over [1e-3, 1e3]
    (condition 1e6), Haar bases, N(0, 100 I) means (em_illcond, seed 5);
    initial mixture = the generating one with means + 0.1 and covariances
    x 1.05; run like the reference with -S (no condition check) and -g 1e-6
    (RegCoef: with Dirichlet(1) weights some components hold fewer than 256
    points, so their sample covariances are singular and the unregularised
    fit stops with a Cholesky failure, in FP64 as in the reference).
    `value` = sweeps/s of the split-precision tensor-core form (em_wide.cu);
    the FP32 CUDA-core and FP64 forms are timed beside it at full size, and
    the logL / posterior errors of mixed and FP32 against FP64 are measured
    over 15 sweeps on the first 2^19 rows."""
    import torch
    from fastem_gb300 import CudaMatrixEM, GaussianMixture, synth
    from fastem_gb300 import _capi as C
    X, info = synth.em_illcond(n=args.n or (1 << 21))
    n, d, k = X.shape[0], X.shape[1], 64
    init = (info["weights"], info["means"] + 0.1, info["covs"] * 1.05)
    cfg = {"workload": "em_illcond N=%d d=256 K=64, one EM sweep per step" % n, "n": n, "d": d, "k": k,
           "init": "generating mixture, means + 0.1, covariances x 1.05", "svd": "off (-S)",
           "reg_coef": ILL_REG, "l2": "inputs larger than L2 (X 2.1 GB, whitened offsets 68.7 GB)"}
    if args.impl == "reference":
        if rank == 0:
            sec, how = cpu_sweep_seconds(X, init, 1 << 13, os.cpu_count())
            v = (1 << 13) / n / sec
            cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": "1 sweep (%s) over the first 8192 rows, scaled x%d" % (how, n >> 13)}
            print(json.dumps({"metric": ILL_METRIC, "impl": "reference", "value": v, "unit": UNIT, "n_gpus": world,
                              "steps": 1, "warmup": 0, "higher_is_better": True, "cpu_baseline": cpu,
                              "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                              "config": cfg}), flush=True)
        return
    dist = Dist(world)
    torch.cuda.set_device(local)
    steps, warm = max(1, args.steps), max(args.warmup, 3)
    G = GaussianMixture(*init)
    clocks = Clocks(local)
    clocks.start()
    with CudaMatrixEM(d, n, k, precision="mixed", device=local) as em:
        em.CopyDataset(X)
        t = time_device_sweeps(em, G.copy(), warm, steps, dist, reg=ILL_REG)
        # end to end through the C-ABI: host rows uploaded, one sweep, mixture read back
        hostX = torch.from_numpy(X).pin_memory()
        em.SetParameters(1, 0.0, 1e12, ILL_REG)
        for _ in range(2):
            C.check(C.lib().fem_em_upload(em.handle, ctypes.c_void_p(hostX.data_ptr()), d))
            em.TrainNoCopy(G.copy())
        e_steps = max(1, min(steps, 3))
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e_steps):
            C.check(C.lib().fem_em_upload(em.handle, ctypes.c_void_p(hostX.data_ptr()), d))
            em.TrainNoCopy(G.copy())
        e_dt = dist.max(time.perf_counter() - t0)
        del hostX
    clk = clocks.stop()
    ms = dist.max(t["train_ms"]) / t["sweeps"]
    value = world * 1e3 / ms
    pbytes = k * (1 + d + d * d) * 8
    e2e = {"value": world * e_steps / e_dt, "unit": UNIT, "h2d_bytes_per_step": n * d * 4 + pbytes,
           "d2h_bytes_per_step": pbytes + 8 + 16}
    # the FP32 CUDA-core and FP64 forms at full size
    other = {}
    for prec, sw in (("fp32", 3), ("fp64", 1)):
        with CudaMatrixEM(d, n, k, precision=prec, device=local) as em:
            em.CopyDataset(X)
            try:
                tt = time_device_sweeps(em, G.copy(), 1, sw, dist, reg=ILL_REG)
                other[prec] = {"status": "ok", "value": world * tt["sweeps"] / (tt["train_ms"] / 1e3),
                               "ms_per_step": tt["train_ms"] / tt["sweeps"], "sweeps_timed": tt["sweeps"]}
            except C.FemError as e:
                other[prec] = {"status": str(e), "failed_at_sweep": em.GetIterCounter()}
    # accuracy against FP64: 15 sweeps on the first 2^19 rows
    m = min(n, 1 << 19)
    Xs = np.ascontiguousarray(X[:m])
    tr, post = {}, {}
    for prec in ("fp64", "mixed", "fp32"):
        with CudaMatrixEM(d, m, k, precision=prec, device=local) as em:
            em.SetParameters(15, 0.0, 1e12, ILL_REG)
            try:
                em.Train(Xs, G.copy())
                tr[prec] = em.logl_trace.copy()
                post[prec] = em.Posteriors()
            except C.FemError as e:
                tr[prec] = str(e)
    acc = {"rows": m, "sweeps": 15, "vs": "fp64 GPU path (oracle-pinned at d = 256)"}
    for prec in ("mixed", "fp32"):
        a, b = tr.get(prec), tr.get("fp64")
        if isinstance(a, np.ndarray) and isinstance(b, np.ndarray):
            L = min(len(a), len(b))
            dl = np.abs(a[:L] - b[:L]) / m
            acc[prec] = {"max_dlogL_per_N": float(dl.max()), "per_sweep": [float("%.3g" % v) for v in dl],
                         "max_dposterior": float(np.max(np.abs(post[prec] - post["fp64"])))}
        else:
            acc[prec] = {"status": a if isinstance(a, str) else b}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sec, how = cpu_sweep_seconds(X, init, 1 << 13, os.cpu_count())
        cpu = {"value": (1 << 13) / n / sec, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": "1 sweep (%s) over the first 8192 rows, scaled x%d" % (how, n >> 13)}
    dist.close()
    if rank != 0:
        return
    fl = em_flops(n, d, k)
    est_ms = t["estep_ms"] / t["sweeps"]
    achieved = fl["estep"] / (est_ms / 1e3) / 1e12
    peak, src = measured_peak_tflops()
    line = {
        "metric": ILL_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": t["sweeps"],
        "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16x3 split products, fp32 accumulate, fp64 factor/logL",
        "data": "synthetic em_illcond (seeded; eigenvalues log-spaced [1e-3, 1e3], Haar bases, N(0,100 I) means)",
        "config": cfg, "fp32": other.get("fp32"), "fp64": other.get("fp64"), "accuracy": acc,
        "precision_note": ("the tensor core's FP32 accumulation truncates addends below the accumulator's ulp; "
                           "at condition 1e6 the running sums of L^-1 (x - mu) are ~1e3 times their result, "
                           "which bounds the mixed form's logL error near 1e-4 per point"),
        "phase_ms_per_step": {"estep_ms": est_ms, "mstep_ms": t["mstep_ms"] / t["sweeps"],
                              "cov_ms": t["cov_ms"] / t["sweeps"], "factor_ms": t["factor_ms"] / t["sweeps"]},
        "roofline": {"kernel": "k_wide_estep", "bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": src, "traffic": None,
                     "algorithmic_flops_per_launch": fl["estep"], "launch_ms": est_ms},
        "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": t["launches"],
    }
    print(json.dumps(line), flush=True)


KM_METRIC = "k-means iter/s N=2^24 d=32 K=256 (labels bit-exact to FP64)"
KM_PROFILE_FILE = os.path.join(ROOT, "profiles", "kmeans_assign_n16m_d32_k256.md")


def km_workload(n, d, k):
    """Equal isotropic blobs (sigma 1, centres U[-20, 20]^d), k-means||
    seeding with seed 3 (KMeansOrOrInitializer, Clust/KMeansOrOrInitializer.cpp:
    143-174) by the library's own host seeder (`em2gpu --seed oror`, the
    reference's draw order on one generator stream; its rows equal the
    oracle's restatement in tests/test_host.py).  Returns (X, C0, seconds the
    seeding took)."""
    import tempfile
    from fastem_gb300 import build as B
    from fastem_gb300 import formats, synth
    X, _ = synth.kmeans_blobs(seed=2, n=n, d=d, k=k)
    B.build_host()
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "x.bin")
        formats.write_bin(f, X)
        t0 = time.perf_counter()
        out = subprocess.run([B.EM2GPU, "--seed", "oror", f, str(k), "3"], capture_output=True, text=True,
                             check=True)
        secs = time.perf_counter() - t0
    C0 = np.array([[float(v) for v in ln.split()] for ln in out.stdout.strip().splitlines()])
    assert C0.shape == (k, d)
    return X, np.ascontiguousarray(C0), secs


def time_km_iterations(km, C, warmup, steps, dist):
    """Device time (library CUDA events: assignment + update kernels) of
    `steps` Lloyd iterations after `warmup`."""
    for _ in range(warmup):
        km.ComputeMSEAndCorrect(C)
    dist.barrier()
    a = u = 0.0
    launches = 0
    for _ in range(steps):
        km.ComputeMSEAndCorrect(C)
        st = km.Stats()
        a += st["assign_ms"]
        u += st["update_ms"]
        launches += 4 if km.precision == "mixed" else 3
    dist.barrier()
    return a, u, launches, st["rechecked"]


def run_kmeans(args, rank, world, local):
    """Lloyd k-means at N = 2^24, d = 32, K = 256 (equal isotropic blobs,
    sigma 1, centres U[-20, 20]^32; k-means|| seeding, seed 3): mixed
    (tcgen05 GEMM + argmin, FP32 refinement, FP64 recheck) against the FP32
    CUDA-core path; roofline = HBM (read X once, write labels).  Outside the
    timed region both paths run the configuration's 30 iterations from the
    same centroids and their labels are compared after every iteration; the
    CPU leg checks the first iteration's labels of its row sample against the
    oracle's FP64 assignment."""
    import torch
    from fastem_gb300 import CudaKMA
    n, d, k = args.n, 32, 256
    if args.impl == "reference":
        if rank == 0:
            X, C0, _ = km_workload(n, d, k)
            cpu = km_cpu_baseline(X, C0)
            print(json.dumps({"metric": KM_METRIC, "impl": "reference", "value": cpu["value"], "unit": UNIT,
                              "n_gpus": world, "steps": 1, "warmup": 1, "higher_is_better": True,
                              "cpu_baseline": cpu, "e2e": {"value": cpu["value"], "unit": UNIT,
                                                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                              "config": {"workload": "kmeans_blobs N=%d d=%d K=%d" % (n, d, k)}}), flush=True)
        return
    dist = Dist(world)
    torch.cuda.set_device(local)
    X, C0, seed_s = km_workload(n, d, k)
    algo_bytes = n * d * 4 + n * 4
    with CudaKMA(d, n, k, precision="mixed", device=local, repair=True) as km:
        km.SetDataset(X)
        km.InitDataStructures()
        C = C0.copy()
        clocks = Clocks(local)
        clocks.start()
        a, u, launches, rech = time_km_iterations(km, C, args.warmup, args.steps, dist)
        clk = clocks.stop()
        ms = dist.max(a + u) / args.steps
        assign_ms = a / args.steps
        # end to end through the C-ABI: dataset upload from pinned host memory + one iteration
        e2e = None
        if not args.no_e2e:
            hostX = torch.from_numpy(X).pin_memory()
            from fastem_gb300 import _capi as Cc
            steps = max(1, min(args.steps, 5))
            Ce = C0.copy()
            # untimed: the first copies out of a freshly pinned buffer are slower
            for _ in range(max(args.warmup, 3)):
                Cc.check(Cc.lib().fem_km_upload(km.handle, ctypes.c_void_p(hostX.data_ptr()), d))
                km.ComputeMSEAndCorrect(C0.copy())
            dist.barrier()
            t0 = time.perf_counter()
            for _ in range(steps):
                Cc.check(Cc.lib().fem_km_upload(km.handle, ctypes.c_void_p(hostX.data_ptr()), d))
                km.ComputeMSEAndCorrect(Ce)
            dt = dist.max(time.perf_counter() - t0)
            e2e = {"value": world * steps / dt, "unit": UNIT, "h2d_bytes_per_step": n * d * 4 + k * d * 8,
                   "d2h_bytes_per_step": (k * d + 2 * k) * 8}
    value = world * 1e3 / ms
    fp32 = None
    if not args.no_fp32:
        with CudaKMA(d, n, k, precision="fp32", device=local, repair=True) as k32:
            k32.SetDataset(X)
            k32.InitDataStructures()
            C32 = C0.copy()
            a32, u32, _, r32 = time_km_iterations(k32, C32, 1, max(2, args.steps // 3), dist)
            ms32 = dist.max(a32 + u32) / max(2, args.steps // 3)
            fp32 = {"value": world * 1e3 / ms32, "ms_per_step": ms32, "rechecked_rows": r32}
    # the configuration's 30 iterations through both GPU paths, labels compared each time
    parity, first_labels = None, None
    if not args.no_fp32:
        iters, mism, dmax, fmax = 30, 0, 0.0, 0.0
        Cm, Cf = C0.copy(), C0.copy()
        with CudaKMA(d, n, k, precision="mixed", device=local, repair=True) as km1, \
                CudaKMA(d, n, k, precision="fp32", device=local, repair=True) as km2:
            km1.SetDataset(X)
            km2.SetDataset(X)
            km1.InitDataStructures()
            km2.InitDataStructures()
            for it in range(iters):
                f1 = km1.ComputeMSEAndCorrect(Cm)
                f2 = km2.ComputeMSEAndCorrect(Cf)
                l1, l2 = km1.Assignment(), km2.Assignment()
                if it == 0:
                    first_labels = l1.copy()
                mism += int((l1 != l2).sum())
                dmax = max(dmax, float(np.max(np.abs(Cm - Cf))))
                fmax = max(fmax, abs(f1 - f2) / abs(f2))
        parity = {"iterations": iters, "label_mismatches_mixed_vs_fp32": mism,
                  "max_centroid_difference": dmax, "max_fit_rel_difference": fmax}
    cpu = km_cpu_baseline(X, C0, first_labels) if (rank == 0 and world == 1 and not args.no_cpu) else None
    dist.close()
    if rank != 0:
        return
    peak = None
    try:
        with open(PEAKS_FILE) as f:
            peak = float(json.load(f)["hbm_gbs"])
        src = "measured (MEASURED_PEAKS hbm_gbs)"
    except Exception:
        peak, src = 6800.0, "fallback 6.8 TB/s"
    achieved = algo_bytes / (assign_ms / 1e3) / 1e9
    traffic = None
    try:
        for line in open(KM_PROFILE_FILE):
            if line.startswith("traffic_bytes_per_launch k_km_assign_tc"):
                traffic = float(line.split("=")[-1])
    except OSError:
        pass
    line = {
        "metric": KM_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16x3 distances, fp32 refinement, fp64 recheck",
        "data": "synthetic kmeans_blobs (seeded; equal isotropic blobs, sigma 1, centres U[-20,20]^32)",
        "config": {"workload": "kmeans_blobs N=%d d=%d K=%d, one Lloyd iteration per step" % (n, d, k),
                   "n": n, "d": d, "k": k, "init": "k-means|| (seed 3, %.1f s on the host)" % seed_s,
                   "l2": "inputs larger than L2 (X 2.1 GB)"},
        "roofline": {"kernel": "k_km_assign_tc", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": assign_ms},
        "rechecked_rows_last_step": rech, "parity": parity, "e2e": e2e, "fp32_plain": fp32,
        "speedup_vs_fp32_plain": (value / fp32["value"]) if fp32 else None,
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def km_cpu_baseline(X, C0, gpu_labels=None):
    """The oracle's Lloyd iteration (FP64, OpenMP, all host cores) on the
    first 2^20 rows, scaled to N.  With `gpu_labels` (the GPU's first-iteration
    assignment of all rows from the same centroids) the sample's labels are
    compared: an assignment depends only on the row and the centroids."""
    from oracle import oracle as O
    O.lib()
    n = len(X)
    sample = min(n, 1 << 20)
    threads = os.cpu_count() or 1
    Xs = np.ascontiguousarray(X[:sample])
    O.km_iterate(Xs[:4096], C0.copy(), repair=False, nthreads=threads)
    t0 = time.perf_counter()
    _, _, _, labels = O.km_iterate(Xs, C0.copy(), repair=False, nthreads=threads)
    dt = (time.perf_counter() - t0) * n / sample
    out = {"value": 1.0 / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": "1 FP64 iteration over the first %d of %d rows, scaled x%d" % (sample, n, n // sample)}
    if gpu_labels is not None:
        out["label_mismatches_vs_gpu_first_iteration"] = int((labels != gpu_labels[:sample]).sum())
    return out


if __name__ == "__main__":
    main()
