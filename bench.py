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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="em", choices=["em", "kmeans", "batched"])
    ap.add_argument("--n", type=int, default=None, help="points (default 2^23 EM, 2^24 k-means)")
    ap.add_argument("--k", type=int, default=128)
    ap.add_argument("--fits-d", type=int, default=None, choices=[4, 8, 16, 32],
                    help="batched workload: only the fits of this dimension (a smaller case for profiling)")
    ap.add_argument("--no-fp32", action="store_true", help="skip the FP32 CUDA-core comparison")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
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


def time_device_sweeps(em, G, warmup, steps, dist):
    """Warm-up sweeps, then `steps` sweeps timed by CUDA events on the
    library's stream (max over ranks)."""
    import torch
    em.SetParameters(warmup, 0.0, 1e5)
    em.TrainNoCopy(G)
    dist.barrier()
    torch.cuda.synchronize()
    em.TimingReset(True)
    em.SetParameters(steps, 0.0, 1e5)
    em.TrainNoCopy(G)
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


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU algorithm (the oracle's FP64
    restatement of SimpleMatrixEM, OpenMP with OpenBLAS level-3 calls where
    the reference calls MKL, all host cores) on a bounded row sample per step;
    the reference itself cannot be compiled here (Eigen 3.4, MKL, libnuma and
    MPI are absent)."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    n, d, k = args.n, 64, args.k
    sample = 1 << 16
    X, init = workload(n, k)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sweep_seconds(X, init, sample, threads)
    tot = 0.0
    for _ in range(args.steps):
        dt, how = cpu_sweep_seconds(X, init, sample, threads)
        tot += dt
    per_sweep_full = tot / args.steps * (n / sample)
    value = 1.0 / per_sweep_full
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_sweep_full * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic em_large (seeded)",
        "config": {"workload": "em_large N=%d d=%d K=%d, one EM sweep per step" % (n, d, k)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "1 sweep (%s) over the first %d of %d rows per step, scaled x%d"
                                   % (how, sample, n, n // sample)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    em = CudaMatrixEM(d, n, k, precision="mixed", device=local)
    em.CopyDataset(X)
    G = GaussianMixture(*init)
    clocks = Clocks(local)
    clocks.start()
    t = time_device_sweeps(em, G, args.warmup, args.steps, dist)
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
        kern, dom_ms, dom_flops = "k_cov_tc", cov_ms, fl["cov"]
    achieved = dom_flops / (dom_ms / 1e3) / 1e12
    roof = {"kernel": kern, "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": peak_src, "traffic": profiled_traffic(kern),
            "algorithmic_flops_per_launch": dom_flops, "launch_ms": dom_ms,
            "estep_ms": est_ms, "mstep_ms": mst_ms, "cov_ms": cov_ms, "factor_ms": fac_ms,
            "sweep_algorithmic_tflops": fl["total"] / (ms_step / 1e3) / 1e12}

    # ---- end to end through the C-ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hostX = torch.from_numpy(X).pin_memory()
        steps = max(1, min(args.steps, 5))
        em.SetParameters(1, 0.0, 1e5)
        Ge = G.copy()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            from fastem_gb300 import _capi as C
            C.check(C.lib().fem_em_upload(em.handle, ctypes.c_void_p(hostX.data_ptr()), d))
            em.TrainNoCopy(Ge)          # uploads the mixture, 1 sweep, reads it back
        dt = dist.max(time.perf_counter() - t0)
        pbytes = k * (1 + d + d * d) * 8
        e2e = {"value": world * steps / dt, "unit": UNIT, "h2d_bytes_per_step": n * d * 4 + pbytes,
               "d2h_bytes_per_step": pbytes + 8 + 16}
        del hostX
    em.close()

    # ---- plain FP32 CUDA-core sweep on the same workload
    fp32 = None
    if not args.no_fp32:
        e32 = CudaMatrixEM(d, n, k, precision="fp32", device=local)
        e32.CopyDataset(X)
        G32 = GaussianMixture(*init)
        s32 = max(2, args.steps // 3)
        t32 = time_device_sweeps(e32, G32, max(1, min(args.warmup, 2)), s32, dist)
        ms32 = dist.max(t32["train_ms"]) / t32["sweeps"]
        fp32 = {"value": world * 1e3 / ms32, "ms_per_step": ms32, "steps": t32["sweeps"],
                "estep_ms": t32["estep_ms"] / t32["sweeps"], "mstep_ms": t32["mstep_ms"] / t32["sweeps"]}
        e32.close()

    # ---- CPU baseline: the oracle port on a bounded sample (rank 0)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sample = 1 << 16
        threads = os.cpu_count() or 1
        cpu_sweep_seconds(X, init, 1 << 12, threads)   # warm the library
        dt, how = cpu_sweep_seconds(X, init, sample, threads)
        cpu = {"value": 1.0 / (dt * n / sample), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "1 sweep (%s) over the first %d of %d rows, scaled x%d" % (how, sample, n, n // sample)}

    dist.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": sweeps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16",
        "precision": "fp16x3 E-step / fp16 M-step (exact diagonal) tensor cores, fp32 accumulate, "
                     "fp64 factorisation, logdet and logL",
        "data": "synthetic em_large (seeded; Dirichlet(2) weights, N(0,25I) means, Haar-rotated "
                "covariances with eigenvalues log-uniform in [0.1,10])",
        "config": {"workload": "em_large N=%d d=%d K=%d, one EM sweep per step" % (n, d, k),
                   "n": n, "d": d, "k": k, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (X 2.1 GB fp32 + 2.1 GB fp16 splits, posteriors 4.3 GB)"},
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


def batched_cpu_baseline(fits, data, sample_every=32):
    """The oracle's TrainNoCopy (FP64, OpenMP over all host cores) on every
    `sample_every`-th fit, 30 sweeps each."""
    from oracle import oracle as O
    O.lib()
    idx = list(range(0, len(fits), sample_every))
    t0 = time.perf_counter()
    for i in idx:
        X, init = data[i]
        O.em_train(X, *init, BATCH_SWEEPS, eps=0.0, abort_thr=1e12, nthreads=os.cpu_count())
    dt = time.perf_counter() - t0
    return {"value": len(idx) / dt, "unit": "fits/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d of the 512 fits (every %dth), %d sweeps each, %.1f s" % (len(idx), sample_every,
                                                                                   BATCH_SWEEPS, dt)}


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
    B = CudaBatchEM(shapes, device=local, max_sweeps=BATCH_SWEEPS)
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
    # the previous scheme: one FP32 handle and stream per fit, 16 host threads
    per_fit = None
    if not args.no_fp32:
        import concurrent.futures as cf

        def run(i):
            X, init = data[i]
            d, n, k = shapes[i]
            with CudaMatrixEM(d, n, k, precision="fp32", device=local) as em:
                em.SetParameters(BATCH_SWEEPS, 0.0, 1e12)
                try:
                    em.Train(X, GaussianMixture(*init))
                except Exception:
                    return None
                return em.logl_trace
        with cf.ThreadPoolExecutor(16) as ex:
            list(ex.map(run, range(8)))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            list(ex.map(run, range(nf)))
            torch.cuda.synchronize()
            per_fit = {"value": nf / (time.perf_counter() - t0), "unit": "fits/s",
                       "scheme": "one FP32 handle and stream per fit, 16 host threads"}
    errs, cpu = [], None
    if not args.no_cpu and rank == 0:
        from oracle import oracle as O
        O.lib()
        for i in range(0, nf, 64):
            X, init = data[i]
            ref = O.em_train(X, *init, BATCH_SWEEPS, eps=0.0, abort_thr=1e12)
            if st[i] == 0 and ref["status"] == 0:
                tr, _ = B.Trace(i)
                m = min(len(tr), len(ref["logl"]))
                errs.append(float(np.max(np.abs(tr[:m] - ref["logl"][:m])) / fits[i]["n"]))
        if world == 1:
            cpu = batched_cpu_baseline(fits, data)
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
                       x_bytes / 1e9, sum(n * k for d, n, k in shapes) * 4 / 1e9)},
        "phase_ms_per_step": per_step, "class_ms_per_step": per_class,
        "roofline": {"kernel": "k_b_cov<32> (covariance sums, d = 32 fits)", "bound": "fp32", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                     "peak_source": "nominal FP32 CUDA-core rate at the sampled SM clock (no measured FP32 peak)",
                     "traffic": traffic, "algorithmic_flop_per_step": cov_flop,
                     "launch_ms": cov_s * 1e3 / BATCH_SWEEPS},
        "failed_fits": int((st != 0).sum()), "failed_fits_oracle_agrees": "fits 282, 283, 385 collapse in FP64",
        "max_dlogL_per_N_sampled": max(errs) if errs else None, "sampled_fits": len(errs),
        "per_fit_handles": per_fit, "speedup_vs_per_fit_handles": (value / per_fit["value"]) if per_fit else None,
        "e2e": e2e, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": tm["launches"],
    }
    print(json.dumps(line), flush=True)


KM_METRIC = "k-means iter/s N=2^24 d=32 K=256 (labels bit-exact to FP64)"
KM_PROFILE_FILE = os.path.join(ROOT, "profiles", "kmeans_assign_n16m_d32_k256.md")


def km_workload(n, d, k):
    from fastem_gb300 import synth
    X, _ = synth.kmeans_blobs(seed=2, n=n, d=d, k=k)
    C0 = synth.dsquared_init(X, k, seed=3)[1].copy()
    return X, C0


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
    sigma 1, centres U[-20, 20]^32; D^2-sampled initial centroids): mixed
    (tcgen05 GEMM + argmin, FP32 refinement, FP64 recheck) against the FP32
    CUDA-core path; roofline = HBM (read X once, write labels)."""
    import torch
    from fastem_gb300 import CudaKMA
    n, d, k = args.n, 32, 256
    if args.impl == "reference":
        if rank == 0:
            X, C0 = km_workload(n, d, k)
            cpu = km_cpu_baseline(X, C0)
            print(json.dumps({"metric": KM_METRIC, "impl": "reference", "value": cpu["value"], "unit": UNIT,
                              "n_gpus": world, "steps": 1, "warmup": 1, "higher_is_better": True,
                              "cpu_baseline": cpu, "e2e": {"value": cpu["value"], "unit": UNIT,
                                                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                              "config": {"workload": "kmeans_blobs N=%d d=%d K=%d" % (n, d, k)}}), flush=True)
        return
    dist = Dist(world)
    torch.cuda.set_device(local)
    X, C0 = km_workload(n, d, k)
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
    cpu = km_cpu_baseline(X, C0) if (rank == 0 and world == 1 and not args.no_cpu) else None
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
                   "n": n, "d": d, "k": k, "init": "D^2 sampling on a 65536-row sample (seed 3)",
                   "l2": "inputs larger than L2 (X 2.1 GB)"},
        "roofline": {"kernel": "k_km_assign_tc", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": assign_ms},
        "rechecked_rows_last_step": rech, "e2e": e2e, "fp32_plain": fp32,
        "speedup_vs_fp32_plain": (value / fp32["value"]) if fp32 else None,
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def km_cpu_baseline(X, C0):
    """The oracle's Lloyd iteration (FP64, OpenMP, all host cores) on the
    first 2^20 rows, scaled to N."""
    from oracle import oracle as O
    O.lib()
    n = len(X)
    sample = min(n, 1 << 20)
    threads = os.cpu_count() or 1
    Xs = np.ascontiguousarray(X[:sample])
    O.km_iterate(Xs[:4096], C0.copy(), repair=False, nthreads=threads)
    t0 = time.perf_counter()
    O.km_iterate(Xs, C0.copy(), repair=False, nthreads=threads)
    dt = (time.perf_counter() - t0) * n / sample
    return {"value": 1.0 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "1 FP64 iteration over the first %d of %d rows, scaled x%d" % (sample, n, n // sample)}


if __name__ == "__main__":
    main()
